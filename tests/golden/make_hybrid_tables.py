"""Writes hybrid_coord_tables.json: the hybrid-coordinate coefficient tables
hyai, hybi of the vertical templates this build supports, as the literal
strings of the reference's source (src/dynamics/vert_coord/
hybrid_coord_test_mod.F90: hybrid_coord_test_l26 :78-147,
hybrid_coord_wrf_l32 :565-647, hybrid_coord_wrf_l64 :734-880).

Run once where the reference's sources are present:
    python tests/golden/make_hybrid_tables.py [path/to/GMCORE]
The tests read only the JSON."""
import json
import os
import re
import sys

TEMPLATES = {"test_l26": "hybrid_coord_test_l26", "wrf_l32": "hybrid_coord_wrf_l32",
             "wrf_l64": "hybrid_coord_wrf_l64"}
NUMBER = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][-+]?\d+)?(?:_r8)?")


def subroutine_lines(lines, name):
    start = next(i for i, ln in enumerate(lines) if re.match(rf"\s*subroutine\s+{name}\s*\(", ln))
    end = next(i for i in range(start, len(lines)) if re.match(rf"\s*end\s+subroutine\s+{name}\b", lines[i]))
    return start, end


def array_literal(lines, start, end, var):
    """Literal strings of `var = [ ... ]` inside lines[start:end], comments
    stripped."""
    body, inside = [], False
    for ln in lines[start:end]:
        code = ln.split("!", 1)[0]
        if not inside:
            m = re.match(rf"\s*{var}\s*=\s*\[(.*)", code)
            if not m:
                continue
            inside, code = True, m.group(1)
        if "]" in code:
            body.append(code.split("]", 1)[0])
            break
        body.append(code)
    return NUMBER.findall(" ".join(s.replace("&", " ") for s in body))


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.sep, "root", "reference")
    rel = os.path.join("src", "dynamics", "vert_coord", "hybrid_coord_test_mod.F90")
    with open(os.path.join(root, rel)) as f:
        lines = f.read().splitlines()
    out = {}
    for key, sub in TEMPLATES.items():
        a, b = subroutine_lines(lines, sub)
        out[key] = {"source": f"{rel}:{a + 1}-{b + 1}",
                    "hyai": array_literal(lines, a, b, "hyai"),
                    "hybi": array_literal(lines, a, b, "hybi")}
        assert len(out[key]["hyai"]) == len(out[key]["hybi"]), key
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "hybrid_coord_tables.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print({k: len(v["hyai"]) for k, v in out.items()})


if __name__ == "__main__":
    main()
