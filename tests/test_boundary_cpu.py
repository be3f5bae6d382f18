"""The drop-in boundary as code, checked without a GPU: every function the
C header declares is bound, under its own name, by the Fortran
iso_c_binding module include/gmcore_gpu_mod.F90 and exported by the library;
the C host program tests/c_driver/step_driver.c compiles warning-free with
gcc against the header and links to the library; the Fortran module's
derived types list the C structures' fields in order.  Where a Fortran
compiler is installed, the module itself is compiled."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gmcore_gpu.h")
MODULE = os.path.join(ROOT, "include", "gmcore_gpu_mod.F90")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gmc_[a-z0-9_]+)\s*\(", text)))


def test_every_header_function_is_bound_in_fortran():
    mod = open(MODULE).read().lower()
    bound = set(re.findall(r"bind\(c,\s*name='(gmc_[a-z0-9_]+)'\)", mod))
    missing = [f for f in header_functions() if f not in bound]
    assert not missing, missing


def test_every_header_function_is_exported():
    from gmcore_gb300 import load
    lib = load()
    for f in header_functions():
        assert hasattr(lib, f), f


def _c_struct_fields(name):
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", text, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        for piece in re.sub(r"\[.*?\]", "", decl).split(","):
            fields.append(re.findall(r"[A-Za-z_]\w*", piece)[-1])   # the declarator's name
    return fields


def _f_type_fields(name):
    mod = open(MODULE).read()
    body = re.search(r"type, bind\(c\) :: " + name + r"\n(.*?)end type " + name, mod, flags=re.S).group(1)
    fields = []
    for line in body.splitlines():
        if "::" in line:
            for n in line.split("::")[1].split(","):
                fields.append(re.sub(r"\(.*\)", "", n.strip()))
    return fields


@pytest.mark.parametrize("name", ["gmc_config", "gmc_diag", "gmc_view", "gmc_ffsl_fields", "gmc_stats"])
def test_fortran_types_match_c_structs(name):
    assert [f.lower() for f in _c_struct_fields(name)] == [f.lower() for f in _f_type_fields(name)]


def test_c_driver_compiles_and_links(tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from c_driver_build import build
    exe = build(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.skipif(shutil.which("gfortran") is None, reason="no Fortran compiler installed")
def test_fortran_module_compiles(tmp_path):
    r = subprocess.run(["gfortran", "-std=f2008", "-c", MODULE, "-J", str(tmp_path), "-o",
                        str(tmp_path / "gmcore_gpu_mod.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
