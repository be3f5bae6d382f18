"""The hybrid-coordinate tables of the vertical templates against the
reference's own source: hyai, hybi as the literals of
src/dynamics/vert_coord/hybrid_coord_test_mod.F90 (tests/golden/
hybrid_coord_tables.json, written by tests/golden/make_hybrid_tables.py).
Literals without a kind suffix or a d exponent are default-kind (single
precision) in Fortran: the reference stores them rounded to float32 and
widened, so that is the expected value.  Then hyam, hybm as the interface
means and the eta levels full_lev = hyam + hybm, half_lev = hyai + hybi
(hybrid_coord_mod.F90:121-132), all bit for bit."""
import json
import os
from fractions import Fraction

import numpy as np
import pytest

from oracle import Oracle

from helpers import baroclinic_config

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "hybrid_coord_tables.json")) as _f:
    TABLES = json.load(_f)
NLEV = {"test_l26": 26, "wrf_l32": 32, "wrf_l64": 64}


def nearest_float32(x):
    """The float32 nearest to the rational x (ties to even)."""
    f = np.float32(float(x))
    best = None
    for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
        d = abs(Fraction(float(c)) - x)
        if best is None or d < best[0] or (d == best[0] and int(c.view(np.uint32)) % 2 == 0):
            best = (d, c)
    return best[1]


def literal_value(s):
    """Value of a Fortran real literal as the reference stores it in real(8)."""
    if s.endswith("_r8") or "d" in s.lower():
        return float(Fraction(s.removesuffix("_r8").lower().replace("d", "e")))
    return float(nearest_float32(Fraction(s)))


@pytest.mark.parametrize("template", sorted(NLEV))
def test_hybrid_tables_match_the_reference_source(template):
    nlev = NLEV[template]
    o = Oracle(baroclinic_config(nlev=nlev))
    try:
        got = {n: o.metric(n, nlev + 1) for n in ("hyai", "hybi", "half_lev")}
        got.update({n: o.metric(n, nlev) for n in ("hyam", "hybm", "full_lev")})
    finally:
        o.close()
    for name in ("hyai", "hybi"):
        want = np.array([literal_value(s) for s in TABLES[template][name]])
        assert len(want) == nlev + 1
        assert np.array_equal(got[name], want), (template, name, np.abs(got[name] - want).max())
    a, b = got["hyai"], got["hybi"]
    assert np.array_equal(got["hyam"], 0.5 * (a[:-1] + a[1:]))
    assert np.array_equal(got["hybm"], 0.5 * (b[:-1] + b[1:]))
    assert np.array_equal(got["full_lev"], got["hyam"] + got["hybm"])
    assert np.array_equal(got["half_lev"], a + b)


def test_single_precision_literals_differ_from_their_double_reading():
    # the widening matters: most table entries are not float32-exact decimals
    lits = TABLES["test_l26"]["hyai"]
    assert sum(literal_value(s) != float(s) for s in lits) > len(lits) // 2
