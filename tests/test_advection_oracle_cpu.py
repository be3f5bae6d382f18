"""Known-answer checks of the oracle's flux-form semi-Lagrangian transport
(ffsl_calc_tracer_hflx_cell, src/dynamics/adv/ffsl_mod.F90) with the
reference's own advection tests, one 12-day period each, m = 1 and
mfx = u, mfy = v, u set on non-pole rows only:

* solid-body rotation of a cosine bell over the poles
  (src/tests/adv/solid_rotation_test_mod.F90): bell height h0 = 1000 and
  radius R0 = a/3 centred at (3 pi/2, 0), rotation axis tilted by
  alpha = 90 degrees (solid_rotation_test_mod.F90:16-20, 43-58, 83-101), and
  the background tracer q0 = 1 (:38, 48);
* the reversing deformational flow of case 2 (src/tests/adv/deform_test_mod.F90):
  hills centred at (5 pi/6, 0) and (7 pi/6, 0) (:42-45), the Gaussian hills
  0.95 exp(-5 |x - x_i|^2) (:113-125) and the cosine hills of radius a/2 on a
  0.1 background (:74-88), winds
  u = k sin^2(lon) sin(2 lat) cos(pi t / T), v = k sin(2 lon) cos(lat) cos(pi t / T),
  k = 10 a / T (:169-207), taken at mid-step.  The flow returns every tracer
  to its initial position at t = T, so the initial field is the exact answer.

With m = 1 the tracer update is the flux divergence of the FFSL face fluxes,
with the pole cells closed by the ring sums of the meridional fluxes.  The
norms are those of the reference's error tool (normalised against the
initial field).  The checks: totals conserved to round-off, no new extrema
beyond round-off and the small undershoots of the split 2-D scheme, the
background kept to the analytic wind's discrete divergence, and the error
falling as the grid is refined."""
import numpy as np
import pytest

from cases import H0, deformational_flow, solid_rotation


@pytest.fixture(scope="module")
def rotation_runs():
    return {res: solid_rotation(*args) for res, args in ((5.0, (72, 37, 3600.0)), (2.5, (144, 73, 1800.0)))}


@pytest.fixture(scope="module")
def deform_runs():
    return {res: deformational_flow(*args) for res, args in ((5.0, (72, 37, 3600.0)), (3.75, (96, 49, 2400.0)))}


@pytest.mark.parametrize("res", [5.0, 2.5])
def test_solid_rotation_conserves_and_stays_monotone(rotation_runs, res):
    tr, q, q0 = rotation_runs[res]
    bell, background = q
    assert tr.mass_change(bell, q0[0]) < 1e-12
    assert bell.min() > -1e-10 * H0
    assert bell.max() <= H0 * (1 + 1e-12)
    assert np.abs(background - 1).max() < 1e-3


def test_solid_rotation_error_converges(rotation_runs):
    e = {res: tr.l2(q[0], q0[0]) for res, (tr, q, q0) in rotation_runs.items()}
    # measured: 0.327 at 5 degrees, 0.077 at 2.5 degrees
    assert e[2.5] < 0.1
    assert e[2.5] < 0.35 * e[5.0]


@pytest.mark.parametrize("res", [5.0, 3.75])
def test_deformational_flow_conserves_and_stays_bounded(deform_runs, res):
    tr, q, q0 = deform_runs[res]
    gauss, cosine = q
    assert tr.mass_change(gauss, q0[0]) < 1e-13
    assert tr.mass_change(cosine, q0[1]) < 1e-13
    assert gauss.min() >= 0.0 and gauss.max() <= q0[0].max()
    # cosine hills on a 0.1 background: undershoots of the split 2-D
    # scheme stay below 1e-4 (measured 6e-6 at 5 degrees)
    assert cosine.min() > 0.1 - 1e-4 and cosine.max() <= 1.0


def test_deformational_flow_error_converges(deform_runs):
    e = {res: tr.l2(q[0], q0[0]) for res, (tr, q, q0) in deform_runs.items()}
    # Gaussian hills, measured: 0.246 at 5 degrees, 0.164 at 3.75 degrees
    assert e[3.75] < 0.2
    assert e[3.75] < 0.8 * e[5.0]
