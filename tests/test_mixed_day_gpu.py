"""One simulated day of the 0.5 degree L32 baroclinic core with 4 tracers:
the mixed FP32/FP64 form against the FP64 form (itself held to the FP64
oracle by the parity tests) on the same seeded initial state.

Target stated for the mixed form: surface-pressure RMS difference
<= 0.05 hPa after one day (480 steps of 180 s); total mass drift of the mixed
form within 1e-8 relative (the FP64 form conserves it to round-off).
"""
import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi

STEPS = 480
PS_RMS_HPA = 0.05


def day_config(precision):
    return abi.default_config(nlon=720, nlat=360, nlev=32, baroclinic=1, dt_dyn=180.0,
                              vert_coord_template=abi.VCOORD_WRF_L32, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, ntracer=4, precision=precision)


@pytest.mark.gpu
@pytest.mark.slow
def test_mixed_form_one_day_surface_pressure():
    st = g.make_ic(day_config(abi.PREC_MIXED), 2, 20240601, 1.0)
    out = {}
    mass = {}
    for prec in (abi.PREC_MIXED, abi.PREC_FP64):
        m = g.Model(day_config(prec))
        m.set_state(st)
        m.prepare()
        tm0 = m.diagnose()["tm"]
        m.step(STEPS)
        mass[prec] = (tm0, m.diagnose()["tm"])
        out[prec] = {name: m.get_field(name) for name in ("phs", "u_lon", "v_lat", "pt")}
        m.close()
    d = out[abi.PREC_MIXED]["phs"] - out[abi.PREC_FP64]["phs"]
    rms_hpa = float(np.sqrt(np.mean(d * d))) / 100.0
    print(f"one day: ps RMS {rms_hpa:.3e} hPa, max {float(np.max(np.abs(d))) / 100.0:.3e} hPa; "
          f"mass drift mixed {abs(mass[abi.PREC_MIXED][1] / mass[abi.PREC_MIXED][0] - 1):.2e}, "
          f"fp64 {abs(mass[abi.PREC_FP64][1] / mass[abi.PREC_FP64][0] - 1):.2e}")
    assert np.all(np.isfinite(out[abi.PREC_MIXED]["phs"]))
    assert rms_hpa <= PS_RMS_HPA, f"ps RMS after one day {rms_hpa:.4g} hPa"
    for name in ("u_lon", "v_lat", "pt"):
        e = out[abi.PREC_MIXED][name] - out[abi.PREC_FP64][name]
        assert float(np.sqrt(np.mean(e * e))) < 0.5, name
    tm0, tm1 = mass[abi.PREC_MIXED]
    assert abs(tm1 - tm0) / tm0 < 1e-8
    tm0, tm1 = mass[abi.PREC_FP64]
    assert abs(tm1 - tm0) / tm0 < 1e-12
