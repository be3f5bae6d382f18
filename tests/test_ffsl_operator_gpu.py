"""The FFSL horizontal-flux operator entry point (gmc_ffsl_hflx) against the
oracle's ffsl_calc_tracer_hflx_cell on seeded inputs."""
import numpy as np
import pytest

from gmcore_gb300 import Model
from oracle import Oracle

from helpers import baroclinic_config, rel_err

pytestmark = pytest.mark.gpu


def ffsl_inputs(cfg, seed, hx):
    rng = np.random.default_rng(seed)
    full = (cfg.nlev, cfg.nlat, cfg.nlon)
    half = (cfg.nlev, cfg.nlat - 1, cfg.nlon)
    f = {
        "q": rng.uniform(0.5, 1.5, full),
        "u": rng.normal(0.0, 20.0, full),
        "v": rng.normal(0.0, 10.0, half),
        "cflx": rng.uniform(-min(hx, 3.0), min(hx, 3.0), full),
        "cfly": rng.uniform(-0.9, 0.9, half),
        "divx": rng.normal(0.0, 1e-5, full),
        "divy": rng.normal(0.0, 1e-5, full),
    }
    f["mfx"] = 5000.0 * f["u"]
    f["mfy"] = 5000.0 * f["v"]
    return f


def device_call(model, f, dt):
    import torch
    dev = {k: torch.tensor(v, dtype=torch.float64, device="cuda") for k, v in f.items()}
    qmfx = torch.zeros_like(dev["q"])
    qmfy = torch.zeros_like(dev["v"])
    torch.cuda.synchronize()
    ptrs = {k: t.data_ptr() for k, t in dev.items()}
    ptrs.update(qmfx=qmfx.data_ptr(), qmfy=qmfy.data_ptr())
    model.ffsl_hflx(ptrs, dt)
    return qmfx.cpu().numpy(), qmfy.cpu().numpy()


def test_ffsl_hflx_operator_matches_oracle():
    pytest.importorskip("torch")
    cfg = baroclinic_config()
    model = Model(cfg)
    orc = Oracle(cfg)
    f = ffsl_inputs(cfg, 3, model.lon_halo_width)
    gx, gy = device_call(model, f, 120.0)
    ox, oy = orc.ffsl_hflx(f["q"], f["u"], f["v"], f["mfx"], f["mfy"], f["cflx"], f["cfly"], f["divx"], f["divy"], 120.0)
    inner = slice(1, cfg.nlat - 1)   # x fluxes exist on rows without the poles
    ex = rel_err(gx[:, inner], ox[:, inner])
    ey = rel_err(gy, oy)
    print("ffsl operator", ex, ey)
    assert ex <= 1e-12 and ey <= 1e-12, (ex, ey)
