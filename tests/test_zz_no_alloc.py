"""gmc_ffsl_hflx_noalloc: the FFSL flux entry point for callers that cannot
allocate device memory during the call (a host model that reserved all device
memory for its own pool, or a time-critical loop that must not wait on an
allocation).  It must give the same fluxes as gmc_ffsl_hflx, call after call,
while its scratch lives in the library's fixed device array; it must not
allocate (the device's default memory pool and its free memory stay as they
were); grids that do not fit that array are refused.  Kept in its own file so
that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from gmcore_gb300 import GmcError, Model, abi

from helpers import baroclinic_config, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the tolerance of the FP64 parity tests


def inputs(cfg, seed, hx):
    rng = np.random.default_rng(seed)
    full = (cfg.nlev, cfg.nlat, cfg.nlon)
    half = (cfg.nlev, cfg.nlat - 1, cfg.nlon)
    f = {"q": rng.uniform(0.5, 1.5, full), "u": rng.normal(0.0, 20.0, full), "v": rng.normal(0.0, 10.0, half),
         "cflx": rng.uniform(-min(hx, 3.0), min(hx, 3.0), full), "cfly": rng.uniform(-0.9, 0.9, half),
         "divx": rng.normal(0.0, 1e-5, full), "divy": rng.normal(0.0, 1e-5, full)}
    f["mfx"] = 5000.0 * f["u"]
    f["mfy"] = 5000.0 * f["v"]
    return f


def on_device(f, dtype):
    import torch
    dev = {k: torch.tensor(v, dtype=dtype, device="cuda") for k, v in f.items()}
    out = {"qmfx": torch.zeros_like(dev["q"]), "qmfy": torch.zeros_like(dev["v"])}
    torch.cuda.synchronize()
    ptrs = {k: t.data_ptr() for k, t in dev.items()}
    ptrs.update({k: t.data_ptr() for k, t in out.items()})
    return dev, out, ptrs


class DevicePool:
    """The current device's default memory pool (the one cudaMallocAsync
    draws from) and the device's free memory, read through the CUDA driver
    API: the used-memory high-water mark can be reset and read back."""

    USED_MEM_HIGH = 8   # CU_MEMPOOL_ATTR_USED_MEM_HIGH

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        assert self.cu.cuInit(0) == 0
        ctx = C.c_void_p()
        assert self.cu.cuCtxGetCurrent(C.byref(ctx)) == 0 and ctx.value, "no current CUDA context"
        dev = C.c_int()
        assert self.cu.cuCtxGetDevice(C.byref(dev)) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def reset_high(self):
        zero = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, C.byref(zero)) == 0

    def used_high(self):
        v = C.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, self.USED_MEM_HIGH, C.byref(v)) == 0
        return v.value

    def free_bytes(self):
        free, total = C.c_size_t(), C.c_size_t()
        assert self.cu.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
        return free.value


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_noalloc_matches_allocating_entry_point_twice(precision):
    torch = pytest.importorskip("torch")
    cfg = baroclinic_config(precision=precision)
    dtype = torch.float64 if precision == abi.PREC_FP64 else torch.float32
    model = Model(cfg)
    hx = model.lon_halo_width
    for call, seed in enumerate((11, 12)):   # two calls in a row, different inputs
        f = inputs(cfg, seed, hx)
        _, ref_out, ref_ptrs = on_device(f, dtype)
        model.ffsl_hflx(ref_ptrs, 120.0)
        _, na_out, na_ptrs = on_device(f, dtype)
        model.ffsl_hflx_noalloc(na_ptrs, 120.0)
        inner = slice(1, cfg.nlat - 1)
        ex = rel_err(na_out["qmfx"].double().cpu().numpy()[:, inner], ref_out["qmfx"].double().cpu().numpy()[:, inner])
        ey = rel_err(na_out["qmfy"].double().cpu().numpy(), ref_out["qmfy"].double().cpu().numpy())
        assert ex <= TOL and ey <= TOL, (call, ex, ey)
    model.close()


def test_noalloc_allocates_nothing():
    torch = pytest.importorskip("torch")
    cfg = baroclinic_config(precision=abi.PREC_FP64)
    model = Model(cfg)
    f = inputs(cfg, 13, model.lon_halo_width)
    _, out, ptrs = on_device(f, torch.float64)
    model.ffsl_hflx_noalloc(ptrs, 120.0)   # first call on the device: looks up the scratch address
    pool = DevicePool()
    # the allocating entry point draws its scratch from the default pool ...
    pool.reset_high()
    model.ffsl_hflx(ptrs, 120.0)
    assert pool.used_high() >= 2 * cfg.nlon * cfg.nlat * cfg.nlev * 8
    # ... the no-allocation one leaves it and the device's free memory alone
    torch.cuda.synchronize()
    pool.reset_high()
    free0 = pool.free_bytes()
    for _ in range(2):
        model.ffsl_hflx_noalloc(ptrs, 120.0)
    assert pool.used_high() == 0
    assert pool.free_bytes() == free0
    model.close()


def test_noalloc_refuses_grids_beyond_its_scratch():
    pytest.importorskip("torch")
    # 360 x 180 x 64 FP64 needs 2 x 4,147,200 x 8 bytes = 66 MB > 32 MiB
    cfg = baroclinic_config(nlon=360, nlat=180, nlev=64, dt=60.0)
    model = Model(cfg)
    fields = {k: 0 for k in ("q", "u", "v", "mfx", "mfy", "cflx", "cfly", "divx", "divy", "qmfx", "qmfy")}
    with pytest.raises(GmcError) as e:
        model.ffsl_hflx_noalloc(fields, 60.0)
    assert e.value.code == abi.GMC_EINVAL
    assert "scratch" in str(e.value)
    model.close()
