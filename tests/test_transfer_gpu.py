"""Host transfers through registered (page-locked, mapped) host ranges
(gmc_host_register): the device-side gather / scatter with FP64 <-> FP32
conversion must give the same values as the host-staged path, for plain
arrays, for views with halos, and for views only partly inside a registered
range (which fall back to the staged path)."""
import ctypes as C

import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi

from helpers import baroclinic_config, initial_state

pytestmark = pytest.mark.gpu

FIELDS = ("u_lon", "v_lat", "pt", "phs")


def paged(x):
    a = g.page_aligned(np.shape(x))
    a[...] = x
    return a


def halo_view(cfg, name, h):
    """Array with an h-wide halo in i and j around the interior and its view."""
    shape = g.field_shape(cfg, name)
    nk = shape[0] if len(shape) == 3 else 1
    nj, ni = shape[-2], shape[-1]
    a = g.page_aligned((nk, nj + 2 * h, ni + 2 * h))
    a[...] = -7.0
    v = abi.View()
    v.data = a.ctypes.data_as(C.POINTER(C.c_double))
    v.lb[0], v.lb[1], v.lb[2] = 1 - h, 1 - h, 1
    v.ub[0], v.ub[1], v.ub[2] = ni + h, nj + h, nk
    return a, v


@pytest.mark.parametrize("precision", [abi.PREC_MIXED, abi.PREC_FP64])
def test_registered_matches_staged(precision):
    cfg = baroclinic_config(ntracer=2, precision=precision)
    st = initial_state(cfg, 5)
    res = {}
    for reg in (False, True):
        arrs = {f: paged(st[f]) for f in FIELDS}
        qs = [paged(st["q"][l]) for l in range(2)]
        outs = {f: g.page_aligned(arrs[f].shape) for f in FIELDS}
        qouts = [g.page_aligned(q.shape) for q in qs]
        pinned = list(arrs.values()) + qs + list(outs.values()) + qouts
        if reg:
            for a in pinned:
                g.host_register(a)
        try:
            m = g.Model(cfg)
            for f in FIELDS:
                m.set_field(f, arrs[f])
            for l in range(2):
                m.set_tracer(l, qs[l])
            m.prepare()
            m.step(3)
            for f in FIELDS:
                m.get_field(f, out=outs[f])
            for l in range(2):
                m.get_tracer(l, out=qouts[l])
            m.close()
        finally:
            if reg:
                for a in pinned:
                    g.host_unregister(a)
        res[reg] = ({f: outs[f].copy() for f in FIELDS}, [q.copy() for q in qouts])
    for f in FIELDS:
        assert np.array_equal(res[False][0][f], res[True][0][f]), f
    for l in range(2):
        assert np.array_equal(res[False][1][l], res[True][1][l]), l


def test_registered_halo_views_and_partial_ranges():
    cfg = baroclinic_config(precision=abi.PREC_MIXED)
    st = initial_state(cfg, 9)
    m = g.Model(cfg)
    m.set_state(st)
    h = 2
    for name in ("u_lon", "v_lat", "phs"):
        ref = m.get_field(name)
        # whole halo'd array registered: device scatter writes the interior only
        a, v = halo_view(cfg, name, h)
        g.host_register(a)
        try:
            assert m.lib.gmc_get_field(m.h, 0, name.encode(), C.byref(v)) == 0
        finally:
            g.host_unregister(a)
        assert np.array_equal(a[:, h:-h, h:-h].reshape(ref.shape), ref), name
        assert np.all(a[:, :h, :] == -7.0) and np.all(a[:, :, :h] == -7.0), name
        assert np.all(a[:, -h:, :] == -7.0) and np.all(a[:, :, -h:] == -7.0), name
        # upload through the registered halo view, read back through a plain array
        a2, v2 = halo_view(cfg, name, h)
        a2[:, h:-h, h:-h] = (ref * 0.5).reshape(a2[:, h:-h, h:-h].shape)
        g.host_register(a2)
        try:
            assert m.lib.gmc_set_field(m.h, 0, name.encode(), C.byref(v2)) == 0
        finally:
            g.host_unregister(a2)
        assert np.array_equal(m.get_field(name), ref * 0.5), name
        m.set_field(name, ref)
    # only the first half of the array registered: the staged path serves it
    ref = m.get_field("pt")
    out = g.page_aligned(ref.shape)
    half = out.reshape(-1)[: out.size // 2]
    g.host_register(half)
    try:
        m.get_field("pt", out=out)
    finally:
        g.host_unregister(half)
    assert np.array_equal(out, ref)
    m.close()


def test_register_rejects_overlap_and_unknown():
    a = g.page_aligned((65536,))
    g.host_register(a)
    try:
        with pytest.raises(g.GmcError):
            g.host_register(a[100:200])
    finally:
        g.host_unregister(a)
    with pytest.raises(g.GmcError):
        g.host_unregister(a)
