"""Tangent-linear and adjoint of the shallow-water step (gmc_tlm_step,
gmc_adjoint): dot-product test between the two, tangent-linear against
centred finite differences of the model, the adjoint gradient of
J = sum (gz_n - gz_target)^2 against centred finite differences, and the
gradient through a torch.autograd.Function wrapper (test harness only).

Tolerances: dot-product test 1e-11 relative (FP64 round-off over the
steps); gradient vs finite differences 1e-6 relative (the stated target).
"""
import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi

from helpers import swm_config

FIELDS = g.TLAD_FIELDS


def c4_config():
    """1 degree shallow water, predict-correct, dt = 60 s (the C4 adjoint case)."""
    return swm_config(nlon=360, nlat=180, dt=60.0)


def initial(cfg, seed=3):
    return g.make_ic(cfg, 1, seed, 0.0)


def model_at(cfg, st, delta=None, eps=0.0):
    m = g.Model(cfg)
    s = dict(st)
    if delta is not None:
        for f in FIELDS:
            s[f] = st[f] + eps * delta[f]
    m.set_state(s)
    m.prepare()
    return m


def run(cfg, st, nsteps, delta=None, eps=0.0):
    m = model_at(cfg, st, delta, eps)
    m.step(nsteps)
    out = {f: m.get_field(f) for f in FIELDS}
    m.close()
    return out


def direction(cfg, seed, scale_u=1.0, scale_gz=50.0):
    """Smooth seeded perturbation of u, v, gz (zonal and meridional harmonics)."""
    rng = np.random.default_rng(seed)
    out = {}
    for f in FIELDS:
        shape = g.field_shape(cfg, f)
        nj, ni = shape[-2], shape[-1]
        jj, ii = np.meshgrid(np.linspace(0, np.pi, nj), np.linspace(0, 2 * np.pi, ni, endpoint=False), indexing="ij")
        a = np.zeros((nj, ni))
        for _ in range(4):
            m, n = rng.integers(1, 6), rng.integers(1, 5)
            a += rng.normal() * np.cos(m * ii + rng.uniform(0, 6.28)) * np.sin(n * jj)
        a *= scale_gz if f == "gz" else scale_u
        out[f] = a.reshape(shape)
    return out


def dot(a, b):
    return sum(float(np.sum(a[f] * b[f])) for f in FIELDS)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [abi.TIME_PC2, abi.TIME_WRFRK3, abi.TIME_EULER])
def test_dot_product_small(scheme):
    cfg = swm_config(nlon=72, nlat=37, dt=600.0, time_scheme=scheme)
    st = initial(cfg)
    n = 12
    dx = direction(cfg, 1)
    lam = direction(cfg, 2, scale_u=1e-3, scale_gz=1e-5)
    m = model_at(cfg, st)
    tl = m.tlm_step(n, dx)
    m.close()
    m = model_at(cfg, st)
    ad = m.adjoint(n, lam, ckpt_every=5)
    m.close()
    lhs, rhs = dot(tl, lam), dot(dx, ad)
    print(f"dot product scheme {scheme}: <M'dx, l> = {lhs:.15e}  <dx, M'^T l> = {rhs:.15e}")
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs))


@pytest.mark.gpu
def test_tlm_against_finite_differences():
    cfg = swm_config(nlon=72, nlat=37, dt=600.0)
    st = initial(cfg)
    n = 12
    dx = direction(cfg, 4)
    m = model_at(cfg, st)
    tl = m.tlm_step(n, dx)
    m.close()
    eps = 1e-4
    xp = run(cfg, st, n, dx, eps)
    xm = run(cfg, st, n, dx, -eps)
    for f in FIELDS:
        fd = (xp[f] - xm[f]) / (2 * eps)
        err = float(np.max(np.abs(fd - tl[f]))) / float(np.max(np.abs(tl[f])))
        print(f"TLM vs FD {f}: {err:.3e}")
        assert err < 1e-5, f


@pytest.mark.gpu
def test_tlm_state_matches_forward():
    """The tangent-linear call advances the model exactly like gmc_step."""
    cfg = swm_config(nlon=72, nlat=37, dt=600.0)
    st = initial(cfg)
    m = model_at(cfg, st)
    m.tlm_step(6, direction(cfg, 5))
    a = {f: m.get_field(f) for f in FIELDS}
    m.close()
    b = run(cfg, st, 6)
    # pole rows of u_lon are never updated (their content is whatever the
    # slot held); every field the step computes must agree bit for bit
    assert np.array_equal(a["u_lon"][..., 1:-1, :], b["u_lon"][..., 1:-1, :])
    assert np.array_equal(a["v_lat"], b["v_lat"])
    assert np.array_equal(a["gz"], b["gz"])


@pytest.mark.gpu
def test_checkpoint_interval_invariance():
    cfg = swm_config(nlon=72, nlat=37, dt=600.0)
    st = initial(cfg)
    lam = direction(cfg, 6, scale_u=1e-3, scale_gz=1e-5)
    res = []
    for k in (1, 4, 16):
        m = model_at(cfg, st)
        res.append(m.adjoint(10, lam, ckpt_every=k))
        m.close()
    for r in res[1:]:
        for f in FIELDS:
            d = float(np.max(np.abs(r[f] - res[0][f]))) / float(np.max(np.abs(res[0][f])))
            assert d < 1e-13, f


def gradient_check(cfg, nsteps, ckpt, seed):
    st = initial(cfg)
    target = st["gz"].copy()
    final = run(cfg, st, nsteps)

    def J(out):
        return float(np.sum((out["gz"] - target) ** 2))

    lam = {"u_lon": np.zeros(g.field_shape(cfg, "u_lon")), "v_lat": np.zeros(g.field_shape(cfg, "v_lat")),
           "gz": 2.0 * (final["gz"] - target)}
    m = model_at(cfg, st)
    grad = m.adjoint(nsteps, lam, ckpt_every=ckpt)
    m.close()
    d = direction(cfg, seed)
    ad = dot(grad, d)
    best = None
    for eps in (1e-3, 3e-4, 1e-4):
        fd = (J(run(cfg, st, nsteps, d, eps)) - J(run(cfg, st, nsteps, d, -eps))) / (2 * eps)
        rel = abs(fd - ad) / abs(ad)
        best = rel if best is None else min(best, rel)
        print(f"gradient {cfg.nlon}x{cfg.nlat} {nsteps} steps eps {eps:g}: adjoint {ad:.12e} fd {fd:.12e} rel {rel:.2e}")
    return best


@pytest.mark.gpu
def test_gradient_small():
    assert gradient_check(swm_config(nlon=72, nlat=37, dt=600.0), 12, 4, 7) < 1e-6


@pytest.mark.gpu
@pytest.mark.slow
def test_gradient_c4_one_degree_96_steps():
    """C4: 1 degree shallow water, 96 steps, checkpoint every 8 steps."""
    assert gradient_check(c4_config(), 96, 8, 8) < 1e-6


@pytest.mark.gpu
def test_autograd_function_wrapper():
    torch = pytest.importorskip("torch")
    cfg = swm_config(nlon=72, nlat=37, dt=600.0)
    st = initial(cfg)
    nsteps = 8
    target = torch.from_numpy(st["gz"].copy())

    class Step(torch.autograd.Function):
        """x0 (u, v, gz) -> x_n through gmc_step; backward through gmc_adjoint."""

        @staticmethod
        def forward(ctx, u, v, gz):
            s = dict(st)
            s.update(u_lon=u.detach().numpy(), v_lat=v.detach().numpy(), gz=gz.detach().numpy())
            ctx.state = s
            m = g.Model(cfg)
            m.set_state(s)
            m.prepare()
            m.step(nsteps)
            out = [torch.from_numpy(m.get_field(f)) for f in FIELDS]
            m.close()
            return tuple(out)

        @staticmethod
        def backward(ctx, gu, gv, ggz):
            m = g.Model(cfg)
            m.set_state(ctx.state)
            m.prepare()
            lam = {"u_lon": gu.numpy(), "v_lat": gv.numpy(), "gz": ggz.numpy()}
            r = m.adjoint(nsteps, lam, ckpt_every=4)
            m.close()
            return tuple(torch.from_numpy(r[f]) for f in FIELDS)

    x = [torch.tensor(st[f], dtype=torch.float64, requires_grad=True) for f in FIELDS]
    u, v, gz = Step.apply(*x)
    loss = ((gz - target) ** 2).sum()
    loss.backward()
    d = direction(cfg, 9)
    ad = sum(float((xi.grad * torch.from_numpy(d[f])).sum()) for xi, f in zip(x, FIELDS))
    eps = 3e-4
    jp = float(((torch.from_numpy(run(cfg, st, nsteps, d, eps)["gz"]) - target) ** 2).sum())
    jm = float(((torch.from_numpy(run(cfg, st, nsteps, d, -eps)["gz"]) - target) ** 2).sum())
    fd = (jp - jm) / (2 * eps)
    assert abs(fd - ad) <= 1e-6 * abs(ad)


@pytest.mark.gpu
def test_adjoint_refuses_unsupported():
    cfg = abi.default_config(nlon=72, nlat=37, nlev=26, baroclinic=1, dt_dyn=120.0,
                             vert_coord_template=abi.VCOORD_TEST_L26, max_wave_speed=400.0)
    m = g.Model(cfg)
    m.set_state(g.make_ic(cfg, 2, 1, 1.0))
    m.prepare()
    with pytest.raises(g.GmcError):
        m.adjoint(2, {"u_lon": np.zeros(g.field_shape(cfg, "u_lon")), "v_lat": np.zeros(g.field_shape(cfg, "v_lat")),
                      "gz": np.zeros((cfg.nlat, cfg.nlon))})
    m.close()
    cfg = swm_config(nlon=72, nlat=37, dt=600.0)
    m = model_at(cfg, initial(cfg))
    m.step(1)   # no longer the prepared state
    with pytest.raises(g.GmcError):
        m.tlm_step(1, direction(cfg, 1))
    m.close()
