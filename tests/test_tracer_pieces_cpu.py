"""The oracle's tracer-step pieces against a separate restatement of adv_run's
negative fixers and the zonal smoother, on seeded fields built to reach every
branch:

* the zonal fixer (adv_mod.F90:236-258): sequential in i over each row; a
  negative cell takes half its deficit from each neighbour when both can
  give it, else from the left or the right neighbour by the reference's own
  formula (q(i-1) = (qm1 - qm0) / m), and is set to zero; at the row ends
  the neighbour is the longitude halo, so what is written there is dropped
  when the halo is refilled;
* the vertical fixer (:275-297): the same along each column, with no
  neighbour above the top or below the bottom level, and a neighbour
  written only if its mass is positive;
* three passes of the order-2 zonal smoother (lon_damp_1d, lon_damp_mod.F90:
  158-241): f = wgt (f + (f(i-1) - 2 f + f(i+1)) / 4) + (1 - wgt) f on the
  rows where the weight is non-zero, each pass from the previous one.

A cell whose neighbours cannot cover it is the reference's 'Negative
tracer!' error, which the oracle reports as GMC_ENEGTRACER."""
import numpy as np
import pytest

from gmcore_gb300 import abi
from oracle import Oracle

from helpers import baroclinic_config

ZONAL, VERTICAL, SMOOTH = 0, 1, 2


def zonal_fixer(q, m, hits, halo=None):
    """halo: the (i = 0, i = nlon + 1) columns of q as last filled, if not
    the wrap of q itself."""
    nlon = q.shape[-1]
    wrap = lambda a: np.concatenate([a[..., -1:], a, a[..., :1]], axis=-1)   # halo cells 0 and nlon+1
    P, M = wrap(q), wrap(m)
    if halo is not None:
        P[..., 0], P[..., -1] = halo
    for i in range(1, nlon + 1):
        neg = P[..., i] < 0
        qm0 = P[..., i] * M[..., i]
        qm1 = P[..., i - 1] * M[..., i - 1]
        qm2 = P[..., i + 1] * M[..., i + 1]
        half = 0.5 * qm0
        both = neg & (qm1 >= half) & (qm2 >= half)
        left = neg & ~both & (qm1 > qm0)
        right = neg & ~both & ~left & (qm2 > qm0)
        hits["both"] += int(both.sum()); hits["left"] += int(left.sum()); hits["right"] += int(right.sum())
        hits["ends"] += int((neg & ((i == 1) | (i == nlon))).sum())
        P[..., i - 1] = np.where(both, (qm1 - half) / M[..., i - 1], np.where(left, (qm1 - qm0) / M[..., i - 1],
                                                                             P[..., i - 1]))
        P[..., i + 1] = np.where(both, (qm2 - half) / M[..., i + 1], np.where(right, (qm2 - qm0) / M[..., i + 1],
                                                                             P[..., i + 1]))
        P[..., i] = np.where(neg, 0.0, P[..., i])
    return P[..., 1:-1]


def vertical_fixer(q, m, hits):
    q = q.copy()
    nlev = q.shape[0]
    for k in range(nlev):
        neg = q[k] < 0
        qm0 = q[k] * m[k]
        qm1 = q[k - 1] * m[k - 1] if k > 0 else np.zeros_like(qm0)
        qm2 = q[k + 1] * m[k + 1] if k < nlev - 1 else np.zeros_like(qm0)
        half = 0.5 * qm0
        both = neg & (qm1 >= half) & (qm2 >= half)
        left = neg & ~both & (qm1 > qm0)
        right = neg & ~both & ~left & (qm2 > qm0)
        hits["both"] += int(both.sum()); hits["left"] += int(left.sum()); hits["right"] += int(right.sum())
        hits["ends"] += int((neg & ((k == 0) | (k == nlev - 1))).sum())
        if k > 0:
            q[k - 1] = np.where(both & (qm1 > 0), (qm1 - half) / m[k - 1],
                                np.where(left & (qm1 > 0), (qm1 - qm0) / m[k - 1], q[k - 1]))
        if k < nlev - 1:
            q[k + 1] = np.where(both & (qm2 > 0), (qm2 - half) / m[k + 1],
                                np.where(right & (qm2 > 0), (qm2 - qm0) / m[k + 1], q[k + 1]))
        q[k] = np.where(neg, 0.0, q[k])
    return q


def zonal_smoother(q, wgt):
    f = q.copy()
    rows = [j for j in range(1, q.shape[1] - 1) if wgt[j] != 0]
    for _ in range(3):
        g = f.copy()
        for j in rows:
            x = f[:, j]
            g[:, j] = wgt[j] * (x + 0.25 * (np.roll(x, 1, -1) - 2.0 * x + np.roll(x, -1, -1))) + (1 - wgt[j]) * x
        f = g
    return f


def fields(cfg, seed):
    """Positive seeded tracer and layer masses with negative cells placed to
    reach every branch: isolated cells, a cell before a deeper one (borrow
    from the left), row ends with a deep cell across the wrap (borrow from the
    right), and the same along columns."""
    rng = np.random.default_rng(seed)
    shape = (cfg.nlev, cfg.nlat, cfg.nlon)
    q = 1.0 + 0.3 * rng.random(shape)
    m = 400.0 + 300.0 * rng.random(shape)
    q[rng.random(shape) < 0.04] *= -0.3
    k, j, i = (rng.integers(0, n, 60) for n in (cfg.nlev, cfg.nlat, cfg.nlon - 3))
    i = i + 1
    q[k, j, i], q[k, j, i + 1] = -0.1, -2.0                    # left borrow at i, then both at i + 1
    rows = rng.integers(0, cfg.nlat, 8)
    q[:, rows, 0], q[:, rows, 1], q[:, rows, -1] = -0.1, 1.0, -2.0   # right borrow at i = 1
    kk = rng.integers(1, cfg.nlev - 2, 40)
    jj, ii = rng.integers(0, cfg.nlat, 40), rng.integers(2, cfg.nlon - 2, 40)
    q[kk, jj, ii], q[kk + 1, jj, ii] = -0.1, -2.0              # column pairs
    q[0, 3, 5], q[-1, 4, 6] = -0.2, -0.3                       # top and bottom cells
    return q, m


@pytest.fixture(scope="module")
def oracle_5deg():
    cfg = baroclinic_config()
    o = Oracle(cfg)
    yield cfg, o
    o.close()


@pytest.mark.parametrize("seed", [1, 2])
def test_zonal_fixer_matches_restatement(oracle_5deg, seed):
    cfg, o = oracle_5deg
    q, m = fields(cfg, seed)
    hits = dict(both=0, left=0, right=0, ends=0)
    want = zonal_fixer(q, m, hits)
    got, rc = o.tracer_piece(ZONAL, q, m)
    assert rc == 0
    assert all(v > 0 for v in hits.values()), hits
    assert np.array_equal(got, want)
    assert got.min() >= 0.0


@pytest.mark.parametrize("seed", [1, 2])
def test_vertical_fixer_matches_restatement(oracle_5deg, seed):
    cfg, o = oracle_5deg
    q, m = fields(cfg, seed)
    hits = dict(both=0, left=0, right=0, ends=0)
    want = vertical_fixer(q, m, hits)
    got, rc = o.tracer_piece(VERTICAL, q, m)
    assert rc == 0
    assert hits["both"] > 0 and hits["left"] > 0 and hits["ends"] > 0, hits
    assert np.array_equal(got, want)
    assert got.min() >= 0.0


def test_uncovered_negative_cell_is_reported(oracle_5deg):
    cfg, o = oracle_5deg
    q, m = np.ones((cfg.nlev, cfg.nlat, cfg.nlon)), np.full((cfg.nlev, cfg.nlat, cfg.nlon), 500.0)
    q[0, 5, 0], q[0, 5, 1], q[0, 5, -1] = -1.0, -2.0, -3.0     # both neighbours deeper: nothing to borrow
    _, rc = o.tracer_piece(ZONAL, q, m)
    assert rc == abi.GMC_ENEGTRACER


def test_zonal_smoother_matches_restatement(oracle_5deg):
    cfg, o = oracle_5deg
    rng = np.random.default_rng(3)
    q = 1.0 + rng.random((cfg.nlev, cfg.nlat, cfg.nlon))
    wgt = o.metric("lon_damp_wgt_full", cfg.nlat)
    assert (wgt > 0).sum() >= 2
    got, rc = o.tracer_piece(SMOOTH, q, np.ones_like(q))
    assert rc == 0
    want = zonal_smoother(q, wgt)
    assert not np.array_equal(want, q)
    assert np.array_equal(got, want)


# ---------------------------------------------------------------------------
# one whole tracer step of adv_run (adv_mod.F90:152-312) from the static
# batch's fields: FFSL fluxes of q(old), the flux-form update from old_m with
# the polar rings, division by the new layer mass, the zonal fixer reading the
# longitude halo of q(new) as it was last filled, copied ghost levels, the
# vertical FFSL update, the vertical fixer and three smoother passes
# ---------------------------------------------------------------------------
def tracer_step(cfg, o, q_old, old_m, halo, m, B, dt):
    from test_operators_cpu import ffsl_fluxes, ring, prev, vertical_flux
    nlat, nlon, nlev = cfg.nlat, cfg.nlon, cfg.nlev
    row = lambda n, rows: o.metric(n, rows)[None, :, None]
    le_lon, le_lat, area = row("le_lon", nlat), row("le_lat", nlat - 1), row("area_cell", nlat)
    I = slice(1, nlat - 1)
    gx, gy = ffsl_fluxes(cfg, o, q_old, B, B["mfx"], B["mfy"], dt)
    qn = np.zeros_like(q_old)
    qn[:, I] = old_m[:, I] * q_old[:, I] - ((gx[:, I] - prev(gx[:, I])) * le_lon[:, I] +
                                             (gy[:, 1:] * le_lat[:, 1:] - gy[:, :-1] * le_lat[:, :-1])) / area[:, I] * dt
    ps = ring(gy[:, 0]) * le_lat[0, 0, 0] / nlon / area[0, 0, 0] * dt
    pn = ring(gy[:, -1]) * le_lat[0, -1, 0] / nlon / area[0, -1, 0] * dt
    qn[:, 0] = old_m[:, 0] * q_old[:, 0] - ps[:, None]
    qn[:, -1] = old_m[:, -1] * q_old[:, -1] + pn[:, None]
    qn = qn / m
    hits = dict(both=0, left=0, right=0, ends=0)
    qn = zonal_fixer(qn, m, hits, halo)
    g = np.concatenate([qn[:1], qn[:1], qn, qn[-1:], qn[-1:]])     # copied ghost levels
    flux = vertical_flux(g, B["we"], B["cflz"])
    qn = qn - ((flux[1:] - flux[:-1]) * dt) / m
    qn = vertical_fixer(qn, m, hits)
    return zonal_smoother(qn, o.metric("lon_damp_wgt_full", nlat)), hits


def test_tracer_steps_match_restatement():
    """Two advected steps (the first step does not advect); the second tracer
    starts with scattered negative cells so that both fixers act inside a
    step, and by the third step the new level's halo is stale."""
    cfg = baroclinic_config(ntracer=2)
    from helpers import initial_state, load_state
    o = Oracle(cfg)
    try:
        st = initial_state(cfg)
        rng = np.random.default_rng(11)
        q1 = st["q"][1] + 0.5
        q1[rng.random(q1.shape) < 0.01] = -0.05
        st["q"][1] = q1
        load_state(o, st)
        o.prepare()
        o.step(1)                                   # no advection at the first step
        dt = cfg.dt_adv if cfg.dt_adv > 0 else cfg.dt_dyn
        fixed = 0
        for _ in range(2):
            old_m = o.get_tracer_batch("old_m")
            before = [(o.get_tracer_level(l, 0)[..., 2:-2], o.get_tracer_level(l, 1)) for l in range(2)]
            o.step(1)
            B = {n: o.get_tracer_batch(n) for n in ("u", "v", "mfx", "mfy", "cflx", "cfly", "divx", "divy", "we", "cflz")}
            m = o.get_field("m")
            for l, (q_old, q_new_prev) in enumerate(before):
                halo = (q_new_prev[..., 1], q_new_prev[..., -2])          # i = 0 and i = nlon + 1
                want, hits = tracer_step(cfg, o, q_old, old_m, halo, m, B, dt)
                fixed += hits["both"] + hits["left"] + hits["right"]
                got = o.get_tracer(l)
                assert not np.array_equal(got, q_old), l
                err = float(np.abs(got - want).max() / np.abs(want).max())
                assert err <= 8 * np.finfo(float).eps, (l, err)
        assert fixed > 0
    finally:
        o.close()


def test_static_batch_cadence():
    """The static tracer batch with dt_adv = dt_dyn (nstep = 1,
    adv_batch_mod.F90:239-252, 389-401, 512-525): the run prologue copies the
    winds, mass fluxes, vertical mass flux and half-level mass in; each step's
    call then alternately averages the held values with the new state's
    ((held + new) / 2, refreshing the Courant numbers from the averages) and
    copies the new state's in (keeping the previous Courant numbers)."""
    from helpers import initial_state, load_state
    from test_operators_cpu import batch_courant, vertical_courant
    cfg = baroclinic_config(ntracer=1)
    dt = cfg.dt_adv if cfg.dt_adv > 0 else cfg.dt_dyn
    o = Oracle(cfg)
    pairs = (("u", "u_f"), ("v", "v_f"), ("mfx", "mfx_lon"), ("mfy", "mfy_lat"), ("we", "we_lev"),
             ("m_lev", "m_lev"))
    try:
        load_state(o, initial_state(cfg))
        o.prepare()
        for b, f in pairs[:2]:
            assert np.array_equal(o.get_tracer_batch(b), o.get_field(f)), b      # prologue copy
        for step in range(1, 5):
            held = {b: o.get_tracer_batch(b) for b in ("u", "v", "mfx", "mfy", "we", "m_lev", "cflx", "cfly", "cflz")}
            o.step(1)
            now = {b: o.get_tracer_batch(b) for b in held}
            average = step % 2 == 1
            for b, f in pairs:
                new = o.get_field(f)
                want = (held[b] + new) / 2 if average else new
                assert np.array_equal(now[b], want), (step, b)
            if average:
                for name, (w, rows) in batch_courant(cfg, o, dt, get=o.get_tracer_batch).items():
                    if name in ("cflx", "cfly"):
                        got = now[name][:, rows] if rows is not None else now[name]
                        assert np.array_equal(got, w), (step, name)
                assert np.array_equal(now["cflz"], vertical_courant(cfg, o, dt, get=o.get_tracer_batch)), step
                assert not np.array_equal(now["cflx"], held["cflx"]), step
            else:
                for name in ("cflx", "cfly", "cflz"):
                    assert np.array_equal(now[name], held[name]), (step, name)
    finally:
        o.close()
