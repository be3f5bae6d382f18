"""The polar-filter rows (tap counts and normalised Gaussian weights of the
big, small1 and small2 filters on full and half latitudes) against an
independent restatement of filter_types_mod.F90:31-147 and exp_two_values
(math_mod.F90:146-159):

  width w = a cfl / max_cfl (c (tanh(90 - |lat_deg|) - 1) + 1),
            cfl = max_wave_speed dt / dx (dx = de_lon on full rows without
            the poles, le_lat on half rows), taps ceiling(w) + 2 made odd;
  small1:   width d w, taps int(d n) made odd;
  small2:   width e2 w, taps int(e2 n) made odd, e2 = exp_two_values(e, d,
            lat0, 80, |lat_deg|), lat0 = -full_lat_deg(2) (full rows) or
            -half_lat_deg(1) (half rows);
  weights   exp(-x^2 / (2 s^2)) / (s sqrt(2 pi)), s = b width / 2,
            x = i - (n+1)/2, normalised by their sum.

Tap counts must agree exactly, weights to a few ulps (both sides evaluate
exp and tanh through the C library; measured: bit for bit)."""
import math

import numpy as np
import pytest

from oracle import Oracle

from helpers import baroclinic_config, swm_config

BIG, SMALL1, SMALL2 = 0, 1, 2


def gaussian(width, n, b):
    s = b * width / 2.0
    # Fortran s**2 is s*s (Python's float ** goes through pow)
    w = [math.exp(-float((i - (n + 1) // 2) ** 2) / (2 * (s * s))) / (s * math.sqrt(2 * math.pi))
         for i in range(1, n + 1)]
    total = 0.0
    for x in w:
        total += x
    return np.array([x / total for x in w])


def exp_two_values(v1, v2, x0, x1, x):
    d, c = x - x0, x1 - x0
    w = math.exp(d * d * math.log(1.0e-3) / (c * c))
    return w * v1 + (1 - w) * v2


def expected_rows(cfg, o, which, lat):
    """[(taps, weights or None)] per row, restated from the reference."""
    nrow = cfg.nlat - 1 if lat else cfg.nlat
    dx_all = o.metric("le_lat" if lat else "de_lon", nrow)
    deg = o.metric("half_lat_deg" if lat else "full_lat_deg", nrow)
    lat0 = -(o.metric("half_lat_deg", cfg.nlat - 1)[0] if lat else o.metric("full_lat_deg", cfg.nlat)[1])
    rows = []
    for j in range(1, nrow + 1):
        dx = dx_all[j - 1]
        if (not lat and (j == 1 or j == nrow)) or not dx > 0 or cfg.max_wave_speed <= 0:
            rows.append((0, None))
            continue
        cfl = cfg.max_wave_speed * cfg.dt_dyn / dx
        w = cfg.filter_coef_a * cfl / cfg.max_cfl * (cfg.filter_coef_c * (math.tanh(90 - abs(deg[j - 1])) - 1) + 1)
        n = math.ceil(w) + 2
        if n % 2 == 0:
            n += 1
        if which != BIG and n > 1:
            f = cfg.filter_coef_d if which == SMALL1 else exp_two_values(cfg.filter_coef_e, cfg.filter_coef_d, lat0,
                                                                            80.0, abs(deg[j - 1]))
            n = int(f * n)
            if n % 2 == 0:
                n += 1
            w = f * w
        rows.append((n, gaussian(w, n, cfg.filter_coef_b) if n > 1 or which != BIG else None))
    return rows


CONFIGS = {
    "swm_1deg_dt60": lambda: swm_config(nlon=360, nlat=180, dt=60.0),
    "baroclinic_2deg_dt600": lambda: baroclinic_config(nlon=180, nlat=90, nlev=26, dt=600.0),
    # the 0.5 degree headline grid (the filters depend on the horizontal grid,
    # dt and the design wave speed only, so a one-level model carries them)
    "grid_0.5deg_dt180": lambda: swm_config(nlon=720, nlat=360, dt=180.0, max_wave_speed=400.0),
}


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_filter_rows_match_restatement(name):
    cfg = CONFIGS[name]()
    o = Oracle(cfg)
    try:
        for which in (BIG, SMALL1, SMALL2):
            for lat in (0, 1):
                taps = o.filter_taps(which, lat)
                for j, (n, want) in enumerate(expected_rows(cfg, o, which, lat), start=1):
                    assert taps[j - 1] == n, (name, which, lat, j, taps[j - 1], n)
                    if want is None or n == 0:
                        continue
                    got = o.filter_weights(which, lat, j)
                    err = np.abs(got - want).max() / want.max()
                    assert err <= 8 * np.finfo(float).eps, (name, which, lat, j, err)
                    assert abs(got.sum() - 1.0) < 1e-14
    finally:
        o.close()
