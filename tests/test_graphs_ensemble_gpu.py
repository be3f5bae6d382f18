"""CUDA-graph replay of gmc_step and ensemble members on their own streams:
both change how kernels are launched, never what they compute, so the
results must equal direct launches and single-member runs bit for bit."""
import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi

from helpers import baroclinic_config, initial_state, swm_config


def run(cfg, states, nsteps, graphs, fields):
    m = g.Model(cfg)
    m.set_graphs(graphs)
    for mem, st in enumerate(states):
        m.set_state(st, member=mem)
    m.prepare()
    m.step(nsteps)
    out = [{f: m.get_field(f, member=mem) for f in fields} for mem in range(len(states))]
    if cfg.ntracer > 0:
        for mem in range(len(states)):
            out[mem]["q0"] = m.get_tracer(0, member=mem)
    m.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_graph_replay_matches_direct_launches(precision):
    cfg = baroclinic_config(ntracer=2, dt_adv=240.0, precision=precision)
    st = [initial_state(cfg)]
    fields = ("u_lon", "v_lat", "pt", "phs")
    a = run(cfg, st, 7, True, fields)[0]
    b = run(cfg, st, 7, False, fields)[0]
    for f in a:
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.gpu
def test_graph_replay_shallow_water():
    cfg = swm_config()
    st = [initial_state(cfg)]
    a = run(cfg, st, 9, True, ("u_lon", "v_lat", "gz"))[0]
    b = run(cfg, st, 9, False, ("u_lon", "v_lat", "gz"))[0]
    for f in a:
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.gpu
@pytest.mark.parametrize("graphs", [True, False])
def test_ensemble_members_match_single_runs(graphs):
    base = baroclinic_config(ntracer=1, precision=abi.PREC_MIXED)
    states = [initial_state(base, seed=s) for s in (11, 12, 13)]
    cfg = baroclinic_config(ntracer=1, precision=abi.PREC_MIXED, n_members=3)
    fields = ("u_lon", "v_lat", "pt", "phs")
    ens = run(cfg, states, 5, graphs, fields)
    for mem, st in enumerate(states):
        single = run(base, [st], 5, graphs, fields)[0]
        for f in single:
            assert np.array_equal(ens[mem][f], single[f]), (mem, f)
