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


def run_layout(cfg, states, nsteps, layout, fields):
    m = g.Model(cfg)
    m.set_member_layout(layout)
    for mem, st in enumerate(states):
        m.set_state(st, member=mem)
    m.prepare()
    m.step(nsteps)
    out = [{f: m.get_field(f, member=mem) for f in fields} for mem in range(len(states))]
    for mem in range(len(states)):
        out[mem]["q0"] = m.get_tracer(0, member=mem)
    st = m.stats()
    m.close()
    return out, st


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_every_member_layout_matches_single_runs(precision):
    """Per-member launches on streams (layout 0) and member-batched launches
    in 1 or 2 groups (grid z = member) compute the same thing: each member
    equals its single run bit for bit, under every layout and under the
    autotuner, which settles on one of them within its first steps."""
    base = baroclinic_config(ntracer=1, precision=precision)
    states = [initial_state(base, seed=s) for s in (21, 22, 23, 24)]
    cfg = baroclinic_config(ntracer=1, precision=precision, n_members=4)
    fields = ("u_lon", "v_lat", "pt", "phs")
    singles = [run(base, [st], 6, True, fields)[0] for st in states]
    for layout in (0, 1, 2):
        ens, st = run_layout(cfg, states, 6, layout, fields)
        assert st["member_layout"] == layout and st["layout_tuned"]
        for mem in range(4):
            for f in singles[mem]:
                assert np.array_equal(ens[mem][f], singles[mem][f]), (layout, mem, f)
    ens, st = run_layout(cfg, states, 30, -1, fields)   # autotuned over 30 steps
    assert st["layout_tuned"] and st["member_layout"] in (0, 1, 2)
    ref = [run(base, [s], 30, True, fields)[0] for s in states]
    for mem in range(4):
        for f in ref[mem]:
            assert np.array_equal(ens[mem][f], ref[mem][f]), ("tuned", mem, f)


@pytest.mark.gpu
def test_member_layout_refuses_what_the_context_cannot_run():
    cfg = baroclinic_config(n_members=2)
    m = g.Model(cfg)
    for bad in (2, 4, 3):   # groups of one member are layout 0; 3 is not a layout
        with pytest.raises(g.GmcError) as e:
            m.set_member_layout(bad)
        assert e.value.code == abi.GMC_EINVAL
    m.set_member_layout(1)
    m.set_member_layout(0)
    m.set_member_layout(-1)
    m.close()
