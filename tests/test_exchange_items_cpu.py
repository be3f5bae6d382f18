"""Host logic of Model.step_io without a GPU: the item arrays of an exchange
are built once per set of arrays and reused while those arrays live, rebuilt
for other arrays, and never reused for a new array that took a dead one's
id; the items carry each field's name and bounds and each tracer's index."""
import gc

import numpy as np

import gmcore_gb300 as g


class FakeLib:
    def __init__(self):
        self.calls = []

    def gmc_step_io(self, h, member, ain, n_in, nsteps, aout, n_out):
        self.calls.append((ain, n_in, nsteps, aout, n_out))
        return 0


def fake_model():
    m = g.Model.__new__(g.Model)
    m.lib, m.h, m._io_cache = FakeLib(), None, {}
    return m


def test_items_are_cached_per_array_set():
    m = fake_model()
    u, phs, q = np.zeros((4, 5, 8)), np.zeros((5, 8)), np.zeros((2, 4, 5, 8))
    items = [("u_lon", u), ("phs", phs), (1, q[1])]
    m.step_io(items, 1, items)
    m.step_io(items, 2, items)
    (a1, n1, s1, o1, _), (a2, _, s2, _, _) = m.lib.calls
    assert a1 is a2 and (s1, s2) == (1, 2) and n1 == 3
    assert a1[0].name == b"u_lon" and a1[0].tracer == -1 and tuple(a1[0].view.ub) == (8, 5, 4)
    assert tuple(a1[1].view.ub) == (8, 5, 1)                 # a 2-D field has one level
    assert a1[2].name is None and a1[2].tracer == 1
    # other arrays: new items
    v = np.zeros((4, 5, 8))
    m.step_io([("u_lon", v)], 1, [])
    assert m.lib.calls[-1][0] is not a1
    assert m.lib.calls[-1][0][0].view.data[0] == 0.0


def test_a_dead_arrays_id_is_not_reused():
    m = fake_model()
    a = np.zeros((4, 5, 8))
    m.step_io([("pt", a)], 1, [])
    first = m.lib.calls[-1][0]
    key_id = id(a)
    del a
    gc.collect()
    # allocate until an array takes the dead one's id (or give up: nothing to check)
    for _ in range(1000):
        b = np.full((4, 5, 8), 7.0)
        if id(b) == key_id:
            m.step_io([("pt", b)], 1, [])
            items = m.lib.calls[-1][0]
            assert items is not first
            assert items[0].view.data[0] == 7.0
            return
        del b


def test_cache_is_bounded():
    m = fake_model()
    keep = [np.zeros((2, 3, 8)) for _ in range(20)]
    for a in keep:
        m.step_io([("pt", a)], 1, [])
    assert len(m._io_cache) <= 8
