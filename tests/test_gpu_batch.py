"""Launch-shape independence, graph-captured runs and the autotuner.

The sweep's result is defined by the schedule, not by how tiles are dealt
out: every tile variant must give the same lattice and tables as the
oracle, a graph-captured run must equal a plain run of the same MCS, and
cpm_autotune must leave the state exactly as it found it."""
import numpy as np
import pytest

import oracle
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu


def _engine(w, seed=0, stream=0):
    import gpucpm
    s = w.lattice.shape
    nx, ny, nz = (s[1], s[0], 1) if w.ndim == 2 else (s[2], s[1], s[0])
    e = gpucpm.create_box(nx, ny, nz, w.ndim, w.ncells, w.temperature)
    e.lattice(0)[...] = w.lattice.view(np.int32)
    w.apply(e, replica=0)
    e.set_seed(seed, stream)
    e.push_to_gpu()
    return e


def _state(e):
    e.synchronize()
    e.pull_from_gpu()
    a, p, c = e.tables(0)
    return e.lattice(0).copy(), a, p, c, e.counters(), e.tick


@pytest.mark.parametrize("shape,ncells", [((70, 66), 50), ((13, 14, 15), 25)])
@pytest.mark.parametrize("variant", [0, 1, 2])
def test_every_tile_variant_matches_oracle(engine_lib, shape, ncells, variant):
    w = W.random_small(shape, ncells, seed=5 + variant, temperature=8.0)
    e = _engine(w, seed=99)
    e.set_variant(variant)
    assert e.sweep_config()["variant"] == variant
    mcs = 6 if len(shape) == 2 else 3
    e.run_mcs(mcs)
    lat, a, p, c, cnt, _ = _state(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=99).run(mcs)
    np.testing.assert_array_equal(lat.view(np.uint32), sim.lattice)
    np.testing.assert_array_equal(a, sim.area)
    np.testing.assert_array_equal(p, sim.perim)
    np.testing.assert_array_equal(c, sim.csum)
    assert cnt["accepted"] == int(sim.counters[2])


def test_graph_run_equals_plain_run(engine_lib):
    w = W.random_small((64, 48), 40, seed=17, temperature=9.0)
    a = _engine(w, seed=3)
    a.run_mcs(4)
    a.run_mcs(4)
    a.run_mcs(4)
    b = _engine(w, seed=3)
    b.run_graph(4)
    b.run_graph(4)
    b.run_graph(4)
    sa, sb = _state(a), _state(b)
    for x, y in zip(sa[:4], sb[:4]):
        np.testing.assert_array_equal(x, y)
    assert sa[4] == sb[4] and sa[5] == sb[5] == 12
    # mixing plain and graph runs keeps the Monte Carlo time consistent
    c = _engine(w, seed=3)
    c.run_graph(4)
    c.run_mcs(4)
    c.run_graph(4)
    sc = _state(c)
    np.testing.assert_array_equal(sa[0], sc[0])
    assert sc[5] == 12


def test_graph_run_on_a_batch(engine_lib):
    import gpucpm
    ws = [W.random_small(s, 30, seed=40 + i, temperature=7.0 + i)
          for i, s in enumerate([(40, 44), (64, 64), (33, 70)])]
    b = gpucpm.Batch(2, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(8, 100)
    b.push_to_gpu()
    b.run_graph(5)
    b.run_graph(5)
    b.synchronize()
    b.pull_from_gpu()
    for r, w in enumerate(ws):
        sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=8,
                               stream=100 + r).run(10)
        np.testing.assert_array_equal(b.lattice(r).view(np.uint32), sim.lattice)


def test_autotune_leaves_state_unchanged(engine_lib):
    w = W.random_small((96, 96), 80, seed=23, temperature=10.0)
    e = _engine(w, seed=5)
    e.run_mcs(3)
    before = _state(e)
    variant, ms = e.autotune(probe_mcs=2)
    assert variant in (0, 1, 2) and ms > 0
    after = _state(e)
    for x, y in zip(before[:4], after[:4]):
        np.testing.assert_array_equal(x, y)
    assert before[4] == after[4] and before[5] == after[5]
    e.run_mcs(4)
    lat = _state(e)[0]
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=5).run(7)
    np.testing.assert_array_equal(lat.view(np.uint32), sim.lattice)
