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
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
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
    assert variant in (0, 1, 2, 3) and ms > 0
    after = _state(e)
    for x, y in zip(before[:4], after[:4]):
        np.testing.assert_array_equal(x, y)
    assert before[4] == after[4] and before[5] == after[5]
    e.run_mcs(4)
    lat = _state(e)[0]
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=5).run(7)
    np.testing.assert_array_equal(lat.view(np.uint32), sim.lattice)


def _batch(ws, seed, stream0):
    import gpucpm
    b = gpucpm.Batch(ws[0].ndim, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(seed, stream0)
    b.push_to_gpu()
    return b


def _batch_state(b, n):
    b.synchronize()
    b.pull_from_gpu()
    return [(b.lattice(r).copy(), *b.tables(r), b.counters(r)) for r in range(n)]


@pytest.mark.parametrize("dims", [2, 3])
@pytest.mark.parametrize("variant", [0, 2, 3])
def test_replica_dispatch_matches_oracle_and_grid(engine_lib, dims, variant):
    """Blocks running whole replicas (largest first) give the same lattices,
    tables and counters as the grid dispatch and as the oracle, for ragged
    sizes including odd sides, plain and graph-captured runs."""
    import gpucpm
    shapes = ([(40, 44), (64, 64), (33, 70), (21, 19), (96, 50)] if dims == 2 else
              [(12, 13, 14), (16, 16, 16), (9, 11, 10)])
    ws = [W.random_small(s, 12 + 6 * i, seed=70 + i, temperature=6.0 + i)
          for i, s in enumerate(shapes)]
    mcs = 5 if dims == 2 else 3
    out = {}
    for d in (gpucpm.DISPATCH_GRID, gpucpm.DISPATCH_REPLICA):
        b = _batch(ws, seed=17, stream0=30)
        b.set_variant(variant)
        b.set_dispatch(d)
        cfg = b.sweep_config()
        assert cfg["dispatch"] == ("replica" if d == gpucpm.DISPATCH_REPLICA else "grid")
        b.run_mcs(mcs)
        b.run_graph(mcs)
        out[d] = _batch_state(b, len(ws))
    for r, w in enumerate(ws):
        sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=17,
                               stream=30 + r).run(2 * mcs)
        for d in out:
            lat, a, p, c, cnt = out[d][r]
            np.testing.assert_array_equal(lat.view(np.uint32), sim.lattice)
            np.testing.assert_array_equal(a, sim.area)
            np.testing.assert_array_equal(p, sim.perim)
            np.testing.assert_array_equal(c, sim.csum)
            assert cnt["accepted"] == int(sim.counters[2])


def test_replica_dispatch_scores_and_autotune(engine_lib):
    """Score launches under replica dispatch equal those under grid dispatch
    (FP32 sums, summation order differs); the autotuner over variants and
    dispatches leaves the batch state unchanged."""
    import torch

    import gpucpm
    ws = [W.sorting_2d(n=40 + 8 * i, ncells=20 + 5 * i, seed=60 + i) for i in range(4)]
    spec = gpucpm.ScoreSpec.make(((1, 1), (2, 2), (1, 2)), lambda_perim=True)
    res = {}
    for d in (gpucpm.DISPATCH_GRID, gpucpm.DISPATCH_REPLICA):
        b = _batch(ws, seed=4, stream0=0)
        b.set_dispatch(d)
        sc = torch.zeros((len(ws), 6, gpucpm.SCORE_MAX), device="cuda")
        torch.cuda.synchronize()
        b.run_scores(6, sc.data_ptr(), 0, 6, spec)
        res[d] = (_batch_state(b, len(ws)), sc.cpu().numpy())
    (sg, scg), (sr, scr) = res[gpucpm.DISPATCH_GRID], res[gpucpm.DISPATCH_REPLICA]
    for r in range(len(ws)):
        np.testing.assert_array_equal(sg[r][0], sr[r][0])
    scale = np.abs(scg).max(axis=(0, 1)) + 1e-6
    assert (np.abs(scg - scr) / scale).max() < 1e-4
    b = _batch(ws, seed=4, stream0=0)
    b.run_mcs(2)
    before = _batch_state(b, len(ws))
    variant, ms = b.autotune(probe_mcs=1)
    assert variant in (0, 1, 2, 3) and ms > 0
    after = _batch_state(b, len(ws))
    for x, y in zip(before, after):
        for u, v in zip(x[:4], y[:4]):
            np.testing.assert_array_equal(u, v)
    b.run_mcs(3)
    fin = _batch_state(b, len(ws))
    for r, w in enumerate(ws):
        sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=4,
                               stream=r).run(5)
        np.testing.assert_array_equal(fin[r][0].view(np.uint32), sim.lattice)


@pytest.mark.parametrize("dims", [2, 3])
def test_hybrid_dispatch_matches_oracle(engine_lib, dims):
    """More replicas than blocks: hybrid dispatch runs the largest ones in
    grid dispatch and whole rounds of the rest in replica dispatch (two
    launches per run, the device tick advanced once).  Lattices, tables and
    counters equal the oracle's for every replica, for plain and graph runs;
    score launches equal grid dispatch's."""
    import torch

    import gpucpm
    n = 160 if dims == 2 else 156
    g = np.random.default_rng(5)
    shapes = [tuple(int(v) for v in g.integers(10, 26, dims)) for _ in range(n)]
    ws = [W.random_small(s, 6, seed=400 + i, temperature=7.0) for i, s in enumerate(shapes)]
    b = _batch(ws, seed=21, stream0=3)
    b.set_dispatch(gpucpm.DISPATCH_HYBRID)
    assert b.sweep_config()["dispatch"] == "hybrid"
    l0 = b.kernel_launches()
    b.run_mcs(3)
    b.run_graph(2)
    b.run_graph(2)
    assert b.tick == 7
    st = _batch_state(b, n)
    assert b.kernel_launches() - l0 >= 6  # two sweep launches per run
    for r, w in enumerate(ws):
        sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=21,
                               stream=3 + r).run(7)
        lat, a, p, c, cnt = st[r]
        np.testing.assert_array_equal(lat.view(np.uint32), sim.lattice)
        np.testing.assert_array_equal(a, sim.area)
        np.testing.assert_array_equal(c, sim.csum)
        assert cnt["accepted"] == int(sim.counters[2])
    if dims == 2:
        spec = gpucpm.ScoreSpec.make(((1, 1), (1, 2)))
        res = {}
        for d in (gpucpm.DISPATCH_GRID, gpucpm.DISPATCH_HYBRID):
            bb = _batch(ws, seed=21, stream0=3)
            bb.set_dispatch(d)
            sc = torch.zeros((n, 4, gpucpm.SCORE_MAX), device="cuda")
            torch.cuda.synchronize()
            bb.run_scores(4, sc.data_ptr(), 0, 4, spec)
            res[d] = (_batch_state(bb, n), sc.cpu().numpy())
        (sg, scg), (sh, sch) = res[gpucpm.DISPATCH_GRID], res[gpucpm.DISPATCH_HYBRID]
        for r in range(n):
            np.testing.assert_array_equal(sg[r][0], sh[r][0])
        scale = np.abs(scg).max(axis=(0, 1)) + 1e-6
        assert (np.abs(scg - sch) / scale).max() < 1e-4
