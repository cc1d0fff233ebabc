"""Persistence (3D): the preferred-direction energy term
(src/kernels3d.cu:327-343) and the per-run direction update
(src/cpm.cu:486-510, src/kernels.cu:159-212).

Bit-exact against the CPU oracle: lattice, tables, counters, the preferred
directions and the mean-coordinate ring after every run call, for single
engines, batches in both dispatch modes, graph runs and checkpoint resume;
and a behavioural check that a strongly persistent cell travels."""
import numpy as np
import pytest

import oracle
from gpucpm import workloads as W
from test_gpu_parity import assert_same, finish, make_engine

pytestmark = pytest.mark.gpu


def _with_persistence(w, lam, diff, history):
    w.persist_lambda = np.asarray(lam, np.float32)
    w.persist_diff = np.asarray(diff, np.float32)
    w.history = history
    return w


def _assert_persistence_state(e, sim, replica=0):
    pd, hist = e.persistence_state(replica)
    np.testing.assert_array_equal(pd, sim.prefdir)
    np.testing.assert_array_equal(hist, np.roll(sim.hist, -sim.hist_slot, axis=0))


@pytest.mark.parametrize("shape,history", [((14, 12, 10), 1), ((13, 15, 11), 3),
                                           ((12, 12, 12), 2)])
def test_persistence_matches_oracle(engine_lib, shape, history):
    w = _with_persistence(W.random_small(shape, 18, ntypes=2, seed=140 + history,
                                         temperature=8.0),
                          [0.0, 9.0, -5.0], [0.0, 0.6, 0.2], history)
    e = make_engine(w, seed=4, stream=2)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=4, stream=2)
    moved = False
    for k in (3, 1, 4, 2, 3):
        e.run_mcs(k)
        sim.run(k)
        finish(e)
        assert_same(e, sim)
        _assert_persistence_state(e, sim)
        moved = moved or (np.abs(sim.hist[0] - sim.hist[-1]).max() > 0)
    if history > 1:
        assert moved


@pytest.mark.parametrize("dispatch", ["grid", "replica"])
def test_persistence_batch(engine_lib, dispatch):
    import gpucpm
    ws = [_with_persistence(W.random_small((12 + 2 * i, 11, 10 + i), 14, ntypes=2,
                                           seed=150 + i, temperature=7.0),
                            [0.0, 6.0 + 2 * i, 4.0], [0.0, 0.5, 0.3 * i], 2)
          for i in range(3)]
    b = gpucpm.Batch(3, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(11, 5)
    b.set_dispatch(gpucpm.DISPATCH_GRID if dispatch == "grid" else gpucpm.DISPATCH_REPLICA)
    b.push_to_gpu()
    sims = [oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=11, stream=5 + r)
            for r, w in enumerate(ws)]
    for k in (2, 3, 2):
        b.run_mcs(k)
        for s in sims:
            s.run(k)
    finish(b)
    for r, s in enumerate(sims):
        np.testing.assert_array_equal(b.lattice(r).view(np.uint32), s.lattice)
        area, perim, cs = b.tables(r)
        np.testing.assert_array_equal(area, s.area)
        np.testing.assert_array_equal(cs, s.csum)
        _assert_persistence_state(b, s, r)


def test_persistence_graph_runs(engine_lib):
    import torch

    import gpucpm
    w = _with_persistence(W.random_small((12, 13, 11), 16, ntypes=2, seed=160,
                                         temperature=8.0), [0.0, 8.0, 8.0], [0.0, 0.4, 0.4], 3)
    e = make_engine(w, seed=2)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=2)
    for _ in range(4):
        e.run_graph(2)
        sim.run(2)
    finish(e)
    assert_same(e, sim)
    _assert_persistence_state(e, sim)
    spec = gpucpm.ScoreSpec.make(((1, 1),))
    sc = torch.zeros((1, 2, gpucpm.SCORE_MAX), device="cuda")
    with pytest.raises(gpucpm.CpmError, match="2D"):  # scores: 2D engines only
        e.run_scores(2, sc.data_ptr(), 0, 2, spec)


def test_checkpoint_resume_with_persistence_and_act(engine_lib, tmp_path):
    from gpucpm import checkpoint
    w = _with_persistence(W.random_small((12, 11, 13), 16, ntypes=2, seed=170,
                                         temperature=8.0), [0.0, 7.0, 5.0], [0.0, 0.5, 0.1], 3)
    w.act_lambda = np.array([0.0, 20.0, 0.0], np.float32)
    w.act_max = np.array([0, 12, 0], np.int32)
    a = make_engine(w, seed=21, stream=3)
    a.run_mcs(3)
    a.run_mcs(2)
    path = tmp_path / "p.npz"
    checkpoint.save(a, path)
    a.run_mcs(2)
    a.run_mcs(3)
    finish(a)
    want_pd = a.persistence_state(0)
    want_act = a.act_lattice(0).copy()

    w2 = W.random_small((12, 11, 13), 16, ntypes=2, seed=999, temperature=1.0)
    b = make_engine(w2, seed=0)
    checkpoint.load(b, path)
    b.run_mcs(2)
    b.run_mcs(3)
    finish(b)
    np.testing.assert_array_equal(b.lattice(0), a.lattice(0))
    for x, y in zip(b.tables(0), a.tables(0)):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(b.act_lattice(0), want_act)
    for x, y in zip(b.persistence_state(0), want_pd):
        np.testing.assert_array_equal(x, y)


def _ball_cell(n=32, r2=16):
    z, y, x = np.mgrid[:n, :n, :n]
    lat = np.zeros((n, n, n), np.uint32)
    ball = (x - n // 2) ** 2 + (y - n // 2) ** 2 + (z - n // 2) ** 2 <= r2
    lat[ball] = 1 | (1 << 24)
    return lat, int(ball.sum())


def test_set_constraints_persistence_moves_a_cell(engine_lib):
    """The reference's keywords (src/python_wrapper.cpp:93-97) and history
    argument; one direction update per inner_iterations chunk.  A single
    cell with lambda 30 travels about 14 sites in 200 MCS (about 0.5
    without persistence), and the run equals the oracle's bit for bit."""
    import gpucpm
    from test_gpu_api import _run_kw
    lat, vol = _ball_cell()
    out = {}
    for lam in (0.0, 30.0):
        sim = gpucpm.Cpm(32, 3, 1, 8, False, 3, 0)
        sim.get_state()[...] = lat.view(np.int32)
        sim.set_constraints(cell_type=1, lambda_area=2, target_area=vol)
        sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=8)
        sim.set_constraints(cell_type=1, lambda_persistence=lam, persistence_diffusion=0.8,
                            persistence_time=5)
        sim.set_seed(1)
        sim.push_to_gpu()
        sim.run(**_run_kw(200, tpb=4, ppt=8, ppc=4) | {"inner_iterations": 10})
        sim.synchronize()
        sim.pull_from_gpu()
        area, _, cs = sim.tables()
        c = cs[1] / area[1]
        d = (c - 16.0 + 16.0) % 32.0 - 16.0  # displacement from the start, nearest image
        out[lam] = float(np.linalg.norm(d))
        if lam:
            J = np.zeros((2, 2), np.float32)
            J[0, 1] = J[1, 0] = 8.0
            ref = oracle.OracleSim(lat, 1, J, [0, 2.0], [0, vol], temperature=8.0,
                                   persist_lambda=[0, lam], persist_diff=[0, 0.8],
                                   history=3, seed=1)
            for _ in range(20):
                ref.run(10)
            np.testing.assert_array_equal(sim.get_state().view(np.uint32), ref.lattice)
            np.testing.assert_array_equal(sim.persistence_state()[0], ref.prefdir)
            assert sim.get_params(0).persistence_time[1] == 5
    assert out[30.0] > 8.0 and out[0.0] < 3.0, out
