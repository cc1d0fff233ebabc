"""Fixed cell types and stickiness (src/kernels2d.cu:280-290, 399-400;
src/kernels3d.cu:251-261, 413-414), and per-replica parameter records.

Bit-exact against the CPU oracle: a fixed target never changes, a fixed
source proposes the medium, stickiness is added to the old configuration's
adhesion only.  Batches whose replicas start from one shared parameter record
and then diverge (copy on write) must still follow each replica's own
parameters."""
import numpy as np
import pytest

import oracle
from gpucpm import workloads as W
from test_gpu_parity import assert_same, finish, make_engine

pytestmark = pytest.mark.gpu


def _with_terms(w, fixed_type, sticky, seed):
    nt = w.J.shape[0]
    g = np.random.default_rng(seed)
    w.stick = np.zeros((nt, nt), np.float32)
    for a, b in sticky:
        w.stick[a, b] = float(g.integers(1, 8))
    w.fixed = np.zeros(nt, bool)
    if fixed_type is not None:
        w.fixed[fixed_type] = True
    return w


@pytest.mark.parametrize("shape,ncells,T,mcs", [((64, 60), 40, 8.0, 20),
                                                 ((35, 33), 25, 5.0, 25),
                                                 ((14, 15, 13), 20, 8.0, 5)])
def test_fixed_and_sticky_match_oracle(engine_lib, shape, ncells, T, mcs):
    w = W.random_small(shape, ncells, ntypes=3, seed=90 + len(shape), temperature=T)
    _with_terms(w, 3, [(1, 2), (2, 1), (1, 0), (2, 3), (3, 1)], seed=4)
    lat0 = w.lattice.copy()
    e = make_engine(w, seed=12)
    e.run_mcs(mcs)
    finish(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=12).run(mcs)
    assert_same(e, sim)
    # the fixed type's sites are exactly where they were
    fixed_sites = (lat0 >> 24) == 3
    assert fixed_sites.any()
    np.testing.assert_array_equal(e.lattice(0).view(np.uint32)[fixed_sites], lat0[fixed_sites])
    assert int(sim.counters[2]) > 0


def test_replica_parameters_copy_on_write(engine_lib):
    """All replicas share one record until single replicas change; each must
    follow its own parameters under both dispatches."""
    import gpucpm
    base = [W.random_small((48, 40), 30, ntypes=3, seed=200 + i, temperature=7.0)
            for i in range(4)]
    for d in (gpucpm.DISPATCH_GRID, gpucpm.DISPATCH_REPLICA):
        b = gpucpm.Batch(2, [w.lattice.shape[::-1] for w in base], [w.ncells for w in base])
        for r, w in enumerate(base):
            b.lattice(r)[...] = w.lattice.view(np.int32)
        w0 = base[0]
        nt = w0.J.shape[0]
        # shared settings for every replica
        for a in range(nt):
            for c in range(nt):
                b.set_adhesion(None, a, c, float(w0.J[a, c]), symmetric=False)
            b.set_area(None, a, int(w0.tgt_area[a]), float(w0.lam_area[a]))
            b.set_perimeter(None, a, int(w0.tgt_perim[a]), float(w0.lam_perim[a]))
        b.set_temperature(None, 7.0)
        # then per-replica changes
        b.set_fixed(1, 3, True)
        b.set_stickiness(2, 1, 2, 4.0)
        b.set_temperature(3, 11.0)
        b.set_stickiness(None, 2, 1, 1.0)  # all replicas again
        b.set_seed(5, 50)
        b.set_dispatch(d)
        b.push_to_gpu()
        b.run_mcs(12)
        b.synchronize()
        b.pull_from_gpu()
        for r, w in enumerate(base):
            stick = np.zeros((nt, nt), np.float32)
            stick[2, 1] = 1.0
            fixed = np.zeros(nt, bool)
            T = 7.0
            if r == 1:
                fixed[3] = True
            if r == 2:
                stick[1, 2] = 4.0
            if r == 3:
                T = 11.0
            sim = oracle.OracleSim(w.lattice, w.ncells, w0.J, w0.lam_area, w0.tgt_area,
                                   w0.lam_perim, w0.tgt_perim, temperature=T, seed=5,
                                   stream=50 + r, stick=stick, fixed=fixed).run(12)
            np.testing.assert_array_equal(b.lattice(r).view(np.uint32), sim.lattice)
            area, perim, cs = b.tables(r)
            np.testing.assert_array_equal(area, sim.area)
            np.testing.assert_array_equal(cs, sim.csum)


def test_set_constraints_fixed_and_stickiness(engine_lib):
    """The reference's keywords reach the engine (src/python_wrapper.cpp:89-91,
    122-125): fixed takes effect on its own, stickiness with other_cell_type."""
    import gpucpm
    sim = gpucpm.Cpm(64, 2, 12, 10, False)
    for k in range(12):
        sim.add_cell(1 + k % 3, 5 + 5 * k, 10 + 4 * (k % 5))
    sim.set_constraints(cell_type=1, lambda_area=2, target_area=60)
    sim.set_constraints(cell_type=2, lambda_area=2, target_area=60)
    sim.set_constraints(cell_type=3, fixed=1)
    sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=12)
    sim.set_constraints(cell_type=0, other_cell_type=2, adhesion=8)
    sim.set_constraints(cell_type=1, other_cell_type=2, adhesion=6)
    sim.set_constraints(cell_type=1, other_cell_type=0, stickiness=3)
    lat0 = sim.get_state().view(np.uint32).copy()
    sim.push_to_gpu()
    sim.run(cell_sync=0, block_sync=0, global_sync=1, threads_per_block=4,
            positions_per_thread=8, positions_per_checkerboard=4,
            updates_per_checkerboard_switch=1, updates_per_barrier=1,
            iterations=100, inner_iterations=100)
    sim.synchronize()
    sim.pull_from_gpu()
    J = np.zeros((4, 4), np.float32)
    J[0, 1] = J[1, 0] = 12
    J[0, 2] = J[2, 0] = 8
    J[1, 2] = J[2, 1] = 6
    S = np.zeros((4, 4), np.float32)
    S[1, 0] = 3
    ref = oracle.OracleSim(lat0, 12, J, [0, 2, 2, 0], [0, 60, 60, 0], temperature=10.0,
                           stick=S, fixed=[False, False, False, True]).run(100)
    np.testing.assert_array_equal(sim.get_state().view(np.uint32), ref.lattice)


def _smooth_field(shape, seed):
    g = np.random.default_rng(seed)
    nd = len(shape)
    f = np.zeros((nd,) + tuple(shape))
    grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    for k in range(nd):
        for _ in range(3):
            kv = [g.integers(1, 3) * 2 * np.pi / n for n in shape]
            ph = g.uniform(0, 2 * np.pi)
            f[k] += g.uniform(0.5, 2.0) * np.sin(sum(a * x for a, x in zip(kv, grids)) + ph)
    return f


@pytest.mark.parametrize("shape,mcs", [((64, 56), 20), ((33, 37), 25), ((14, 12, 15), 5)])
def test_chemotaxis_matches_oracle(engine_lib, shape, mcs):
    """The chemotaxis term (src/kernels2d.cu:302-334, src/kernels3d.cu:
    275-324) against the oracle, bit for bit, including the 2D seam."""
    w = W.random_small(shape, 30 if len(shape) == 2 else 20, ntypes=2, seed=70 + len(shape),
                       temperature=8.0)
    w.chemo = np.array([0.0, 4.0, -2.5], np.float32)
    w.field = _smooth_field(shape, seed=3)
    e = make_engine(w, seed=21)
    e.run_mcs(mcs)
    finish(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=21).run(mcs)
    assert_same(e, sim)
    # and the term changes the dynamics
    w0 = W.random_small(shape, 30 if len(shape) == 2 else 20, ntypes=2, seed=70 + len(shape),
                        temperature=8.0)
    plain = oracle.OracleSim(w0.lattice, w0.ncells, **w0.oracle_kwargs(), seed=21).run(mcs)
    assert (plain.lattice != sim.lattice).any()


def test_chemotaxis_moves_cells_up_the_field(engine_lib):
    """A uniform field along +x with lambda > 0 drives cells toward +x."""
    import gpucpm
    drift = {}
    for lam in (0.0, 20.0):
        sim = gpucpm.Cpm(128, 2, 4, 10, True)
        for k in range(4):
            sim.add_cell(1, 40 + 12 * k, 30 + 20 * k)
        sim.set_constraints(cell_type=1, lambda_area=5, target_area=80)
        sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=10)
        sim.set_constraints(cell_type=1, lambda_chemotaxis=lam)
        f = sim.get_field()
        assert f.shape == (2, 128, 128)
        f[0] = 1.0
        sim.push_to_gpu()
        sim.run_mcs(60)
        sim.synchronize()
        c0 = sim.get_centroids()[:, 0].copy()
        sim.run_mcs(300)
        sim.synchronize()
        drift[lam] = float(np.mean(sim.get_centroids()[:, 0] - c0))
    assert drift[20.0] > drift[0.0] + 5.0, drift


def _with_act(w, lam, amax):
    w.act_lambda = np.asarray(lam, np.float32)
    w.act_max = np.asarray(amax, np.int32)
    return w


@pytest.mark.parametrize("shape,mcs", [((48, 44), 12), ((33, 35), 10), ((12, 14, 13), 4)])
def test_act_matches_oracle(engine_lib, shape, mcs):
    """The act model (src/kernels2d.cu:312-473, src/kernels3d.cu:301-470) and
    its stamps against the oracle, bit for bit: copies of act runs land after
    their phase in both."""
    w = W.random_small(shape, 24 if len(shape) == 2 else 16, ntypes=2, seed=110 + len(shape),
                       temperature=9.0)
    _with_act(w, [0.0, 30.0, 18.0], [0, 15, 10])
    e = make_engine(w, seed=8)
    e.run_mcs(mcs)
    finish(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=8).run(mcs)
    assert_same(e, sim)
    np.testing.assert_array_equal(e.act_lattice(0).view(np.uint32), sim.act)
    assert sim.act.max() == mcs - 1


def test_act_batch_replica_dispatch_and_scores_refused(engine_lib):
    import torch

    import gpucpm
    ws = [_with_act(W.random_small((40 + 4 * i, 36), 20, ntypes=2, seed=130 + i,
                                   temperature=8.0), [0.0, 20.0 + 5 * i, 10.0], [0, 12, 9])
          for i in range(3)]
    for d in (gpucpm.DISPATCH_GRID, gpucpm.DISPATCH_REPLICA):
        b = gpucpm.Batch(2, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
        for r, w in enumerate(ws):
            b.lattice(r)[...] = w.lattice.view(np.int32)
            w.apply(b, replica=r)
        b.set_seed(6, 20)
        b.set_dispatch(d)
        b.push_to_gpu()
        b.run_mcs(8)
        b.synchronize()
        b.pull_from_gpu()
        for r, w in enumerate(ws):
            sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=6,
                                   stream=20 + r).run(8)
            np.testing.assert_array_equal(b.lattice(r).view(np.uint32), sim.lattice)
            np.testing.assert_array_equal(b.act_lattice(r).view(np.uint32), sim.act)
            area, perim, cs = b.tables(r)
            np.testing.assert_array_equal(cs, sim.csum)
    spec = gpucpm.ScoreSpec.make(((1, 1),))
    sc = torch.zeros((3, 2, gpucpm.SCORE_MAX), device="cuda")
    with pytest.raises(gpucpm.CpmError, match="act"):
        b.run_scores(2, sc.data_ptr(), 0, 2, spec)


def test_set_constraints_act_and_get_act_state(engine_lib):
    """The reference's keywords (src/python_wrapper.cpp:113-115) and its
    act-state view."""
    import gpucpm
    sim = gpucpm.Cpm(64, 2, 6, 10, False, 1, 1)
    for k in range(6):
        sim.add_cell(1, 8 + 9 * k, 12 + 7 * k)
    sim.set_constraints(cell_type=1, lambda_area=5, target_area=60)
    sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=10)
    sim.set_constraints(cell_type=1, lambda_act=40, max_act=20)
    lat0 = sim.get_state().view(np.uint32).copy()
    sim.push_to_gpu()
    sim.run_mcs(30)
    sim.synchronize()
    sim.pull_from_gpu()
    st = sim.get_act_state()
    assert st.dtype == np.int32 and st.shape == (64, 64)
    J = np.zeros((2, 2), np.float32)
    J[0, 1] = J[1, 0] = 10
    ref = oracle.OracleSim(lat0, 6, J, [0, 5], [0, 60], temperature=10.0,
                           act_lambda=[0, 40], act_max=[0, 20]).run(30)
    np.testing.assert_array_equal(sim.get_state().view(np.uint32), ref.lattice)
    np.testing.assert_array_equal(st.view(np.uint32), ref.act)


def _all_terms(w, seed):
    """Every Hamiltonian term at once: fixed type 3, stickiness, chemotaxis,
    act, persistence (3D) on top of adhesion, area and perimeter."""
    nt = w.J.shape[0]
    _with_terms(w, 3 if nt > 3 else None, [(1, 2), (2, 1), (1, 0)], seed)
    w.chemo = np.array([0.0, 3.0, -2.0, 1.0][:nt], np.float32)
    w.field = _smooth_field(w.lattice.shape, seed=seed)
    _with_act(w, [0.0, 25.0, 0.0, 10.0][:nt], [0, 14, 0, 6][:nt])
    if w.ndim == 3:
        w.persist_lambda = np.array([0.0, 6.0, -4.0, 0.0][:nt], np.float32)
        w.persist_diff = np.array([0.0, 0.5, 0.2, 0.0][:nt], np.float32)
        w.history = 2
    return w


@pytest.mark.parametrize("shape", [(46, 40), (13, 12, 14)])
def test_all_terms_together_match_oracle(engine_lib, shape):
    w = _all_terms(W.random_small(shape, 26 if len(shape) == 2 else 18, ntypes=3,
                                  seed=190 + len(shape), temperature=9.0), seed=5)
    e = make_engine(w, seed=12, stream=4)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=12, stream=4)
    for k in (3, 2, 4):
        e.run_mcs(k)
        sim.run(k)
    finish(e)
    assert_same(e, sim)
    np.testing.assert_array_equal(e.act_lattice(0).view(np.uint32), sim.act)
    if len(shape) == 3:
        pd, hist = e.persistence_state(0)
        np.testing.assert_array_equal(pd, sim.prefdir)
        np.testing.assert_array_equal(hist, np.roll(sim.hist, -sim.hist_slot, axis=0))


@pytest.mark.parametrize("dims,dispatch", [(2, "grid"), (2, "replica"), (3, "grid"),
                                           (3, "replica")])
def test_all_terms_batch_matches_oracle(engine_lib, dims, dispatch):
    """Replicas with diverging records (one without act, one without
    chemotaxis) under both dispatches."""
    import gpucpm
    shapes = [(40, 36), (33, 45), (30, 30)] if dims == 2 else [(12, 11, 13), (14, 10, 12)]
    ws = [_all_terms(W.random_small(s, 18, ntypes=3, seed=200 + i, temperature=8.0 + i),
                     seed=i) for i, s in enumerate(shapes)]
    ws[0].act_lambda = None
    ws[1].chemo = None
    b = gpucpm.Batch(dims, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(3, 9)
    b.set_dispatch(gpucpm.DISPATCH_GRID if dispatch == "grid" else gpucpm.DISPATCH_REPLICA)
    b.push_to_gpu()
    sims = [oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=3, stream=9 + r)
            for r, w in enumerate(ws)]
    for k in (2, 3):
        b.run_mcs(k)
        for s in sims:
            s.run(k)
    finish(b)
    for r, s in enumerate(sims):
        np.testing.assert_array_equal(b.lattice(r).view(np.uint32), s.lattice)
        area, perim, cs = b.tables(r)
        np.testing.assert_array_equal(area, s.area)
        np.testing.assert_array_equal(perim, s.perim)
        np.testing.assert_array_equal(cs, s.csum)
        if s.act is not None:
            np.testing.assert_array_equal(b.act_lattice(r).view(np.uint32), s.act)


@pytest.mark.parametrize("dims", [2, 3])
def test_all_terms_hybrid_dispatch_matches_oracle(engine_lib, dims):
    """Hybrid dispatch (grid over the largest replicas, replica dispatch over
    whole rounds of the rest) with every term on, act's deferred copies and
    3D persistence included; more replicas than blocks."""
    import gpucpm
    n = 158 if dims == 2 else 154
    g = np.random.default_rng(11)
    shapes = [tuple(int(v) for v in g.integers(10, 18, dims)) for _ in range(n)]
    ws = [_all_terms(W.random_small(s, 6, ntypes=3, seed=600 + i, temperature=8.0), seed=i)
          for i, s in enumerate(shapes)]
    b = gpucpm.Batch(dims, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(2, 40)
    b.set_dispatch(gpucpm.DISPATCH_HYBRID)
    b.push_to_gpu()
    b.run_mcs(2)
    b.run_graph(2)
    finish(b)
    for r, w in enumerate(ws):
        s = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=2, stream=40 + r)
        s.run(2)
        s.run(2)
        np.testing.assert_array_equal(b.lattice(r).view(np.uint32), s.lattice)
        area, perim, cs = b.tables(r)
        np.testing.assert_array_equal(area, s.area)
        np.testing.assert_array_equal(cs, s.csum)
        np.testing.assert_array_equal(b.act_lattice(r).view(np.uint32), s.act)
        if dims == 3:
            pd, hist = b.persistence_state(r)
            np.testing.assert_array_equal(pd, s.prefdir)
