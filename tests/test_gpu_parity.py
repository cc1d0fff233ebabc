"""Bit-exact parity of the CUDA sweep with the CPU oracle.

Every test runs the same seeded input through libgpucpm_gb300.so (via the C-ABI)
and through oracle/cpm_oracle.cpp, then requires the lattice, the cell tables
(area, perimeter, exact centroid sums) and the evaluated / accepted counters
to be identical.  Integer and index results admit no tolerance; the FP32 dH
and Metropolis test are specified to the operation, so the accept decisions
must agree exactly as well."""
import numpy as np
import pytest

import oracle
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu


def make_engine(w, seed=0, stream=0):
    import gpucpm
    shape = w.lattice.shape
    if w.ndim == 2:
        e = gpucpm.create_box(shape[1], shape[0], 1, 2, w.ncells, w.temperature)
    else:
        e = gpucpm.create_box(shape[2], shape[1], shape[0], 3, w.ncells, w.temperature)
    e.lattice(0)[...] = w.lattice.view(np.int32)
    w.apply(e, replica=0)
    e.set_seed(seed, stream)
    e.push_to_gpu()
    return e


def finish(e):
    e.synchronize()
    e.pull_from_gpu()
    return e


def assert_same(e, sim, replica=0):
    lat = e.lattice(replica).view(np.uint32)
    assert lat.shape == sim.lattice.shape
    mism = np.argwhere(lat != sim.lattice)
    assert mism.size == 0, f"{len(mism)} sites differ, first at {mism[:5].tolist()}"
    area, perim, cs = e.tables(replica)
    np.testing.assert_array_equal(area, sim.area)
    np.testing.assert_array_equal(perim, sim.perim)
    np.testing.assert_array_equal(cs, sim.csum)
    c = e.counters(replica)
    assert c["attempts"] == int(sim.counters[0])
    assert c["evaluated"] == int(sim.counters[1])
    assert c["accepted"] == int(sim.counters[2])


CASES = [
    ("2d_even_perim", (64, 64), 40, True, 8.0, 25),
    ("2d_odd_box", (37, 41), 30, True, 6.0, 30),
    ("2d_odd_both", (33, 35), 20, False, 12.0, 30),
    ("2d_no_perim", (96, 64), 60, False, 10.0, 20),
    ("2d_cold", (48, 48), 30, True, 0.0, 15),
    ("3d_even", (16, 16, 16), 20, True, 10.0, 6),
    ("3d_odd", (9, 13, 11), 16, True, 7.0, 8),
]


@pytest.mark.parametrize("name,shape,ncells,perim,T,mcs", CASES,
                         ids=[c[0] for c in CASES])
def test_sweep_matches_oracle(engine_lib, name, shape, ncells, perim, T, mcs):
    w = W.random_small(shape, ncells, seed=sum(name.encode()) % 1000, temperature=T,
                       perim=perim)
    e = make_engine(w, seed=12345, stream=3)
    e.run_mcs(mcs)
    finish(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=12345,
                           stream=3).run(mcs)
    assert sim.counters[2] > 0
    assert_same(e, sim)


def test_sorting_2d_full_config(engine_lib):
    """200x200 Graner-Glazier sorting, 1000 MCS, Philox seed 0."""
    w = W.sorting_2d()
    e = make_engine(w, seed=0)
    e.run_mcs(w.mcs)
    finish(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=0).run(w.mcs)
    assert_same(e, sim)


def test_chunked_runs_equal_one_run_and_tick_resume(engine_lib):
    w = W.random_small((40, 44), 25, seed=21, temperature=9.0)
    a = make_engine(w, seed=5)
    a.run_mcs(12)
    finish(a)
    b = make_engine(w, seed=5)
    b.run_mcs(7)
    b.run_mcs(5)
    finish(b)
    np.testing.assert_array_equal(a.lattice(0), b.lattice(0))
    # resume: new engine from b's state after 7 MCS, tick set to 7
    c = make_engine(w, seed=5)
    c.run_mcs(7)
    finish(c)
    d = make_engine(W.Workload(**{**w.__dict__, "lattice": c.lattice(0).view(np.uint32).copy()}),
                    seed=5)
    d.tick = 7
    d.run_mcs(5)
    finish(d)
    np.testing.assert_array_equal(a.lattice(0), d.lattice(0))


def test_batch_matches_oracle_and_single_engines(engine_lib):
    import gpucpm
    shapes = [(37, 41), (64, 64), (33, 50), (96, 80), (5, 7), (128, 31)]
    ws = []
    for r, (ny, nx) in enumerate(shapes):
        w = W.random_small((ny, nx), max(1, nx * ny // 60), seed=100 + r,
                           temperature=4.0 + 3 * r, perim=r % 2 == 0)
        ws.append(w)
    b = gpucpm.Batch(2, [(w.lattice.shape[1], w.lattice.shape[0]) for w in ws],
                     [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(77, 10)
    b.push_to_gpu()
    b.run_mcs(9)
    finish(b)
    for r, w in enumerate(ws):
        sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=77,
                               stream=10 + r).run(9)
        assert_same(b, sim, replica=r)
        single = make_engine(w, seed=77, stream=10 + r)
        single.run_mcs(9)
        finish(single)
        np.testing.assert_array_equal(single.lattice(0), b.lattice(r))


def test_batch_3d(engine_lib):
    import gpucpm
    shapes = [(9, 10, 11), (16, 12, 8), (7, 7, 7)]
    ws = [W.random_small(s, 12 + 3 * r, seed=200 + r, temperature=9.0)
          for r, s in enumerate(shapes)]
    b = gpucpm.Batch(3, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(3, 0)
    b.push_to_gpu()
    b.run_mcs(5)
    finish(b)
    for r, w in enumerate(ws):
        sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=3,
                               stream=r).run(5)
        assert_same(b, sim, replica=r)


def test_reference_api_path_matches_oracle(engine_lib):
    """gpucpm.Cpm driven exactly like the reference's examples."""
    import gpucpm
    sim = gpucpm.Cpm(64, 2, 10, 20, False)
    sim.add_cell(1, 10, 10)
    sim.add_cell(1, 40, 40)
    sim.add_cell(1, 40, 10)
    sim.set_constraints(cell_type=1, lambda_area=10, target_area=200)
    sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=10)
    lat0 = sim.get_state().view(np.uint32).copy()
    sim.push_to_gpu()
    sim.run(cell_sync=0, block_sync=0, global_sync=1, threads_per_block=4,
            positions_per_thread=8, positions_per_checkerboard=4,
            updates_per_checkerboard_switch=1, updates_per_barrier=1,
            iterations=200, inner_iterations=200)
    sim.synchronize()
    sim.pull_from_gpu()
    J = np.zeros((2, 2), np.float32)
    J[0, 1] = J[1, 0] = 10
    ref = oracle.OracleSim(lat0, 10, J, [0, 10], [0, 200], temperature=20.0).run(200)
    np.testing.assert_array_equal(sim.get_state().view(np.uint32), ref.lattice)
    cen = sim.get_centroids()
    assert cen.shape == (3, 2)
    area = ref.area[1:4]
    want = ref.csum[1:4] / area[:, None]
    want -= 64 * np.floor(want / 64)
    np.testing.assert_allclose(cen, want, rtol=0, atol=1e-12)
