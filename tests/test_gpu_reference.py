"""Parity with the reference's own CUDA build (oracle/_ref, built from the
reference sources by oracle/ref_gpu/build.py and driven by ref_driver.cpp).

1. Table recount: the reference's calculateAreasAndCircumferences and this
   engine's push compute identical area and perimeter tables.
2. A one-thread reference run (deterministic for a given seed) equals
   tests/refmodel.py's restatement of the reference's sequential algorithm,
   bit for bit.  That restatement's dH is the one tests/test_oracle.py
   replays against the oracle, so the oracle's dH is pinned to the
   reference's outputs through it.
(Statistical parity with the reference's parallel runs is
tests/test_gpu_reference_stats.py.)
"""
import numpy as np
import pytest

import refmodel
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu

ref_gpu = pytest.importorskip("oracle.ref_gpu")
if not ref_gpu.available():
    pytest.skip("reference cubin not built (needs the reference checkout)",
                allow_module_level=True)


def _ours(w, seed=0, stream=0):
    import gpucpm
    n = w.lattice.shape[0]
    e = gpucpm.Cpm(n, w.ndim, w.ncells, w.temperature, False)
    e.get_state()[...] = w.lattice.view(np.int32)
    w.apply(e)
    e.set_seed(seed, stream)
    e.push_to_gpu()
    return e


def _ref(w):
    r = ref_gpu.RefGpu(w.lattice.shape[0], w.ndim, w.ncells, w.temperature)
    r.apply(w)
    r.push(w.lattice)
    return r


@pytest.mark.parametrize("case", ["sorting256", "tissue2d", "tissue3d"])
def test_table_recount_matches_reference(engine_lib, case):
    if case == "sorting256":
        w = W.sorting_2d(n=256, ncells=655)
    elif case == "tissue2d":
        w = W.tissue_2d(n=512, area=100)
    else:
        w = W.tissue_3d(n=64, volume=500)
    ours = _ours(w)
    area, perim, _ = ours.tables()
    ra, rp = _ref(w).tables()
    np.testing.assert_array_equal(area, ra.astype(np.int32))
    np.testing.assert_array_equal(perim, rp.astype(np.int32))


@pytest.mark.parametrize("D,perimeter,seed,terms", [(16, False, 12345, None),
                                                    (16, True, 777, None),
                                                    (32, True, 31337, None),
                                                    (32, True, 4242, "fixed_sticky"),
                                                    (32, False, 2024, "chemotaxis")])
def test_one_thread_reference_run_equals_restatement(engine_lib, D, perimeter, seed, terms):
    """`terms`: with stickiness and a fixed type (src/kernels2d.cu:280-290,
    399-400), run by the reference's fixed-toggle variant; or with a
    chemotaxis field (:302-334), run by its chemotaxis-toggle variant."""
    nt = 3 if terms == "fixed_sticky" else 2
    w = W.random_small((D, D), D * D // 20, ntypes=nt, seed=D + seed % 97, temperature=6.0,
                       perim=perimeter)
    J = np.rint(w.J).astype(int)
    lam_a = [0.0] + [1.0] * nt
    tgt_a = [0] + [20] * nt
    lam_p = ([0.0] + [0.5] * nt) if perimeter else [0.0] * (nt + 1)
    tgt_p = [0] + [18] * nt
    stick = fixed = chemo = field = None
    if terms == "fixed_sticky":
        stick = np.zeros((nt + 1, nt + 1), np.float32)
        stick[1, 2], stick[2, 1], stick[1, 0], stick[0, 2] = 3, 2, 4, 1
        fixed = np.array([False, False, False, True])
    if terms == "chemotaxis":
        chemo = np.array([0.0, 3.0, -2.0], np.float32)
        g = np.random.default_rng(seed)
        field = g.uniform(-2.0, 2.0, (2, D, D))
    wi = W.Workload("one_thread", w.lattice, w.ncells, J.astype(np.float32),
                    np.array(lam_a, np.float32), np.array(tgt_a, np.int32),
                    np.array(lam_p, np.float32), np.array(tgt_p, np.int32), 6.0, 0,
                    stick=stick, fixed=fixed, chemo=chemo, field=field)
    ref = _ref(wi)
    a0, p0 = ref.tables()
    mcs = 3
    ref.run(mcs, threads_per_block=1, positions_per_thread=D, positions_per_checkerboard=D,
            seed=seed)
    ref.synchronize()
    got = ref.pull()
    ra, rp = ref.tables()

    lat = w.lattice.copy()
    area, perim = a0.astype(np.int64), p0.astype(np.int64)
    acc = refmodel.sequential_run(lat, area, perim, J, lam_a, tgt_a, lam_p, tgt_p, 6.0,
                                  seed, mcs, perimeter_on=perimeter, stick=stick, fixed=fixed,
                                  chemo=chemo, field=field)
    assert acc > 10
    np.testing.assert_array_equal(got, lat)
    np.testing.assert_array_equal(ra.astype(np.int64), area)
    if perimeter:
        np.testing.assert_array_equal(rp.astype(np.int64), perim)


def one_thread_case_3d(D, perimeter, seed, terms):
    """Inputs of a one-thread 3D reference run (shared with the golden
    fixture generator)."""
    nt = 3 if terms == "fixed_sticky" else 2
    w = W.random_small((D, D, D), D ** 3 // 40, ntypes=nt, seed=D + seed % 89,
                       temperature=6.0, perim=perimeter)
    J = np.rint(w.J).astype(int)
    lam_a = [0.0] + [1.0] * nt
    tgt_a = [0] + [40] * nt
    lam_p = ([0.0] + [0.5] * nt) if perimeter else [0.0] * (nt + 1)
    tgt_p = [0] + [90] * nt
    stick = fixed = None
    if terms == "fixed_sticky":
        stick = np.zeros((nt + 1, nt + 1), np.float32)
        stick[1, 2], stick[2, 1], stick[1, 0], stick[0, 2] = 3, 2, 4, 1
        fixed = np.array([False, False, False, True])
    wi = W.Workload("one_thread_3d", w.lattice, w.ncells, J.astype(np.float32),
                    np.array(lam_a, np.float32), np.array(tgt_a, np.int32),
                    np.array(lam_p, np.float32), np.array(tgt_p, np.int32), 6.0, 0,
                    stick=stick, fixed=fixed)
    return wi, J, lam_a, tgt_a, lam_p, tgt_p


@pytest.mark.parametrize("D,perimeter,seed,terms", [(8, False, 999, None),
                                                    (16, True, 555, None),
                                                    (16, True, 8080, "fixed_sticky")])
def test_one_thread_reference_run_3d_equals_restatement(engine_lib, D, perimeter, seed, terms):
    """The reference's 3D sweep (src/kernels3d.cu:51-594, non-shared
    branch, with its neighbour redraw test that compares nz with y, :208)
    run by one thread equals tests/refmodel.py's sequential_run_3d."""
    wi, J, lam_a, tgt_a, lam_p, tgt_p = one_thread_case_3d(D, perimeter, seed, terms)
    ref = _ref(wi)
    a0, p0 = ref.tables()
    mcs = 2
    ref.run(mcs, threads_per_block=1, positions_per_thread=D, positions_per_checkerboard=D,
            seed=seed)
    ref.synchronize()
    got = ref.pull()
    ra, rp = ref.tables()
    lat = wi.lattice.copy()
    area, perim = a0.astype(np.int64), p0.astype(np.int64)
    acc = refmodel.sequential_run_3d(lat, area, perim, J, lam_a, tgt_a, lam_p, tgt_p, 6.0,
                                     seed, mcs, perimeter_on=perimeter, stick=wi.stick,
                                     fixed=wi.fixed)
    assert acc > 10
    np.testing.assert_array_equal(got, lat)
    np.testing.assert_array_equal(ra.astype(np.int64), area)
    if perimeter:
        np.testing.assert_array_equal(rp.astype(np.int64), perim)
