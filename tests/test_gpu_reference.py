"""Parity with the reference's own CUDA build (oracle/_ref, built from the
reference sources by oracle/ref_gpu/build.py and driven by ref_driver.cpp).

1. Table recount: the reference's calculateAreasAndCircumferences and this
   engine's push compute identical area and perimeter tables.
2. A one-thread reference run (deterministic for a given seed) equals
   tests/refmodel.py's restatement of the reference's sequential algorithm,
   bit for bit.  That restatement's dH is the one tests/test_oracle.py
   replays against the oracle, so the oracle's dH is pinned to the
   reference's outputs through it.
3. Statistics of the sorting workload after 1000 MCS (the reference's own
   example geometry, racy updates and Park-Miller draws, against this
   engine's deterministic schedule): mean area, area spread, perimeter,
   surviving cells, heterotypic boundary fraction and site activity agree
   within the tolerances below.
"""
import json
import os
import pathlib

import numpy as np
import pytest

import refmodel
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu

ref_gpu = pytest.importorskip("oracle.ref_gpu")
if not ref_gpu.available():
    pytest.skip("reference cubin not built (needs the reference checkout)",
                allow_module_level=True)

REPORT = pathlib.Path(os.environ.get("CPM_TEST_REPORT_DIR",
                                    pathlib.Path(__file__).resolve().parents[1] / "test_reports"))


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


def _observables(lat, prev):
    ids = (lat & 0xFFFFFF).astype(np.int64)
    areas = np.bincount(ids.ravel())[1:]
    alive = areas[areas > 0]
    lat64 = lat.astype(np.int64)
    per = np.zeros_like(areas)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            if dy == 0 and dx == 0:
                continue
            nb = np.roll(np.roll(lat64, -dy, 0), -dx, 1)
            diff = (nb != lat64) & (ids > 0)
            per += np.bincount(ids[diff], minlength=len(areas) + 1)[1:]
    return {"mean_area": float(alive.mean()), "sd_area": float(alive.std()),
            "mean_perimeter": float(per[areas > 0].mean()), "cells": int(len(alive)),
            "heterotypic": refmodel.heterotypic_fraction(lat),
            "activity": float((lat != prev).mean())}


def test_sorting_statistics_match_reference(engine_lib):
    """The sorting recipe at 256^2 (655 cells of 5x5, J_ll=14 J_dd=2 J_ld=11
    J_lm=J_dm=16, A=25, lambda=1, T=10) after 1000 MCS, 6 seeds each.  The
    reference runs its own examples/sorting.py geometry (32x32 threads, 4x4
    sites per thread, 2x2 checkerboard squares, grid sync per attempt)."""
    w = W.sorting_2d(n=256, ncells=655)
    mcs, tail = 1000, 10
    ours, refs = [], []
    for seed in range(1, 7):
        e = _ours(w, seed=seed)
        e.run_mcs(mcs - tail)
        e.synchronize()
        e.pull_from_gpu()
        prev = e.get_state().view(np.uint32).copy()
        e.run_mcs(tail)
        e.synchronize()
        e.pull_from_gpu()
        ours.append(_observables(e.get_state().view(np.uint32), prev))

        r = _ref(w)
        kw = dict(threads_per_block=32, positions_per_thread=4, positions_per_checkerboard=2)
        r.run(mcs - tail, seed=seed, **kw)
        r.synchronize()
        prev = r.pull()
        r.run(tail, seed=seed + 1000, **kw)
        r.synchronize()
        refs.append(_observables(r.pull(), prev))

    summary = {}
    for k in ours[0]:
        a = np.array([o[k] for o in ours], float)
        b = np.array([o[k] for o in refs], float)
        summary[k] = {"ours_mean": a.mean(), "ours_sd": a.std(ddof=1),
                      "ref_mean": b.mean(), "ref_sd": b.std(ddof=1)}
    REPORT.mkdir(exist_ok=True)
    (REPORT / "reference_sorting_stats.json").write_text(json.dumps(summary, indent=1))
    # Stated tolerances (relative to the reference's mean over seeds):
    #   mean area, mean perimeter          5 %
    #   sorting order parameter           10 %
    #   area spread, site activity        15 %
    #   surviving cells                   10 %
    # Cells shrink and die in this workload (655 -> ~340).  Reading area
    # from a per-phase snapshot lets a shrinking cell lose several sites in
    # one phase at a slightly too small area penalty, which costs about 5 %
    # more cells by MCS 1000 than the reference's live reads; the oracle
    # with tables updated after every attempt instead reproduces the
    # reference's survival.
    for k, tol in (("mean_area", 0.05), ("sd_area", 0.15), ("mean_perimeter", 0.05),
                   ("cells", 0.10), ("heterotypic", 0.10), ("activity", 0.15)):
        o, r = summary[k]["ours_mean"], summary[k]["ref_mean"]
        assert abs(o - r) <= tol * abs(r), (k, summary[k])


def _observables_3d(lat, prev):
    ids = (lat & 0xFFFFFF).astype(np.int64)
    vols = np.bincount(ids.ravel())[1:]
    alive = vols > 0
    lat64 = lat.astype(np.int64)
    surf = np.zeros_like(vols)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                if dz == dy == dx == 0:
                    continue
                nb = np.roll(lat64, (-dz, -dy, -dx), axis=(0, 1, 2))
                diff = (nb != lat64) & (ids > 0)
                surf += np.bincount(ids[diff], minlength=len(vols) + 1)[1:]
    return {"mean_volume": float(vols[alive].mean()), "sd_volume": float(vols[alive].std()),
            "mean_surface": float(surf[alive].mean()), "cells": int(alive.sum()),
            "activity": float((lat != prev).mean())}


def test_tissue3d_statistics_match_reference(engine_lib):
    """A 64^3 Voronoi tissue (2 types, integer J in [4, 16], V* = 500,
    lambda_V = 1, S* = 350, lambda_S = 0.2, T = 20) after 200 MCS, 8 seeds
    each.  The reference runs its 3D kernel (src/kernels3d.cu, non-shared,
    grid sync per attempt) with 4^3-thread blocks, 4 sites per thread and
    2x2x2 checkerboard squares."""
    w = W.tissue_3d(n=64, volume=500, seed=6)
    w.J = np.rint(w.J).astype(np.float32)
    mcs, tail = 200, 5
    ours, refs = [], []
    for seed in range(1, 9):
        e = _ours(w, seed=seed)
        e.run_mcs(mcs - tail)
        e.synchronize()
        e.pull_from_gpu()
        prev = e.get_state().view(np.uint32).copy()
        e.run_mcs(tail)
        e.synchronize()
        e.pull_from_gpu()
        ours.append(_observables_3d(e.get_state().view(np.uint32), prev))

        r = _ref(w)
        kw = dict(threads_per_block=4, positions_per_thread=4, positions_per_checkerboard=2)
        r.run(mcs - tail, seed=seed, **kw)
        r.synchronize()
        prev = r.pull()
        r.run(tail, seed=seed + 1000, **kw)
        r.synchronize()
        refs.append(_observables_3d(r.pull(), prev))

    summary = {}
    for k in ours[0]:
        a = np.array([o[k] for o in ours], float)
        b = np.array([o[k] for o in refs], float)
        summary[k] = {"ours_mean": a.mean(), "ours_sd": a.std(ddof=1),
                      "ref_mean": b.mean(), "ref_sd": b.std(ddof=1)}
    REPORT.mkdir(exist_ok=True)
    (REPORT / "reference_tissue3d_stats.json").write_text(json.dumps(summary, indent=1))
    # Stated tolerances (relative to the reference's mean over seeds):
    #   mean volume, mean surface, surviving cells   5 %
    #   volume spread                                 15 %
    #   site activity                                 50 %
    # The tissue nearly freezes (cells shrink to ~62 voxels under the steep
    # surface term), and the rare moves left are sensitive to the schedule.
    # An oracle run that commits every copy at once, as the reference's
    # live reads do, has 12 % less activity than the phase-snapshot rule
    # this engine follows.  The rest of the gap comes from the reference's
    # random site per attempt and its self-picks of :208.  The state
    # itself (volumes, surfaces, cells) agrees within a few percent.
    # The systematic activity gap is about 40 %, and the racy reference's
    # activity varies ~13 % from seed to seed (~9 % at 2 sigma for a mean
    # over 8 seeds), so 50 % holds the gap and that noise.
    for k, tol in (("mean_volume", 0.05), ("mean_surface", 0.05), ("cells", 0.05),
                   ("sd_volume", 0.15), ("activity", 0.50)):
        o, r = summary[k]["ours_mean"], summary[k]["ref_mean"]
        assert abs(o - r) <= tol * abs(r), (k, summary[k])
