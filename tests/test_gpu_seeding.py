"""Seeding and analysis kernels: periodic Voronoi seeding on the device and
boundary lengths by type pair.

The seeding kernel must equal the brute-force nearest-point labelling of the
oracle bit for bit (ties to the lowest point index), including degenerate
point sets (one point, duplicates, points on bucket edges, clusters that
force wide ring searches), and reproduce the full-size 4096^2 and 256^3
workload lattices that the CPU k-d tree builds.  Boundary counts must equal
the oracle's count on every replica of a batch, and agree with the sorting
order parameter."""
import time

import numpy as np
import pytest

import oracle
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu


def _engine_for(shape, ncells):
    import gpucpm
    if len(shape) == 2:
        return gpucpm.create_box(shape[1], shape[0], 1, 2, ncells, 10.0)
    return gpucpm.create_box(shape[2], shape[1], shape[0], 3, ncells, 10.0)


def _point_sets(shape, seed):
    rng = np.random.default_rng(seed)
    dims = np.array(shape[::-1], np.float64)
    nd = len(shape)
    sets = {"uniform": rng.random((300, nd)) * dims,
            "one": rng.random((1, nd)) * dims,
            # integer points sit on bucket edges and give exact distance ties
            "lattice_points": np.floor(rng.random((120, nd)) * dims),
            "cluster": 0.05 * rng.random((40, nd)) * dims + 1.0}
    dup = rng.random((60, nd)) * dims
    sets["duplicates"] = np.concatenate([dup, dup[::-1]])  # every point twice
    return sets


@pytest.mark.parametrize("shape", [(96, 120), (31, 17), (3, 3), (18, 20, 22), (5, 4, 3)])
def test_voronoi_matches_brute_force(engine_lib, shape):
    for name, pts in _point_sets(shape, sum(shape)).items():
        n = len(pts)
        rng = np.random.default_rng(n)
        ncells = n
        values = ((np.arange(n) + 1) | (rng.integers(1, 4, n) << 24)).astype(np.uint32)
        e = _engine_for(shape, ncells)
        e.seed_voronoi(0, pts, values)
        e.recount()
        e.synchronize()
        e.pull_from_gpu()
        want = oracle.voronoi(shape, pts, values)
        got = e.lattice(0).view(np.uint32)
        bad = np.argwhere(got != want)
        assert bad.size == 0, f"{name}: {len(bad)} sites differ, first {bad[:3].tolist()}"
        sim = oracle.OracleSim(want, ncells, np.zeros((4, 4), np.float32), [0] * 4, [0] * 4)
        area, perim, cs = e.tables(0)
        np.testing.assert_array_equal(area, sim.area)
        np.testing.assert_array_equal(perim, sim.perim)


def test_voronoi_rejects_bad_input(engine_lib):
    import gpucpm
    e = _engine_for((16, 16), 4)
    with pytest.raises(gpucpm.CpmError, match="outside"):
        e.seed_voronoi(0, [[16.0, 2.0]], [1])
    with pytest.raises(gpucpm.CpmError, match="value"):
        e.seed_voronoi(0, [[1.0, 2.0]], [9])  # id above ncells
    with pytest.raises(gpucpm.CpmError, match="value"):
        e.seed_voronoi(0, [[1.0, 2.0]], [2 << 24])  # medium with a type


@pytest.mark.parametrize("which", ["tissue_2d", "tissue_3d"])
def test_voronoi_reproduces_full_size_workloads(engine_lib, which):
    """4096^2 from 167,772 points and 256^3 from 33,554 points: the device
    seeding gives the k-d tree's lattice (distance ties, which could differ,
    have probability ~0 with random points)."""
    w = getattr(W, which)()
    e = _engine_for(w.lattice.shape, w.ncells)
    e.seed_voronoi(0, w.meta["points"], w.meta["values"])  # first call: warm-up
    e.synchronize()
    t0 = time.perf_counter()
    e.seed_voronoi(0, w.meta["points"], w.meta["values"])
    dt = time.perf_counter() - t0
    e.recount()
    e.synchronize()
    e.pull_from_gpu()
    got = e.lattice(0).view(np.uint32)
    assert np.array_equal(got, w.lattice), int((got != w.lattice).sum())
    print(f"{which}: seeded {w.lattice.size} sites from {len(w.meta['values'])} points "
          f"in {dt * 1e3:.1f} ms (host binning and copies included)")


def test_boundaries_match_oracle_on_a_batch(engine_lib):
    import gpucpm
    ws = [W.random_small((40, 36), 25, ntypes=3, seed=180),
          W.random_small((33, 47), 30, ntypes=2, seed=181),
          W.random_small((64, 64), 50, ntypes=3, seed=182)]
    b = gpucpm.Batch(2, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.push_to_gpu()
    b.run_mcs(10)
    b.synchronize()
    counts = b.boundary_counts(4)
    ratio = b.observe_heterotypic()
    b.pull_from_gpu()
    for r in range(3):
        lat = b.lattice(r).view(np.uint32)
        np.testing.assert_array_equal(counts[r], oracle.boundaries(lat, 4))
        cc = counts[r][1:, 1:]
        total, hetero = int(np.triu(cc).sum()), int(np.triu(cc, 1).sum())
        assert abs(ratio[r] - hetero / total) < 1e-6
    # types above ntypes are skipped
    np.testing.assert_array_equal(b.boundary_counts(2)[0], counts[0][:2, :2])


def test_boundaries_3d(engine_lib):
    w = W.random_small((14, 12, 16), 30, ntypes=3, seed=183)
    e = _engine_for(w.lattice.shape, w.ncells)
    e.lattice(0)[...] = w.lattice.view(np.int32)
    w.apply(e, replica=0)
    e.push_to_gpu()
    e.run_mcs(4)
    e.synchronize()
    c = e.boundary_counts(4)[0]
    e.pull_from_gpu()
    np.testing.assert_array_equal(c, oracle.boundaries(e.lattice(0).view(np.uint32), 4))


def test_voronoi_seeds_one_replica_of_a_batch(engine_lib):
    """Seeding replica 1 writes only its own lattice region."""
    import gpucpm
    shapes = [(20, 24), (31, 26), (17, 17)]
    b = gpucpm.Batch(2, [s[::-1] for s in shapes], [30, 40, 10])
    for r in range(3):
        b.lattice(r)[...] = 0
    b.push_to_gpu()
    rng = np.random.default_rng(9)
    pts = rng.random((40, 2)) * np.array(shapes[1][::-1], np.float64)
    vals = ((np.arange(40) + 1) | (2 << 24)).astype(np.uint32)
    b.seed_voronoi(1, pts, vals)
    b.recount()
    b.synchronize()
    b.pull_from_gpu()
    np.testing.assert_array_equal(b.lattice(1).view(np.uint32), oracle.voronoi(shapes[1], pts, vals))
    assert not b.lattice(0).any() and not b.lattice(2).any()
    area, _, _ = b.tables(1)
    assert area[1:].sum() == shapes[1][0] * shapes[1][1]


def test_voronoi_refuses_clustered_points_before_launch(engine_lib):
    """2M points crowded into one corner of a 4096^2 lattice would make the
    ring search scan ~10^13 buckets; the host bound refuses the call before
    any kernel runs, and the engine stays usable."""
    import gpucpm
    e = _engine_for((4096, 4096), 2_000_000)
    rng = np.random.default_rng(1)
    pts = rng.random((2_000_000, 2)) * 2.0
    vals = (np.arange(2_000_000, dtype=np.uint32) + 1) | (1 << 24)
    with pytest.raises(gpucpm.CpmError, match="unevenly"):
        e.seed_voronoi(0, pts, vals)
    ok = rng.random((1000, 2)) * 4096.0
    e.seed_voronoi(0, ok, (np.arange(1000, dtype=np.uint32) + 1) | (1 << 24))
    e.recount()
    e.synchronize()
