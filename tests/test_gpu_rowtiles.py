"""The row-tile sweeps of single lattices (cpm_sweep2d.cu, cpm_sweep3d.cu)
against the oracle, bit for bit, under each way of staging tiles:

  parity  the general sweep_kernel (scalar loads, parity-split tiles)
  vector  row-major tiles from 16-byte vector loads
  tma     row-major tiles, interior tiles copied by cp.async.bulk.tensor
  cluster (2D) the lattice held in the shared memory of one thread-block
          cluster, a strip of rows per block with copies of its
          neighbours' edge rows, tiles read in place

Shapes cover partial tiles in x (nx = 76: 38 target columns, a full and a
6-wide tile), odd heights and depths (one-row or one-plane slots of the last
class), every tile variant in 2D and 3D, and the periodic seam on every
side; terms cover the perimeter, stickiness, a fixed type and a chemotaxis
field.  Graph-captured
runs and plain runs agree."""
import numpy as np
import pytest

import oracle
from gpucpm import workloads as W
from test_gpu_parity import assert_same, finish, make_engine

pytestmark = pytest.mark.gpu

FILLS = ("parity", "vector", "tma", "cluster")


def _fill_code(name):
    import gpucpm
    return {"parity": gpucpm.FILL_PARITY, "vector": gpucpm.FILL_VECTOR,
            "tma": gpucpm.FILL_TMA, "cluster": gpucpm.FILL_CLUSTER}[name]


def _terms(w, seed):
    nt = w.J.shape[0]
    g = np.random.default_rng(seed)
    w.stick = np.zeros((nt, nt), np.float32)
    w.stick[1, 2], w.stick[2, 1], w.stick[1, 0] = g.integers(1, 6, 3).astype(np.float32)
    w.fixed = np.zeros(nt, bool)
    w.fixed[nt - 1] = True
    if w.ndim == 2:
        ny, nx = w.lattice.shape
        yy, xx = np.mgrid[0:ny, 0:nx]
        w.field = np.stack([np.sin(2 * np.pi * yy / ny) * 3.0, np.cos(2 * np.pi * xx / nx)])
    else:
        nz, ny, nx = w.lattice.shape
        zz, yy, xx = np.mgrid[0:nz, 0:ny, 0:nx]
        w.field = np.stack([np.sin(2 * np.pi * yy / ny) * 3.0, np.cos(2 * np.pi * xx / nx),
                            np.sin(2 * np.pi * zz / nz) * 1.5])
    w.chemo = np.zeros(nt, np.float32)
    w.chemo[1] = 2.5
    return w


@pytest.mark.parametrize("fill", FILLS)
@pytest.mark.parametrize("shape,ncells,variant,terms,mcs", [
    ((256, 256), 300, 0, False, 12),   # the sorting size, 32 x 6 tiles
    ((67, 76), 40, 0, True, 15),       # odd ny, partial x tiles, every term
    ((130, 144), 120, 1, True, 10),    # 32 x 8 tiles
    ((132, 200), 150, 2, False, 10),   # 32 x 16 tiles
    ((96, 72), 50, 3, True, 20),       # one-row tiles, nx = one staged row
    ((66, 72), 40, 0, False, 12),      # cluster: a last block of one row (both its edges)
    ((18, 20, 72), 60, 0, True, 6),    # 3D, 32 x 2 x 2 tiles, every term
    ((19, 21, 76), 60, 1, False, 5),   # 3D, odd ny and nz, partial x tiles
    ((20, 18, 80), 50, 2, True, 4),    # 3D, 32 x 4 x 4 tiles
    ((18, 19, 72), 40, 3, False, 6),   # 3D, one-row tiles
])
def test_row_tiles_match_oracle(engine_lib, fill, shape, ncells, variant, terms, mcs):
    if fill == "cluster" and len(shape) == 3:
        pytest.skip("the cluster sweep is 2D")
    w = W.random_small(shape, ncells, ntypes=3, seed=500 + ncells, temperature=9.0)
    if terms:
        _terms(w, ncells)
    e = make_engine(w, seed=77, stream=3)
    e.set_variant(variant)
    e.set_fill(_fill_code(fill))
    assert e.sweep_config()["fill"] == fill
    e.run_mcs(mcs)
    finish(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=77, stream=3)
    sim.run(mcs)
    assert_same(e, sim)
    assert int(sim.counters[2]) > 0


def test_cluster_sweep_graph_runs_and_autotune(engine_lib):
    """The 256^2 sorting lattice in the cluster sweep: graph replays and plain
    runs continue one trajectory, and the autotuner (which tries the cluster
    sweep) leaves the state as it was."""
    import gpucpm
    w = W.sorting_2d(n=256, ncells=655)
    e = make_engine(w, seed=9)
    e.set_fill(gpucpm.FILL_CLUSTER)
    e.run_graph(5)
    e.run_mcs(3)
    e.autotune(probe_mcs=2)
    e.run_graph(4)
    finish(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=9).run(12)
    assert_same(e, sim)


def test_row_tiles_graph_runs_and_default_fill(engine_lib):
    import gpucpm
    w = W.tissue_2d(n=512, area=100, seed=4)
    e = make_engine(w, seed=5)
    assert e.fill == gpucpm.FILL_TMA  # the default for lattices that fit
    e.run_graph(4)
    e.run_graph(4)
    e.run_mcs(3)
    finish(e)
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=5).run(11)
    assert_same(e, sim)


def test_row_tiles_need_a_fitting_lattice(engine_lib):
    import gpucpm
    w = W.random_small((80, 70), 30, seed=3)  # nx = 70 is not a multiple of 4
    e = make_engine(w)
    assert e.fill == gpucpm.FILL_PARITY
    with pytest.raises(gpucpm.CpmError):
        e.set_fill(gpucpm.FILL_TMA)
    b = gpucpm.Batch(2, [(128, 128), (128, 128)], [10, 10])  # batches keep the general sweep
    assert b.fill == gpucpm.FILL_PARITY
    with pytest.raises(gpucpm.CpmError):
        b.set_fill(gpucpm.FILL_VECTOR)
