"""Bit-exact parity at every timed configuration, at full length.

The GPU engine and the CPU oracle run the same workloads as the benchmark
for the same number of MCS, and must end with identical lattices, area /
perimeter tables, exact centroid sums and evaluated / accepted counters:

  4096^2 tissue (167,772 cells, area + perimeter terms)  500 MCS
  256^3 tissue (26,844 cells, volume + surface terms)    200 MCS
  256 ragged replicas, sides 64..1024, own parameters     500 MCS, grid dispatch
  512 replicas of the 256^2 two-type sorting grid         500 MCS, hybrid dispatch

The batches run through graph-captured launches, as the benchmark times
them.  The oracle runs the single lattices on every host thread and the
batches one replica per thread (each replica draws Philox stream r of its
batch, so it equals a single lattice with that stream id).  On a 16-core
host the oracle side takes about two and a half minutes in all.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import oracle
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu


def _compare(lat, tables, counters, sim, label):
    area, perim, cs = tables
    diff = int((lat != sim.lattice).sum())
    assert diff == 0, f"{label}: {diff} sites differ from the oracle"
    np.testing.assert_array_equal(area, sim.area, err_msg=label)
    np.testing.assert_array_equal(perim, sim.perim, err_msg=label)
    np.testing.assert_array_equal(cs, sim.csum, err_msg=label)
    assert (counters["evaluated"], counters["accepted"]) == (
        int(sim.counters[1]), int(sim.counters[2])), label


@pytest.mark.parametrize("name", ["tissue_2d", "tissue_3d"])
def test_single_lattice_full_length(engine_lib, name):
    import gpucpm
    w = W.tissue_2d() if name == "tissue_2d" else W.tissue_3d()
    mcs, seed = w.mcs, 5
    n = w.lattice.shape[0]
    e = gpucpm.Cpm(n, w.ndim, w.ncells, w.temperature, False)
    e.get_state()[...] = w.lattice.view(np.int32)
    w.apply(e)
    e.set_seed(seed)
    e.push_to_gpu()
    e.autotune(probe_mcs=2)  # the benchmark's tile choice; the state is restored
    e.run_mcs(mcs)
    e.synchronize()
    e.pull_from_gpu()
    lat = e.get_state().view(np.uint32).copy()
    tables, counters = e.tables(), e.counters()
    del e
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=seed)
    sim.run(mcs, nthreads=os.cpu_count() or 1)
    _compare(lat, tables, counters, sim, f"{name} {mcs} MCS")


def _batch_full_length(ws, mcs, seed, dispatch):
    import gpucpm
    sizes = [w.lattice.shape[::-1] for w in ws]
    b = gpucpm.Batch(2, sizes, [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(seed, 0)
    b.set_dispatch(dispatch)
    b.push_to_gpu()
    b.run_graph(mcs)
    b.synchronize()
    b.pull_from_gpu()
    got = [(b.lattice(r).view(np.uint32).copy(), b.tables(r), b.counters(r))
           for r in range(len(ws))]
    del b

    def one(r):
        w = ws[r]
        sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=seed, stream=r)
        return sim.run(mcs, nthreads=1)

    # largest replicas first, so that the pool ends evenly
    order = sorted(range(len(ws)), key=lambda r: -ws[r].nsites)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        sims = dict(zip(order, ex.map(one, order)))
    for r in range(len(ws)):
        _compare(*got[r], sims[r], f"replica {r} of {len(ws)}, {mcs} MCS")


def test_ragged_ensemble_full_length(engine_lib):
    import gpucpm
    ws = W.ensemble_2d(nrep=256, seed=3)
    _batch_full_length(ws, 500, seed=9, dispatch=gpucpm.DISPATCH_GRID)


def test_sorting_batch_full_length(engine_lib):
    import gpucpm
    ws = [W.sorting_grid(n=256, ncells=2600, seed=0)] * 512
    _batch_full_length(ws, 500, seed=11, dispatch=gpucpm.DISPATCH_HYBRID)
