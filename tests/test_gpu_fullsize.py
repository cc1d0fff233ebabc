"""Parity at the benchmark sizes: the 4096^2 tissue and the 256^3 tissue,
bit-exact against the multi-threaded oracle for a few MCS, plus table
invariants after longer GPU-only runs (tables equal a from-scratch recount of
the final lattice; total area equals the number of non-medium sites)."""
import numpy as np
import pytest

import oracle
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tissue2d():
    return W.tissue_2d()


@pytest.fixture(scope="module")
def tissue3d():
    return W.tissue_3d()


def _engine(w, seed):
    import gpucpm
    n = w.lattice.shape[0]
    e = gpucpm.Cpm(n, w.ndim, w.ncells, w.temperature, False)
    e.get_state()[...] = w.lattice.view(np.int32)
    w.apply(e)
    e.set_seed(seed)
    e.push_to_gpu()
    return e


def _bit_exact(w, mcs, seed):
    e = _engine(w, seed)
    e.run_mcs(mcs)
    e.synchronize()
    e.pull_from_gpu()
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=seed).run(mcs)
    lat = e.get_state().view(np.uint32)
    assert int((lat != sim.lattice).sum()) == 0
    area, perim, cs = e.tables()
    np.testing.assert_array_equal(area, sim.area)
    np.testing.assert_array_equal(perim, sim.perim)
    np.testing.assert_array_equal(cs, sim.csum)
    c = e.counters()
    assert (c["evaluated"], c["accepted"]) == (int(sim.counters[1]), int(sim.counters[2]))


def _invariants(w, mcs, seed):
    e = _engine(w, seed)
    e.run_mcs(mcs)
    e.synchronize()
    e.pull_from_gpu()
    lat = e.get_state().view(np.uint32)
    area, perim, cs = e.tables()
    rec = oracle.OracleSim(lat, w.ncells, **w.oracle_kwargs())
    np.testing.assert_array_equal(area, rec.area)
    np.testing.assert_array_equal(perim, rec.perim)
    assert ((cs - rec.csum) % lat.shape[0] == 0).all()
    assert int(area[1:].sum()) == int(((lat & 0xFFFFFF) != 0).sum())
    c = e.counters()
    assert c["attempts"] == lat.size * mcs
    assert 0 < c["accepted"] <= c["evaluated"] <= c["attempts"]


def test_tissue2d_4096_bit_exact(engine_lib, tissue2d):
    _bit_exact(tissue2d, 3, seed=1)


def test_tissue2d_4096_invariants(engine_lib, tissue2d):
    _invariants(tissue2d, 50, seed=2)


def test_tissue3d_256_bit_exact(engine_lib, tissue3d):
    _bit_exact(tissue3d, 2, seed=1)


def test_tissue3d_256_invariants(engine_lib, tissue3d):
    _invariants(tissue3d, 20, seed=2)
