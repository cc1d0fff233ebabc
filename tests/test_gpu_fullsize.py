"""Table invariants at the benchmark sizes: after GPU-only runs of the 4096^2
and 256^3 tissues, the tables equal a from-scratch recount of the final
lattice and the total area equals the number of non-medium sites.  (The
bit-exact comparison with the oracle at full length is
tests/test_gpu_fulllength.py.)"""
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


def test_tissue2d_4096_invariants(engine_lib, tissue2d):
    _invariants(tissue2d, 50, seed=2)


def test_tissue3d_256_invariants(engine_lib, tissue3d):
    _invariants(tissue3d, 20, seed=2)
