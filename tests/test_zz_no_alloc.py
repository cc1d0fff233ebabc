"""cpm_sweep_static: the sweep for callers that cannot allocate device memory.

The entry point works on caller-owned device buffers and takes all other
working memory from a fixed array inside the library.  Here the caller's
buffers come from torch; the entry point itself must allocate nothing.  Its
results must equal, bit for bit, those of the handle-based entry points
(cpm_create_box / cpm_push / cpm_run) with the same seed, stream id and
tick, over two calls in a row: the first recounts the tables from the
lattice, the second continues from the tables the first one left.

This file is collected last on purpose, so that a run that stops at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from gpucpm import workloads as W

pytestmark = pytest.mark.gpu


def _params(w):
    import gpucpm
    p = gpucpm.StaticParams()
    nt = w.J.shape[0]
    J = np.zeros((gpucpm.MAX_TYPES, gpucpm.MAX_TYPES), np.float32)
    J[:nt, :nt] = w.J
    p.J[:] = J.ravel().tolist()

    def fill(dst, src, dt):
        a = np.zeros(gpucpm.MAX_TYPES, dt)
        a[:len(src)] = src
        dst[:] = a.tolist()
    fill(p.lambda_area, w.lam_area, np.float32)
    fill(p.target_area, w.tgt_area, np.int32)
    fill(p.lambda_perimeter, w.lam_perim, np.float32)
    fill(p.target_perimeter, w.tgt_perim, np.int32)
    p.temperature = w.temperature
    return p


@pytest.mark.parametrize("shape,ncells", [((96, 80), 60), ((14, 12, 10), 30)])
def test_static_sweep_matches_handle_over_two_calls(engine_lib, shape, ncells):
    import torch

    import gpucpm
    w = W.random_small(shape, ncells, seed=31 + ncells, temperature=9.0)
    ndim = w.ndim
    dims = w.lattice.shape[::-1]  # (nx, ny[, nz])
    seed, stream_id, mcs = 4242, 7, 6

    # Reference results through the handle-based entry points.
    e = gpucpm.create_box(dims[0], dims[1], dims[2] if ndim == 3 else 1, ndim,
                          w.ncells, w.temperature)
    e.lattice(0)[...] = w.lattice.view(np.int32)
    w.apply(e, replica=0)
    e.set_seed(seed, stream_id)
    e.push_to_gpu()
    expected = []
    for _ in range(2):
        e.reset_counters()
        e.run_mcs(mcs)
        e.synchronize()
        e.pull_from_gpu()
        c = e.counters()
        expected.append((e.lattice(0).copy(), *e.tables(0), (c["evaluated"], c["accepted"])))

    # The same two steps through the allocation-free entry point, on device
    # buffers owned by the caller.
    dev = torch.device("cuda", 0)
    lat = torch.from_numpy(w.lattice.view(np.int32).copy()).to(dev)
    area = torch.full((w.ncells + 1,), -1, dtype=torch.int32, device=dev)
    perim = torch.full((w.ncells + 1,), -1, dtype=torch.int32, device=dev)
    cs = torch.full((w.ncells + 1, ndim), -1, dtype=torch.int64, device=dev)
    torch.cuda.synchronize()
    params = _params(w)
    for call in range(2):
        counters = gpucpm.sweep_static(
            ndim, dims, w.ncells, lat.data_ptr(), area.data_ptr(), perim.data_ptr(),
            cs.data_ptr(), params, seed=seed, stream_id=stream_id, tick=call * mcs,
            mcs=mcs, recount=(call == 0))
        want_lat, want_area, want_perim, want_cs, want_counters = expected[call]
        np.testing.assert_array_equal(lat.cpu().numpy().reshape(want_lat.shape), want_lat)
        np.testing.assert_array_equal(area.cpu().numpy(), want_area)
        np.testing.assert_array_equal(perim.cpu().numpy(), want_perim)
        np.testing.assert_array_equal(cs.cpu().numpy(), want_cs)
        assert counters == want_counters
        assert counters[1] > 0


def test_static_sweep_rejects_sizes_beyond_its_array(engine_lib):
    import gpucpm
    lib = gpucpm.library()
    p = gpucpm.StaticParams()
    nul = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.cpm_sweep_static(2, 1024, 1024, 1, 10, nul, nul, nul, nul, 1,
                              ctypes.byref(p), 0, 0, 0, 1, None, None)
    assert rc == gpucpm.CPM_ERR_INVALID
    assert b"CPM_STATIC_MAX_SITES" in lib.cpm_last_error(None)
    rc = lib.cpm_sweep_static(2, 64, 64, 1, 20000, nul, nul, nul, nul, 1,
                              ctypes.byref(p), 0, 0, 0, 1, None, None)
    assert rc == gpucpm.CPM_ERR_INVALID
    assert b"CPM_STATIC_MAX_CELLS" in lib.cpm_last_error(None)
