"""cpm_sweep_static: the sweep for callers that cannot allocate device memory.

The entry point works on caller-owned device buffers and takes all other
working memory from a fixed array inside the library.  Here the caller's
buffers come from torch; the entry point itself must allocate nothing.  Its
results must equal, bit for bit, those of the handle-based entry points
(cpm_create_box / cpm_push / cpm_run) with the same seed, stream id and
tick, over two calls in a row: the first recounts the tables from the
lattice, the second continues from the tables the first one left.  Device
memory in use must not change across calls once the library's kernels are
loaded.

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
    if w.stick is not None:
        S = np.zeros((gpucpm.MAX_TYPES, gpucpm.MAX_TYPES), np.float32)
        S[:nt, :nt] = w.stick
        p.stickiness[:] = S.ravel().tolist()
    if w.fixed is not None:
        for t, f in enumerate(w.fixed):
            p.fixed[t] = 1 if f else 0
    return p


def _workload(shape, ncells, terms):
    w = W.random_small(shape, ncells, ntypes=3, seed=31 + ncells, temperature=9.0)
    if terms == "sticky_fixed":
        nt = w.J.shape[0]
        S = np.zeros((nt, nt), np.float32)
        S[1, 2], S[2, 1], S[1, 1] = 3.5, 1.25, 0.75
        w.stick = S
        fixed = np.zeros(nt, bool)
        fixed[3] = True
        w.fixed = fixed
    return w


def _handle_run(w, seed, stream_id, mcs, calls):
    import gpucpm
    dims = w.lattice.shape[::-1]  # (nx, ny[, nz])
    e = gpucpm.create_box(dims[0], dims[1], dims[2] if w.ndim == 3 else 1, w.ndim,
                          w.ncells, w.temperature)
    e.lattice(0)[...] = w.lattice.view(np.int32)
    w.apply(e, replica=0)
    e.set_seed(seed, stream_id)
    e.push_to_gpu()
    expected = []
    for _ in range(calls):
        e.reset_counters()
        e.run_mcs(mcs)
        e.synchronize()
        e.pull_from_gpu()
        c = e.counters()
        expected.append((e.lattice(0).copy(), *e.tables(0), (c["evaluated"], c["accepted"])))
    return expected


@pytest.mark.parametrize("shape,ncells,terms", [
    ((96, 80), 60, "plain"),
    ((14, 12, 10), 30, "plain"),
    ((90, 72), 50, "sticky_fixed"),
    ((32768, 8), 1500, "plain"),   # narrow: nx = 8, far below the 64-site tile width
])
def test_static_sweep_matches_handle_over_two_calls(engine_lib, shape, ncells, terms):
    import torch

    import gpucpm
    w = _workload(shape, ncells, terms)
    ndim = w.ndim
    dims = w.lattice.shape[::-1]
    seed, stream_id, mcs = 4242, 7, 6
    expected = _handle_run(w, seed, stream_id, mcs, calls=2)

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


def test_static_sweep_leaves_device_memory_unchanged(engine_lib):
    """After one call (which loads the library's kernels), further calls do
    not change the device's free memory: the entry point allocates nothing."""
    import gc

    import torch

    import gpucpm
    w = _workload((96, 80), 60, "plain")
    dims = w.lattice.shape[::-1]
    dev = torch.device("cuda", 0)
    lat = torch.from_numpy(w.lattice.view(np.int32).copy()).to(dev)
    area = torch.zeros((w.ncells + 1,), dtype=torch.int32, device=dev)
    perim = torch.zeros((w.ncells + 1,), dtype=torch.int32, device=dev)
    cs = torch.zeros((w.ncells + 1, 2), dtype=torch.int64, device=dev)
    params = _params(w)
    ptrs = (lat.data_ptr(), area.data_ptr(), perim.data_ptr(), cs.data_ptr())
    gpucpm.sweep_static(2, dims, w.ncells, *ptrs, params, seed=1, tick=0, mcs=3,
                        recount=True)
    torch.cuda.synchronize()
    # engines of earlier tests free their memory when collected: collect them
    # now and keep the collector off while measuring
    gc.collect()
    gc.disable()
    try:
        free0, _ = torch.cuda.mem_get_info(dev)
        frees = []
        for call in range(1, 3):
            gpucpm.sweep_static(2, dims, w.ncells, *ptrs, params, seed=1, tick=3 * call,
                                mcs=3, recount=False)
            frees.append(torch.cuda.mem_get_info(dev)[0])
    finally:
        gc.enable()
    assert frees == [free0, free0]


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
