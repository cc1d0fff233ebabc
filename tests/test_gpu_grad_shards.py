"""Sharded likelihood-ratio gradients on the GPU, end to end.

Two processes (gloo ranks, both on cuda:0) each hold half of an ensemble
through gpucpm.grad.Ensemble(..., group=WORLD), run the score-accumulating
forward and the backward kernel through torch.autograd, and exchange the
observable totals and the gradient.  Their gradient must equal the one of a
single process that holds every replica (same seed; rank k's replicas carry
the stream ids k * R .. k * R + R - 1 of the single process's batch, so
every replica follows the same trajectory in both runs).  Only the order of
the FP32 sums over replicas differs, hence the 1e-4 tolerance.
"""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

R_SHARD, MCS, WORLD = 48, 10, 2


def _workload():
    from gpucpm import workloads as W
    return W.sorting_grid(n=60, ncells=143, seed=0)


def _grad(ens, mcs):
    import torch

    from gpucpm import grad as G
    th = ens.theta0().clone().requires_grad_(True)
    O = G.LikelihoodRatio.apply(th, ens, mcs, [mcs])
    O.mean().backward()
    torch.cuda.synchronize()
    return th.grad.double().numpy().copy(), O.detach().double().cpu().numpy().copy()


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "gpu-cpm_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        torch.cuda.set_device(0)
        from gpucpm import grad as G
        ens = G.Ensemble([_workload()] * R_SHARD, seed=3, stream_id=rank * R_SHARD,
                         group=dist.group.WORLD)
        out[rank] = _grad(ens, MCS)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_ensemble_equals_single_process(engine_lib):
    import torch.multiprocessing as mp

    from gpucpm import grad as G
    ens = G.Ensemble([_workload()] * (WORLD * R_SHARD), seed=3, stream_id=0)
    want, O_all = _grad(ens, MCS)
    del ens
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(WORLD, _free_port(), out), nprocs=WORLD,
                           start_method="spawn")
        res = dict(out)
    assert sorted(res) == list(range(WORLD))
    # each shard followed its replicas' trajectories exactly
    for r in range(WORLD):
        np.testing.assert_array_equal(res[r][1], O_all[r * R_SHARD:(r + 1) * R_SHARD])
    scale = np.abs(want).max()
    for r in range(WORLD):
        np.testing.assert_allclose(res[r][0], want, rtol=1e-4, atol=1e-4 * scale)
    np.testing.assert_array_equal(res[0][0], res[1][0])
