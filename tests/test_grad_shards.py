"""Sharded likelihood-ratio gradients: the host protocol of gpucpm.grad
(one all-reduce of per-checkpoint observable sums and replica counts before
the backward kernel, one all-reduce of the gradient after it) on two gloo
ranks on CPU.  The backward kernel is stood in for by its formula in NumPy
(the GPU tests check the kernel against that formula); the sharded result
must equal the estimator over all replicas in one process."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

R, C, K = 6, 3, 5


def _data(seed):
    g = np.random.default_rng(seed)
    O = g.uniform(0.2, 0.6, (R, C))
    cum = g.normal(0.0, 3.0, (R, C, K))  # cumulative scores up to each checkpoint
    return O, cum


def _estimator(O, cum, dl, total=None, ntotal=None):
    """The backward kernel's formula (leave-one-out baseline)."""
    n = O.shape[0] if ntotal is None else ntotal
    s = O.sum(axis=0) if total is None else np.asarray(total)
    b = (s[None, :] - O) / (n - 1)
    return np.einsum("rc,rck->k", dl * (O - b), cum)


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from gpucpm import grad as G
    O, cum = _data(100 + rank)
    tot, ntot = G.shard_totals(torch.tensor(O, dtype=torch.float32))
    dl = np.full((R, C), 1.0 / R)  # this shard's loss: mean over its replicas
    g = torch.tensor(_estimator(O, cum, dl, tot, ntot), dtype=torch.float64)
    G.reduce_gradient(g)
    out[rank] = (tot, ntot, g.numpy().copy())
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_gradient_equals_single_process():
    world = 2
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world,
                           start_method="spawn")
        res = dict(out)
    parts = [_data(100 + r) for r in range(world)]
    O = np.concatenate([p[0] for p in parts])
    cum = np.concatenate([p[1] for p in parts])
    for r in range(world):
        tot, ntot, _ = res[r]
        assert ntot == world * R
        np.testing.assert_allclose(tot, O.sum(axis=0), rtol=1e-6)
    # one process over all replicas, loss = mean over all of them
    want = _estimator(O, cum, np.full((world * R, C), 1.0 / (world * R)))
    for r in range(world):
        np.testing.assert_allclose(res[r][2], want, rtol=1e-5)
    np.testing.assert_array_equal(res[0][2], res[1][2])


def test_estimator_without_totals_is_local():
    O, cum = _data(1)
    dl = np.full((R, C), 1.0 / R)
    np.testing.assert_allclose(_estimator(O, cum, dl),
                               _estimator(O, cum, dl, O.sum(axis=0), R))
