"""State I/O and resume: checkpoints, the zero-copy device view, recount and
parameter records.

A run restored from a checkpoint must continue bit for bit like the
uninterrupted run (lattice, area, perimeter, centroid sums); a lattice
edited in place through the torch view must get tables equal to the
oracle's recount of the edited lattice."""
import gc

import numpy as np
import pytest

import oracle
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu


def _state(e):
    e.synchronize()
    e.pull_from_gpu()
    return [(e.host_lattice(r).copy(), *e.tables(r)) for r in range(e.n_replicas)]


def _assert_states_equal(a, b):
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)


def _batch(ws, seed):
    import gpucpm
    b = gpucpm.Batch(ws[0].ndim, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(seed, 7)
    return b


@pytest.mark.parametrize("dims", [2, 3])
def test_checkpoint_resume_is_bit_exact(engine_lib, tmp_path, dims):
    from gpucpm import checkpoint
    shapes = [(48, 40), (37, 52), (30, 30)] if dims == 2 else [(12, 10, 14), (11, 13, 9)]
    ws = [W.random_small(s, 20 + 5 * i, ntypes=3, seed=300 + i, temperature=6.0 + i)
          for i, s in enumerate(shapes)]
    ws[0].fixed = np.array([False, False, False, True])
    ws[1].stick = np.zeros((4, 4), np.float32)
    ws[1].stick[1, 2] = 3.0
    a = _batch(ws, seed=9)
    a.push_to_gpu()
    a.run_mcs(6)
    path = tmp_path / "state.npz"
    checkpoint.save(a, path)
    a.run_mcs(5)
    want = _state(a)

    b = _batch([W.random_small(s, 20 + 5 * i, ntypes=3, seed=999, temperature=1.0)
                for i, s in enumerate(shapes)], seed=0)  # other contents everywhere
    checkpoint.load(b, path)
    assert b.tick == 6 and b.seed == (9, 7)
    b.run_mcs(5)
    _assert_states_equal(_state(b), want)


def test_device_view_and_recount(engine_lib):
    import torch

    import gpucpm
    w = W.random_small((64, 48), 40, seed=17, temperature=8.0)
    e = gpucpm.create_box(48, 64, 1, 2, w.ncells, w.temperature)
    e.lattice(0)[...] = w.lattice.view(np.int32)
    w.apply(e, replica=0)
    e.push_to_gpu()
    e.run_mcs(3)
    e.synchronize()
    t = e.device_lattice(0)
    assert t.dtype == torch.int32 and tuple(t.shape) == (64, 48) and t.is_cuda
    e.pull_from_gpu()
    np.testing.assert_array_equal(t.cpu().numpy(), e.lattice(0))
    # dissolve one cell into the medium, in place on the device
    victim = int(t[10, 10].item())
    assert victim & 0xFFFFFF
    t[t == victim] = 0
    torch.cuda.synchronize()
    e.recount()
    e.pull_from_gpu()
    lat = e.lattice(0).view(np.uint32).copy()
    assert not (lat == np.uint32(victim)).any()
    sim = oracle.OracleSim(lat, w.ncells, **w.oracle_kwargs())
    area, perim, cs = e.tables(0)
    np.testing.assert_array_equal(area, sim.area)
    np.testing.assert_array_equal(perim, sim.perim)
    np.testing.assert_array_equal(cs, sim.csum)
    # the tensor keeps its engine alive
    del e
    gc.collect()
    assert int((t != 0).sum().item()) > 0


def test_params_roundtrip_and_sharing(engine_lib):
    import gpucpm
    ws = [W.random_small((32, 32), 20, seed=40 + i) for i in range(4)]
    b = _batch(ws, seed=1)  # apply() per replica: one record each
    p = b.get_params(2)
    b.set_params(None, p)   # every replica: one shared record again
    b.set_temperature(3, 3.5)
    b.push_to_gpu()
    b.run_mcs(1)            # uploads (and drops unused records)
    idx = b.param_index()
    assert idx[0] == idx[1] == idx[2] != idx[3]
    q = b.get_params(3)
    assert q.temperature == np.float32(3.5)
    assert bytes(b.get_params(0)) == bytes(p)
