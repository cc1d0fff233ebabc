"""gpucpm.checkpoint's file format and restore order, on CPU.

The engine is stood in for by an in-memory fake with the methods the module
calls (its push recounts the tables with the oracle, as the engine's push
does on the device).  The GPU test of the same module checks that a resumed
run continues bit for bit."""
import ctypes

import numpy as np
import pytest

import oracle
from gpucpm import StaticParams, checkpoint
from gpucpm import workloads as W


class FakeEngine:
    def __init__(self, ws, dimensionality=2):
        self.ws = ws
        self.dimensionality = dimensionality
        self.n_replicas = len(ws)
        self.lat = [w.lattice.view(np.int32).copy() for w in ws]
        self.params = [StaticParams() for _ in ws]
        self.tab = [None] * len(ws)
        self.tick = 0
        self._seed = (0, 0)
        self.pushed = False

    def synchronize(self):
        pass

    def pull_from_gpu(self):
        pass

    def host_lattice(self, r):
        return self.lat[r]

    def _ncells(self, r):
        return self.ws[r].ncells

    def tables(self, r):
        return self.tab[r]

    def param_index(self):
        keys, out = {}, []
        for p in self.params:
            out.append(keys.setdefault(bytes(p), len(keys)))
        return np.array(out, np.int32)

    def get_params(self, r):
        q = StaticParams()
        ctypes.memmove(ctypes.addressof(q), bytes(self.params[r]), ctypes.sizeof(q))
        return q

    def set_params(self, r, p):
        for k in (range(self.n_replicas) if r is None else [r]):
            self.params[k] = self.get_params_from(p)

    @staticmethod
    def get_params_from(p):
        q = StaticParams()
        ctypes.memmove(ctypes.addressof(q), bytes(p), ctypes.sizeof(q))
        return q

    @property
    def seed(self):
        return self._seed

    def set_seed(self, s, k):
        self._seed = (s, k)

    def push_to_gpu(self):
        for r, w in enumerate(self.ws):
            sim = oracle.OracleSim(self.lat[r].view(np.uint32), w.ncells, **w.oracle_kwargs())
            self.tab[r] = (sim.area.copy(), sim.perim.copy(), sim.csum.copy())
        self.pushed = True

    def set_centroid_sums(self, r, cs):
        a, p, _ = self.tab[r]
        self.tab[r] = (a, p, np.array(cs, np.int64))

    def reset_counters(self):
        pass


def _engine(seed):
    ws = [W.random_small(s, 15 + i, seed=seed + i) for i, s in enumerate([(24, 20), (17, 31)])]
    e = FakeEngine(ws)
    e.push_to_gpu()
    return e


def test_checkpoint_roundtrip(tmp_path):
    a = _engine(5)
    for r, p in enumerate(a.params):
        p.temperature = 3.0 + r
        p.J[1] = 7.0
    a.params.append(a.get_params(0))  # a third replica sharing replica 0's record
    a.ws.append(a.ws[0])
    a.lat.append(a.lat[0].copy())
    a.tab.append(tuple(x.copy() for x in a.tab[0]))
    a.n_replicas = 3
    a.tab[0] = (a.tab[0][0], a.tab[0][1], a.tab[0][2] + 24)  # a shifted periodic image
    a.tick, a._seed = 123, (77, 8)
    path = tmp_path / "c.npz"
    checkpoint.save(a, path)
    d = np.load(path)
    assert d["params"].shape[0] == 2 and list(d["param_index"]) == [0, 1, 0]

    b = _engine(5)
    b.ws.append(b.ws[0])
    b.lat.append(np.zeros_like(b.lat[0]))
    b.params.append(StaticParams())
    b.tab.append(None)
    b.n_replicas = 3
    checkpoint.load(b, path)
    assert b.tick == 123 and b.seed == (77, 8)
    for r in range(3):
        np.testing.assert_array_equal(b.lat[r], a.lat[r])
        for x, y in zip(b.tab[r], a.tab[r]):
            np.testing.assert_array_equal(x, y)
        assert bytes(b.params[r]) == bytes(a.params[r])


def test_checkpoint_rejects_other_shapes(tmp_path):
    a = _engine(5)
    path = tmp_path / "c.npz"
    checkpoint.save(a, path)
    b = FakeEngine([W.random_small((24, 22), 15, seed=1), a.ws[1]])
    b.push_to_gpu()
    with pytest.raises(Exception, match="size or cell count"):
        checkpoint.load(b, path)


def test_checkpoint_rejects_tables_of_another_lattice(tmp_path):
    a = _engine(5)
    a.tab[1] = (a.tab[1][0] + 1, a.tab[1][1], a.tab[1][2])
    path = tmp_path / "c.npz"
    checkpoint.save(a, path)
    b = _engine(5)
    with pytest.raises(Exception, match="do not describe"):
        checkpoint.load(b, path)
