"""Checkpoints of an engine's complete state (gpucpm.Cpm or gpucpm.Batch).

`save(engine, path)` writes one .npz file; `load(engine, path)` restores it
into an engine of the same shape (same replica sizes and cell counts), after
which runs continue exactly as the uninterrupted run would have: the sweep
is a pure function of (lattice, tables, parameters, seed, stream, Monte
Carlo time).  The file holds:

  dimensionality, shapes [R, d], ncells [R]
  lattice        uint32, every replica's lattice, concatenated
  area, perimeter, centroid_sums   the tables, concatenated per replica
  params         uint8 [P, sizeof(StaticParams)]: each parameter record once
  param_index    [R]: the record of each replica
  tick, seed, stream_id
  act            uint32, the act stamps (only when the engine has them)
  prefdir, history, history_size   the persistence state: preferred
                 directions [rows, 3] and the mean-coordinate ring
                 [history_size, rows, 3] oldest slot first, rows of all
                 replicas concatenated (only when the engine has it)

Area and perimeter are recomputed by the push on load and checked against
the file; centroid sums are restored as saved (they record which periodic
image each site joined as, which a recount cannot know).  The reference
keeps its state only in host <-> device copies (src/cpm.cu:531-597) and has
no checkpoint of its own.
"""
import ctypes

import numpy as np

from . import CPM_ERR_INVALID, CpmError, StaticParams

FORMAT = 2


def save(engine, path):
    engine.synchronize()
    engine.pull_from_gpu()
    n = engine.n_replicas
    shapes, ncells, lats, areas, perims, css = [], [], [], [], [], []
    for r in range(n):
        lat = engine.host_lattice(r)
        shapes.append(lat.shape)
        ncells.append(engine._ncells(r))
        lats.append(lat.view(np.uint32).ravel().copy())
        a, p, c = engine.tables(r)
        areas.append(a)
        perims.append(p)
        css.append(c)
    index = engine.param_index()
    uniq, inverse = np.unique(index, return_inverse=True)
    first = {int(u): int(np.flatnonzero(index == u)[0]) for u in uniq}
    params = np.stack([np.frombuffer(bytes(engine.get_params(first[int(u)])), np.uint8)
                       for u in uniq])
    seed, stream_id = engine.seed
    extra = {}
    if getattr(engine, "act_exists", False):
        extra["act"] = np.concatenate([engine.act_lattice(r).view(np.uint32).ravel()
                                       for r in range(n)])
    if getattr(engine, "persistence_exists", False):
        states = [engine.persistence_state(r) for r in range(n)]
        extra["prefdir"] = np.concatenate([s[0] for s in states])
        extra["history"] = np.concatenate([s[1] for s in states], axis=1)
        extra["history_size"] = np.array([engine.history], np.int64)
    np.savez(path, format=np.array([FORMAT]), dimensionality=np.array([engine.dimensionality]),
             shapes=np.array(shapes, np.int64), ncells=np.array(ncells, np.int64),
             lattice=np.concatenate(lats), area=np.concatenate(areas),
             perimeter=np.concatenate(perims), centroid_sums=np.concatenate(css),
             params=params, param_index=inverse.astype(np.int64),
             tick=np.array([engine.tick], np.uint64), seed=np.array([seed], np.uint64),
             stream_id=np.array([stream_id], np.uint64), **extra)


def load(engine, path):
    d = np.load(path)
    if int(d["format"][0]) not in (1, FORMAT):
        raise CpmError(CPM_ERR_INVALID, f"unknown checkpoint format {int(d['format'][0])}")
    n = engine.n_replicas
    shapes, ncells = d["shapes"], d["ncells"]
    if int(d["dimensionality"][0]) != engine.dimensionality or len(shapes) != n:
        raise CpmError(CPM_ERR_INVALID, "checkpoint and engine differ in dimensionality "
                                        "or replica count")
    for r in range(n):
        if (tuple(int(v) for v in shapes[r]) != tuple(engine.host_lattice(r).shape)
                or int(ncells[r]) != engine._ncells(r)):
            raise CpmError(CPM_ERR_INVALID, f"replica {r}: size or cell count differs")
    lat, off = d["lattice"], 0
    for r in range(n):
        view = engine.host_lattice(r)
        view[...] = lat[off:off + view.size].view(np.int32).reshape(view.shape)
        if "act" in d.files:  # pushed with the lattice
            act = engine.act_lattice(r)
            act[...] = d["act"][off:off + view.size].view(np.int32).reshape(act.shape)
        off += view.size
    if "history_size" in d.files:
        engine.set_history(int(d["history_size"][0]))
    params = d["params"]
    index = d["param_index"]

    def record(i):
        p = StaticParams()
        ctypes.memmove(ctypes.addressof(p), params[i].tobytes(), ctypes.sizeof(p))
        return p

    counts = np.bincount(index, minlength=len(params))
    common = int(np.argmax(counts))
    engine.set_params(None, record(common))
    for r in np.flatnonzero(index != common):
        engine.set_params(int(r), record(int(index[r])))
    engine.push_to_gpu()
    rows = 0
    area, perim, cs = d["area"], d["perimeter"], d["centroid_sums"]
    for r in range(n):
        n1 = int(ncells[r]) + 1
        a, p, _ = engine.tables(r)
        if (not np.array_equal(a, area[rows:rows + n1])
                or not np.array_equal(p, perim[rows:rows + n1])):
            raise CpmError(CPM_ERR_INVALID, f"replica {r}: the tables of the checkpoint do "
                                            "not describe its lattice")
        engine.set_centroid_sums(r, cs[rows:rows + n1])
        if "prefdir" in d.files:
            engine.set_persistence_state(r, d["prefdir"][rows:rows + n1],
                                         d["history"][:, rows:rows + n1])
        rows += n1
    engine.tick = int(d["tick"][0])
    engine.set_seed(int(d["seed"][0]), int(d["stream_id"][0]))
    engine.reset_counters()
