"""CPU oracle of the checkerboard Cellular Potts sweep.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product.  See cpm_oracle.cpp for
the algorithm, its reference citations and its parity status: the reference
ships no golden vectors and its parallel runs are nondeterministic, so the
pin is the reference's own deterministic one-thread runs and table recounts,
kept in tests/golden/.
"""
import ctypes

import numpy as np

from .build import LIB_PATH, build

MAX_TYPES = 32


class Params(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("nz", ctypes.c_int), ("ncells", ctypes.c_int),
        ("J", ctypes.c_float * (MAX_TYPES * MAX_TYPES)),
        ("lam_area", ctypes.c_float * MAX_TYPES),
        ("tgt_area", ctypes.c_int * MAX_TYPES),
        ("lam_perim", ctypes.c_float * MAX_TYPES),
        ("tgt_perim", ctypes.c_int * MAX_TYPES),
        ("temperature", ctypes.c_float),
        ("seed", ctypes.c_uint64),
        ("stream", ctypes.c_uint32),
        ("stick", ctypes.c_float * (MAX_TYPES * MAX_TYPES)),
        ("fixed_mask", ctypes.c_uint32),
        ("chemo", ctypes.c_float * MAX_TYPES),
        ("field", ctypes.c_void_p),
        ("act_lambda", ctypes.c_float * MAX_TYPES),
        ("act_max", ctypes.c_int * MAX_TYPES),
        ("act", ctypes.c_void_p),
        ("persist_lambda", ctypes.c_float * MAX_TYPES),
        ("prefdir", ctypes.c_void_p),
    ]


class ScoreSpec(ctypes.Structure):
    """Layout of cpm_score_spec: J type pairs, lambda_area, lambda_perim and
    T flags."""
    _fields_ = [("n_pairs", ctypes.c_int), ("pair_a", ctypes.c_int * 6),
                ("pair_b", ctypes.c_int * 6), ("lambda_area", ctypes.c_int),
                ("lambda_perim", ctypes.c_int), ("temperature", ctypes.c_int)]

    @classmethod
    def make(cls, pairs, lambda_area=True, temperature=True, lambda_perim=False):
        s = cls()
        s.n_pairs = len(pairs)
        for k, (a, b) in enumerate(pairs):
            s.pair_a[k], s.pair_b[k] = int(a), int(b)
        s.lambda_area = 1 if lambda_area else 0
        s.lambda_perim = 1 if lambda_perim else 0
        s.temperature = 1 if temperature else 0
        return s


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        l = ctypes.CDLL(str(path))
        u32p = ctypes.POINTER(ctypes.c_uint32)
        l.orc_philox4x32_10.argtypes = [u32p, u32p, u32p]
        l.orc_exp_neg.argtypes = [ctypes.c_float]
        l.orc_exp_neg.restype = ctypes.c_float
        for name in ("orc_log2_pos", "orc_exp2"):
            getattr(l, name).argtypes = [ctypes.c_float]
            getattr(l, name).restype = ctypes.c_float
        l.orc_init_tables.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
        l.orc_run.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                              ctypes.c_int, ctypes.c_void_p]
        l.orc_run_scores.argtypes = l.orc_run.argtypes + [ctypes.c_void_p,
                                                          ctypes.c_void_p]
        l.orc_voronoi.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p] * 3
        l.orc_boundaries.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_int,
                                                           ctypes.c_void_p]
        l.orc_init_prefdir.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_int, ctypes.c_void_p]
        l.orc_mean_coords.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]
        l.orc_persist_update.argtypes = [ctypes.POINTER(Params)] + [ctypes.c_void_p] * 6 + [
            ctypes.c_int, ctypes.c_int]
        l.orc_dh_error.argtypes = [ctypes.POINTER(Params)] + [ctypes.c_void_p] * 3 + [
            ctypes.c_int, ctypes.c_void_p]
        _lib = l
    return _lib


def philox4x32_10(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [int(v) for v in o]


def exp_neg(x: float) -> float:
    return float(lib().orc_exp_neg(float(x)))


def log2_pos(v: float) -> float:
    return float(lib().orc_log2_pos(float(v)))


def exp2(y: float) -> float:
    return float(lib().orc_exp2(float(y)))


class OracleSim:
    """One lattice plus its cell tables, advanced by the CPU oracle.

    `lattice` is a uint32 array of shape (ny, nx) or (nz, ny, nx) holding
    id | type << 24.  Parameters follow the engine's conventions: J[a][b] is
    the adhesion seen by a site of type a next to a site of type b; stick
    (optional, [a][b]) the stickiness, fixed (optional, per type) the
    unmovable types, chemo (optional, per type) the chemotaxis lambdas,
    field (optional, [ndim, (nz,) ny, nx]) the chemotaxis field, act_lambda /
    act_max (optional, per type) the act model and act (optional) its
    starting stamps (kept in self.act).  persist_lambda / persist_diff
    (optional, per type, 3D) the persistence term with a ring of `history`
    mean-coordinate slots: self.prefdir [ncells+1, 3] starts from
    (seed, stream) and every run() call ends with one update, as every
    engine run call does.
    """

    def __init__(self, lattice, ncells, J, lam_area, tgt_area,
                 lam_perim=None, tgt_perim=None, temperature=1.0, seed=0,
                 stream=0, stick=None, fixed=None, chemo=None, field=None,
                 act_lambda=None, act_max=None, act=None, persist_lambda=None,
                 persist_diff=None, history=1):
        lat = np.ascontiguousarray(lattice, dtype=np.uint32).copy()
        self.ndim = lat.ndim
        self.lattice = lat
        self.ncells = int(ncells)
        p = Params()
        p.ndim = self.ndim
        if self.ndim == 2:
            p.nz, (p.ny, p.nx) = 1, lat.shape
        else:
            p.nz, p.ny, p.nx = lat.shape
        p.ncells = self.ncells
        Jm = np.zeros((MAX_TYPES, MAX_TYPES), np.float32)
        Jin = np.asarray(J, np.float32)
        Jm[:Jin.shape[0], :Jin.shape[1]] = Jin
        p.J[:] = Jm.ravel().tolist()

        def fill(dst, src, dt):
            arr = np.zeros(MAX_TYPES, dt)
            if src is not None:
                s = np.asarray(src, dt).ravel()
                arr[:s.size] = s
            dst[:] = arr.tolist()
        fill(p.lam_area, lam_area, np.float32)
        fill(p.tgt_area, tgt_area, np.int32)
        fill(p.lam_perim, lam_perim, np.float32)
        fill(p.tgt_perim, tgt_perim, np.int32)
        p.temperature = float(temperature)
        p.seed = int(seed)
        p.stream = int(stream)
        Sm = np.zeros((MAX_TYPES, MAX_TYPES), np.float32)
        if stick is not None:
            Sin = np.asarray(stick, np.float32)
            Sm[:Sin.shape[0], :Sin.shape[1]] = Sin
        p.stick[:] = Sm.ravel().tolist()
        mask = 0
        for t, f in enumerate(np.zeros(0) if fixed is None else np.asarray(fixed).ravel()):
            if f:
                mask |= 1 << t
        p.fixed_mask = mask
        fill(p.chemo, chemo, np.float32)
        self.field = None
        if field is not None:  # [ndim, (nz,) ny, nx], rounded to float as the engine does
            self.field = np.ascontiguousarray(field, dtype=np.float32)
            if self.field.shape != (self.ndim,) + lat.shape:
                raise ValueError("field must have shape (ndim,) + lattice shape")
            p.field = self.field.ctypes.data
        fill(p.act_lambda, act_lambda, np.float32)
        fill(p.act_max, act_max, np.int32)
        self.act = None
        if act is not None or (act_lambda is not None and np.any(np.asarray(act_lambda) != 0)):
            # act stamps (MCS of the last copy into each site), zero to start
            self.act = (np.zeros(lat.shape, np.uint32) if act is None
                        else np.ascontiguousarray(act, dtype=np.uint32).copy())
            p.act = self.act.ctypes.data
        fill(p.persist_lambda, persist_lambda, np.float32)
        self.persist_diff = np.zeros(MAX_TYPES, np.float32)
        if persist_diff is not None:
            d = np.asarray(persist_diff, np.float32).ravel()
            self.persist_diff[:d.size] = d
        self.prefdir = None
        persist = (self.ndim == 3 and persist_lambda is not None
                   and np.any(np.asarray(persist_lambda) != 0))
        if persist:
            self.prefdir = np.zeros((self.ncells + 1, 3), np.float64)
            lib().orc_init_prefdir(ctypes.c_uint64(int(seed)), ctypes.c_uint32(int(stream)),
                                   ctypes.c_uint32(0), self.ncells, self.prefdir.ctypes.data)
            p.prefdir = self.prefdir.ctypes.data
        self.params = p
        n1 = self.ncells + 1
        self.area = np.zeros(n1, np.int32)
        self.perim = np.zeros(n1, np.int32)
        self.csum = np.zeros((n1, self.ndim), np.int64)
        self.tick = 0
        self.counters = np.zeros(3, np.uint64)
        err = lib().orc_init_tables(ctypes.byref(p), self.lattice.ctypes.data,
                                    self.area.ctypes.data,
                                    self.perim.ctypes.data,
                                    self.csum.ctypes.data)
        if err:
            raise ValueError(f"invalid lattice (oracle error bits {err})")
        if self.prefdir is not None:
            # the type of every id (-1 for ids without sites), and every
            # history slot holding the means at the start
            self.ctype = np.full(self.ncells + 1, -1, np.int32)
            self.ctype[self.lattice.ravel() & 0xFFFFFF] = self.lattice.ravel() >> 24
            self.history = int(history)
            self.hist = np.empty((self.history, self.ncells + 1, 3), np.float64)
            self.hist[:] = self.mean_coords()
            self.hist_slot = 0

    def mean_coords(self):
        """[ncells+1, 3] mean coordinate of every cell, in [0, n) per axis."""
        out = np.zeros((self.ncells + 1, 3), np.float64)
        lib().orc_mean_coords(ctypes.byref(self.params), self.area.ctypes.data,
                              self.csum.ctypes.data, out.ctypes.data)
        return out

    def run(self, mcs: int, nthreads: int = 0):
        lib().orc_run(ctypes.byref(self.params), self.lattice.ctypes.data,
                      self.area.ctypes.data, self.perim.ctypes.data,
                      self.csum.ctypes.data, self.tick, int(mcs),
                      int(nthreads), self.counters.ctypes.data)
        self.tick += int(mcs)
        if self.prefdir is not None and int(mcs) > 0:
            lib().orc_persist_update(ctypes.byref(self.params), self.area.ctypes.data,
                                     self.csum.ctypes.data, self.ctype.ctypes.data,
                                     self.persist_diff.ctypes.data, self.prefdir.ctypes.data,
                                     self.hist.ctypes.data, self.history, self.hist_slot)
            self.hist_slot = (self.hist_slot + 1) % self.history
        return self

    def run_scores(self, mcs: int, spec, nthreads: int = 0):
        """run() that also returns the FP64 likelihood-ratio scores, one row
        of 8 (parameters in the spec's order) per MCS.  `spec` is a
        ctypes structure with cpm_score_spec's layout."""
        scores = np.zeros((int(mcs), 8), np.float64)
        lib().orc_run_scores(ctypes.byref(self.params), self.lattice.ctypes.data,
                             self.area.ctypes.data, self.perim.ctypes.data,
                             self.csum.ctypes.data, self.tick, int(mcs),
                             int(nthreads), self.counters.ctypes.data,
                             ctypes.byref(spec), scores.ctypes.data)
        self.tick += int(mcs)
        return scores

    def dh_error(self, nthreads=0):
        """FP32 dH (the sweep's arithmetic) against an FP64 recomputation over
        every (target, neighbouring source of another id) pair of the current
        state: dict(pairs, max_abs, max_rel, max_rel_dh, max_accept_prob_diff,
        sign_flips); max_rel divides by the sum of the terms' magnitudes,
        max_rel_dh by max(|dH64|, 1).  Adhesion, stickiness, perimeter and
        area terms."""
        out = np.zeros(6, np.float64)
        lib().orc_dh_error(ctypes.byref(self.params), self.lattice.ctypes.data,
                           self.area.ctypes.data, self.perim.ctypes.data, int(nthreads),
                           out.ctypes.data)
        return {"pairs": int(out[0]), "max_abs": float(out[1]), "max_rel": float(out[2]),
                "max_rel_dh": float(out[5]), "max_accept_prob_diff": float(out[3]),
                "sign_flips": int(out[4])}

    def recount(self):
        """Tables recomputed from scratch from the current lattice."""
        n1 = self.ncells + 1
        area = np.zeros(n1, np.int32)
        perim = np.zeros(n1, np.int32)
        csum = np.zeros((n1, self.ndim), np.int64)
        err = lib().orc_init_tables(ctypes.byref(self.params),
                                    self.lattice.ctypes.data, area.ctypes.data,
                                    perim.ctypes.data, csum.ctypes.data)
        if err:
            raise ValueError(f"invalid lattice (oracle error bits {err})")
        return area, perim, csum


def voronoi(shape, points, values):
    """Brute-force periodic Voronoi lattice (uint32, shape [(nz,) ny, nx]):
    each site takes values[k] of its nearest point (min-image distance in
    double, ties to the lowest k); points [npoints, ndim], x first."""
    shape = tuple(int(v) for v in shape)
    ndim = len(shape)
    nx, ny = shape[-1], shape[-2]
    nz = shape[0] if ndim == 3 else 1
    pts = np.ascontiguousarray(points, np.float64)
    vals = np.ascontiguousarray(values, np.uint32)
    out = np.zeros(shape, np.uint32)
    lib().orc_voronoi(ndim, nx, ny, nz, len(vals), pts.ctypes.data, vals.ctypes.data,
                      out.ctypes.data)
    return out


def boundaries(lattice, ntypes):
    """[ntypes, ntypes] uint64 boundary counts by unordered type pair (a <= b)
    of one lattice: Moore pairs, each once, of sites with different values."""
    lat = np.ascontiguousarray(lattice, np.uint32)
    ndim = lat.ndim
    nx, ny = lat.shape[-1], lat.shape[-2]
    nz = lat.shape[0] if ndim == 3 else 1
    out = np.zeros((ntypes, ntypes), np.uint64)
    lib().orc_boundaries(ndim, nx, ny, nz, lat.ctypes.data, int(ntypes), out.ctypes.data)
    return out
