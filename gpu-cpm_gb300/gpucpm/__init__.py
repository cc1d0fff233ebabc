"""gpucpm — drop-in replacement for shabaz/gpu-cpm's Python module, on GB300.

`gpucpm.Cpm` keeps the reference's constructor and method set
(src/python_wrapper.cpp:365-380): set_constraints, add_cell, push_to_gpu,
run, synchronize, pull_from_gpu, get_state, get_centroids, get_act_state and
get_field.  Every call goes through the C-ABI of libgpucpm_gb300.so
(include/gpucpm.h); there is no CPU fallback — importing this module on a
machine without the built library raises ImportError, and a CUDA failure
raises CpmError.

Differences from the reference, all deliberate:
  * errors raise CpmError instead of printing and continuing
    (src/cpm.cu:52-56) or returning False (src/python_wrapper.cpp:87,138,217);
  * adhesion and temperature accept floats (the reference parses int);
  * set_adhesion_symmetric is honoured (the reference parses an int into a
    double that stays non-zero, so it always sets both entries,
    src/python_wrapper.cpp:81-86);
  * runs are reproducible: the random stream is keyed by a seed (default 0,
    see set_seed) instead of std::random_device (src/cpm.cu:347-350);
  * get_state's array keeps its Cpm alive (the reference's view dangles
    once the object is freed);
  * stickiness accepts floats; fixed and stickiness apply whatever the
    run() toggles (the reference applies fixed types only when
    partial_dispatch is off or some type is fixed, src/cpm.cu:308-320,
    which for a non-zero fixed flag is the same);
  * the chemotaxis field is float on the device (the reference keeps
    doubles) and the chemotaxis energy is summed in FP32, rounded step by
    step; get_field's array exists whether or not has_field was set.
  * the act model's geometric means use this library's own FP32 log2 /
    exp2 (the reference uses the fast __powf), and copies of runs with an
    act lambda are written at the end of their phase (see cpm_set_act).
  * persistence (3D only, as in the reference) draws the initial preferred
    directions from (seed, stream) instead of std::random_device, and its
    energy is summed in FP32 like chemotaxis.  Cpm.run makes one engine run
    per inner_iterations chunk when persistence is on, because the
    preferred directions are updated once per engine run (the reference
    updates them once per launch of its run loop).
"""
import ctypes
import os
import pathlib

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE.parent / "libgpucpm_gb300.so"

CPM_OK = 0
CPM_ERR_INVALID = 1
CPM_ERR_CUDA = 2
CPM_ERR_ALLOC = 3
CPM_ERR_STATE = 4
CPM_ERR_TIMEOUT = 5
CPM_ERR_UNSUPPORTED = 6
MAX_TYPES = 32
CPM_FLAG_FIELD = 1
CPM_FLAG_ACT = 2
DISPATCH_GRID = 0
DISPATCH_REPLICA = 1
DISPATCH_HYBRID = 2
FILL_PARITY = 0
FILL_VECTOR = 1
FILL_TMA = 2
FILL_CLUSTER = 3
FILL_NAMES = {FILL_PARITY: "parity", FILL_VECTOR: "vector", FILL_TMA: "tma",
              FILL_CLUSTER: "cluster"}


class CpmError(RuntimeError):
    """A libgpucpm_gb300 call returned a non-zero status."""

    def __init__(self, code, message):
        super().__init__(f"[status {code}] {message}")
        self.code = code


class _Counters(ctypes.Structure):
    _fields_ = [("attempts", ctypes.c_uint64), ("evaluated", ctypes.c_uint64),
                ("accepted", ctypes.c_uint64)]


SCORE_MAX = 8


class ScoreSpec(ctypes.Structure):
    """cpm_score_spec: J type pairs, then lambda_area, lambda_perim, T (flags)."""
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

    @property
    def nparam(self):
        return self.n_pairs + self.lambda_area + self.lambda_perim + self.temperature


class StaticParams(ctypes.Structure):
    """cpm_static_params of include/gpucpm.h (parameters of sweep_static)."""
    _fields_ = [("J", ctypes.c_float * (MAX_TYPES * MAX_TYPES)),
                ("lambda_area", ctypes.c_float * MAX_TYPES),
                ("target_area", ctypes.c_int * MAX_TYPES),
                ("lambda_perimeter", ctypes.c_float * MAX_TYPES),
                ("target_perimeter", ctypes.c_int * MAX_TYPES),
                ("temperature", ctypes.c_float),
                ("stickiness", ctypes.c_float * (MAX_TYPES * MAX_TYPES)),
                ("fixed", ctypes.c_int * MAX_TYPES),
                ("chemotaxis", ctypes.c_float * MAX_TYPES),
                ("act_lambda", ctypes.c_float * MAX_TYPES),
                ("act_max", ctypes.c_int * MAX_TYPES),
                ("persistence_lambda", ctypes.c_float * MAX_TYPES),
                ("persistence_diffusion", ctypes.c_float * MAX_TYPES),
                ("persistence_time", ctypes.c_int * MAX_TYPES)]


class _DeviceArray:
    """__cuda_array_interface__ (version 3) of engine-owned device memory;
    a tensor made from it holds this object, which holds the engine."""

    def __init__(self, ptr, shape, owner, typestr="<i4"):
        self._owner = owner
        self.__cuda_array_interface__ = {"shape": tuple(int(v) for v in shape),
                                         "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None, "stream": None}


_lib = None


def library():
    """The loaded C-ABI library (ctypes.CDLL); raises ImportError if absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("GPUCPM_LIB", str(LIB_PATH))
    if not os.path.exists(path):
        raise ImportError(
            f"libgpucpm_gb300.so not found at {path}; build it with "
            "`python gpu-cpm_gb300/build.py` (no CPU fallback exists)")
    L = ctypes.CDLL(path)
    H = ctypes.c_void_p
    ip = ctypes.POINTER(ctypes.c_int)
    sig = {
        "cpm_create": [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                       ctypes.c_int, ctypes.POINTER(H)],
        "cpm_create_box": [ctypes.c_int] * 5 + [ctypes.c_float, ctypes.POINTER(H)],
        "cpm_create_batch": [ctypes.c_int, ctypes.c_int, ip, ip, ip, ip,
                             ctypes.POINTER(H)],
        "cpm_destroy": [H],
        "cpm_set_temperature": [H, ctypes.c_float],
        "cpm_set_temperature_r": [H, ctypes.c_int, ctypes.c_float],
        "cpm_set_area": [H, ctypes.c_int, ctypes.c_int, ctypes.c_float],
        "cpm_set_area_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float],
        "cpm_set_perimeter": [H, ctypes.c_int, ctypes.c_int, ctypes.c_float],
        "cpm_set_perimeter_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_float],
        "cpm_set_adhesion": [H, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int],
        "cpm_set_adhesion_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                               ctypes.c_float, ctypes.c_int],
        "cpm_set_fixed": [H, ctypes.c_int, ctypes.c_int],
        "cpm_set_chemotaxis": [H, ctypes.c_int, ctypes.c_float],
        "cpm_set_act": [H, ctypes.c_int, ctypes.c_int, ctypes.c_float],
        "cpm_set_act_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float],
        "cpm_host_act_r": [H, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                           ctypes.POINTER(ctypes.c_int64)],
        "cpm_has_act": [H, ctypes.POINTER(ctypes.c_int)],
        "cpm_set_chemotaxis_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_float],
        "cpm_set_persistence": [H, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float],
        "cpm_set_persistence_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                  ctypes.c_float],
        "cpm_set_history": [H, ctypes.c_int],
        "cpm_has_persistence": [H, ip, ip],
        "cpm_get_persistence_r": [H, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
        "cpm_set_persistence_state_r": [H, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
        "cpm_host_field_r": [H, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                             ctypes.POINTER(ctypes.c_int64)],
        "cpm_set_fixed_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int],
        "cpm_set_stickiness": [H, ctypes.c_int, ctypes.c_int, ctypes.c_float],
        "cpm_set_stickiness_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float],
        "cpm_add_cell": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int],
        "cpm_host_lattice": [H, ctypes.POINTER(ctypes.c_void_p),
                             ctypes.POINTER(ctypes.c_int64)],
        "cpm_host_lattice_r": [H, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                               ctypes.POINTER(ctypes.c_int64)],
        "cpm_device_lattice_r": [H, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)],
        "cpm_push": [H],
        "cpm_pull": [H],
        "cpm_run": [H, ctypes.c_int],
        "cpm_synchronize": [H],
        "cpm_set_stream": [H, ctypes.c_void_p],
        "cpm_set_seed": [H, ctypes.c_uint64, ctypes.c_uint32],
        "cpm_get_tick": [H, ctypes.POINTER(ctypes.c_uint64)],
        "cpm_set_tick": [H, ctypes.c_uint64],
        "cpm_get_centroids": [H, ctypes.c_void_p, ctypes.c_int, ip],
        "cpm_get_tables_r": [H, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.c_void_p],
        "cpm_get_counters": [H, ctypes.POINTER(_Counters)],
        "cpm_get_counters_r": [H, ctypes.c_int, ctypes.POINTER(_Counters)],
        "cpm_reset_counters": [H],
        "cpm_info": [H, ip, ip, ip, ctypes.POINTER(ctypes.c_uint64)],
        "cpm_run_graph": [H, ctypes.c_int],
        "cpm_autotune": [H, ctypes.c_int, ip, ctypes.POINTER(ctypes.c_float)],
        "cpm_set_variant": [H, ctypes.c_int],
        "cpm_sweep_config": [H, ip, ip, ip, ip, ip, ip, ip],
        "cpm_set_dispatch": [H, ctypes.c_int],
        "cpm_set_fill": [H, ctypes.c_int],
        "cpm_get_fill": [H, ip],
        "cpm_recount": [H],
        "cpm_set_centroid_sums_r": [H, ctypes.c_int, ctypes.c_void_p],
        "cpm_get_params_r": [H, ctypes.c_int, ctypes.POINTER(StaticParams)],
        "cpm_set_params_r": [H, ctypes.c_int, ctypes.POINTER(StaticParams)],
        "cpm_set_params": [H, ctypes.POINTER(StaticParams)],
        "cpm_get_param_index": [H, ctypes.c_void_p],
        "cpm_get_seed": [H, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32)],
        "cpm_get_device": [H, ctypes.POINTER(ctypes.c_int)],
        "cpm_run_scores": [H, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                           ctypes.POINTER(ScoreSpec)],
        "cpm_observe_heterotypic": [H, ctypes.c_void_p],
        "cpm_observe_boundaries": [H, ctypes.c_int, ctypes.c_void_p],
        "cpm_seed_voronoi_r": [H, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.cpm_sweep_static.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p] * 4 + [
        ctypes.c_int, ctypes.POINTER(StaticParams), ctypes.c_uint64, ctypes.c_uint32,
        ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
    L.cpm_sweep_static.restype = ctypes.c_int
    L.cpm_lr_backward.argtypes = [ctypes.c_void_p] * 3 + [ctypes.POINTER(ctypes.c_int)] + [
        ctypes.c_int] * 4 + [ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_void_p,
                             ctypes.c_void_p]
    L.cpm_lr_backward.restype = ctypes.c_int
    L.cpm_set_device.argtypes = [ctypes.c_int]
    L.cpm_set_device.restype = ctypes.c_int
    L.cpm_debug_barrier_timeout.argtypes = [ctypes.c_uint64, ip]
    L.cpm_debug_barrier_timeout.restype = ctypes.c_int
    L.cpm_last_error.argtypes = [H]
    L.cpm_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def _check(rc, handle=None):
    if rc != CPM_OK:
        msg = library().cpm_last_error(handle)
        raise CpmError(rc, msg.decode() if msg else "unknown error")


def _int_array(values):
    a = (ctypes.c_int * len(values))(*[int(v) for v in values])
    return a


class _Engine:
    """Owner of one C handle (a single lattice or a batch of replicas)."""

    def __init__(self, handle):
        self._h = handle
        self._lib = library()
        n, d, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(self._lib.cpm_info(self._h, ctypes.byref(n), ctypes.byref(d),
                                  ctypes.byref(g), None), self._h)
        self.n_replicas, self.dimensionality, self.sweep_grid = n.value, d.value, g.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.cpm_destroy(h)
            self._h = None

    def _call(self, name, *args):
        _check(getattr(self._lib, name)(self._h, *args), self._h)

    # -- shared helpers ---------------------------------------------------
    def _host_view(self, replica, shape):
        ptr, n = ctypes.c_void_p(), ctypes.c_int64()
        self._call("cpm_host_lattice_r", int(replica), ctypes.byref(ptr),
                   ctypes.byref(n))
        buf = (ctypes.c_int32 * n.value).from_address(ptr.value)
        buf._owner = self  # the array keeps this engine (and its memory) alive
        return np.ctypeslib.as_array(buf).reshape(shape)

    def field(self, replica=0):
        """Writable host view of a replica's chemotaxis field, float64
        [ndim, (nz,) ny, nx] (component k = x, y, z), zero until written;
        pushed with the lattice."""
        ptr, n = ctypes.c_void_p(), ctypes.c_int64()
        self._call("cpm_host_field_r", int(replica), ctypes.byref(ptr), ctypes.byref(n))
        buf = (ctypes.c_double * n.value).from_address(ptr.value)
        buf._owner = self
        return np.ctypeslib.as_array(buf).reshape((self.dimensionality,)
                                                  + tuple(self._replica_shape(replica)))

    def act_lattice(self, replica=0):
        """Writable host view (int32, as the reference's get_act_state) of a
        replica's act stamps: the MCS of the last copy into each site."""
        ptr, n = ctypes.c_void_p(), ctypes.c_int64()
        self._call("cpm_host_act_r", int(replica), ctypes.byref(ptr), ctypes.byref(n))
        buf = (ctypes.c_int32 * n.value).from_address(ptr.value)
        buf._owner = self
        return np.ctypeslib.as_array(buf).reshape(tuple(self._replica_shape(replica)))

    def set_history(self, history):
        """Slots of the mean-coordinate ring of the persistence update (the
        reference's `history` constructor argument), >= 1."""
        self._call("cpm_set_history", int(history))

    @property
    def history(self):
        v = ctypes.c_int()
        self._call("cpm_has_persistence", None, ctypes.byref(v))
        return v.value

    @property
    def persistence_exists(self):
        """Whether preferred directions exist (a 3D run with persistence)."""
        v = ctypes.c_int()
        self._call("cpm_has_persistence", ctypes.byref(v), None)
        return bool(v.value)

    def persistence_state(self, replica=0):
        """(prefdir [ncells+1, 3], history [history, ncells+1, 3] oldest
        first), float64 copies; None while no persistence state exists."""
        if not self.persistence_exists:
            return None
        n1 = self._ncells(replica) + 1
        pd = np.empty((n1, 3), np.float64)
        hist = np.empty((self.history, n1, 3), np.float64)
        self._call("cpm_get_persistence_r", int(replica), pd.ctypes.data, hist.ctypes.data)
        return pd, hist

    def set_persistence_state(self, replica, prefdir, history=None):
        """Restore a replica's preferred directions (and optionally its
        ring, oldest slot first); the engine must be pushed and 3D."""
        n1 = self._ncells(replica) + 1
        pd = np.ascontiguousarray(prefdir, np.float64)
        if pd.shape != (n1, 3):
            raise CpmError(CPM_ERR_INVALID, f"prefdir must have shape ({n1}, 3)")
        hp = None
        if history is not None:
            hist = np.ascontiguousarray(history, np.float64)
            if hist.shape != (self.history, n1, 3):
                raise CpmError(CPM_ERR_INVALID,
                               f"history must have shape ({self.history}, {n1}, 3)")
            hp = hist.ctypes.data
        self._call("cpm_set_persistence_state_r", int(replica), pd.ctypes.data, hp)

    @property
    def act_exists(self):
        """Whether the act stamps are allocated (has_act, or first use)."""
        v = ctypes.c_int()
        self._call("cpm_has_act", ctypes.byref(v))
        return bool(v.value)

    def host_lattice(self, replica=0):
        """Writable host view of a replica's lattice ([y, x] / [z, y, x])."""
        return self._host_view(replica, self._replica_shape(replica))

    def device_lattice(self, replica=0):
        """Zero-copy torch.int32 CUDA tensor of a replica's device lattice
        (shape as host_lattice; values id | type << 24).  It shows the state
        after the last completed run: call synchronize() first.  Writing to
        it changes the engine's lattice; call recount() afterwards so that
        the tables describe it again.  The tensor keeps the engine alive."""
        import torch
        view = _DeviceArray(self.device_lattice_ptr(replica), self._replica_shape(replica), self)
        return torch.as_tensor(view, device=torch.device("cuda", self.device))

    @property
    def device(self):
        d = ctypes.c_int()
        self._call("cpm_get_device", ctypes.byref(d))
        return d.value

    def recount(self):
        """Revalidate the device lattices and recompute all tables from
        them (push_to_gpu without the host copy)."""
        self._call("cpm_recount")

    def set_centroid_sums(self, replica, centroid_sums):
        """Restore a replica's centroid sums (as tables() returned them),
        after a push: they depend on the path, area and perimeter do not."""
        cs = np.ascontiguousarray(centroid_sums, dtype=np.int64)
        if cs.shape != (self._ncells(replica) + 1, self.dimensionality):
            raise CpmError(CPM_ERR_INVALID, f"centroid sums must have shape "
                           f"{(self._ncells(replica) + 1, self.dimensionality)}")
        self._call("cpm_set_centroid_sums_r", int(replica), cs.ctypes.data)

    def get_params(self, replica=0):
        """A replica's parameters as a StaticParams record."""
        p = StaticParams()
        self._call("cpm_get_params_r", int(replica), ctypes.byref(p))
        return p

    def set_params(self, replica, params):
        """Set a replica's parameters from a StaticParams record (replica
        None: every replica)."""
        if replica is None:
            self._call("cpm_set_params", ctypes.byref(params))
        else:
            self._call("cpm_set_params_r", int(replica), ctypes.byref(params))

    def param_index(self):
        """Per replica, the parameter record it uses (equal values share)."""
        out = np.empty(self.n_replicas, np.int32)
        self._call("cpm_get_param_index", out.ctypes.data)
        return out

    @property
    def seed(self):
        """(seed, stream_id) of the Philox stream."""
        s, k = ctypes.c_uint64(), ctypes.c_uint32()
        self._call("cpm_get_seed", ctypes.byref(s), ctypes.byref(k))
        return s.value, k.value

    def device_lattice_ptr(self, replica=0):
        """Device address of a replica's lattice (uint32, row-major)."""
        p = ctypes.c_void_p()
        self._call("cpm_device_lattice_r", int(replica), ctypes.byref(p))
        return p.value

    def set_stream(self, stream):
        """Enqueue work on a caller-owned CUDA stream (a cudaStream_t as int,
        e.g. torch.cuda.Stream().cuda_stream); None restores the own stream."""
        self._call("cpm_set_stream", ctypes.c_void_p(int(stream) if stream else None))

    def set_seed(self, seed, stream_id=0):
        """Key of the Philox stream; replica r of a batch uses stream_id + r."""
        self._call("cpm_set_seed", ctypes.c_uint64(int(seed)), ctypes.c_uint32(int(stream_id)))

    @property
    def tick(self):
        t = ctypes.c_uint64()
        self._call("cpm_get_tick", ctypes.byref(t))
        return t.value

    @tick.setter
    def tick(self, value):
        self._call("cpm_set_tick", ctypes.c_uint64(int(value)))

    def tables(self, replica=0):
        """(area, perimeter, centroid_sums) of every id 0..number_of_cells."""
        n1 = self._ncells(replica) + 1
        area = np.empty(n1, np.int32)
        perim = np.empty(n1, np.int32)
        cs = np.empty((n1, self.dimensionality), np.int64)
        self._call("cpm_get_tables_r", int(replica), area.ctypes.data,
                   perim.ctypes.data, cs.ctypes.data)
        return area, perim, cs

    def counters(self, replica=None):
        """dict(attempts, evaluated, accepted) since the last reset."""
        c = _Counters()
        if replica is None:
            self._call("cpm_get_counters", ctypes.byref(c))
        else:
            self._call("cpm_get_counters_r", int(replica), ctypes.byref(c))
        return {"attempts": c.attempts, "evaluated": c.evaluated, "accepted": c.accepted}

    def reset_counters(self):
        self._call("cpm_reset_counters")

    def kernel_launches(self):
        k = ctypes.c_uint64()
        self._call("cpm_info", None, None, None, ctypes.byref(k))
        return k.value

    def push_to_gpu(self):
        self._call("cpm_push")

    def pull_from_gpu(self):
        self._call("cpm_pull")

    def synchronize(self):
        self._call("cpm_synchronize")

    def run_mcs(self, mcs):
        """Enqueue `mcs` Monte Carlo steps (asynchronous)."""
        self._call("cpm_run", int(mcs))

    def run_graph(self, mcs):
        """Enqueue `mcs` MCS as one replay of a captured CUDA graph."""
        self._call("cpm_run_graph", int(mcs))

    def autotune(self, probe_mcs=2):
        """Pick the fastest tile variant on the current state (state kept).
        Returns (variant, ms per MCS)."""
        v, ms = ctypes.c_int(), ctypes.c_float()
        self._call("cpm_autotune", int(probe_mcs), ctypes.byref(v), ctypes.byref(ms))
        return v.value, ms.value

    def set_variant(self, variant):
        """Warp tile in targets: 0 = 32x6 (3D 32x2x2), 1 = 32x8 (32x4x2),
        2 = 32x16 (32x4x4), 3 = 32x1 (32x1x1, for lattices too small to
        give every warp a wider tile).  The result does not depend on it."""
        self._call("cpm_set_variant", int(variant))

    def set_dispatch(self, dispatch):
        """DISPATCH_GRID (all warps on every slot of all replicas),
        DISPATCH_REPLICA (a block runs whole replicas) or DISPATCH_HYBRID
        (grid over the largest replicas, then replica dispatch over whole
        rounds of the rest); same results."""
        self._call("cpm_set_dispatch", int(dispatch))

    def run_scores(self, mcs, scores_ptr, score_base, score_len, spec):
        """cpm_run plus likelihood-ratio scores into a device float buffer
        [n_replicas][score_len][SCORE_MAX] (2D engines)."""
        self._call("cpm_run_scores", int(mcs), ctypes.c_void_p(int(scores_ptr)),
                   ctypes.c_uint64(int(score_base)), int(score_len), ctypes.byref(spec))

    def observe_heterotypic(self):
        """Per replica: fraction of Moore pairs of two different cells whose
        types differ (the sorting order parameter).  Synchronous."""
        out = np.empty(self.n_replicas, np.float32)
        self._call("cpm_observe_heterotypic", out.ctypes.data)
        return out

    def boundary_counts(self, ntypes):
        """uint64 [n_replicas, ntypes, ntypes]: Moore neighbour pairs (each
        once) of sites with different values, by unordered type pair (a <= b)
        — the boundary lengths between types, medium (type 0) included.
        Read from the device lattices.  Synchronous."""
        out = np.empty((self.n_replicas, int(ntypes), int(ntypes)), np.uint64)
        self._call("cpm_observe_boundaries", int(ntypes), out.ctypes.data)
        return out

    def seed_voronoi(self, replica, points, values):
        """Fill a replica's device lattice with the periodic Voronoi tiling of
        `points` ([npoints, ndim] in [0, n), x first): each site takes
        values[k] (id | type << 24) of its nearest point, ties to the lowest
        k.  The tables are stale until recount() (or pull + push)."""
        pts = np.ascontiguousarray(points, np.float64)
        vals = np.ascontiguousarray(values, np.uint32)
        if pts.ndim != 2 or pts.shape[1] != self.dimensionality or len(vals) != len(pts):
            raise CpmError(CPM_ERR_INVALID, "points must be [npoints, ndim] with one value each")
        self._call("cpm_seed_voronoi_r", int(replica), len(vals), pts.ctypes.data,
                   vals.ctypes.data)

    def sweep_config(self):
        """dict(variant, tile, warps_per_block, grid, dispatch, fill) of the
        launch runs use."""
        vals = [ctypes.c_int() for _ in range(7)]
        self._call("cpm_sweep_config", *[ctypes.byref(v) for v in vals])
        v, tx, ty, tz, w, g, d = (x.value for x in vals)
        return {"variant": v, "tile": (tx, ty, tz), "warps_per_block": w, "grid": g,
                "dispatch": {DISPATCH_REPLICA: "replica",
                             DISPATCH_HYBRID: "hybrid"}.get(d, "grid"),
                "fill": FILL_NAMES[self.fill]}

    @property
    def fill(self):
        """How the sweep stages its tiles: FILL_PARITY, FILL_VECTOR, FILL_TMA
        or FILL_CLUSTER (see cpm_set_fill)."""
        f = ctypes.c_int()
        self._call("cpm_get_fill", ctypes.byref(f))
        return f.value

    def set_fill(self, fill):
        self._call("cpm_set_fill", int(fill))


class Cpm(_Engine):
    """Cellular Potts simulation on one lattice (reference: gpucpm.Cpm).

    Cpm(dimension, dimensionality, number_of_cells, temperature, has_field,
        history=1, has_act=1) — the argument order of PyCpm_init
    (src/python_wrapper.cpp:27-41).  has_field allocates the chemotaxis
    field and has_act the act stamps up front (both also appear on first
    use); history sets the ring of the 3D persistence update.
    """

    def __init__(self, dimension, dimensionality, number_of_cells, temperature,
                 has_field=False, history=1, has_act=1):
        lib = library()
        h = ctypes.c_void_p()
        _check(lib.cpm_create(int(dimension), int(dimensionality),
                              int(number_of_cells), float(temperature),
                              (CPM_FLAG_FIELD if has_field else 0)
                              | (CPM_FLAG_ACT if has_act else 0), ctypes.byref(h)), None)
        super().__init__(h)
        self.dimension = int(dimension)
        self.number_of_cells = int(number_of_cells)
        self.has_field = bool(has_field)
        self.has_act = bool(has_act)
        self._shape = (self.dimension,) * self.dimensionality
        self._persistence = False
        self.set_history(history)

    def _ncells(self, replica):
        return self.number_of_cells

    def _replica_shape(self, replica):
        return self._shape

    def set_constraints(self, cell_type, *, other_cell_type=-1,
                        lambda_perimeter=-1, target_perimeter=-1,
                        lambda_area=-1, target_area=-1, lambda_act=-1,
                        max_act=-1, adhesion=-1, fixed=-1,
                        lambda_chemotaxis=-1, lambda_persistence=-1,
                        persistence_diffusion=-1, persistence_time=-1,
                        set_adhesion_symmetric=1, stickiness=-1):
        """Set per-type Hamiltonian parameters (src/python_wrapper.cpp:55-129).

        A group is applied only when all of its fields differ from -1, as in
        the reference (fixed: any value >= 0).  Groups of terms outside this
        engine raise CpmError.
        """
        ct = int(cell_type)
        if (lambda_persistence != -1 and persistence_diffusion != -1
                and persistence_time != -1):
            self._call("cpm_set_persistence", ct, int(persistence_time),
                       float(persistence_diffusion), float(lambda_persistence))
            if float(lambda_persistence) != 0.0:
                self._persistence = True
        if lambda_perimeter != -1 and target_perimeter != -1:
            self._call("cpm_set_perimeter", ct, int(target_perimeter), float(lambda_perimeter))
        if lambda_area != -1 and target_area != -1:
            self._call("cpm_set_area", ct, int(target_area), float(lambda_area))
        if fixed >= 0:
            self._call("cpm_set_fixed", ct, int(fixed))
        if lambda_act != -1 and max_act != -1:
            self._call("cpm_set_act", ct, int(max_act), float(lambda_act))
        if lambda_chemotaxis != -1:
            self._call("cpm_set_chemotaxis", ct, float(lambda_chemotaxis))
        if other_cell_type != -1 and adhesion != -1:
            self._call("cpm_set_adhesion", ct, int(other_cell_type), float(adhesion),
                       1 if set_adhesion_symmetric else 0)
        if other_cell_type != -1 and stickiness != -1:
            self._call("cpm_set_stickiness", ct, int(other_cell_type), float(stickiness))

    def set_temperature(self, temperature):
        self._call("cpm_set_temperature", float(temperature))

    def add_cell(self, type, x, y, z=-1):  # noqa: A002 - reference's keyword
        """Seed the next cell id of `type` at one site (src/cpm.cu:160-174)."""
        if self.dimensionality == 3 and z == -1:
            raise CpmError(CPM_ERR_INVALID, "add_cell needs z on a 3D lattice")
        self._call("cpm_add_cell", int(type), int(x), int(y), int(z if z != -1 else 0))

    def run(self, cell_sync, block_sync, global_sync, threads_per_block,
            positions_per_thread, positions_per_checkerboard,
            updates_per_checkerboard_switch, updates_per_barrier, iterations,
            inner_iterations, shared=0, partial_dispatch=0,
            centroid_tracking=0):
        """Run (iterations // inner_iterations) * inner_iterations MCS.

        Same arguments as the reference (src/python_wrapper.cpp:182-227).
        The launch-geometry, synchronisation and dispatch knobs have no
        meaning for this engine's schedule and are accepted for
        compatibility.  Asynchronous, like the reference's 2D run.
        """
        for name, v in (("cell_sync", cell_sync), ("block_sync", block_sync),
                        ("global_sync", global_sync),
                        ("threads_per_block", threads_per_block),
                        ("positions_per_thread", positions_per_thread),
                        ("positions_per_checkerboard", positions_per_checkerboard),
                        ("updates_per_checkerboard_switch", updates_per_checkerboard_switch),
                        ("updates_per_barrier", updates_per_barrier),
                        ("iterations", iterations), ("inner_iterations", inner_iterations)):
            if not isinstance(v, (int, np.integer)) or isinstance(v, bool):
                raise TypeError(f"{name} must be an int")
        inner = int(inner_iterations)
        if inner <= 0:
            raise CpmError(CPM_ERR_INVALID, "inner_iterations must be positive")
        total = (int(iterations) // inner) * inner
        if self._persistence and self.dimensionality == 3:
            for _ in range(total // inner):  # one direction update per chunk
                self.run_mcs(inner)
        elif total > 0:
            self.run_mcs(total)

    def get_state(self):
        """Writable int32 view of the host lattice, shape (D, D[, D]),
        indexed [y, x] / [z, y, x]; values are id | type << 24."""
        return self._host_view(0, self._shape)

    def get_centroids(self):
        """(n, d) float64 mean coordinates of the cells made by add_cell."""
        n = ctypes.c_int()
        self._call("cpm_get_centroids", None, 0, ctypes.byref(n))
        out = np.empty((n.value, self.dimensionality), np.float64)
        if n.value:
            self._call("cpm_get_centroids", out.ctypes.data, n.value, ctypes.byref(n))
        return out

    def get_act_state(self):
        """Writable int32 view of the act stamps, shape (D, D[, D]) as the
        reference's (src/python_wrapper.cpp:310-326)."""
        return self.act_lattice(0)

    def get_field(self):
        """Writable float64 view of the chemotaxis field, shape (d, D, D[, D])
        as the reference's (src/python_wrapper.cpp:274-290)."""
        return self.field(0)


class Batch(_Engine):
    """Many independent replicas advanced by one persistent launch.

    sizes: list of (nx, ny) in 2D or (nx, ny, nz) in 3D; ncells: list of
    cell counts.  Parameters are set per replica with the *_r setters.
    """

    def __init__(self, dimensionality, sizes, ncells):
        lib = library()
        n = len(sizes)
        if n == 0 or len(ncells) != n:
            raise CpmError(CPM_ERR_INVALID, "sizes and ncells must have equal, non-zero length")
        nx = _int_array([s[0] for s in sizes])
        ny = _int_array([s[1] for s in sizes])
        nz = _int_array([s[2] if dimensionality == 3 else 1 for s in sizes])
        nc = _int_array(ncells)
        h = ctypes.c_void_p()
        _check(lib.cpm_create_batch(n, int(dimensionality), nx, ny, nz, nc,
                                    ctypes.byref(h)), None)
        super().__init__(h)
        self.sizes = [tuple(int(v) for v in s) for s in sizes]
        self.ncells = [int(c) for c in ncells]

    def _ncells(self, replica):
        return self.ncells[replica]

    def _replica_shape(self, replica):
        return tuple(reversed(self.sizes[replica]))

    def lattice(self, replica):
        """Writable host view of one replica's lattice ([y, x] / [z, y, x])."""
        return self._host_view(replica, tuple(reversed(self.sizes[replica])))

    # replica None: every replica of the batch
    def set_temperature(self, replica, temperature):
        if replica is None:
            self._call("cpm_set_temperature", float(temperature))
        else:
            self._call("cpm_set_temperature_r", int(replica), float(temperature))

    def set_area(self, replica, cell_type, target, lam):
        if replica is None:
            self._call("cpm_set_area", int(cell_type), int(target), float(lam))
        else:
            self._call("cpm_set_area_r", int(replica), int(cell_type), int(target), float(lam))

    def set_perimeter(self, replica, cell_type, target, lam):
        if replica is None:
            self._call("cpm_set_perimeter", int(cell_type), int(target), float(lam))
        else:
            self._call("cpm_set_perimeter_r", int(replica), int(cell_type), int(target),
                       float(lam))

    def set_act(self, replica, cell_type, max_act, lam):
        if replica is None:
            self._call("cpm_set_act", int(cell_type), int(max_act), float(lam))
        else:
            self._call("cpm_set_act_r", int(replica), int(cell_type), int(max_act), float(lam))

    def set_persistence(self, replica, cell_type, time, diffusion, lam):
        """Persistence of a type (3D): lambda, diffusion and the stored-only
        time.  Preferred directions change once per run_mcs call."""
        if replica is None:
            self._call("cpm_set_persistence", int(cell_type), int(time), float(diffusion),
                       float(lam))
        else:
            self._call("cpm_set_persistence_r", int(replica), int(cell_type), int(time),
                       float(diffusion), float(lam))

    def set_chemotaxis(self, replica, cell_type, lam):
        if replica is None:
            self._call("cpm_set_chemotaxis", int(cell_type), float(lam))
        else:
            self._call("cpm_set_chemotaxis_r", int(replica), int(cell_type), float(lam))

    def set_fixed(self, replica, cell_type, fixed=True):
        if replica is None:
            self._call("cpm_set_fixed", int(cell_type), 1 if fixed else 0)
        else:
            self._call("cpm_set_fixed_r", int(replica), int(cell_type), 1 if fixed else 0)

    def set_stickiness(self, replica, cell_type, other, S):
        if replica is None:
            self._call("cpm_set_stickiness", int(cell_type), int(other), float(S))
        else:
            self._call("cpm_set_stickiness_r", int(replica), int(cell_type), int(other),
                       float(S))

    def set_adhesion(self, replica, cell_type, other, J, symmetric=True):
        if replica is None:
            self._call("cpm_set_adhesion", int(cell_type), int(other), float(J),
                       1 if symmetric else 0)
        else:
            self._call("cpm_set_adhesion_r", int(replica), int(cell_type), int(other),
                       float(J), 1 if symmetric else 0)


def sweep_static(dimensionality, shape, number_of_cells, lattice_ptr, area_ptr,
                 perimeter_ptr, centroid_sums_ptr, params, seed=0, stream_id=0,
                 tick=0, mcs=1, recount=False, stream=None):
    """Run `mcs` MCS on caller-owned device buffers without allocating.

    For callers that cannot allocate device memory (a framework-owned memory
    pool, a loop that must not allocate after start-up): the lattice and the
    tables are device pointers the caller owns, all other working memory is a
    fixed array inside the library (see cpm_sweep_static in
    include/gpucpm.h for the size limits).  `shape` is (nx, ny) or
    (nx, ny, nz); `params` a StaticParams.  Returns (evaluated, accepted).
    Synchronous; calls must not overlap on the GPU.
    """
    nx, ny = int(shape[0]), int(shape[1])
    nz = int(shape[2]) if dimensionality == 3 else 1
    c = (ctypes.c_uint64 * 2)()
    _check(library().cpm_sweep_static(
        int(dimensionality), nx, ny, nz, int(number_of_cells), lattice_ptr, area_ptr,
        perimeter_ptr, centroid_sums_ptr, 1 if recount else 0, ctypes.byref(params),
        int(seed), int(stream_id), int(tick), int(mcs),
        ctypes.c_void_p(int(stream) if stream else None), c), None)
    return int(c[0]), int(c[1])


def lr_backward(scores_ptr, dl_do_ptr, obs_ptr, checkpoints, nrep, length, nparam,
                grad_ptr, stream=None, obs_total=None, nrep_total=0):
    """Backward kernel of the likelihood-ratio estimator (device pointers):
    grad[k] = sum_r sum_c dL/dO[r,c] (O[r,c] - b[r,c])
                        * sum_{t < checkpoints[c]} scores[r,t,k],
    b[r,c] = mean of O[.,c] over the other replicas (0 for one replica).
    obs_total (host floats, one per checkpoint) and nrep_total extend "the
    other replicas" to every shard of a sharded ensemble."""
    cp = (ctypes.c_int * len(checkpoints))(*[int(c) for c in checkpoints])
    tot = None
    if obs_total is not None:
        tot = (ctypes.c_float * len(checkpoints))(*[float(v) for v in obs_total])
    _check(library().cpm_lr_backward(
        ctypes.c_void_p(int(scores_ptr)), ctypes.c_void_p(int(dl_do_ptr)),
        ctypes.c_void_p(int(obs_ptr)), cp, int(nrep), int(length), int(nparam),
        len(checkpoints), tot, int(nrep_total), ctypes.c_void_p(int(grad_ptr)),
        ctypes.c_void_p(int(stream) if stream else None)), None)


def set_device(device):
    """CUDA device that engines created later by this thread live on."""
    _check(library().cpm_set_device(int(device)), None)


def barrier_timeout_selftest(timeout_ns=50_000_000):
    """Status produced by a grid barrier that can never complete (expects
    CPM_ERR_TIMEOUT after about timeout_ns); the CUDA context stays usable."""
    st = ctypes.c_int()
    _check(library().cpm_debug_barrier_timeout(int(timeout_ns), ctypes.byref(st)), None)
    return st.value


def create_box(nx, ny, nz, dimensionality, number_of_cells, temperature):
    """A single lattice of any box shape (nz = 1 in 2D), as a Batch of one."""
    lib = library()
    h = ctypes.c_void_p()
    _check(lib.cpm_create_box(int(nx), int(ny), int(nz), int(dimensionality),
                              int(number_of_cells), float(temperature),
                              ctypes.byref(h)), None)
    b = Batch.__new__(Batch)
    _Engine.__init__(b, h)
    b.sizes = [(int(nx), int(ny)) if dimensionality == 2 else (int(nx), int(ny), int(nz))]
    b.ncells = [int(number_of_cells)]
    return b
