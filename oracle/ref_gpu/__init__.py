"""The reference's own CUDA sweep, driven from Python (test infrastructure).

`RefGpu` loads oracle/_ref/gpucpm_ref_sm103a.cubin (the reference's
src/kernels.cu compiled unchanged, see build.py) through ref_driver.cpp and
offers the reference's Cpm workflow: create, set parameters (short J, int T,
double lambdas, as src/settings.h stores them), push, run with the reference's
run() knobs and an explicit seed, synchronize, pull, and the area /
circumference tables.  Only one instance exists per process.
"""
import ctypes

import numpy as np

from .build import CUBIN, DRIVER, build

_lib = None


def available():
    return CUBIN.exists()


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(DRIVER))
        i, d = ctypes.c_int, ctypes.c_double
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_open.argtypes = [ctypes.c_char_p, i]
        L.ref_create.argtypes = [i, i, i, i]
        L.ref_set_area.argtypes = [i, i, d]
        L.ref_set_perimeter.argtypes = [i, i, d]
        L.ref_set_adhesion.argtypes = [i, i, i]
        L.ref_set_temperature.argtypes = [i]
        L.ref_set_stickiness.argtypes = [i, i, i]
        L.ref_set_fixed.argtypes = [i, i]
        L.ref_set_chemotaxis.argtypes = [i, d]
        L.ref_set_field.argtypes = [ctypes.c_void_p]
        L.ref_push.argtypes = [ctypes.c_void_p]
        L.ref_run.argtypes = [i] * 16
        L.ref_pull.argtypes = [ctypes.c_void_p]
        L.ref_tables.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ref_max_coop_blocks.argtypes = [i, i, i, ctypes.POINTER(i)]
        _lib = L
    return _lib


def _check(rc):
    if rc:
        raise RuntimeError(lib().ref_last_error().decode())


class RefGpu:
    def __init__(self, dimension, dimensionality, ncells, temperature, device=0):
        L = lib()
        _check(L.ref_open(str(CUBIN).encode(), int(device)))
        _check(L.ref_create(int(dimension), int(dimensionality), int(ncells),
                            int(round(temperature))))
        self.dimension, self.ndim, self.ncells = int(dimension), int(dimensionality), int(ncells)
        self.perimeter = False
        self.fixed = False
        self.chemotaxis = False

    def set_area(self, t, target, lam):
        _check(lib().ref_set_area(int(t), int(target), float(lam)))

    def set_perimeter(self, t, target, lam):
        _check(lib().ref_set_perimeter(int(t), int(target), float(lam)))
        self.perimeter = self.perimeter or lam != 0

    def set_adhesion(self, a, b, J):
        _check(lib().ref_set_adhesion(int(a), int(b), int(round(J))))

    def set_stickiness(self, a, b, S):
        _check(lib().ref_set_stickiness(int(a), int(b), int(round(S))))

    def set_chemotaxis(self, t, lam):
        _check(lib().ref_set_chemotaxis(int(t), float(lam)))
        self.chemotaxis = self.chemotaxis or lam != 0

    def set_field(self, field):
        """Chemotaxis field [ndim, D, D(, D)] (doubles, as the reference keeps it)."""
        f = np.ascontiguousarray(field, dtype=np.float64)
        _check(lib().ref_set_field(f.ctypes.data))

    def set_fixed(self, t, fixed=True):
        _check(lib().ref_set_fixed(int(t), 1 if fixed else 0))
        self.fixed = self.fixed or bool(fixed)

    def apply(self, w):
        """Parameters of a gpucpm.workloads.Workload, rounded as the
        reference stores them (short J, int T)."""
        nt = w.J.shape[0]
        for a in range(nt):
            for b in range(a, nt):
                self.set_adhesion(a, b, w.J[a, b])
            if w.lam_area[a] != 0:
                self.set_area(a, int(w.tgt_area[a]), float(w.lam_area[a]))
            if w.lam_perim[a] != 0:
                self.set_perimeter(a, int(w.tgt_perim[a]), float(w.lam_perim[a]))
            if w.fixed is not None and w.fixed[a]:
                self.set_fixed(a)
            if w.chemo is not None and w.chemo[a] != 0:
                self.set_chemotaxis(a, float(w.chemo[a]))
            for b in range(nt):
                if w.stick is not None and w.stick[a, b] != 0:
                    self.set_stickiness(a, b, w.stick[a, b])
        _check(lib().ref_set_temperature(int(round(w.temperature))))
        if w.field is not None:
            self.set_field(w.field)

    def push(self, lattice):
        lat = np.ascontiguousarray(lattice, dtype=np.uint32)
        _check(lib().ref_push(lat.ctypes.data))

    def run(self, iterations, threads_per_block, positions_per_thread,
            positions_per_checkerboard, updates_per_checkerboard_switch=1,
            updates_per_barrier=1, global_sync=1, block_sync=0, cell_sync=0,
            inner_iterations=None, shared=0, centroid_tracking=0, seed=1):
        inner = iterations if inner_iterations is None else inner_iterations
        _check(lib().ref_run(cell_sync, block_sync, global_sync, threads_per_block,
                             positions_per_thread, positions_per_checkerboard,
                             updates_per_checkerboard_switch, updates_per_barrier,
                             int(iterations), int(inner), int(shared),
                             1 if self.perimeter else 0, int(centroid_tracking), int(seed),
                             1 if self.fixed else 0, 1 if self.chemotaxis else 0))

    def synchronize(self):
        _check(lib().ref_synchronize())

    def pull(self):
        shape = (self.dimension,) * self.ndim
        out = np.empty(shape, np.uint32)
        _check(lib().ref_pull(out.ctypes.data))
        return out

    def tables(self):
        a = np.empty(self.ncells + 1, np.uint32)
        c = np.empty(self.ncells + 1, np.uint32)
        _check(lib().ref_tables(a.ctypes.data, c.ctypes.data))
        return a, c

    def max_coop_blocks(self, threads_per_block, shared=0):
        n = ctypes.c_int()
        _check(lib().ref_max_coop_blocks(int(threads_per_block), int(shared),
                                         1 if self.perimeter else 0, ctypes.byref(n)))
        return n.value
