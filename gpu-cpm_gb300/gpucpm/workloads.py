"""Seeded synthetic initial states and parameters of the benchmark workloads.

Each builder returns a `Workload`: the initial lattice (uint32, id | type <<
24), the cell count, and per-type parameters in the engine's convention
(J[a][b] = adhesion of a site of type a against a neighbour of type b; type
0 is the medium).  All randomness comes from numpy's Philox generator under
the given seed, so every process and machine builds identical inputs.

  sorting_2d   200x200, 400 cells as 5x5 squares, light/dark 50/50,
               J_ll=14 J_dd=2 J_ld=11 J_lm=J_dm=16, A=25 lambda=1, T=10
  tissue_2d    4096x4096 Voronoi tiling at 100 sites per cell, 3 types,
               symmetric J ~ U[2,20], A=100 lambda=1, P*=40 lambda_P=0.5, T=20
  tissue_3d    256^3 Voronoi, 80% of regions cells / 20% medium, 2 types,
               J ~ U[4,16], V*=500 lambda=1, S*=350 lambda_S=0.2, T=20
  ensemble_2d  ragged replicas, side log-uniform in [64,1024], cells=side^2/50
  sorting_grid 256x256 two-type sorting: 2600 of the 2601 slots of a 51x51
               grid of 5x5 squares
"""
from dataclasses import dataclass, field

import numpy as np

MAX_TYPES = 32


def _rng(seed):
    return np.random.Generator(np.random.Philox(int(seed)))


@dataclass
class Workload:
    name: str
    lattice: np.ndarray          # uint32, shape (ny, nx) or (nz, ny, nx)
    ncells: int
    J: np.ndarray                # float32 [ntypes, ntypes]
    lam_area: np.ndarray         # float32 [ntypes]
    tgt_area: np.ndarray         # int32 [ntypes]
    lam_perim: np.ndarray        # float32 [ntypes]
    tgt_perim: np.ndarray        # int32 [ntypes]
    temperature: float
    mcs: int
    meta: dict = field(default_factory=dict)
    stick: np.ndarray = None     # float32 [ntypes, ntypes] stickiness, or None
    fixed: np.ndarray = None     # bool [ntypes]: fixed (unmovable) types, or None
    chemo: np.ndarray = None     # float32 [ntypes]: chemotaxis lambdas, or None
    field: np.ndarray = None     # float64 [ndim, (nz,) ny, nx] chemotaxis field, or None
    act_lambda: np.ndarray = None  # float32 [ntypes]: act lambdas, or None
    act_max: np.ndarray = None     # int32 [ntypes]: act maxima, or None
    persist_lambda: np.ndarray = None  # float32 [ntypes]: persistence lambdas (3D), or None
    persist_diff: np.ndarray = None    # float32 [ntypes]: persistence diffusion, or None
    history: int = 1                   # mean-coordinate ring slots (engine-wide)

    @property
    def ndim(self):
        return self.lattice.ndim

    @property
    def nsites(self):
        return int(self.lattice.size)

    def apply(self, engine, replica=None):
        """Set parameters on a gpucpm.Cpm (replica None) or one Batch replica."""
        nt = self.J.shape[0]
        for a in range(nt):
            for b in range(nt):
                if replica is None:
                    engine._call("cpm_set_adhesion", a, b, float(self.J[a, b]), 0)
                else:
                    engine.set_adhesion(replica, a, b, float(self.J[a, b]), symmetric=False)
            if replica is None:
                engine._call("cpm_set_area", a, int(self.tgt_area[a]), float(self.lam_area[a]))
                engine._call("cpm_set_perimeter", a, int(self.tgt_perim[a]),
                             float(self.lam_perim[a]))
            else:
                engine.set_area(replica, a, int(self.tgt_area[a]), float(self.lam_area[a]))
                engine.set_perimeter(replica, a, int(self.tgt_perim[a]), float(self.lam_perim[a]))
        if replica is None:
            engine.set_temperature(self.temperature)
        else:
            engine.set_temperature(replica, self.temperature)
        if self.field is not None:
            view = engine.field(0 if replica is None else replica)
            view[...] = self.field
        if self.persist_lambda is not None and self.history != engine.history:
            engine.set_history(self.history)
        for a in range(nt):
            if self.act_lambda is not None and self.act_lambda[a] != 0:
                mx = int(self.act_max[a]) if self.act_max is not None else 0
                if replica is None:
                    engine._call("cpm_set_act", a, mx, float(self.act_lambda[a]))
                else:
                    engine.set_act(replica, a, mx, float(self.act_lambda[a]))
            if self.chemo is not None and self.chemo[a] != 0:
                if replica is None:
                    engine._call("cpm_set_chemotaxis", a, float(self.chemo[a]))
                else:
                    engine.set_chemotaxis(replica, a, float(self.chemo[a]))
            if self.persist_lambda is not None and self.persist_lambda[a] != 0:
                df = float(self.persist_diff[a]) if self.persist_diff is not None else 0.0
                if replica is None:
                    engine._call("cpm_set_persistence", a, 0, df, float(self.persist_lambda[a]))
                else:
                    engine.set_persistence(replica, a, 0, df, float(self.persist_lambda[a]))
            if self.fixed is not None and self.fixed[a]:
                if replica is None:
                    engine._call("cpm_set_fixed", a, 1)
                else:
                    engine.set_fixed(replica, a, True)
            for b in range(nt):
                if self.stick is not None and self.stick[a, b] != 0:
                    if replica is None:
                        engine._call("cpm_set_stickiness", a, b, float(self.stick[a, b]))
                    else:
                        engine.set_stickiness(replica, a, b, float(self.stick[a, b]))

    def oracle_kwargs(self):
        return dict(J=self.J, lam_area=self.lam_area, tgt_area=self.tgt_area,
                    lam_perim=self.lam_perim, tgt_perim=self.tgt_perim,
                    temperature=self.temperature, stick=self.stick, fixed=self.fixed,
                    chemo=self.chemo, field=self.field, act_lambda=self.act_lambda,
                    act_max=self.act_max, persist_lambda=self.persist_lambda,
                    persist_diff=self.persist_diff, history=self.history)


def _params(nt, J, lam_area=0.0, tgt_area=0, lam_perim=0.0, tgt_perim=0):
    la = np.full(nt, lam_area, np.float32)
    ta = np.full(nt, tgt_area, np.int32)
    lp = np.full(nt, lam_perim, np.float32)
    tp = np.full(nt, tgt_perim, np.int32)
    la[0] = ta[0] = lp[0] = tp[0] = 0  # the medium has no constraints
    return np.asarray(J, np.float32), la, ta, lp, tp


def sorting_J():
    """Graner-Glazier sorting adhesion: light (1) / dark (2) / medium (0)."""
    J = np.zeros((3, 3), np.float32)
    J[1, 1], J[2, 2] = 14, 2
    J[1, 2] = J[2, 1] = 11
    J[1, 0] = J[0, 1] = 16
    J[2, 0] = J[0, 2] = 16
    return J


def place_squares(n, side, count, size, rng):
    """`count` non-overlapping size x size squares on a periodic n x n lattice.

    Returns top-left corners; placement by rejection sampling in `rng` order.
    """
    occ = np.zeros((n, n), bool)
    corners = []
    tries = 0
    while len(corners) < count:
        tries += 1
        if tries > 200 * count:
            raise RuntimeError("could not place squares without overlap")
        x, y = (int(v) for v in rng.integers(0, n, 2))
        ys = (np.arange(y, y + size) % n)[:, None]
        xs = (np.arange(x, x + size) % n)[None, :]
        if occ[ys, xs].any():
            continue
        occ[ys, xs] = True
        corners.append((x, y))
    return corners


def _paint_squares(lat, corners, size, types):
    n = lat.shape[0]
    for i, (x, y) in enumerate(corners):
        ys = (np.arange(y, y + size) % n)[:, None]
        xs = (np.arange(x, x + size) % lat.shape[1])[None, :]
        lat[ys, xs] = np.uint32((i + 1) | (int(types[i]) << 24))


def sorting_2d(n=200, ncells=400, size=5, seed=0, mcs=1000, temperature=10.0):
    rng = _rng(seed)
    corners = place_squares(n, n, ncells, size, rng)
    types = rng.permutation(np.repeat([1, 2], [ncells // 2, ncells - ncells // 2]))
    lat = np.zeros((n, n), np.uint32)
    _paint_squares(lat, corners, size, types)
    J, la, ta, lp, tp = _params(3, sorting_J(), 1.0, size * size)
    return Workload("sorting_2d", lat, ncells, J, la, ta, lp, tp, float(temperature), mcs,
                    {"n": n, "cell_side": size})


def sorting_grid(n=256, ncells=2600, size=5, seed=0, mcs=500, temperature=10.0):
    """2600 of the 2601 slots of the 51x51 grid of 5-strided 5x5 squares."""
    rng = _rng(seed)
    per = n // size
    slots = rng.permutation(per * per)[:ncells]
    corners = [(int(s % per) * size, int(s // per) * size) for s in slots]
    types = rng.permutation(np.repeat([1, 2], [ncells // 2, ncells - ncells // 2]))
    lat = np.zeros((n, n), np.uint32)
    _paint_squares(lat, corners, size, types)
    J, la, ta, lp, tp = _params(3, sorting_J(), 1.0, size * size)
    return Workload("sorting_grid", lat, ncells, J, la, ta, lp, tp, float(temperature), mcs,
                    {"n": n})


def voronoi_labels(shape, npoints, rng, return_points=False):
    """Periodic Voronoi labels 0..npoints-1 of every site of `shape` (and the
    points, [npoints, ndim] x first, when asked)."""
    from scipy.spatial import cKDTree
    dims = np.array(shape[::-1], np.float64)  # (nx, ny[, nz])
    pts = rng.random((npoints, len(shape))) * dims
    tree = cKDTree(pts, boxsize=dims)
    grids = np.meshgrid(*[np.arange(d, dtype=np.float64) for d in shape[::-1]],
                        indexing="ij")
    coords = np.stack([g.ravel() for g in grids], axis=1)
    _, idx = tree.query(coords, k=1, workers=-1)
    # meshgrid with indexing="ij" over (x, y[, z]) puts x slowest; bring the
    # labels back to row-major [z, y, x].
    lab = idx.reshape(tuple(int(d) for d in dims)).transpose()
    lab = np.ascontiguousarray(lab).astype(np.int64)
    return (lab, pts) if return_points else lab


def _sym_uniform(nt, lo, hi, rng):
    J = rng.uniform(lo, hi, (nt, nt)).astype(np.float32)
    return np.triu(J) + np.triu(J, 1).T


def tissue_2d(n=4096, area=100, ntypes=3, seed=1, mcs=500):
    rng = _rng(seed)
    ncells = (n * n) // area
    lab, pts = voronoi_labels((n, n), ncells, rng, return_points=True)
    types = rng.integers(1, ntypes + 1, ncells)
    values = ((np.arange(ncells) + 1) | (types << 24)).astype(np.uint32)
    lat = values[lab]
    J, la, ta, lp, tp = _params(ntypes + 1, _sym_uniform(ntypes + 1, 2.0, 20.0, rng),
                                1.0, area, 0.5, 40)
    return Workload("tissue_2d", lat, ncells, J, la, ta, lp, tp, 20.0, mcs,
                    {"n": n, "area": area, "points": pts, "values": values})


def tissue_3d(n=256, volume=500, fill=0.8, ntypes=2, seed=2, mcs=200):
    rng = _rng(seed)
    nreg = (n ** 3) // volume
    lab, pts = voronoi_labels((n, n, n), nreg, rng, return_points=True)
    is_cell = rng.random(nreg) < fill
    ids = np.zeros(nreg, np.int64)
    ncells = int(is_cell.sum())
    ids[is_cell] = np.arange(1, ncells + 1)
    types = np.zeros(nreg, np.int64)
    types[is_cell] = rng.integers(1, ntypes + 1, ncells)
    values = (ids | (types << 24)).astype(np.uint32)
    lat = values[lab]
    J, la, ta, lp, tp = _params(ntypes + 1, _sym_uniform(ntypes + 1, 4.0, 16.0, rng),
                                1.0, volume, 0.2, 350)
    return Workload("tissue_3d", lat, ncells, J, la, ta, lp, tp, 20.0, mcs,
                    {"n": n, "volume": volume, "points": pts, "values": values})


def ensemble_2d(nrep=256, lo=64, hi=1024, sites_per_cell=50, seed=3, mcs=500):
    """Ragged replicas: side log-uniform in [lo, hi], per-replica J, lambda, T."""
    rng = _rng(seed)
    sides = np.exp(rng.uniform(np.log(lo), np.log(hi), nrep)).round().astype(int)
    out = []
    for r, side in enumerate(sides):
        ncells = max(1, int(side) * int(side) // sites_per_cell)
        lab = voronoi_labels((int(side), int(side)), ncells, rng)
        types = rng.integers(1, 3, ncells)
        lat = ((lab + 1) | (types[lab] << 24)).astype(np.uint32)
        J = _sym_uniform(3, 2.0, 20.0, rng)
        lam = float(rng.uniform(0.5, 2.0))
        T = float(rng.uniform(5.0, 30.0))
        Jp, la, ta, lp, tp = _params(3, J, lam, sites_per_cell)
        out.append(Workload(f"ensemble_2d[{r}]", lat, ncells, Jp, la, ta, lp, tp, T, mcs,
                            {"side": int(side)}))
    return out


def random_small(shape, ncells, ntypes=2, seed=0, temperature=8.0, perim=True,
                 area=None, medium_fraction=0.25):
    """Small Voronoi test lattice with medium patches (any shape, 2D or 3D)."""
    rng = _rng(seed)
    nreg = ncells + max(1, int(ncells * medium_fraction))
    lab = voronoi_labels(tuple(shape), nreg, rng)
    ids = np.zeros(nreg, np.int64)
    ids[:ncells] = np.arange(1, ncells + 1)
    rng.shuffle(ids)
    types = np.where(ids > 0, rng.integers(1, ntypes + 1, nreg), 0)
    lat = (ids[lab] | (types[lab] << 24)).astype(np.uint32)
    nsites = int(np.prod(shape))
    A = area if area is not None else max(1, nsites // nreg)
    J = _sym_uniform(ntypes + 1, 2.0, 20.0, rng)
    J[0, 0] = 0
    P = int(4 * np.sqrt(A)) if len(shape) == 2 else int(6 * A ** (2 / 3))
    J, la, ta, lp, tp = _params(ntypes + 1, J, 1.0, A, 0.3 if perim else 0.0, P)
    return Workload("random_small", lat, ncells, J, la, ta, lp, tp, float(temperature), 0,
                    {"shape": tuple(shape)})
