"""CPU tests of the oracle: known-answer vectors, exp error bound, table
recount on hand-computed lattices, hand-computed dH against the reference's
formula, invariants after sweeps and thread-count independence."""
import ctypes
import math

import numpy as np
import pytest

import oracle
from gpucpm import workloads as W


# Philox4x32-10 known-answer vectors (Random123 kat_vectors, philox4x32_10).
KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2,
     [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(ctr, key, want):
    assert oracle.philox4x32_10(ctr, key) == want


def test_exp_neg_error_bound():
    xs = np.concatenate([np.linspace(-20.0, 0.0, 40001, dtype=np.float32),
                         np.float32(-np.logspace(-8, np.log10(20), 2000))])
    worst = 0.0
    for x in xs:
        got = oracle.exp_neg(float(x))
        ref = math.exp(float(x))
        worst = max(worst, abs(got - ref) / float(np.spacing(np.float32(ref))))
    assert worst <= 1.0, worst  # at most 1 ulp of FP32 over [-20, 0]
    assert oracle.exp_neg(0.0) == 1.0
    assert oracle.exp_neg(-20.5) == 0.0


def _sim(lat, ncells, J=None, **kw):
    if J is None:
        J = np.zeros((3, 3), np.float32)
    kw.setdefault("lam_area", [0, 1, 1])
    kw.setdefault("tgt_area", [0, 9, 9])
    return oracle.OracleSim(np.asarray(lat, np.uint32), ncells, J, **kw)


def test_recount_single_square_2d():
    lat = np.zeros((8, 8), np.uint32)
    lat[2:5, 3:6] = 1 | (1 << 24)
    s = _sim(lat, 1)
    # 3x3 block in medium: 4 corners x 5 + 4 edges x 3 foreign Moore neighbours
    assert s.area[1] == 9 and s.perim[1] == 32
    assert list(s.csum[1]) == [3 * (3 + 4 + 5), 3 * (2 + 3 + 4)]


def test_recount_wrapped_cell_uses_nearest_images():
    lat = np.zeros((10, 10), np.uint32)
    lat[4, [9, 0, 1]] = 1 | (1 << 24)  # straddles the periodic x boundary
    s = _sim(lat, 1)
    assert s.area[1] == 3
    # anchor is the first site in raster order (x=0); x=9 maps to -1
    assert s.csum[1][0] == -1 + 0 + 1 and s.csum[1][1] == 12


def test_recount_3d_cube():
    lat = np.zeros((6, 6, 6), np.uint32)
    lat[1:3, 1:3, 1:3] = 1 | (2 << 24)
    s = _sim(lat, 1)
    # each site of a 2x2x2 cube has 7 same-cell and 19 foreign neighbours
    assert s.area[1] == 8 and s.perim[1] == 8 * 19


def test_invalid_lattices_rejected():
    lat = np.zeros((6, 6), np.uint32)
    lat[0, 0] = 5 | (1 << 24)
    with pytest.raises(ValueError):
        _sim(lat, 3)  # id above ncells
    lat[0, 0] = 1 << 24
    with pytest.raises(ValueError):
        _sim(lat, 3)  # medium with a type
    lat[0, 0] = 1 | (1 << 24)
    lat[0, 1] = 1 | (2 << 24)
    with pytest.raises(ValueError):
        _sim(lat, 3)  # one id, two types


def _reference_dh(lat, ax, ay, sx, sy, area, perim, J, lam_a, tgt_a, lam_p, tgt_p,
                  stick=None, s=None):
    """dH of copying (sx, sy) into (ax, ay), restated from the reference
    (src/kernels2d.cu:346-519): integer adhesion sums (stickiness added to
    the old configuration's, :399-400), double lambda terms.  `s` overrides
    the source value (the medium proposed by a fixed source type)."""
    n = lat.shape[0]
    t = int(lat[ay, ax])
    s = int(lat[sy, sx]) if s is None else s
    ts, tt = s >> 24, t >> 24
    e_old = e_new = 0
    ops = nps = opt = npt = 0
    for j in (-1, 0, 1):
        for i in (-1, 0, 1):
            if i == 0 and j == 0:
                continue
            v = int(lat[(ay + j) % n, (ax + i) % n])
            tv = v >> 24
            if t != v:
                e_old += J[tt][tv] + (stick[tt][tv] if stick is not None else 0)
            if s != v:
                e_new += J[ts][tv]
            ops += v == s
            nps += v != s
            opt += v != t
            npt += v == t
    e = float(e_new - e_old)
    if s:
        P = perim[s & 0xFFFFFF]
        Pn = P - ops + nps
        e += lam_p[ts] * ((Pn - tgt_p[ts]) ** 2 - (P - tgt_p[ts]) ** 2)
    if t:
        P = perim[t & 0xFFFFFF]
        Pn = P - opt + npt
        e += lam_p[tt] * ((Pn - tgt_p[tt]) ** 2 - (P - tgt_p[tt]) ** 2)
    if s:
        e += lam_a[ts] * (1 + 2 * area[s & 0xFFFFFF] - 2 * tgt_a[ts])
    if t:
        e += lam_a[tt] * (1 - 2 * area[t & 0xFFFFFF] + 2 * tgt_a[tt])
    return e


@pytest.mark.parametrize("case", ["plain", "fixed_sticky"])
def test_first_mcs_matches_reference_dh_formula(case):
    """Replay one MCS in Python with the reference's dH formula and the same
    Philox draws, and compare the result with the oracle.  The second case
    adds stickiness and a fixed type (src/kernels2d.cu:280-290, 399-400)."""
    w = W.random_small((16, 16), 10, ntypes=3, seed=11, temperature=6.0)
    J = np.rint(w.J).astype(int)            # integer J: both sides exact
    lam_a = [1.0] * 4
    lam_p = [0.5] * 4
    tgt_a, tgt_p = [0, 20, 20, 20], [0, 18, 18, 18]
    T = 6.0
    stick = fixed = None
    if case == "fixed_sticky":
        stick = np.zeros((4, 4), int)
        stick[1, 2], stick[2, 1], stick[1, 0], stick[2, 3] = 3, 5, 2, 4
        fixed = [False, False, False, True]
    sim = oracle.OracleSim(w.lattice, w.ncells, J.astype(np.float32), lam_a, tgt_a,
                           lam_p, tgt_p, temperature=T, seed=7, stick=stick, fixed=fixed)
    lat = w.lattice.copy()
    area, perim = sim.area.copy(), sim.perim.copy()
    n = 16
    accepted = 0
    for cy in (0, 1):
        for cx in (0, 1):
            slot = cy * 3 + cx
            changes = []
            for y in range(cy, n, 2):
                for x in range(cx, n, 2):
                    t = int(lat[y, x])
                    nbs = [(x + i, y + j) for j in (-1, 0, 1) for i in (-1, 0, 1)
                           if (i, j) != (0, 0)]
                    vals = [int(lat[b % n, a % n]) for a, b in nbs]
                    if all(v == t for v in vals):
                        continue
                    r = oracle.philox4x32_10([y * n + x, slot, 0, 0], [7, 0])
                    k = (r[0] * 8) >> 32
                    if vals[k] == t:
                        continue
                    s = vals[k]
                    if fixed is not None:
                        if fixed[t >> 24]:
                            continue
                        if fixed[s >> 24]:
                            s = 0
                            if s == t:
                                continue
                    sx, sy = nbs[k][0] % n, nbs[k][1] % n
                    dH = _reference_dh(lat, x, y, sx, sy, area, perim, J, lam_a,
                                       tgt_a, lam_p, tgt_p, stick, s)
                    u = ((r[1] >> 8) | 1) * 2.0 ** -24
                    if dH < 0 or u < math.exp(-dH / T):
                        changes.append((x, y, s, t, vals))
            for x, y, s, t, vals in changes:
                lat[y, x] = s
                accepted += 1
                if s:
                    area[s & 0xFFFFFF] += 1
                    perim[s & 0xFFFFFF] += 8 - 2 * sum(v == s for v in vals)
                if t:
                    area[t & 0xFFFFFF] -= 1
                    perim[t & 0xFFFFFF] += 2 * sum(v == t for v in vals) - 8
    sim.run(1)
    assert accepted > 5
    assert int(sim.counters[2]) == accepted
    np.testing.assert_array_equal(sim.lattice, lat)
    np.testing.assert_array_equal(sim.area, area)
    np.testing.assert_array_equal(sim.perim, perim)


@pytest.mark.parametrize("shape,ncells", [((64, 64), 40), ((37, 41), 30),
                                          ((12, 10, 14), 25), ((9, 13, 11), 20)])
def test_tables_match_recount_after_sweeps(shape, ncells):
    w = W.random_small(shape, ncells, seed=len(shape) * 7 + ncells)
    s = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=3)
    s.run(30 if len(shape) == 2 else 10)
    a, p, c = s.recount()
    np.testing.assert_array_equal(a, s.area)
    np.testing.assert_array_equal(p, s.perim)
    dims = np.array(shape[::-1])
    assert ((c - s.csum) % dims == 0).all()
    assert int(s.area[1:].sum()) == int(((s.lattice & 0xFFFFFF) != 0).sum())


def test_thread_count_does_not_change_result():
    w = W.random_small((48, 52), 35, seed=4)
    a = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=9).run(20, 1)
    b = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=9).run(20, 5)
    np.testing.assert_array_equal(a.lattice, b.lattice)
    np.testing.assert_array_equal(a.csum, b.csum)
    np.testing.assert_array_equal(a.counters, b.counters)


def test_run_is_resumable_by_tick():
    w = W.random_small((32, 32), 20, seed=8)
    a = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=2).run(12)
    b = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=2).run(5).run(7)
    np.testing.assert_array_equal(a.lattice, b.lattice)


def test_zero_temperature_accepts_only_downhill():
    w = W.random_small((32, 32), 20, seed=12, temperature=0.0)
    s = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs())
    e0 = _total_energy(s)
    s.run(5)
    assert _total_energy(s) <= e0


def _total_energy(s):
    lat = s.lattice.astype(np.int64)
    J = np.asarray(s.params.J).reshape(32, 32)
    e = 0.0
    n0, n1 = lat.shape
    for j in (-1, 0, 1):
        for i in (-1, 0, 1):
            if (i, j) == (0, 0):
                continue
            nb = np.roll(np.roll(lat, -j, 0), -i, 1)
            diff = nb != lat
            e += J[lat >> 24, nb >> 24][diff].sum()
    e /= 2
    la = np.asarray(s.params.lam_area)
    ta = np.asarray(s.params.tgt_area)
    ids = np.arange(1, s.ncells + 1)
    ty = np.zeros(s.ncells + 1, int)
    ty[lat.ravel() & 0xFFFFFF] = lat.ravel() >> 24
    e += (la[ty[ids]] * (s.area[ids] - ta[ty[ids]]) ** 2).sum()
    lp = np.asarray(s.params.lam_perim)
    tp = np.asarray(s.params.tgt_perim)
    e += (lp[ty[ids]] * (s.perim[ids] - tp[ty[ids]]) ** 2).sum()
    return e


PAIRS = ((1, 1), (2, 2), (1, 2), (1, 0), (2, 0))


def _log_p(dH, T, accepted):
    """log of P(decision), P(accept) = min(1, exp(-dH/T))."""
    x = max(dH, 0.0) / T
    return -x if accepted else math.log(-math.expm1(-x))


@pytest.mark.parametrize("case", ["voronoi_perimeter", "sorting_integer"])
def test_oracle_scores_are_derivatives_of_the_decision_log_likelihood(case):
    """Replay one MCS with the reference's dH formula (as above); for every
    evaluated attempt with dH >= 0 differentiate log P(its decision) by
    central differences in each parameter, with the lattice and tables of
    that moment held fixed, and compare the sum with the oracle's FP64
    scores for that MCS.  At dH = 0 (frequent with integer parameters) the
    central difference is the mean of the two one-sided slopes, the value
    the scores use there."""
    if case == "voronoi_perimeter":
        w = W.random_small((16, 16), 10, seed=11, temperature=6.0)
        J = np.rint(w.J).astype(float)
        lam_a, tgt_a = [0.0, 1.0, 1.0], [0, 20, 20]
        lam_p, tgt_p = [0.0, 0.5, 0.5], [0, 18, 18]
        T = 6.0
    else:  # integer J and area terms, no perimeter term: many dH = 0 exactly
        w = W.sorting_grid(n=30, ncells=35, seed=2)
        J = w.J.astype(float)
        lam_a, tgt_a = [0.0, 1.0, 1.0], [0, 25, 25]
        lam_p, tgt_p = [0.0, 0.0, 0.0], [0, 0, 0]
        T = 10.0
    sim = oracle.OracleSim(w.lattice, w.ncells, J.astype(np.float32), lam_a, tgt_a,
                           lam_p, tgt_p, temperature=T, seed=7)
    # the sorting case replays MCS 6, once the squares have roughened
    tick0 = 5 if case == "sorting_integer" else 0
    sim.run(tick0)
    spec = oracle.ScoreSpec.make(PAIRS, lambda_perim=True)
    lat = sim.lattice.copy()
    area, perim = sim.area.copy(), sim.perim.copy()
    n = lat.shape[0]
    want = np.zeros(8)
    evaluated_pos = zero_dh = 0

    def dH_of(theta, ax, ay, sx, sy):
        Jt = J.copy()
        for k, (a, b) in enumerate(PAIRS):
            Jt[a, b] = Jt[b, a] = theta[k]
        la = [0.0, theta[5], theta[5]]
        lp = [0.0, theta[6], theta[6]]
        return _reference_dh(lat, ax, ay, sx, sy, area, perim, Jt, la, tgt_a, lp, tgt_p)

    theta = np.array([J[a, b] for a, b in PAIRS] + [1.0, lam_p[1], T])
    for cy in (0, 1):
        for cx in (0, 1):
            slot = cy * 3 + cx
            changes = []
            for y in range(cy, n, 2):
                for x in range(cx, n, 2):
                    t = int(lat[y, x])
                    nbs = [(x + i, y + j) for j in (-1, 0, 1) for i in (-1, 0, 1)
                           if (i, j) != (0, 0)]
                    vals = [int(lat[b % n, a % n]) for a, b in nbs]
                    if all(v == t for v in vals):
                        continue
                    r = oracle.philox4x32_10([y * n + x, tick0 * 9 + slot, 0, 0], [7, 0])
                    k = (r[0] * 8) >> 32
                    if vals[k] == t:
                        continue
                    sx, sy = nbs[k][0] % n, nbs[k][1] % n
                    dH = dH_of(theta, x, y, sx, sy)
                    u = ((r[1] >> 8) | 1) * 2.0 ** -24
                    acc = dH < 0 or u < math.exp(-dH / T)
                    if dH == 0:
                        zero_dh += 1
                    if dH >= 0:
                        evaluated_pos += 1
                        for q in range(8):
                            h = 1e-4 * max(1.0, abs(theta[q]))
                            if case == "sorting_integer" and q == 6:
                                # lambda_perim = 0; perimeter terms of ~700 and
                                # a large cancellation between accepted and
                                # rejected attempts call for a small step
                                h = 1e-6
                            tp, tm = theta.copy(), theta.copy()
                            tp[q] += h
                            tm[q] -= h
                            lp = _log_p(dH_of(tp, x, y, sx, sy), tp[7], acc)
                            lm = _log_p(dH_of(tm, x, y, sx, sy), tm[7], acc)
                            want[q] += (lp - lm) / (2 * h)
                    if acc:
                        changes.append((x, y, vals[k], t, vals))
            for x, y, s, t, vals in changes:
                lat[y, x] = s
                if s:
                    area[s & 0xFFFFFF] += 1
                    perim[s & 0xFFFFFF] += 8 - 2 * sum(v == s for v in vals)
                if t:
                    area[t & 0xFFFFFF] -= 1
                    perim[t & 0xFFFFFF] += 2 * sum(v == t for v in vals) - 8
    got = sim.run_scores(1, spec)[0, :8]
    assert evaluated_pos > 20
    if case == "sorting_integer":
        assert zero_dh > 0
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(sim.lattice, lat)


def test_own_log2_and_exp2_error_bounds():
    """The act model's FP32 log2 / exp2 (the sweep kernel's log2_pos /
    exp2_own, restated in the oracle): within 1.5 ulp of FP32."""
    vs = np.unique(np.concatenate([np.arange(1, 5000), np.geomspace(1, 1e7, 3000).astype(int)]))
    worst = 0.0
    for v in vs:
        got = oracle.log2_pos(float(v))
        ref = math.log2(float(np.float32(v)))
        worst = max(worst, abs(got - ref) / float(np.spacing(np.float32(max(abs(ref), 1.0)))))
    assert worst <= 1.5, worst
    worst = 0.0
    for y in np.linspace(-30.0, 60.0, 9001, dtype=np.float32):
        got = oracle.exp2(float(y))
        ref = 2.0 ** float(y)
        worst = max(worst, abs(got - ref) / float(np.spacing(np.float32(ref))))
    assert worst <= 1.5, worst
    assert oracle.exp2(0.0) == 1.0 and oracle.log2_pos(1.0) == 0.0


def _act_mean_py(lat, act, x, y, ident, amax, tick):
    """Geometric mean of max(amax + act - tick, 0) over (x, y) and its
    neighbours holding `ident`, as exp2 of the FP32 mean log2 (restated)."""
    n = lat.shape[0]
    f32 = np.float32
    a0 = amax + int(act[y, x]) - tick
    if a0 <= 0:
        return f32(0.0)
    s, count = f32(oracle.log2_pos(a0)), 1
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            if dx == 0 and dy == 0:
                continue
            xx, yy = (x + dx) % n, (y + dy) % n
            if int(lat[yy, xx]) != ident:
                continue
            v = amax + int(act[yy, xx]) - tick
            if v <= 0:
                return f32(0.0)
            s = f32(s + f32(oracle.log2_pos(v)))
            count += 1
    return f32(oracle.exp2(f32(s / f32(count))))


def test_act_mcs_matches_restatement():
    """One MCS of the act model (src/kernels2d.cu:312-473), replayed in
    Python from the phase's starting state, against the oracle: act term
    first, lambda and max of the target type (source type for a medium
    target), every copy and its stamp written after its phase."""
    w = W.random_small((20, 20), 12, ntypes=2, seed=31, temperature=8.0)
    J = np.rint(w.J).astype(int)
    lam_a, tgt_a = [0.0, 1.0, 1.0], [0, 30, 30]
    lam_p, tgt_p = [0.0, 0.0, 0.0], [0, 0, 0]
    act_lambda = np.array([0.0, 40.0, 25.0], np.float32)
    act_max = np.array([0, 20, 12], np.int32)
    T, seed = 8.0, 3
    sim = oracle.OracleSim(w.lattice, w.ncells, J.astype(np.float32), lam_a, tgt_a, lam_p, tgt_p,
                           temperature=T, seed=seed, act_lambda=act_lambda, act_max=act_max)
    sim.run(4)  # stamps up to MCS 3
    assert sim.act.max() == 3
    lat, act = sim.lattice.copy(), sim.act.copy()
    area = sim.area.copy()
    n, tick, f32 = 20, 4, np.float32
    accepted = 0
    for cy in (0, 1):
        for cx in (0, 1):
            slot = cy * 3 + cx
            changes = []
            for y in range(cy, n, 2):
                for x in range(cx, n, 2):
                    t = int(lat[y, x])
                    nbs = [(x + i, y + j) for j in (-1, 0, 1) for i in (-1, 0, 1)
                           if (i, j) != (0, 0)]
                    vals = [int(lat[b % n, a % n]) for a, b in nbs]
                    if all(v == t for v in vals):
                        continue
                    r = oracle.philox4x32_10([y * n + x, tick * 9 + slot, 0, 0], [seed, 0])
                    k = (r[0] * 8) >> 32
                    s = vals[k]
                    if s == t:
                        continue
                    sx, sy = nbs[k][0] % n, nbs[k][1] % n
                    ts, tt = s >> 24, t >> 24
                    e_old = sum(J[tt][v >> 24] for v in vals if v != t)
                    e_new = sum(J[ts][v >> 24] for v in vals if v != s)
                    lead = f32(0.0)
                    ta = tt if tt else ts
                    if act_lambda[ta] != 0 and act_max[ta] != 0:
                        tgt = _act_mean_py(lat, act, x, y, t, int(act_max[tt]), tick) if t else f32(0)
                        src = _act_mean_py(lat, act, sx, sy, s, int(act_max[ts]), tick) if s else f32(0)
                        lead = f32(lead + f32(f32(-act_lambda[ta] / f32(act_max[ta])) * f32(src - tgt)))
                    dH = f32(lead + f32(e_new - e_old))
                    if s:
                        dH = f32(float(dH) + lam_a[ts] * (1 + 2 * (int(area[s & 0xFFFFFF]) - tgt_a[ts])))
                    if t:
                        dH = f32(float(dH) + lam_a[tt] * (1 - 2 * (int(area[t & 0xFFFFFF]) - tgt_a[tt])))
                    u = f32(((r[1] >> 8) | 1) * 2.0 ** -24)
                    ok = dH < 0 or u < f32(oracle.exp_neg(float(f32(-dH / f32(T)))))
                    if ok:
                        changes.append((x, y, s, t))
            for x, y, s, t in changes:
                lat[y, x] = s
                act[y, x] = tick
                accepted += 1
                if s:
                    area[s & 0xFFFFFF] += 1
                if t:
                    area[t & 0xFFFFFF] -= 1
    sim.run(1)
    assert accepted > 10
    np.testing.assert_array_equal(sim.lattice, lat)
    np.testing.assert_array_equal(sim.act, act)
    np.testing.assert_array_equal(sim.area, area)


def test_initial_preferred_directions():
    """Unit vectors, a pure function of (seed, stream + replica), spread
    over the sphere (the reference draws normalised normal deviates,
    src/cpm.cu:224-251)."""
    lib = oracle.lib()
    n = 3000
    a = np.zeros((n + 1, 3))
    b = np.zeros((n + 1, 3))
    c = np.zeros((n + 1, 3))
    lib.orc_init_prefdir(7, 3, 0, n, a.ctypes.data)
    lib.orc_init_prefdir(7, 2, 1, n, b.ctypes.data)
    lib.orc_init_prefdir(8, 3, 0, n, c.ctypes.data)
    np.testing.assert_array_equal(a, b)  # stream + replica is one counter word
    assert not np.array_equal(a, c)
    np.testing.assert_allclose(np.linalg.norm(a, axis=1), 1.0, rtol=0, atol=1e-15)
    assert np.linalg.norm(a.mean(axis=0)) < 0.06
    np.testing.assert_allclose(np.abs(a).mean(axis=0), 0.5, atol=0.03)  # E|x| on the sphere


def test_preferred_direction_update_known_answer():
    """src/kernels.cu:159-212 restated with numpy: displacement from the
    oldest ring slot, divided by its length taken BEFORE the per-axis wrap
    into (-n/2, n/2], blended with the old direction by the diffusion and
    normalised; the medium, empty cells and resting cells keep theirs."""
    n = (10, 8, 12)
    p = oracle.Params()
    p.ndim, p.nx, p.ny, p.nz, p.ncells = 3, n[0], n[1], n[2], 4
    area = np.array([900, 4, 5, 0, 3], np.int32)
    rng = np.random.default_rng(4)
    csum = rng.integers(-50, 200, size=(5, 3)).astype(np.int64)
    csum[3] = 0
    ctype = np.array([0, 1, 2, -1, 1], np.int32)
    diff = np.zeros(32, np.float32)
    diff[1], diff[2] = 0.75, 0.25
    pref = rng.normal(size=(5, 3))
    pref /= np.linalg.norm(pref, axis=1, keepdims=True)
    H, slot = 3, 1
    hist = rng.uniform(0, 8, size=(H, 5, 3))
    cur = np.zeros((5, 3))
    for c in range(5):
        if area[c] > 0:
            m = csum[c] / area[c]
            cur[c] = m - np.array(n) * np.floor(m / np.array(n))
    hist[(slot + 1) % H, 4] = cur[4]  # cell 4 has not moved since the oldest slot
    want = pref.copy()
    old = hist[(slot + 1) % H].copy()
    for c in (1, 2):
        d = cur[c] - old[c]
        length = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
        w = d.copy()
        for k in range(3):
            if w[k] > n[k] // 2:
                w[k] -= n[k]
            if w[k] < -(n[k] // 2):
                w[k] += n[k]
        q = float(diff[ctype[c]])
        v = (w / length) * (1 - q) + pref[c] * q
        want[c] = v / np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    got, h2 = pref.copy(), hist.copy()
    oracle.lib().orc_persist_update(ctypes.byref(p), area.ctypes.data, csum.ctypes.data,
                                    ctype.ctypes.data, diff.ctypes.data, got.ctypes.data,
                                    h2.ctypes.data, H, slot)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(h2[slot], cur)


def test_persistence_steers_a_single_cell():
    """A lone cell with a strong persistence term keeps going: its net
    displacement over several direction updates is several times that of
    the same cell without the term."""
    nn = 20
    z, y, x = np.mgrid[:nn, :nn, :nn]
    lat = np.zeros((nn, nn, nn), np.uint32)
    ball = (x - 10) ** 2 + (y - 10) ** 2 + (z - 10) ** 2 <= 9
    lat[ball] = 1 | (1 << 24)
    J = np.zeros((2, 2), np.float32)
    J[0, 1] = J[1, 0] = 8.0
    out = []
    for lam in (0.0, 30.0):
        s = oracle.OracleSim(lat, 1, J, [0, 2.0], [0, int(ball.sum())], temperature=8.0,
                             persist_lambda=[0, lam], persist_diff=[0, 0.8], history=3,
                             seed=1)
        start = np.array([10.0, 10.0, 10.0])
        for _ in range(10):
            s.run(8)
        m = s.csum[1] / s.area[1]
        out.append(np.linalg.norm((m - start + nn / 2) % nn - nn / 2))
    assert out[1] > 3 * max(out[0], 1.0), out


@pytest.mark.parametrize("shape", [(40, 52), (12, 10, 14)])
def test_oracle_voronoi_matches_kdtree_and_breaks_ties_low(shape):
    """The brute-force labelling equals scipy's periodic k-d tree (the
    workloads' seeding) on random points; with every point duplicated the
    lower index of each pair wins."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(len(shape))
    dims = np.array(shape[::-1], np.float64)
    pts = rng.random((90, len(shape))) * dims
    vals = np.arange(1, 91, dtype=np.uint32)
    lab = oracle.voronoi(shape, pts, vals)
    grids = np.meshgrid(*[np.arange(d, dtype=np.float64) for d in shape[::-1]], indexing="ij")
    coords = np.stack([g.ravel() for g in grids], axis=1)
    _, idx = cKDTree(pts, boxsize=dims).query(coords, k=1)
    kd = np.ascontiguousarray(idx.reshape(tuple(int(d) for d in dims)).transpose()) + 1
    np.testing.assert_array_equal(lab, kd)
    dup = np.concatenate([pts, pts])
    lab2 = oracle.voronoi(shape, dup, np.arange(1, 181, dtype=np.uint32))
    np.testing.assert_array_equal(lab2, lab)


@pytest.mark.parametrize("shape", [(30, 26), (9, 11, 10)])
def test_oracle_boundaries_match_numpy(shape):
    w = W.random_small(shape, 20, ntypes=3, seed=7)
    lat = w.lattice
    T = 4
    want = np.zeros((T, T), np.uint64)
    offs = ([(0, 1), (1, -1), (1, 0), (1, 1)] if lat.ndim == 2 else
            [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)
             if (dz, dy, dx) > (0, 0, 0)])
    for off in offs:
        nb = np.roll(lat, tuple(-o for o in off), axis=tuple(range(lat.ndim)))
        diff = nb != lat
        a, b = (lat >> 24)[diff], (nb >> 24)[diff]
        np.add.at(want, (np.minimum(a, b), np.maximum(a, b)), 1)
    np.testing.assert_array_equal(oracle.boundaries(lat, T), want)


@pytest.mark.parametrize("case", ["plain", "fixed_sticky"])
def test_first_mcs_3d_matches_reference_dh_formula(case):
    """3D: replay one MCS of the oracle's schedule (8 slots of an even box,
    26-neighbour source pick from the same Philox draws) with the
    reference's 3D dH (tests/refmodel.py reference_dh_nb, restating
    src/kernels3d.cu:355-541), copies landing after their slot."""
    import refmodel
    n = 8
    w = W.random_small((n, n, n), 12, ntypes=3, seed=21, temperature=6.0)
    J = np.rint(w.J).astype(int)
    lam_a, lam_p = [1.0] * 4, [0.5] * 4
    tgt_a, tgt_p = [0, 40, 40, 40], [0, 90, 90, 90]
    T = 6.0
    stick = fixed = None
    if case == "fixed_sticky":
        stick = np.zeros((4, 4), int)
        stick[1, 2], stick[2, 1], stick[1, 0], stick[2, 3] = 3, 5, 2, 4
        fixed = [False, False, False, True]
    sim = oracle.OracleSim(w.lattice, w.ncells, J.astype(np.float32), lam_a, tgt_a,
                           lam_p, tgt_p, temperature=T, seed=9, stick=stick, fixed=fixed)
    lat = w.lattice.copy()
    area, perim = sim.area.copy(), sim.perim.copy()
    offs = [(m % 3 - 1, (m // 3) % 3 - 1, m // 9 - 1) for m in range(27) if m != 13]
    accepted = 0
    for cz in (0, 1):
        for cy in (0, 1):
            for cx in (0, 1):
                slot = cz * 9 + cy * 3 + cx
                changes = []
                for z in range(cz, n, 2):
                    for y in range(cy, n, 2):
                        for x in range(cx, n, 2):
                            t = int(lat[z, y, x])
                            nbs = [((x + i) % n, (y + j) % n, (z + k) % n) for i, j, k in offs]
                            vals = [int(lat[c, b, a]) for a, b, c in nbs]
                            if all(v == t for v in vals):
                                continue
                            r = oracle.philox4x32_10([(z * n + y) * n + x, slot, 0, 0], [9, 0])
                            kd = (r[0] * 26) >> 32
                            if vals[kd] == t:
                                continue
                            s = vals[kd]
                            if fixed is not None:
                                if fixed[t >> 24]:
                                    continue
                                if fixed[s >> 24]:
                                    s = 0
                                    if s == t:
                                        continue
                            dH, dps, dpt = refmodel.reference_dh_nb(
                                t, s, vals, area, perim, J, lam_a, tgt_a, lam_p, tgt_p,
                                True, stick)
                            u = ((r[1] >> 8) | 1) * 2.0 ** -24
                            if dH < 0 or u < math.exp(-dH / T):
                                changes.append((x, y, z, s, t, dps, dpt))
                for x, y, z, s, t, dps, dpt in changes:
                    lat[z, y, x] = s
                    accepted += 1
                    if s:
                        area[s & 0xFFFFFF] += 1
                        perim[s & 0xFFFFFF] += dps
                    if t:
                        area[t & 0xFFFFFF] -= 1
                        perim[t & 0xFFFFFF] += dpt
    sim.run(1)
    assert accepted > 5
    assert int(sim.counters[2]) == accepted
    np.testing.assert_array_equal(sim.lattice, lat)
    np.testing.assert_array_equal(sim.area, area)
    np.testing.assert_array_equal(sim.perim, perim)


def test_fp32_dh_error_on_the_4096_tissue():
    """The sweep's FP32 dH against an FP64 recomputation on the 4096^2 tissue
    (FP32 J ~ U[2,20], lambda_area 1, lambda_P 0.5, T 20), over every
    (target, source of another id) pair of the seeded state and of the state
    after 5 MCS, about 2e7 pairs each.  The error is a few FP32 roundings on
    the scale of the terms summed (adhesion ~20 per neighbour, constraint
    terms up to ~1e3 in the seeded state), so it is bounded relative to the
    sum of the terms' magnitudes, not to dH itself, which can be small after
    cancellation.  Bounds: 1e-6 of that scale, and no Metropolis probability
    moved by more than 1e-5.  The figures go to
    test_reports/dh_fp32_vs_fp64.json."""
    import json
    import os
    import pathlib
    from gpucpm import workloads as W
    w = W.tissue_2d()
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=3)
    res = {"seeded": sim.dh_error()}
    sim.run(5)
    res["after_5_mcs"] = sim.dh_error()
    report = pathlib.Path(os.environ.get("CPM_TEST_REPORT_DIR",
                                         pathlib.Path(__file__).resolve().parents[1] /
                                         "test_reports"))
    report.mkdir(exist_ok=True)
    (report / "dh_fp32_vs_fp64.json").write_text(json.dumps(res, indent=1))
    for r in res.values():
        assert r["pairs"] > 10_000_000
        assert r["max_rel"] < 1e-6, r
        assert r["max_accept_prob_diff"] < 1e-5, r
