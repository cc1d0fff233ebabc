"""Python restatement of the reference's sequential copy-attempt algorithm.

Used by the tests to pin the engine's semantics against the reference's own
outputs.  With one thread (threads_per_block = 1, positions_per_thread =
positions_per_checkerboard = D) the reference sweep src/kernels2d.cu:44-583
is an ordinary sequential Cellular Potts model driven by its Park-Miller
generator, and therefore deterministic for a given seed.  `sequential_run`
repeats that run step by step:
  seed mixing          src/kernels2d.cu:99
  site pick            :199-202 (a = r % ppc, b = r % ppc)
  neighbour pick       :232-241 and src/random.cu:22-28 (dx = r % 3 - 1,
                       wrap with & (D - 1), redraw while it is the site)
  dH                   :346-519 via reference_dh()
  Metropolis test      :522-525 (r = seed / (2^31 - 1))
  commit + tables      :548-569
"""
import math

import numpy as np

M = 2147483647


def next_random(seed):
    """Park-Miller step of src/random.cu:5-12 (exact in integers)."""
    return (seed * 16807) % M


def reference_dh(lat, ax, ay, sx, sy, area, perim, J, lam_a, tgt_a, lam_p, tgt_p,
                 perimeter_on=True, stick=None, s=None, chemo=None):
    """dH of copying (sx, sy) into (ax, ay) as src/kernels2d.cu:346-519
    computes it: integer adhesion sums (stickiness added to the old
    configuration's, :399-400), double lambda terms.  `s` overrides the
    source value (the medium that a fixed source type proposes).  `chemo`
    is the chemotaxis term (:325-334), computed first; the reference's
    energy is a float, so with it every addition is rounded to float (the
    other terms are integers or half-integers, exact either way)."""
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
                e_old += J[tt][tv] + (int(stick[tt][tv]) if stick is not None else 0)
            if s != v:
                e_new += J[ts][tv]
            ops += v == s
            nps += v != s
            opt += v != t
            npt += v == t
    f32 = np.float32
    e = float(e_new - e_old) if chemo is None else float(f32(f32(chemo) + f32(e_new - e_old)))
    if perimeter_on:
        if s:
            P = int(perim[s & 0xFFFFFF])
            Pn = P - ops + nps
            e += lam_p[ts] * ((Pn - tgt_p[ts]) ** 2 - (P - tgt_p[ts]) ** 2)
            e = e if chemo is None else float(f32(e))
        if t:
            P = int(perim[t & 0xFFFFFF])
            Pn = P - opt + npt
            e += lam_p[tt] * ((Pn - tgt_p[tt]) ** 2 - (P - tgt_p[tt]) ** 2)
            e = e if chemo is None else float(f32(e))
    if s:
        e += lam_a[ts] * (1 + 2 * int(area[s & 0xFFFFFF]) - 2 * tgt_a[ts])
        e = e if chemo is None else float(f32(e))
    if t:
        e += lam_a[tt] * (1 - 2 * int(area[t & 0xFFFFFF]) + 2 * tgt_a[tt])
        e = e if chemo is None else float(f32(e))
    return e, (nps - ops), (npt - opt)


def sequential_run(lat, area, perim, J, lam_a, tgt_a, lam_p, tgt_p, T, seed, mcs,
                   perimeter_on=True, stick=None, fixed=None, chemo=None, field=None):
    """The reference's one-thread run (in place); returns the accept count.
    fixed (per type): the checks of src/kernels2d.cu:280-290, after the
    id comparison; a fixed source becomes the medium and is still evaluated
    (and accepted, as a no-op, when the target is the medium too)."""

    D = lat.shape[0]
    seed = next_random(0 + seed)  # calculateIndex(0, 0) + seed
    accepted = 0
    for _ in range(mcs):
        for _ in range(D * D):
            seed = next_random(seed)
            x = seed % D
            seed = next_random(seed)
            y = seed % D
            while True:
                seed = next_random(seed)
                nx = (x + seed % 3 - 1) & (D - 1)
                seed = next_random(seed)
                ny = (y + seed % 3 - 1) & (D - 1)
                if not (nx == x and ny == y):
                    break
            s, t = int(lat[y, x]), int(lat[ny, nx])
            if s == t:
                continue
            if fixed is not None:
                if fixed[t >> 24]:
                    continue
                if fixed[s >> 24]:
                    s = 0
            chem = None
            if chemo is not None:
                # src/kernels2d.cu:302-334: direction from the wrapped
                # coordinates (float), field at the source, double product
                lam = chemo[s >> 24] if (s >> 24) else chemo[t >> 24]
                chem = 0.0
                if lam != 0:
                    dx, dy = np.float32(nx - x), np.float32(ny - y)
                    dl = np.float32(math.sqrt(np.float32(dx * dx + dy * dy)))
                    dx, dy = np.float32(dx / dl), np.float32(dy / dl)
                    chem = -lam * (float(dx) * field[0][y, x] + float(dy) * field[1][y, x])
            dH, dps, dpt = reference_dh(lat, nx, ny, x, y, area, perim, J, lam_a, tgt_a,
                                        lam_p, tgt_p, perimeter_on, stick, s, chem)
            e = np.float32(dH)
            seed = next_random(seed)
            r = np.float32(seed / M)
            if e < 0 or (T > 0 and r < np.float32(math.exp(-float(e) / T))):
                lat[ny, nx] = s
                accepted += 1
                if s:
                    area[s & 0xFFFFFF] += 1
                    if perimeter_on:
                        perim[s & 0xFFFFFF] += dps
                if t:
                    area[t & 0xFFFFFF] -= 1
                    if perimeter_on:
                        perim[t & 0xFFFFFF] += dpt
    return accepted


def heterotypic_fraction(lat):
    """Fraction of Moore-8 neighbour pairs of two different non-medium cells
    whose types differ (the sorting order parameter)."""
    lat = np.asarray(lat).astype(np.int64)
    hetero = total = 0
    for dy, dx in ((0, 1), (1, -1), (1, 0), (1, 1)):
        nb = np.roll(np.roll(lat, -dy, 0), -dx, 1)
        both = ((lat & 0xFFFFFF) != 0) & ((nb & 0xFFFFFF) != 0) & (lat != nb)
        total += int(both.sum())
        hetero += int((both & ((lat >> 24) != (nb >> 24))).sum())
    return hetero / max(total, 1)


def reference_dh_nb(t, s, nb_vals, area, perim, J, lam_a, tgt_a, lam_p, tgt_p,
                    perimeter_on=True, stick=None):
    """dH of copying value s into a target holding t, from the values of the
    target's neighbours (8 in 2D, 26 in 3D), as src/kernels3d.cu:355-541
    (and src/kernels2d.cu:346-519) sum it: integer adhesion (stickiness added
    to the old configuration's), double lambda terms, rounded to float once
    at the end (every term here is an integer or half-integer, exact in
    float either way).  Returns (dH, source perimeter change, target
    perimeter change)."""
    ts, tt = s >> 24, t >> 24
    e_old = e_new = 0
    ops = nps = opt = npt = 0
    for v in nb_vals:
        tv = v >> 24
        if t != v:
            e_old += J[tt][tv] + (int(stick[tt][tv]) if stick is not None else 0)
        if s != v:
            e_new += J[ts][tv]
        ops += v == s
        nps += v != s
        opt += v != t
        npt += v == t
    e = float(e_new - e_old)
    if perimeter_on:
        if s:
            P = int(perim[s & 0xFFFFFF])
            Pn = P - ops + nps
            e += lam_p[ts] * ((Pn - tgt_p[ts]) ** 2 - (P - tgt_p[ts]) ** 2)
        if t:
            P = int(perim[t & 0xFFFFFF])
            Pn = P - opt + npt
            e += lam_p[tt] * ((Pn - tgt_p[tt]) ** 2 - (P - tgt_p[tt]) ** 2)
    if s:
        e += lam_a[ts] * (1 + 2 * int(area[s & 0xFFFFFF]) - 2 * tgt_a[ts])
    if t:
        e += lam_a[tt] * (1 - 2 * int(area[t & 0xFFFFFF]) + 2 * tgt_a[tt])
    return e, (nps - ops), (npt - opt)


def sequential_run_3d(lat, area, perim, J, lam_a, tgt_a, lam_p, tgt_p, T, seed, mcs,
                      perimeter_on=True, stick=None, fixed=None):
    """The reference's one-thread 3D run (src/kernels3d.cu:51-594 with one
    thread, positions_per_thread = positions_per_checkerboard = D,
    non-shared branch), in place; returns the accept count.  lat is
    [z, y, x] with a power-of-two side D.
      seed mixing       :85 (calculateIndex(0, 0, 0) + seed)
      source site       :159-164, 196-199 (three draws, a, b, c = r % D)
      target neighbour  :202-212 (dx = r % 3 - 1 per axis, wrap with
                        & (D - 1), src/random.cu:18-26), redrawn while
                        nx == x && ny == y && nz == y: the reference compares
                        nz with y (:208), so a zero displacement with
                        z != y is kept (and is a no-op) while some true
                        neighbours are redrawn
      fixed types       :251-261
      dH                :355-541 via reference_dh_nb()
      Metropolis test   :544-546 (r = seed / (2^31 - 1))
      commit + tables   :549-582"""
    D = lat.shape[0]
    seed = next_random(0 + seed)
    accepted = 0
    for _ in range(mcs):
        for _ in range(D * D * D):
            seed = next_random(seed)
            x = seed % D
            seed = next_random(seed)
            y = seed % D
            seed = next_random(seed)
            z = seed % D
            while True:
                seed = next_random(seed)
                nx = (x + seed % 3 - 1) & (D - 1)
                seed = next_random(seed)
                ny = (y + seed % 3 - 1) & (D - 1)
                seed = next_random(seed)
                nz = (z + seed % 3 - 1) & (D - 1)
                if not (nx == x and ny == y and nz == y):
                    break
            s, t = int(lat[z, y, x]), int(lat[nz, ny, nx])
            if s == t:
                continue
            if fixed is not None:
                if fixed[t >> 24]:
                    continue
                if fixed[s >> 24]:
                    s = 0
            nb = [int(lat[(nz + k) % D, (ny + j) % D, (nx + i) % D])
                  for k in (-1, 0, 1) for j in (-1, 0, 1) for i in (-1, 0, 1)
                  if (i, j, k) != (0, 0, 0)]
            dH, dps, dpt = reference_dh_nb(t, s, nb, area, perim, J, lam_a, tgt_a, lam_p,
                                           tgt_p, perimeter_on, stick)
            e = np.float32(dH)
            seed = next_random(seed)
            r = np.float32(seed / M)
            if e < 0 or (T > 0 and r < np.float32(math.exp(-float(e) / T))):
                lat[nz, ny, nx] = s
                accepted += 1
                if s:
                    area[s & 0xFFFFFF] += 1
                    if perimeter_on:
                        perim[s & 0xFFFFFF] += dps
                if t:
                    area[t & 0xFFFFFF] -= 1
                    if perimeter_on:
                        perim[t & 0xFFFFFF] += dpt
    return accepted
