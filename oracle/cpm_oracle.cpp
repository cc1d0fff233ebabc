// cpm_oracle.cpp — CPU oracle of the checkerboard Cellular Potts sweep.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file:
// it is loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU
// baseline, as the checker the CUDA engine is compared against bit for bit.
//
// Parity status: the reference (shabaz/gpu-cpm) ships no tests or fixtures,
// and its production runs are nondeterministic (std::random_device seed per
// run, src/cpm.cu:347-350; racy area reads, src/kernels2d.cu:297-298).  Its
// one-thread runs are deterministic: tests/golden/ holds five of them and
// three table recounts, made by the reference's own CUDA build, and the CPU
// tests check this file's table recount against them and, through
// tests/refmodel.py, its dH, test and bookkeeping.  This file restates the
// reference's per-attempt algorithm on a deterministic schedule; the
// restatement is checked against the reference's parallel runs
// statistically on the GPU.
//
// What follows the reference, function by function:
//   * site pick / neighbour pick:  src/kernels2d.cu:199-243 (target and a
//     uniformly random Moore neighbour as source, as in the shared-memory
//     branch :212-226), 3D src/kernels3d.cu:203-243
//   * early out when source id == target id: src/kernels2d.cu:276
//   * fixed types (target fixed: no change; source fixed: the medium is
//     proposed instead): src/kernels2d.cu:280-290, src/kernels3d.cu:251-261
//   * stickiness added to the old configuration's adhesion:
//     src/kernels2d.cu:399-400, src/kernels3d.cu:413-414
//   * adhesion, perimeter, area dH:  src/kernels2d.cu:346-519,
//     src/kernels3d.cu:368-541 (same term order: adhesion, perimeter source,
//     perimeter target, area source, area target)
//   * Metropolis test `dH < 0 || r < exp(-dH/T)`: src/kernels2d.cu:522-525
//   * commit + area / perimeter bookkeeping: src/kernels2d.cu:544-569
//   * centroid add / subtract with periodic unwrapping about the running
//     mean: src/kernels.cu:63-119 (kept as exact int64 sums here)
//   * table initialisation (area, Moore interface count, centroid):
//     src/kernels2d.cu:5-41, src/kernels3d.cu:3-47
//
// Deterministic schedule (the engine's, not the reference's):
//   * Sites are coloured by (x mod 2, y mod 2[, z mod 2]); on an axis of odd
//     length the last coordinate gets a third class 2.  Slot
//     (cz, cy, cx) in lexicographic order is one phase; an MCS runs every
//     non-empty slot once, so each site is the target of exactly one attempt
//     per MCS.  Two targets of one phase are >= 2 apart on every axis (with
//     wrap), so no attempt reads another attempt's target.
//   * Every attempt of a phase reads the cell tables as they were when the
//     phase began; integer deltas are summed after the phase.
//   * The random numbers of an attempt are Philox4x32-10 (Salmon et al.,
//     SC'11, "Parallel random numbers: as easy as 1, 2, 3") of counter
//     (site, phase lo, stream, phase hi) under key (seed lo, seed hi), with
//     phase = tick * 3^d + slot.  Word 0 picks the neighbour (mulhi by the
//     neighbour count); word 1 gives the uniform ((w1 >> 8) | 1) * 2^-24.
//   * dH is FP32: adhesion summed in neighbour order, then each constraint
//     added with one fused multiply-add of lambda and an exact integer.
//     exp is computed by exp_neg() below, an own Cody-Waite + Taylor kernel.
//
// Build: oracle/build.py (g++ -O2 -ffp-contract=off -fopenmp).  Contraction
// must stay off so that no a*b+c is fused behind the code's back.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

constexpr int kMaxTypes = 32;

struct Params {
  int ndim, nx, ny, nz, ncells;
  float J[kMaxTypes * kMaxTypes];  // J[own type][neighbour type]
  float lam_area[kMaxTypes];
  int tgt_area[kMaxTypes];
  float lam_perim[kMaxTypes];
  int tgt_perim[kMaxTypes];
  float temperature;
  uint64_t seed;
  uint32_t stream;
  // stickiness S[own][neighbour], added to the old configuration's
  // adhesion (src/kernels2d.cu:399-400); fixed types (bit t), which never
  // move (src/kernels2d.cu:280-290)
  float stick[kMaxTypes * kMaxTypes];
  uint32_t fixed_mask;
  // chemotaxis lambda per type and the field ([k][z][y][x] floats, or null)
  // (src/kernels2d.cu:302-334, src/kernels3d.cu:275-324)
  float chemo[kMaxTypes];
  const float* field;
  // act model (src/kernels2d.cu:312-473): lambda and max per type, and the
  // act stamps (MCS of the last copy into each site, or null)
  float act_lambda[kMaxTypes];
  int act_max[kMaxTypes];
  uint32_t* act;
  // persistence (3D, src/kernels3d.cu:327-343): lambda per type and the
  // preferred direction of every cell ([ncells+1][3] doubles, or null)
  float persist_lambda[kMaxTypes];
  const double* prefdir;
};

// log2(v), v >= 1, and 2^y in FP32, the library's own (act model): log2 by
// the atanh series after reducing the mantissa to [1/sqrt(2), sqrt(2)),
// 2^y by Cody-Waite reduction and Taylor terms to degree 7.  Written step
// for step as the sweep kernel's log2_pos / exp2_own.
float log2_pos(float v) {
  uint32_t b;
  std::memcpy(&b, &v, 4);
  int e = (int)((b >> 23) & 0xFFu) - 127;
  const uint32_t mb = (b & 0x7FFFFFu) | (127u << 23);
  float m;
  std::memcpy(&m, &mb, 4);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e += 1;
  }
  const float z = (m - 1.0f) / (m + 1.0f);
  const float z2 = z * z;
  float p = 1.0f / 11.0f;
  p = std::fma(p, z2, 1.0f / 9.0f);
  p = std::fma(p, z2, 1.0f / 7.0f);
  p = std::fma(p, z2, 0.2f);
  p = std::fma(p, z2, 1.0f / 3.0f);
  p = std::fma(p, z2, 1.0f);
  return (float)e + (z * p) * 2.8853900817779268f;
}

float exp2_own(float y) {
  const float kf = std::nearbyint(y);
  const float f = y - kf;
  const float r = std::fma(f, 0x1.62e430p-1f, f * -0x1.05c610p-29f);
  float p = 1.0f / 5040.0f;
  p = std::fma(p, r, 1.0f / 720.0f);
  p = std::fma(p, r, 1.0f / 120.0f);
  p = std::fma(p, r, 1.0f / 24.0f);
  p = std::fma(p, r, 1.0f / 6.0f);
  p = std::fma(p, r, 0.5f);
  p = std::fma(p, r, 1.0f);
  p = std::fma(p, r, 1.0f);
  const int k = (int)kf;
  const uint32_t bits = (uint32_t)(k + 127) << 23;
  float s;
  std::memcpy(&s, &bits, 4);
  return p * s;
}

// Geometric mean of max(amax + act[i] - tick, 0) over site (x, y, z) and its
// neighbours holding `id` (src/kernels2d.cu:338-473), as exp2 of the mean
// log2 in neighbour order; 0 when a factor is 0.
float act_mean(const Params& p, const uint32_t* lat, int x, int y, int z, uint32_t id,
               int amax, int64_t tick) {
  const int nx = p.nx, ny = p.ny, nz = p.ndim == 3 ? p.nz : 1;
  auto at = [&](int xx, int yy, int zz) { return ((int64_t)zz * ny + yy) * nx + xx; };
  auto wrapc = [](int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); };
  const int64_t a0 = (int64_t)amax + (int64_t)p.act[at(x, y, z)] - tick;
  if (a0 <= 0) return 0.0f;
  float sum = log2_pos((float)a0);
  int count = 1;
  const int zlo = p.ndim == 3 ? -1 : 0, zhi = p.ndim == 3 ? 1 : 0;
  for (int dz = zlo; dz <= zhi; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dz && !dy && !dx) continue;
        const int64_t n = at(wrapc(x + dx, nx), wrapc(y + dy, ny),
                             p.ndim == 3 ? wrapc(z + dz, nz) : 0);
        if (lat[n] != id) continue;
        const int64_t v = (int64_t)amax + (int64_t)p.act[n] - tick;
        if (v <= 0) return 0.0f;
        sum = sum + log2_pos((float)v);
        ++count;
      }
  return exp2_own(sum / (float)count);
}

// Unit copy direction (target minus source): the raw difference of wrapped
// coordinates in 2D (src/kernels2d.cu:302-309), the nearest image in 3D
// (src/kernels3d.cu:275-299); FP32, rounded step by step.  Returns the
// source site's index.
int64_t unit_dir(const Params& p, int x, int y, int z, int kdir, float& ux, float& uy,
                 float& uz) {
  int ox, oy, oz;
  if (p.ndim == 2) {
    const int m = kdir + (kdir >= 4);
    oz = 0;
    oy = m / 3 - 1;
    ox = m % 3 - 1;
  } else {
    const int m = kdir + (kdir >= 13);
    oz = m / 9 - 1;
    oy = (m / 3) % 3 - 1;
    ox = m % 3 - 1;
  }
  const int nx = p.nx, ny = p.ny, nz = p.ndim == 3 ? p.nz : 1;
  auto wrapc = [](int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); };
  const int sx = wrapc(x + ox, nx), sy = wrapc(y + oy, ny), sz = p.ndim == 3 ? wrapc(z + oz, nz) : 0;
  int dx = x - sx, dy = y - sy, dz = z - sz;
  if (p.ndim == 3) {
    if (dx > nx / 2) dx -= nx;
    if (dx < -(nx / 2)) dx += nx;
    if (dy > ny / 2) dy -= ny;
    if (dy < -(ny / 2)) dy += ny;
    if (dz > nz / 2) dz -= nz;
    if (dz < -(nz / 2)) dz += nz;
  }
  const float fx = (float)dx, fy = (float)dy, fz = (float)dz;
  float s2 = fx * fx;
  s2 = std::fma(fy, fy, s2);
  if (p.ndim == 3) s2 = std::fma(fz, fz, s2);
  const float len = std::sqrt(s2);
  ux = fx / len;
  uy = fy / len;
  uz = p.ndim == 3 ? fz / len : 0.0f;
  return ((int64_t)sz * ny + sy) * nx + sx;
}

// The unit copy direction dotted with the chemotaxis field at the source.
float chemo_dot(const Params& p, int x, int y, int z, int kdir) {
  float ux, uy, uz;
  const int64_t site = unit_dir(p, x, y, z, kdir, ux, uy, uz);
  const int64_t sites = (int64_t)p.nx * p.ny * (p.ndim == 3 ? p.nz : 1);
  float c = ux * p.field[site];
  c = std::fma(uy, p.field[sites + site], c);
  if (p.ndim == 3) c = std::fma(uz, p.field[2 * sites + site], c);
  return c;
}

// The unit copy direction dotted with a preferred direction, each component
// rounded to FP32 (persistence, src/kernels3d.cu:327-343).
float persist_dot(const Params& p, int x, int y, int z, int kdir, const double* pd) {
  float ux, uy, uz;
  unit_dir(p, x, y, z, kdir, ux, uy, uz);
  float c = ux * (float)pd[0];
  c = std::fma(uy, (float)pd[1], c);
  c = std::fma(uz, (float)pd[2], c);
  return c;
}

// ---- Philox4x32-10 --------------------------------------------------------
inline void philox_round(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  const uint32_t n0 = hi1 ^ c[1] ^ k0;
  const uint32_t n2 = hi0 ^ c[3] ^ k1;
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}

inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    philox_round(c, k0, k1);
  }
}

// ---- exp(x) for x <= 0 in FP32 --------------------------------------------
// Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, with ln2 split into its
// FP32 rounding and the remainder; exp(r) by the degree-7 Taylor polynomial
// (1/n! coefficients) in Horner form; 2^k applied by building the exponent.
// Below x = -20 the result is 0: every uniform used by the sweep is at least
// 2^-24 > exp(-20), so the Metropolis test rejects there either way.
inline float exp_neg(float x) {
  if (x < -20.0f) return 0.0f;
  const float kf = std::nearbyint(x * 0x1.715476p+0f);  // x * log2(e)
  float r = std::fma(-kf, 0x1.62e430p-1f, x);           // ln2 (FP32)
  r = std::fma(-kf, -0x1.05c610p-29f, r);               // ln2 - FP32(ln2)
  float p = 0x1.a01a02p-13f;                            // 1/7!
  p = std::fma(p, r, 0x1.6c16c2p-10f);                  // 1/6!
  p = std::fma(p, r, 0x1.111112p-7f);                   // 1/5!
  p = std::fma(p, r, 0x1.555556p-5f);                   // 1/4!
  p = std::fma(p, r, 0x1.555556p-3f);                   // 1/3!
  p = std::fma(p, r, 0x1.000000p-1f);                   // 1/2!
  p = std::fma(p, r, 1.0f);
  p = std::fma(p, r, 1.0f);
  const int k = (int)kf;  // in [-29, 0]
  uint32_t bits = (uint32_t)(k + 127) << 23;
  float scale;
  std::memcpy(&scale, &bits, 4);
  return p * scale;
}

// ---- schedule helpers -------------------------------------------------------
inline int class_count(int n, int c) {
  if (n == 1) return c == 0 ? 1 : 0;
  if (c < 2) return n / 2;
  return n & 1;
}
inline int class_coord(int n, int c, int i) {
  if (n == 1) return 0;
  return c < 2 ? 2 * i + c : n - 1;
}
inline int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// Periodic image of coordinate xc nearest to mean S/a (a >= 1).
inline int64_t image(int xc, int n, int64_t a, int64_t S) {
  const int64_t d = (int64_t)xc * a - S;
  if (2 * d > (int64_t)n * a) return (int64_t)xc - n;
  if (2 * d < -(int64_t)n * a) return (int64_t)xc + n;
  return xc;
}

struct Accepted {
  int64_t site;   // written after the phase, as all of the phase's copies
  uint32_t s, t;  // full site values (id | type << 24)
  int dps, dpt;
  int64_t img_s[3], img_t[3];
};

struct Tables {
  int32_t* area;
  int32_t* perim;
  int64_t* csum;
};

// Parameters the likelihood-ratio scores differentiate (layout of
// cpm_score_spec): J of symmetric type pairs, then a lambda_area and a
// lambda_perim shared by all cell types, then T.  Score slots: pairs at
// 0..5, lambda_area at 6, lambda_perim at 7, T at 8.
constexpr int kScoreSlots = 9;
struct ScoreSpec {
  int n_pairs;
  int pair_a[6];
  int pair_b[6];
  int lambda_area;
  int lambda_perim;
  int temperature;
};

// d log P(decision)/d theta of one evaluated attempt with dH >= 0, in FP64
// from the attempt's (FP32) decision: P(accept) = min(1, exp(-x)), x = dH / T;
// accept contributes -dx/dtheta, reject exp(-x)/(1-exp(-x)) dx/dtheta.  At
// dH = 0 exactly P has a kink (slope -dx/dtheta on one side, 0 on the
// other) and the score is the mean of the two, -dx/dtheta / 2.
// dx/dJ_ab = (changes of the a-b contact count) / T, dx/dlambda_area and
// dx/dlambda_perim = (the integer area / perimeter terms) / T, dx/dT = -x / T.
void add_score(const ScoreSpec& sp, const uint32_t* nb, int N, uint32_t s, uint32_t t,
               int64_t da, int64_t dp, double dH, double T, bool accepted,
               double* sc) {
  const double x = dH / T;
  const double coef = dH == 0.0 ? -0.5 : accepted ? -1.0 : std::exp(-x) / -std::expm1(-x);
  const double cT = coef / T;
  const int ts = (int)(s >> 24), tt = (int)(t >> 24);
  for (int k = 0; k < sp.n_pairs; ++k) {
    const int a = sp.pair_a[k], b = sp.pair_b[k];
    int d = 0;
    for (int m = 0; m < N; ++m) {
      const int tn = (int)(nb[m] >> 24);
      const bool pair_new = (ts == a && tn == b) || (a != b && ts == b && tn == a);
      const bool pair_old = (tt == a && tn == b) || (a != b && tt == b && tn == a);
      if (nb[m] != s && pair_new) ++d;
      if (nb[m] != t && pair_old) --d;
    }
    sc[k] += cT * d;
  }
  if (sp.lambda_area) sc[6] += cT * (double)da;
  if (sp.lambda_perim) sc[7] += cT * (double)dp;
  if (sp.temperature) sc[8] += -cT * x;
}

// One copy attempt at target (x, y, z).  Returns 0 for a no-op, 1 for an
// evaluated and rejected attempt, 2 for an accepted one (lattice written,
// *acc filled).  With `sp`, adds the attempt's score to sc[8].
inline int attempt(const Params& p, uint32_t* lat, const Tables& tb, int x,
                   int y, int z, uint64_t phase, bool perim_on, bool stick_on,
                   Accepted* acc, const ScoreSpec* sp = nullptr,
                   double* sc = nullptr) {
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const int N = p.ndim == 2 ? 8 : 26;
  uint32_t nb[26];
  int m = 0;
  const int zlo = p.ndim == 3 ? -1 : 0, zhi = p.ndim == 3 ? 1 : 0;
  for (int dz = zlo; dz <= zhi; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dz && !dy && !dx) continue;
        const int xx = wrap(x + dx, nx), yy = wrap(y + dy, ny),
                  zz = p.ndim == 3 ? wrap(z + dz, nz) : 0;
        nb[m++] = lat[((int64_t)zz * ny + yy) * nx + xx];
      }
  const int64_t site = ((int64_t)z * ny + y) * nx + x;
  const uint32_t t = lat[site];
  bool interior = true;
  for (int k = 0; k < N; ++k) interior &= (nb[k] == t);
  if (interior) return 0;

  uint32_t r[4] = {(uint32_t)site, (uint32_t)phase, p.stream,
                   (uint32_t)(phase >> 32)};
  philox4x32_10(r, (uint32_t)p.seed, (uint32_t)(p.seed >> 32));
  const int kdir = (int)(((uint64_t)r[0] * (uint64_t)N) >> 32);
  uint32_t s = nb[kdir];
  if (s == t) return 0;
  // a target of a fixed type never changes; a source of a fixed type
  // proposes the medium instead
  if ((p.fixed_mask >> ((t >> 24) & (kMaxTypes - 1))) & 1u) return 0;
  if ((p.fixed_mask >> ((s >> 24) & (kMaxTypes - 1))) & 1u) {
    s = 0;
    if (s == t) return 0;
  }

  const int ts = (int)(s >> 24), tt = (int)(t >> 24);
  float e_old = 0.0f, e_new = 0.0f;
  int cnt_s = 0, cnt_t = 0;
  for (int k = 0; k < N; ++k) {
    const int tn = (int)(nb[k] >> 24);
    if (nb[k] != t) e_old = e_old + p.J[tt * kMaxTypes + tn];
    if (nb[k] != s) e_new = e_new + p.J[ts * kMaxTypes + tn];
    cnt_s += nb[k] == s;
    cnt_t += nb[k] == t;
  }
  if (stick_on) {  // the old configuration's stickiness, as one term
    float e_st = 0.0f;
    for (int k = 0; k < N; ++k)
      if (nb[k] != t) e_st = e_st + p.stick[tt * kMaxTypes + (int)(nb[k] >> 24)];
    e_old = e_old + e_st;
  }
  float dH = e_new - e_old;
  {
    float chemo = 0.0f;
    const float lam = p.chemo[ts ? ts : tt];
    if (lam != 0.0f && p.field) chemo = -lam * chemo_dot(p, x, y, z, kdir);
    if (p.prefdir && p.ndim == 3) {  // persistence next: the source cell's
      // direction and type, the target's for a medium source
      const float lamP = p.persist_lambda[ts ? ts : tt];
      const uint32_t own = (s & 0xFFFFFFu) ? (s & 0xFFFFFFu) : (t & 0xFFFFFFu);
      if (lamP != 0.0f) chemo = chemo + -lamP * persist_dot(p, x, y, z, kdir, p.prefdir + 3 * own);
    }
    if (p.act) {  // act next: of the target type, of the source type for a medium target
      const int ta = tt ? tt : ts;
      const float lamA = p.act_lambda[ta];
      const int amax_a = p.act_max[ta];
      if (lamA != 0.0f && amax_a != 0) {
        int ox, oy, oz;
        if (p.ndim == 2) {
          const int m = kdir + (kdir >= 4);
          oz = 0;
          oy = m / 3 - 1;
          ox = m % 3 - 1;
        } else {
          const int m = kdir + (kdir >= 13);
          oz = m / 9 - 1;
          oy = (m / 3) % 3 - 1;
          ox = m % 3 - 1;
        }
        const int sx = wrap(x + ox, nx), sy = wrap(y + oy, ny),
                  sz = p.ndim == 3 ? wrap(z + oz, nz) : 0;
        const int64_t tk = (int64_t)(phase / (uint64_t)(p.ndim == 2 ? 9 : 27));
        const float tgt = t ? act_mean(p, lat, x, y, z, t, p.act_max[tt], tk) : 0.0f;
        const float src = s ? act_mean(p, lat, sx, sy, sz, s, p.act_max[ts], tk) : 0.0f;
        chemo = chemo + (-lamA / (float)amax_a) * (src - tgt);
      }
    }
    dH = chemo + dH;
  }
  const int dps = N - 2 * cnt_s;  // source cell gains the target site
  const int dpt = 2 * cnt_t - N;  // target cell loses it
  const uint32_t is = s & 0xFFFFFFu, it = t & 0xFFFFFFu;
  if (perim_on) {
    if (s != 0) {
      const int64_t P = tb.perim[is];
      const int64_t q = (int64_t)dps * (2 * (P - p.tgt_perim[ts]) + dps);
      dH = std::fma(p.lam_perim[ts], (float)q, dH);
    }
    if (t != 0) {
      const int64_t P = tb.perim[it];
      const int64_t q = (int64_t)dpt * (2 * (P - p.tgt_perim[tt]) + dpt);
      dH = std::fma(p.lam_perim[tt], (float)q, dH);
    }
  }
  if (s != 0) {
    const int64_t q = 1 + 2 * ((int64_t)tb.area[is] - p.tgt_area[ts]);
    dH = std::fma(p.lam_area[ts], (float)q, dH);
  }
  if (t != 0) {
    const int64_t q = 1 - 2 * ((int64_t)tb.area[it] - p.tgt_area[tt]);
    dH = std::fma(p.lam_area[tt], (float)q, dH);
  }

  bool ok;
  if (dH < 0.0f) {
    ok = true;
  } else if (!(p.temperature > 0.0f)) {
    ok = false;
  } else {
    const float u = (float)((r[1] >> 8) | 1u) * 0x1p-24f;
    ok = u < exp_neg(-dH / p.temperature);
  }
  if (sp && dH >= 0.0f && p.temperature > 0.0f) {
    const int64_t da = (s ? 1 + 2 * ((int64_t)tb.area[is] - p.tgt_area[ts]) : 0) +
                       (t ? 1 - 2 * ((int64_t)tb.area[it] - p.tgt_area[tt]) : 0);
    const int64_t dp =
        (s ? (int64_t)dps * (2 * ((int64_t)tb.perim[is] - p.tgt_perim[ts]) + dps) : 0) +
        (t ? (int64_t)dpt * (2 * ((int64_t)tb.perim[it] - p.tgt_perim[tt]) + dpt) : 0);
    add_score(*sp, nb, N, s, t, da, dp, dH, p.temperature, ok, sc);
  }
  if (!ok) return 1;

  acc->site = site;
  acc->s = s;
  acc->t = t;
  acc->dps = dps;
  acc->dpt = dpt;
  const int coord[3] = {x, y, z};
  const int dims[3] = {nx, ny, nz};
  for (int a = 0; a < p.ndim; ++a) {
    acc->img_s[a] = s ? image(coord[a], dims[a], tb.area[is],
                              tb.csum[(int64_t)is * p.ndim + a])
                      : 0;
    acc->img_t[a] = t ? image(coord[a], dims[a], tb.area[it],
                              tb.csum[(int64_t)it * p.ndim + a])
                      : 0;
  }
  return 2;
}

bool perimeter_enabled(const Params& p) {
  for (int k = 0; k < kMaxTypes; ++k)
    if (p.lam_perim[k] != 0.0f) return true;
  return false;
}

}  // namespace

extern "C" {

// Parameter block shared with oracle/__init__.py (ctypes.Structure).
typedef Params orc_params;

// Philox4x32-10 of one counter block (known-answer tests).
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  philox4x32_10(c, key[0], key[1]);
  std::memcpy(out, c, sizeof c);
}

float orc_exp_neg(float x) { return exp_neg(x); }
float orc_log2_pos(float v) { return log2_pos(v); }
float orc_exp2(float y) { return exp2_own(y); }

// Recompute every table from the lattice.  Returns 0, or a bit set of
// 1: id above ncells, 2: type >= 32, 4: non-zero type on id 0,
// 8: one id carries two types.
int orc_init_tables(const orc_params* pp, const uint32_t* lat, int32_t* area,
                    int32_t* perim, int64_t* csum) {
  const Params& p = *pp;
  const int nx = p.nx, ny = p.ny, nz = p.ndim == 3 ? p.nz : 1;
  const int64_t nsites = (int64_t)nx * ny * nz;
  const int64_t ncell1 = (int64_t)p.ncells + 1;
  std::vector<int64_t> first(ncell1, -1);
  std::vector<int> type(ncell1, -1);
  int err = 0;
  for (int64_t i = 0; i < nsites; ++i) {
    const uint32_t v = lat[i];
    const uint32_t id = v & 0xFFFFFFu;
    const int ty = (int)(v >> 24);
    if (id > (uint32_t)p.ncells) { err |= 1; continue; }
    if (ty >= kMaxTypes) err |= 2;
    if (id == 0 && ty != 0) err |= 4;
    if (type[id] < 0) type[id] = ty;
    else if (type[id] != ty) err |= 8;
    if (first[id] < 0) first[id] = i;
  }
  if (err) return err;
  std::memset(area, 0, sizeof(int32_t) * ncell1);
  std::memset(perim, 0, sizeof(int32_t) * ncell1);
  std::memset(csum, 0, sizeof(int64_t) * ncell1 * p.ndim);
  const int dims[3] = {nx, ny, nz};
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int64_t i = ((int64_t)z * ny + y) * nx + x;
        const uint32_t v = lat[i];
        const uint32_t id = v & 0xFFFFFFu;
        if (id == 0) continue;
        int foreign = 0;
        const int zlo = p.ndim == 3 ? -1 : 0, zhi = p.ndim == 3 ? 1 : 0;
        for (int dz = zlo; dz <= zhi; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              if (!dz && !dy && !dx) continue;
              const int xx = wrap(x + dx, nx), yy = wrap(y + dy, ny),
                        zz = p.ndim == 3 ? wrap(z + dz, nz) : 0;
              foreign += lat[((int64_t)zz * ny + yy) * nx + xx] != v;
            }
        area[id] += 1;
        perim[id] += foreign;
        const int64_t f = first[id];
        const int anchor[3] = {(int)(f % nx), (int)((f / nx) % ny),
                               (int)(f / ((int64_t)nx * ny))};
        const int c[3] = {x, y, z};
        for (int a = 0; a < p.ndim; ++a)
          csum[(int64_t)id * p.ndim + a] += image(c[a], dims[a], 1, anchor[a]);
      }
  return 0;
}

}  // extern "C"

namespace {

int run_impl(const orc_params* pp, uint32_t* lat, int32_t* area, int32_t* perim,
             int64_t* csum, uint64_t tick0, int mcs, int nthreads,
             uint64_t* counters, const ScoreSpec* sp, double* scores) {
  const Params& p = *pp;
  const int nx = p.nx, ny = p.ny, nz = p.ndim == 3 ? p.nz : 1;
  const int nslots = p.ndim == 2 ? 9 : 27;
  const bool perim_on = perimeter_enabled(p);
  bool stick_on = false;
  for (int k = 0; k < kMaxTypes * kMaxTypes; ++k) stick_on = stick_on || p.stick[k] != 0.0f;
  // act stamps are kept when some type has an act lambda (the sweep then
  // writes every copy, and its stamp, after its phase)
  bool act_on = false;
  for (int k = 0; k < kMaxTypes; ++k) act_on = act_on || (p.act && p.act_lambda[k] != 0.0f);
  Tables tb{area, perim, csum};
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  std::vector<std::vector<Accepted>> logs(nthreads);
  std::vector<double> tsc((size_t)nthreads * kScoreSlots, 0.0);
  uint64_t n_att = 0, n_eval = 0, n_acc = 0;
  for (int m = 0; m < mcs; ++m) {
    const uint64_t tick = tick0 + (uint64_t)m;
    for (int cz = 0; cz < (p.ndim == 3 ? 3 : 1); ++cz)
      for (int cy = 0; cy < 3; ++cy)
        for (int cx = 0; cx < 3; ++cx) {
          const int ncx = class_count(nx, cx), ncy = class_count(ny, cy),
                    ncz = class_count(nz, cz);
          if (!ncx || !ncy || !ncz) continue;
          const int slot = (cz * 3 + cy) * 3 + cx;
          const uint64_t phase = tick * (uint64_t)nslots + (uint64_t)slot;
          const int64_t nrows = (int64_t)ncy * ncz;
          uint64_t e = 0, a = 0;
#pragma omp parallel num_threads(nthreads) reduction(+ : e, a)
          {
            const int th = omp_get_thread_num();
            std::vector<Accepted>& log = logs[th];
            double* sc = sp ? &tsc[(size_t)th * kScoreSlots] : nullptr;
            log.clear();
#pragma omp for schedule(static)
            for (int64_t row = 0; row < nrows; ++row) {
              const int z = class_coord(nz, cz, (int)(row / ncy));
              const int y = class_coord(ny, cy, (int)(row % ncy));
              for (int i = 0; i < ncx; ++i) {
                const int x = class_coord(nx, cx, i);
                Accepted acc;
                const int res = attempt(p, lat, tb, x, y, z, phase, perim_on, stick_on,
                                        &acc, sp, sc);
                if (res >= 1) ++e;
                if (res == 2) {
                  ++a;
                  log.push_back(acc);
                }
              }
            }
          }
          n_att += (uint64_t)ncx * ncy * ncz;
          n_eval += e;
          n_acc += a;
          if (sp) {  // scores of this MCS, in the slot order of the spec
            double* row = scores + (size_t)m * 8;
            for (int th = 0; th < nthreads; ++th) {
              double* sc = &tsc[(size_t)th * kScoreSlots];
              int k = 0;
              for (int q = 0; q < sp->n_pairs; ++q) row[k++] += sc[q];
              if (sp->lambda_area) row[k++] += sc[6];
              if (sp->lambda_perim) row[k++] += sc[7];
              if (sp->temperature) row[k++] += sc[8];
              for (int q = 0; q < kScoreSlots; ++q) sc[q] = 0.0;
            }
          }
          // Apply the phase's deltas; integer sums, so order is irrelevant.
          for (auto& log : logs)
            for (const Accepted& c : log) {
              lat[c.site] = c.s;
              if (act_on) p.act[c.site] = (uint32_t)tick;
              if (c.s) {
                const uint32_t is = c.s & 0xFFFFFFu;
                area[is] += 1;
                perim[is] += c.dps;
                for (int d = 0; d < p.ndim; ++d)
                  csum[(int64_t)is * p.ndim + d] += c.img_s[d];
              }
              if (c.t) {
                const uint32_t it = c.t & 0xFFFFFFu;
                area[it] -= 1;
                perim[it] += c.dpt;
                for (int d = 0; d < p.ndim; ++d)
                  csum[(int64_t)it * p.ndim + d] -= c.img_t[d];
              }
            }
          for (auto& log : logs) log.clear();
        }
  }
  if (counters) {
    counters[0] += n_att;
    counters[1] += n_eval;
    counters[2] += n_acc;
  }
  return 0;
}

}  // namespace

extern "C" {

// Run `mcs` Monte Carlo steps from tick `tick0` in place.  counters[0..2]
// receive attempts, evaluated and accepted counts (added to).  `nthreads`
// <= 0 uses every OpenMP thread; the result does not depend on it.
int orc_run(const orc_params* pp, uint32_t* lat, int32_t* area, int32_t* perim,
            int64_t* csum, uint64_t tick0, int mcs, int nthreads,
            uint64_t* counters) {
  return run_impl(pp, lat, area, perim, csum, tick0, mcs, nthreads, counters, nullptr,
                  nullptr);
}

// orc_run that also sums, per MCS, the likelihood-ratio score of every
// evaluated attempt with dH > 0 (FP64, from the attempts' own decisions):
// scores[m * 8 + k] for parameter k of the spec's order, m < mcs (added to).
int orc_run_scores(const orc_params* pp, uint32_t* lat, int32_t* area,
                   int32_t* perim, int64_t* csum, uint64_t tick0, int mcs,
                   int nthreads, uint64_t* counters, const void* spec,
                   double* scores) {
  return run_impl(pp, lat, area, perim, csum, tick0, mcs, nthreads, counters,
                  static_cast<const ScoreSpec*>(spec), scores);
}

// Periodic Voronoi labels by brute force: site (x, y, z) takes values[k] of
// the point with the smallest min-image squared distance, summed x, y, z in
// double; ties go to the lowest k.  points[k*ndim + a], x first.
void orc_voronoi(int ndim, int nx, int ny, int nz, int npoints, const double* points,
                 const uint32_t* values, uint32_t* out) {
  if (ndim == 2) nz = 1;
  const int n[3] = {nx, ny, nz};
  const int64_t sites = (int64_t)nx * ny * nz;
  auto min_image = [](double a, double b, int len) {
    const double d = std::fabs(a - b);
    const double e = (double)len - d;
    return e < d ? e : d;
  };
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < sites; ++s) {
    const double c[3] = {(double)(s % nx), (double)((s / nx) % ny), (double)(s / ((int64_t)nx * ny))};
    double best = 1e300;
    int bk = -1;
    for (int k = 0; k < npoints; ++k) {
      double d2 = 0.0;
      for (int a = 0; a < ndim; ++a) {
        const double d = min_image(c[a], points[(int64_t)k * ndim + a], n[a]);
        d2 = a == 0 ? d * d : d2 + d * d;
      }
      if (d2 < best) {
        best = d2;
        bk = k;
      }
    }
    out[s] = bk >= 0 ? values[bk] : 0u;
  }
}

// Boundary counts by unordered type pair: every Moore pair (each once: the
// forward half of the neighbourhood of every site) of sites with different
// values and types a, b < T adds 1 to out[min*T + max].
void orc_boundaries(int ndim, int nx, int ny, int nz, const uint32_t* lat, int T,
                    uint64_t* out) {
  if (ndim == 2) nz = 1;
  std::memset(out, 0, sizeof(uint64_t) * T * T);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const uint32_t v = lat[((int64_t)z * ny + y) * nx + x];
        for (int m = ndim == 3 ? 14 : 5; m < (ndim == 3 ? 27 : 9); ++m) {
          const int ox = m % 3 - 1, oy = (m / 3) % 3 - 1, oz = ndim == 3 ? m / 9 - 1 : 0;
          const int xx = (x + ox + nx) % nx, yy = (y + oy + ny) % ny, zz = (z + oz + nz) % nz;
          const uint32_t w = lat[((int64_t)zz * ny + yy) * nx + xx];
          if (w == v) continue;
          const int a = (int)(v >> 24), b = (int)(w >> 24);
          if (a >= T || b >= T) continue;
          ++out[(a < b ? a : b) * T + (a < b ? b : a)];
        }
      }
}

// Initial preferred directions of cells 0..ncells of replica `replica`:
// uniform on the sphere (the reference normalises three normal deviates,
// src/cpm.cu:224-251; this library draws by rejection in the cube instead).
// Try k of cell c uses the Philox block (c, 0xFFFFFFF0 - k, stream +
// replica, 0xFFFFFFFF): x, y, z = (word >> 8) * 2^-23 - 1 from its first
// three words, kept when 0 < |v|^2 <= 1; (1, 0, 0) after 64 failed tries.
void orc_init_prefdir(uint64_t seed, uint32_t stream, uint32_t replica, int ncells,
                      double* prefdir) {
  for (int c = 0; c <= ncells; ++c) {
    double d[3] = {1.0, 0.0, 0.0};
    for (uint32_t k = 0; k < 64; ++k) {
      uint32_t w[4] = {(uint32_t)c, 0xFFFFFFF0u - k, stream + replica, 0xFFFFFFFFu};
      philox4x32_10(w, (uint32_t)seed, (uint32_t)(seed >> 32));
      const double x = (double)(w[0] >> 8) * 0x1p-23 - 1.0;
      const double y = (double)(w[1] >> 8) * 0x1p-23 - 1.0;
      const double z = (double)(w[2] >> 8) * 0x1p-23 - 1.0;
      const double r2 = x * x + y * y + z * z;
      if (r2 > 0.0 && r2 <= 1.0) {
        const double l = std::sqrt(r2);
        d[0] = x / l;
        d[1] = y / l;
        d[2] = z / l;
        break;
      }
    }
    std::memcpy(prefdir + 3 * c, d, sizeof d);
  }
}

// Mean coordinate of every cell on every axis, in [0, n): sum / area
// reduced modulo n (0 for cells without sites).  out[(ncells+1)*3].
void orc_mean_coords(const orc_params* pp, const int32_t* area, const int64_t* csum,
                     double* out) {
  const Params& p = *pp;
  const int dims[3] = {p.nx, p.ny, p.nz};
  for (int c = 0; c <= p.ncells; ++c)
    for (int k = 0; k < 3; ++k) {
      double m = 0.0;
      if (area[c] > 0) {
        m = (double)csum[3 * c + k] / (double)area[c];
        m = m - (double)dims[k] * std::floor(m / (double)dims[k]);
      }
      out[3 * c + k] = m;
    }
}

// One preferred-direction update after a run (src/cpm.cu:486-510,
// src/kernels.cu:159-212): the current means go into history slot `slot`
// (hist [H][ncells+1][3]); the displacement d from slot (slot + 1) % H is
// divided by its length taken before the per-axis wrap into (-n/2, n/2],
// and p <- normalize(d (1 - diff) + p diff), diff of the cell's type
// (ctype[c], -1 for none).  Cell 0, empty cells and zero displacements keep
// their direction.
void orc_persist_update(const orc_params* pp, const int32_t* area, const int64_t* csum,
                        const int32_t* ctype, const float* diffusion, double* prefdir,
                        double* hist, int H, int slot) {
  const Params& p = *pp;
  const int n1 = p.ncells + 1;
  const int dims[3] = {p.nx, p.ny, p.nz};
  std::vector<double> cur((size_t)n1 * 3);
  orc_mean_coords(pp, area, csum, cur.data());
  const int prev = (slot + 1) % H;
  for (int c = 0; c < n1; ++c) {
    double d[3];
    for (int k = 0; k < 3; ++k) {
      hist[((int64_t)slot * n1 + c) * 3 + k] = cur[3 * c + k];
      d[k] = cur[3 * c + k] - hist[((int64_t)prev * n1 + c) * 3 + k];
    }
    if (c == 0 || area[c] <= 0) continue;
    const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (len == 0.0) continue;
    const int ty = ctype[c];
    if (ty < 0 || ty >= kMaxTypes) continue;
    const double q = (double)diffusion[ty];
    double np[3];
    for (int k = 0; k < 3; ++k) {
      double v = d[k];
      if (v > (double)(dims[k] / 2)) v = v - (double)dims[k];
      if (v < (double)(-(dims[k] / 2))) v = v + (double)dims[k];
      v = v / len;
      np[k] = v * (1.0 - q) + prefdir[3 * c + k] * q;
    }
    const double l2 = std::sqrt(np[0] * np[0] + np[1] * np[1] + np[2] * np[2]);
    if (l2 == 0.0) continue;
    for (int k = 0; k < 3; ++k) prefdir[3 * c + k] = np[k] / l2;
  }
}

// FP32 dH of the sweep against an FP64 recomputation, over every (target,
// source) pair a sweep could evaluate in the current state: each site and
// each Moore neighbour holding another id.  The FP32 value follows attempt()
// step for step (adhesion and stickiness summed in neighbour order, one
// fused multiply-add per constraint); the FP64 value sums the same terms
// (parameters widened from their FP32 values, integers exact) in double.
// Terms covered: adhesion, stickiness, perimeter and area (the tissue
// workloads').  out[0] pairs, out[1] max |dH32 - dH64|, out[2] max of that
// over the sum of the terms' magnitudes (the scale FP32 rounding works on),
// out[3] max |min(1, e^(-dH32/T)) - min(1, e^(-dH64/T))|, out[4] pairs whose
// sign of dH differs, out[5] max |dH32 - dH64| / max(|dH64|, 1).  Test
// infrastructure.
void orc_dh_error(const orc_params* pp, const uint32_t* lat, const int32_t* area,
                  const int32_t* perim, int nthreads, double* out) {
  const Params& p = *reinterpret_cast<const Params*>(pp);
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const int N = p.ndim == 2 ? 8 : 26;
  const bool perim_on = perimeter_enabled(p);
  const int64_t sites = (int64_t)nx * ny * nz;
  double n_all = 0, max_abs = 0, max_rel = 0, max_pd = 0, flips = 0, max_rel_dh = 0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : n_all, flips) \
    reduction(max : max_abs, max_rel, max_pd, max_rel_dh)
  for (int64_t site = 0; site < sites; ++site) {
    const int x = (int)(site % nx), y = (int)((site / nx) % ny), z = (int)(site / ((int64_t)nx * ny));
    uint32_t nb[26];
    int m = 0;
    const int zlo = p.ndim == 3 ? -1 : 0, zhi = p.ndim == 3 ? 1 : 0;
    for (int dz = zlo; dz <= zhi; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          if (!dz && !dy && !dx) continue;
          nb[m++] = lat[((int64_t)wrap(z + dz, nz) * ny + wrap(y + dy, ny)) * nx + wrap(x + dx, nx)];
        }
    const uint32_t t = lat[site];
    const int tt = (int)(t >> 24);
    for (int kdir = 0; kdir < N; ++kdir) {
      const uint32_t s = nb[kdir];
      if (s == t) continue;
      const int ts = (int)(s >> 24);
      float e_old = 0.0f, e_new = 0.0f, e_st = 0.0f;
      double d_old = 0.0, d_new = 0.0, scale = 0.0;
      int cnt_s = 0, cnt_t = 0;
      for (int k = 0; k < N; ++k) {
        const int tn = (int)(nb[k] >> 24);
        if (nb[k] != t) {
          e_old = e_old + p.J[tt * kMaxTypes + tn];
          e_st = e_st + p.stick[tt * kMaxTypes + tn];
          d_old += (double)p.J[tt * kMaxTypes + tn] + (double)p.stick[tt * kMaxTypes + tn];
          scale += std::fabs((double)p.J[tt * kMaxTypes + tn]) +
                   std::fabs((double)p.stick[tt * kMaxTypes + tn]);
        }
        if (nb[k] != s) {
          e_new = e_new + p.J[ts * kMaxTypes + tn];
          d_new += (double)p.J[ts * kMaxTypes + tn];
          scale += std::fabs((double)p.J[ts * kMaxTypes + tn]);
        }
        cnt_s += nb[k] == s;
        cnt_t += nb[k] == t;
      }
      e_old = e_old + e_st;
      float dH = e_new - e_old;
      double dD = d_new - d_old;
      const int dps = N - 2 * cnt_s, dpt = 2 * cnt_t - N;
      const uint32_t is = s & 0xFFFFFFu, it = t & 0xFFFFFFu;
      if (perim_on) {
        if (s) {
          const int64_t q = (int64_t)dps * (2 * ((int64_t)perim[is] - p.tgt_perim[ts]) + dps);
          dH = std::fma(p.lam_perim[ts], (float)q, dH);
          dD += (double)p.lam_perim[ts] * (double)q;
          scale += std::fabs((double)p.lam_perim[ts] * (double)q);
        }
        if (t) {
          const int64_t q = (int64_t)dpt * (2 * ((int64_t)perim[it] - p.tgt_perim[tt]) + dpt);
          dH = std::fma(p.lam_perim[tt], (float)q, dH);
          dD += (double)p.lam_perim[tt] * (double)q;
          scale += std::fabs((double)p.lam_perim[tt] * (double)q);
        }
      }
      if (s) {
        const int64_t q = 1 + 2 * ((int64_t)area[is] - p.tgt_area[ts]);
        dH = std::fma(p.lam_area[ts], (float)q, dH);
        dD += (double)p.lam_area[ts] * (double)q;
        scale += std::fabs((double)p.lam_area[ts] * (double)q);
      }
      if (t) {
        const int64_t q = 1 - 2 * ((int64_t)area[it] - p.tgt_area[tt]);
        dH = std::fma(p.lam_area[tt], (float)q, dH);
        dD += (double)p.lam_area[tt] * (double)q;
        scale += std::fabs((double)p.lam_area[tt] * (double)q);
      }
      const double err = std::fabs((double)dH - dD);
      n_all += 1;
      max_abs = std::max(max_abs, err);
      max_rel = std::max(max_rel, err / std::max(scale, 1.0));
      max_rel_dh = std::max(max_rel_dh, err / std::max(std::fabs(dD), 1.0));
      if ((dH < 0.0f) != (dD < 0.0)) flips += 1;
      if (p.temperature > 0.0f) {
        const double T = (double)p.temperature;
        const double p32 = dH < 0.0f ? 1.0 : std::exp(-(double)dH / T);
        const double p64 = dD < 0.0 ? 1.0 : std::exp(-dD / T);
        max_pd = std::max(max_pd, std::fabs(p32 - p64));
      }
    }
  }
  out[0] = n_all;
  out[1] = max_abs;
  out[2] = max_rel;
  out[3] = max_pd;
  out[4] = flips;
  out[5] = max_rel_dh;
}

}  // extern "C"
