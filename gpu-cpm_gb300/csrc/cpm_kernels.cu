// cpm_kernels.cu — sm_103a kernels of the Cellular Potts engine.
//
//   sweep_kernel<NDIM, PERIM>  the checkerboard Metropolis sweep, persistent
//                              over all MCS of a run and all replicas of a
//                              batch.  Replaces copyAttempt
//                              (src/kernels2d.cu:44-583) and copyAttempt3d
//                              (src/kernels3d.cu:51-594).
//   init_pass1 / init_pass2    lattice validation and the table recount
//                              (area, perimeter, centroid sums).  Replaces
//                              calculateAreasAndCircumferences{,3d}
//                              (src/kernels2d.cu:5-41, src/kernels3d.cu:3-47).
//   init_prefdir_kernel, persist_fill_kernel, persist_update_kernel
//                              3D persistence: initial preferred directions,
//                              the mean-coordinate ring and the per-run
//                              direction update (src/kernels.cu:159-212).
//   lr_backward_kernel         likelihood-ratio gradient from score sums.
//   voronoi_kernel             periodic Voronoi seeding (bucketed, exact).
//   observe_heterotypic_kernel, observe_boundaries_kernel
//                              sorting order parameter and boundary lengths
//                              by type pair.
//
// Sweep schedule.  Sites are coloured by their class on every axis (even /
// odd / last coordinate of an odd axis); one phase ("slot") is one colour,
// and one MCS runs every non-empty slot in lexicographic (cz, cy, cx) order.
// All targets of a slot are >= 2 apart on each axis, so an attempt never
// reads a site another attempt of the same slot may write; the cell tables
// are read as they stood when the slot began (double-buffered, see
// cpm_internal.h) and the integer deltas are exact and order-free.  The
// result is independent of thread, block and replica order, which is what
// makes the CPU oracle (oracle/cpm_oracle.cpp) reproduce it bit for bit.
//
// Work decomposition.  One block per SM (24 warps at 80 registers in 2D; at
// most 20 at 96 registers in 3D and in score launches), one grid barrier
// per slot.  The unit of work is a warp tile: CX x CY (x CZ)
// targets of one slot of one replica, staged with a one-site halo in the
// warp's own shared memory (periodic wrap resolved while loading; even and
// odd lattice columns kept in separate halves so that 32 consecutive
// targets read 32 consecutive words).  A warp then works its tile in three
// compacted passes, so lanes stay busy although most attempts end early:
//   1. boundary test: a target whose Moore neighbours all carry its own id
//      cannot change; the others are queued;
//   2. Philox draw and source pick for the queued targets; attempts whose
//      source id equals the target's are dropped, the rest are queued with
//      their direction and uniform;
//   3. dH, Metropolis test, lattice write and table deltas.
// A warp never waits for another warp inside a slot, so the warps of an SM
// hide each other's load latencies.  Tiles of a slot are flattened over
// replicas (prefix table per slot).  A single lattice gives each block one
// contiguous band of tile rows, the same in every slot (3D warps claim the
// band's tiles from a shared counter); a batch deals its tiles warp-strided
// over the grid, which balances ragged replicas by work.  Replica dispatch
// instead lets each block run whole replicas with block barriers, and
// hybrid runs (two launches, cpm_engine.cu) combine the two.
//
// Memory.  Mutable data (lattice, tables, deltas, dirty lists) is read with
// ld.global.cg so that no SM serves a stale L1 line after a barrier; the
// per-replica parameters are read-only for the kernel's lifetime.
#include <algorithm>
#include <cstdint>

#include "cpm_device.cuh"
#include "cpm_sweep_common.cuh"

namespace gpucpm {
namespace {


__device__ __forceinline__ int find_task_replica(const int* pre, int nrep,
                                                 int task) {
  // largest r < nrep with pre[r] <= task; empty replicas (pre[r] ==
  // pre[r + 1]) are skipped because a later r shares their prefix.
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pre + mid) <= task)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_site_replica(const DevReplica* reps,
                                                 int nrep, long long g) {
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&reps[mid].lat_off) <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}


// Shared-memory layout of a staged warp tile.  Logical column c of a staged
// row lives at (c & 1) * HALF + (c >> 1): target columns (odd logical
// columns) in the upper half, their left / right neighbours in the lower.
template <int NDIM, int V>
struct Stage {
  using G = TileGeom<NDIM, V>;
  static constexpr int HALF = G::CX + 1;
  static constexpr int SXP = 2 * HALF;
  static constexpr int SY = 2 * G::CY + 1;
  static constexpr int SZ = NDIM == 3 ? 2 * G::CZ + 1 : 1;
  static constexpr int WORDS = SXP * SY * SZ;
  static constexpr int NT = G::CX * G::CY * G::CZ;
  static constexpr int NB = NDIM == 2 ? 8 : 26;

  // shared-memory index of target q's own site (qx = q % CX is the lane)
  __device__ static __forceinline__ int center(int q) {
    const int qx = q % G::CX, qy = (q / G::CX) % G::CY, qz = q / (G::CX * G::CY);
    const int zz = NDIM == 3 ? 2 * qz + 1 : 0;
    return (zz * SY + 2 * qy + 1) * SXP + HALF + qx;
  }
  // offset of neighbour (dz, dy, dx) from a target's own site
  __host__ __device__ static constexpr int offset(int dz, int dy, int dx) {
    return (dz * SY + dy) * SXP + (dx == 0 ? 0 : (dx < 0 ? -HALF : 1 - HALF));
  }
  // offset of the k-th neighbour in (dz, dy, dx) lexicographic order
  __device__ static __forceinline__ int nb_offset(int k) {
    if (NDIM == 2) {
      const int m = k + (k >= 4);
      return offset(0, m / 3 - 1, m % 3 - 1);
    }
    const int m = k + (k >= 13);
    return offset(m / 9 - 1, (m / 3) % 3 - 1, m % 3 - 1);
  }
};

template <int NDIM, int V>
struct WarpSmem {
  uint2 qb[Stage<NDIM, V>::NT];                // (q | dir << 16, uniform word)
  uint32_t tile[Stage<NDIM, V>::WORDS];
  uint16_t qa[Stage<NDIM, V>::NT];
};

// Warps per block of a variant: as many warp tiles as fit in shared memory,
// at most max_sweep_warps (the register file's limit).
template <int NDIM, int V, bool SCORE = false>
constexpr int variant_warps() {
  const size_t w = kSweepSmemMax / sizeof(WarpSmem<NDIM, V>);
  return w < (size_t)max_sweep_warps<NDIM, SCORE>() ? (int)w : max_sweep_warps<NDIM, SCORE>();
}

template <int NDIM, int V, bool SCORE = false>
SweepShape shape_of() {
  using G = TileGeom<NDIM, V>;
  SweepShape s;
  s.variant = V;
  s.cx = G::CX;
  s.cy = G::CY;
  s.cz = G::CZ;
  s.warps = variant_warps<NDIM, V, SCORE>();
  s.smem = sizeof(WarpSmem<NDIM, V>) * (size_t)s.warps;
  return s;
}

// Act model (src/kernels2d.cu:338-473, src/kernels3d.cu:347-470): the
// geometric mean of max(amax + act[i] - tick, 0) over site (x, y, z) and
// those of its neighbours that hold `id`, as exp2 of the mean log2 (own
// log2_pos / exp2_own, summed in neighbour order); 0 when a factor is 0.
// L and A are the replica's lattice and act stamps, read as they stood when
// the phase began (copies of an act run are written after the phase).
template <int NDIM>
__device__ __forceinline__ float act_mean(const uint32_t* L, const uint32_t* A, int x, int y,
                                          int z, int nx, int ny, int nz, uint32_t id, int amax,
                                          long long tick) {
  auto at = [&](int xx, int yy, int zz) { return ((long long)zz * ny + yy) * nx + xx; };
  const long long a0 = (long long)amax + (long long)__ldcg(A + at(x, y, z)) - tick;
  if (a0 <= 0) return 0.0f;
  float sum = log2_pos((float)a0);
  int count = 1;
  const int zlo = NDIM == 3 ? -1 : 0, zhi = NDIM == 3 ? 1 : 0;
  for (int dz = zlo; dz <= zhi; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dz && !dy && !dx) continue;
        const long long n = at(wrap_coord(x + dx, nx), wrap_coord(y + dy, ny),
                               NDIM == 3 ? wrap_coord(z + dz, nz) : 0);
        if (__ldcg(L + n) != id) continue;
        const long long v = (long long)amax + (long long)__ldcg(A + n) - tick;
        if (v <= 0) return 0.0f;
        sum = __fadd_rn(sum, log2_pos((float)v));
        ++count;
      }
  return exp2_own(__fdiv_rn(sum, (float)count));
}

// Warp-reduces a lane's score partial sums and adds them, by lane 0, to the
// (replica, MCS) row of the score buffer: J pairs at their index, then
// lambda_area, lambda_perim and T in that order when enabled.  Clears the
// partial sums.
__device__ __forceinline__ void flush_scores(const SweepArgs& a, float* sc, int rep,
                                             unsigned long long tick) {
#pragma unroll
  for (int k = 0; k < kScoreRegs; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sc[k] += __shfl_xor_sync(kFull, sc[k], o);
  const long long row = (long long)tick - (long long)a.score_base;
  if ((threadIdx.x & 31) == 0 && rep >= 0 && row >= 0 && row < a.score_len) {
    float* dst = a.scores + ((long long)rep * a.score_len + row) * kScoreMax;
    int k = 0;
#pragma unroll
    for (int p = 0; p < kScorePairsMax; ++p)
      if (p < a.score_spec.n_pairs) atomicAdd(dst + k++, sc[p]);
    if (a.score_spec.lambda_area) atomicAdd(dst + k++, sc[kScorePairsMax]);
    if (a.score_spec.lambda_perim) atomicAdd(dst + k++, sc[kScorePairsMax + 1]);
    if (a.score_spec.temperature) atomicAdd(dst + k++, sc[kScorePairsMax + 2]);
  }
#pragma unroll
  for (int k = 0; k < kScoreRegs; ++k) sc[k] = 0.0f;
}

// EXT: the instantiation (variant 0, no scores) with the act term and 3D
// persistence; with act (a.act_on) every accepted copy is deferred to the
// end of its phase.  Kept apart so that the other kernels carry none of its
// registers.  ONE: the instantiation of single-lattice grid launches (tile
// bands per block, the replica index a constant), apart from the batch one
// so that neither carries the other's loop.
template <int NDIM, bool PERIM, int V, bool SCORE, bool EXT = false, bool ONE = false>
__global__ void __launch_bounds__(32 * max_sweep_warps<NDIM, SCORE>(), 1)
    sweep_kernel(const SweepArgs a) {
  using G = TileGeom<NDIM, V>;
  using S = Stage<NDIM, V>;
  constexpr int NB = S::NB;
  constexpr int NT = S::NT;
  constexpr unsigned long long NSLOTS = NDIM == 2 ? 9 : 27;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_ok;
  __shared__ unsigned s_cnt[2];
  __shared__ unsigned long long s_tick0;
  __shared__ int s_claim;
  __shared__ unsigned s_next[2];  // next unclaimed tile of the phase (parity of claim_phase)
  __shared__ unsigned s_pend;  // (act runs) entries on this block's pending list

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wpb = blockDim.x >> 5;  // warps (tiles in flight) per block
  WarpSmem<NDIM, V>& ws = reinterpret_cast<WarpSmem<NDIM, V>*>(smem_raw)[warp];
  const uint32_t k0 = (uint32_t)a.seed, k1 = (uint32_t)(a.seed >> 32);
  int* err = reinterpret_cast<int*>(&a.ctl[kCtlErr]);
  // (kernel-parameter arrays are selected with ?: rather than indexed with
  // a runtime value, which would copy the parameter block to local memory)
  auto blist = [&](int b) { return a.dlist + (2LL * blockIdx.x + b) * a.list_cap; };
  unsigned episode = 0;
  int cnt_rep = -1;
  unsigned long long n_eval = 0, n_acc = 0;  // warp-uniform
  // (score launches) per-lane score sums of replica sc_rep at MCS sc_tick
  float sc[kScoreRegs];
#pragma unroll
  for (int k = 0; k < kScoreRegs; ++k) sc[k] = 0.0f;
  int sc_rep = -1;
  unsigned long long sc_tick = 0;
  if (tid < 2) s_cnt[tid] = 0;
  if (NDIM == 3 && tid < 2) s_next[tid] = 0;
  if (tid == 0) s_pend = 0;
  // Every block reads *tick_ptr before its first barrier arrival, and block
  // 0 advances it only after its last barrier, so all blocks see one value.
  if (tid == 0) s_tick0 = a.tick_ptr ? __ldcg(a.tick_ptr) : a.tick0;
  __syncthreads();

  // Tables of the phase with double-buffer index `cur`.
  auto tables = [&](int cur) {
    PhaseTables<NDIM> pt;
    pt.rap = cur ? a.ap[1] : a.ap[0];
    pt.rcs = cur ? a.cs[1] : a.cs[0];
    pt.wap = cur ? a.ap[0] : a.ap[1];
    pt.wcs = cur ? a.cs[0] : a.cs[1];
    pt.dap = cur ? a.dap[1] : a.dap[0];
    pt.dcs = cur ? a.dcs[1] : a.dcs[0];
    pt.list = blist(cur);
    pt.cnt = &s_cnt[cur];
    return pt;
  };
  // Replay of the deltas of the phase with index `prv` into the copy it
  // read (rows on this block's list only).
  auto replay_phase = [&](int prv) {
    const unsigned n = min(s_cnt[prv], (unsigned)a.list_cap);  // see kErrListFull
    replay<NDIM>(blist(prv), n, prv ? a.dap[1] : a.dap[0],
                 prv ? a.dcs[1] : a.dcs[0], prv ? a.ap[1] : a.ap[0],
                 prv ? a.cs[1] : a.cs[0]);
  };

  // (act runs) the phase's deferred copies and their act stamps, written by
  // the block that made them; callers put a barrier before and after.
  auto apply_pending = [&](unsigned long long tick) {
    const unsigned n = min(s_pend, (unsigned)a.pend_cap);  // see kErrListFull
    const long long base = (long long)blockIdx.x * a.pend_cap;
    for (unsigned j = tid; j < n; j += blockDim.x) {
      const unsigned long long site = __ldcg(a.pend_site + base + j);
      a.lat[site] = __ldcg(a.pend_val + base + j);
      a.act[site] = (uint32_t)tick;
    }
  };

  // One warp tile of replica r (its `local`-th tile of the slot): stage the
  // tile, then boundary test, source pick and dH / test / commit.
  // A tile by its coordinates in the replica's tile grid of the slot (tz is
  // the third coordinate in 3D; in 2D the grid has one layer).
  auto run_tile_at = [&](const PhaseTables<NDIM>& pt, const int r, const int tx,
                         const int ty, const int tz, const int cx, const int cy,
                         const int cz, const unsigned long long tick,
                         const unsigned long long phase) {
    if (r != cnt_rep) {
      if (lane == 0 && cnt_rep >= 0) {
        if (n_eval) atomicAdd(&a.counters[2 * cnt_rep], n_eval);
        if (n_acc) atomicAdd(&a.counters[2 * cnt_rep + 1], n_acc);
      }
      n_eval = n_acc = 0;
      cnt_rep = r;
    }
    if (SCORE && (r != sc_rep || tick != sc_tick)) {  // warp-uniform
      flush_scores(a, sc, sc_rep, sc_tick);
      sc_rep = r;
      sc_tick = tick;
    }
    const DevParams* P = a.params + __ldg(&a.reps[r].pset);
    const unsigned fixed_mask = __ldg(&P->fixed_mask);
    const bool stick_on = __ldg(&P->stick_on) != 0;
    const bool chemo_on = __ldg(&P->chemo_on) != 0;
    const bool act_rec = EXT && __ldg(&P->act_on) != 0;
    const bool persist_rec = EXT && NDIM == 3 && __ldg(&P->persist_on) != 0;
    const int nx = __ldg(&a.reps[r].nx), ny = __ldg(&a.reps[r].ny),
              nz = __ldg(&a.reps[r].nz), ncells = __ldg(&a.reps[r].ncells);
    const long long lat_off = __ldg(&a.reps[r].lat_off);
    const long long cell_off = __ldg(&a.reps[r].cell_off);
    const int ncx = class_count(nx, cx), ncy = class_count(ny, cy),
              ncz = class_count(nz, cz);
    const int i0 = tx * G::CX, j0 = ty * G::CY, l0 = tz * G::CZ;
    const int cntx = min(G::CX, ncx - i0), cnty = min(G::CY, ncy - j0),
              cntz = min(G::CZ, ncz - l0);
    const int xorig = class_coord(nx, cx, i0) - 1;
    const int yorig = class_coord(ny, cy, j0) - 1;
    const int zorig = NDIM == 3 ? class_coord(nz, cz, l0) - 1 : 0;
    const int ux = 2 * cntx + 1, uy = 2 * cnty + 1,
              uz = NDIM == 3 ? 2 * cntz + 1 : 1;
    uint32_t* L = a.lat + lat_off;

    // ---- stage the tile and its halo (periodic wrap applied here) ----
    int gx[3];
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      int v = xorig + lane + 32 * u;
      gx[u] = v < 0 ? v + nx : (v >= nx ? v - nx : v);
    }
    for (int zz = 0; zz < uz; ++zz) {
      int gz = zorig + zz;
      gz = gz < 0 ? gz + nz : (gz >= nz ? gz - nz : gz);
#pragma unroll
      for (int yy = 0; yy < uy; ++yy) {
        int gy = yorig + yy;
        gy = gy < 0 ? gy + ny : (gy >= ny ? gy - ny : gy);
        const uint32_t* src = L + ((long long)gz * ny + gy) * nx;
        uint32_t* dst = ws.tile + (zz * S::SY + yy) * S::SXP;
#pragma unroll
        for (int u = 0; u < 3; ++u) {
          const int c = lane + 32 * u;
          if (c < ux) dst[(c & 1) * S::HALF + (c >> 1)] = __ldcg(src + gx[u]);
        }
      }
    }
    __syncwarp();

    // ---- pass 1: boundary test ---------------------------------------
    int na = 0;
#pragma unroll
    for (int it = 0; it < NT / 32; ++it) {
      const int q = it * 32 + lane;
      const int qy = it % G::CY, qz = it / G::CY;
      bool bnd = false;
      if (lane < cntx && qy < cnty && qz < cntz) {
        const int c = S::center(q);
        const uint32_t t = ws.tile[c];
#pragma unroll
        for (int k = 0; k < NB; ++k) bnd |= ws.tile[c + S::nb_offset(k)] != t;
      }
      const unsigned ball = __ballot_sync(kFull, bnd);
      if (bnd) ws.qa[na + __popc(ball & lanemask_lt())] = (uint16_t)q;
      na += __popc(ball);
    }
    __syncwarp();

    // ---- pass 2: random draw and source pick -------------------------
    int nb = 0;
    for (int base = 0; base < na; base += 32) {
      const int j = base + lane;
      bool keep = false;
      uint2 entry = make_uint2(0u, 0u);
      if (j < na) {
        const int q = ws.qa[j];
        const int qx = q % G::CX, qy = (q / G::CX) % G::CY,
                  qz = q / (G::CX * G::CY);
        const int x = class_coord(nx, cx, i0 + qx);
        const int y = class_coord(ny, cy, j0 + qy);
        const int z = NDIM == 3 ? class_coord(nz, cz, l0 + qz) : 0;
        const long long site = ((long long)z * ny + y) * nx + x;
        uint32_t c0 = (uint32_t)site, c1 = (uint32_t)phase,
                 c2 = a.stream0 + (uint32_t)r, c3 = (uint32_t)(phase >> 32);
        philox4x32_10(c0, c1, c2, c3, k0, k1);
        const int kdir = (int)__umulhi(c0, (unsigned)NB);
        const int c = S::center(q);
        const uint32_t tv = ws.tile[c], sv = ws.tile[c + S::nb_offset(kdir)];
        keep = sv != tv;
        uint32_t medium = 0;  // 1: the source is replaced by the medium
        if (fixed_mask && keep) {
          // a target of a fixed type never changes; a source of a fixed type
          // proposes the medium instead (src/kernels2d.cu:280-290)
          if ((fixed_mask >> ((tv >> 24) & (kMaxTypes - 1))) & 1u) {
            keep = false;
          } else if ((fixed_mask >> ((sv >> 24) & (kMaxTypes - 1))) & 1u) {
            medium = 1;
            keep = tv != 0u;
          }
        }
        entry = make_uint2((uint32_t)q | ((uint32_t)kdir << 16) | (medium << 24), c1);
      }
      const unsigned ball = __ballot_sync(kFull, keep);
      if (keep) ws.qb[nb + __popc(ball & lanemask_lt())] = entry;
      nb += __popc(ball);
    }
    __syncwarp();

    // ---- pass 3: dH, Metropolis test, commit -------------------------
    for (int base = 0; base < nb; base += 32) {
      const int j = base + lane;
      bool accepted = false;
      long long push_s = -1, push_t = -1;  // table rows this lane changed
      if (j < nb) {
        const uint2 entry = ws.qb[j];
        const int q = (int)(entry.x & 0xFFFFu), kdir = (int)((entry.x >> 16) & 0xFFu);
        const int c = S::center(q);
        const uint32_t t = ws.tile[c];
        const uint32_t s = (entry.x >> 24) ? 0u : ws.tile[c + S::nb_offset(kdir)];
        const uint32_t is = s & 0xFFFFFFu, it = t & 0xFFFFFFu;
        if (is > (uint32_t)ncells || it > (uint32_t)ncells) {
          atomicOr(err, kErrBadId);
        } else {
          const int ts = (int)(s >> 24) & (kMaxTypes - 1);
          const int tt = (int)(t >> 24) & (kMaxTypes - 1);
          const long long rs = cell_off + is, rt = cell_off + it;
          const unsigned long long aps = s ? __ldcg(pt.rap + rs) : 0ull;
          const unsigned long long apt = t ? __ldcg(pt.rap + rt) : 0ull;
          // centroid sums, needed only on acceptance: in 2D fetched with the
          // row so that an accepted attempt waits on one L2 round trip; in
          // 3D (three words a side, fewer acceptances) on acceptance
          constexpr bool kEarlyCs = NDIM == 2;
          long long cs_s[NDIM], cs_t[NDIM];
#pragma unroll
          for (int k = 0; k < NDIM; ++k) {
            cs_s[k] = kEarlyCs && s ? __ldcg(pt.rcs + rs * NDIM + k) : 0;
            cs_t[k] = kEarlyCs && t ? __ldcg(pt.rcs + rt * NDIM + k) : 0;
          }
          float e_old = 0.0f, e_new = 0.0f;
          int cnt_s = 0, cnt_t = 0;
          // (score launches) neighbours by type < kScoreTypes, one byte
          // per type: of the new configuration (n != s), of the old (n != t)
          unsigned by_new = 0, by_old = 0;
#pragma unroll
          for (int k = 0; k < NB; ++k) {
            const uint32_t v = ws.tile[c + S::nb_offset(k)];
            const int tn = (int)(v >> 24) & (kMaxTypes - 1);
            if (v != t) e_old = __fadd_rn(e_old, __ldg(&P->J[tt * kMaxTypes + tn]));
            if (v != s) e_new = __fadd_rn(e_new, __ldg(&P->J[ts * kMaxTypes + tn]));
            cnt_s += v == s;
            cnt_t += v == t;
            if (SCORE && tn < kScoreTypes) {
              if (v != s) by_new += 1u << (8 * tn);
              if (v != t) by_old += 1u << (8 * tn);
            }
          }
          if (stick_on) {  // uniform over the tile (one replica)
            // stickiness of the old configuration, summed in neighbour order
            // and added to its adhesion as one term
            float e_st = 0.0f;
#pragma unroll
            for (int k = 0; k < NB; ++k) {
              const uint32_t v = ws.tile[c + S::nb_offset(k)];
              const int tn = (int)(v >> 24) & (kMaxTypes - 1);
              if (v != t) e_st = __fadd_rn(e_st, __ldg(&P->stick[tt * kMaxTypes + tn]));
            }
            e_old = __fadd_rn(e_old, e_st);
          }
          float dH = __fsub_rn(e_new, e_old);
          {
            // chemotaxis first, as in the reference's sum; lambda of the
            // source type, of the target type for a medium source
            float chemo = 0.0f;
            if (chemo_on) {  // uniform over the tile
              const float lam = __ldg(&P->chemo[ts ? ts : tt]);
              if (lam != 0.0f) {
                const int qx = q % G::CX, qy = (q / G::CX) % G::CY,
                          qz = q / (G::CX * G::CY);
                const int x = class_coord(nx, cx, i0 + qx);
                const int y = class_coord(ny, cy, j0 + qy);
                const int z = NDIM == 3 ? class_coord(nz, cz, l0 + qz) : 0;
                const long long sites = (long long)nx * ny * nz;
                chemo = __fmul_rn(-lam, chemo_dot<NDIM>(a.field + NDIM * lat_off, sites, x, y,
                                                          z, kdir, nx, ny, nz));
              }
            }
            // persistence next (3D): lambda of the source type (target type for
            // a medium source), preferred direction of the source cell (of the
            // target cell for a medium source), src/kernels3d.cu:327-343
            if (EXT && NDIM == 3 && persist_rec) {  // uniform over the tile
              const float lam = __ldg(&P->persist_lambda[ts ? ts : tt]);
              if (lam != 0.0f) {
                const int qx = q % G::CX, qy = (q / G::CX) % G::CY,
                          qz = q / (G::CX * G::CY);
                const int x = class_coord(nx, cx, i0 + qx);
                const int y = class_coord(ny, cy, j0 + qy);
                const int z = NDIM == 3 ? class_coord(nz, cz, l0 + qz) : 0;
                float ux, uy, uz;
                int sx, sy, sz;
                unit_dir<NDIM>(kdir, x, y, z, nx, ny, nz, ux, uy, uz, sx, sy, sz);
                const double* pd = a.prefdir + 3 * (is ? rs : rt);
                float c = __fmul_rn(ux, (float)__ldg(pd));
                c = __fmaf_rn(uy, (float)__ldg(pd + 1), c);
                c = __fmaf_rn(uz, (float)__ldg(pd + 2), c);
                chemo = __fadd_rn(chemo, __fmul_rn(-lam, c));
              }
            }
            // act next: lambda and max of the target type, of the source type
            // for a medium target
            if (EXT && act_rec) {  // uniform over the tile
              const int ta = tt ? tt : ts;
              const float lam = __ldg(&P->act_lambda[ta]);
              const int amax_a = __ldg(&P->act_max[ta]);
              if (lam != 0.0f && amax_a != 0) {
                const int qx = q % G::CX, qy = (q / G::CX) % G::CY,
                          qz = q / (G::CX * G::CY);
                const int x = class_coord(nx, cx, i0 + qx);
                const int y = class_coord(ny, cy, j0 + qy);
                const int z = NDIM == 3 ? class_coord(nz, cz, l0 + qz) : 0;
                int sx, sy, sz;
                source_coords<NDIM>(kdir, x, y, z, nx, ny, nz, sx, sy, sz);
                const uint32_t* A = a.act + lat_off;
                const long long tk = (long long)tick;
                const float tgt = t ? act_mean<NDIM>(L, A, x, y, z, nx, ny, nz, t,
                                                     __ldg(&P->act_max[tt]), tk)
                                    : 0.0f;
                const float src = s ? act_mean<NDIM>(L, A, sx, sy, sz, nx, ny, nz, s,
                                                     __ldg(&P->act_max[ts]), tk)
                                    : 0.0f;
                chemo = __fadd_rn(chemo, __fmul_rn(__fdiv_rn(-lam, (float)amax_a),
                                                   __fsub_rn(src, tgt)));
              }
            }
            dH = __fadd_rn(chemo, dH);
          }
          const int dps = NB - 2 * cnt_s;
          const int dpt = 2 * cnt_t - NB;
          if (PERIM && __ldg(&P->perim_on)) {
            if (s) {
              const long long qv = (long long)dps *
                  (2LL * (unpack_perim(aps) - __ldg(&P->tgt_perim[ts])) + dps);
              dH = __fmaf_rn(__ldg(&P->lam_perim[ts]), __ll2float_rn(qv), dH);
            }
            if (t) {
              const long long qv = (long long)dpt *
                  (2LL * (unpack_perim(apt) - __ldg(&P->tgt_perim[tt])) + dpt);
              dH = __fmaf_rn(__ldg(&P->lam_perim[tt]), __ll2float_rn(qv), dH);
            }
          }
          if (s) {
            const long long qv =
                1 + 2LL * (unpack_area(aps) - __ldg(&P->tgt_area[ts]));
            dH = __fmaf_rn(__ldg(&P->lam_area[ts]), __ll2float_rn(qv), dH);
          }
          if (t) {
            const long long qv =
                1 - 2LL * (unpack_area(apt) - __ldg(&P->tgt_area[tt]));
            dH = __fmaf_rn(__ldg(&P->lam_area[tt]), __ll2float_rn(qv), dH);
          }
          const float T = __ldg(&P->temperature);
          bool ok;
          float ex = 1.0f;  // exp(-dH/T) when 0 <= dH and T > 0
          if (dH < 0.0f) {
            ok = true;
          } else if (!(T > 0.0f)) {
            ok = false;
          } else {
            const float u =
                __fmul_rn(__uint2float_rn((entry.y >> 8) | 1u), 0x1p-24f);
            ex = exp_neg(__fdiv_rn(-dH, T));
            ok = u < ex;
          }
          if (SCORE && dH >= 0.0f && T > 0.0f) {
            // d log P(decision) / d theta with P(accept) = min(1, exp(-dH/T)):
            // accept: -g, reject: e/(1-e) g, g = d(dH/T)/d theta.  At
            // dH = 0 exactly (integer parameters make it common) P has a
            // kink, slope -g on one side and 0 on the other; the score takes
            // the mean of the two one-sided derivatives, -g/2.
            const float x = dH / T;
            const float om = x < 1e-2f
                                 ? x * (1.0f - 0.5f * x * (1.0f - (x / 3.0f) *
                                                                      (1.0f - 0.25f * x)))
                                 : 1.0f - ex;  // 1 - exp(-x)
            const float cT = (dH == 0.0f ? -0.5f : (ok ? -1.0f : ex / om)) / T;
#pragma unroll
            for (int p = 0; p < kScorePairsMax; ++p) {
              if (p < a.score_spec.n_pairs) {
                const int pa = a.score_spec.pair_a[p], pb = a.score_spec.pair_b[p];
                int d = 0;
                if (ts == pa) d += (by_new >> (8 * pb)) & 0xFF;
                if (pa != pb && ts == pb) d += (by_new >> (8 * pa)) & 0xFF;
                if (tt == pa) d -= (by_old >> (8 * pb)) & 0xFF;
                if (pa != pb && tt == pb) d -= (by_old >> (8 * pa)) & 0xFF;
                sc[p] += cT * (float)d;
              }
            }
            if (a.score_spec.lambda_area) {
              const int da =
                  (s ? 1 + 2 * (unpack_area(aps) - __ldg(&P->tgt_area[ts])) : 0) +
                  (t ? 1 - 2 * (unpack_area(apt) - __ldg(&P->tgt_area[tt])) : 0);
              sc[kScorePairsMax] += cT * (float)da;
            }
            if (a.score_spec.lambda_perim) {
              const long long dp =
                  (s ? (long long)dps * (2LL * (unpack_perim(aps) -
                                                __ldg(&P->tgt_perim[ts])) + dps)
                     : 0LL) +
                  (t ? (long long)dpt * (2LL * (unpack_perim(apt) -
                                                __ldg(&P->tgt_perim[tt])) + dpt)
                     : 0LL);
              sc[kScorePairsMax + 1] += cT * __ll2float_rn(dp);
            }
            if (a.score_spec.temperature) sc[kScorePairsMax + 2] -= cT * x;
          }
          if (ok) {
            accepted = true;
            const int qx = q % G::CX, qy = (q / G::CX) % G::CY,
                      qz = q / (G::CX * G::CY);
            const int x = class_coord(nx, cx, i0 + qx);
            const int y = class_coord(ny, cy, j0 + qy);
            const int z = NDIM == 3 ? class_coord(nz, cz, l0 + qz) : 0;
            const long long site = ((long long)z * ny + y) * nx + x;
            if (EXT && a.act_on) {  // written after the phase
              const unsigned j = atomicAdd(&s_pend, 1u);
              if ((long long)j < a.pend_cap) {
                const long long e = (long long)blockIdx.x * a.pend_cap + j;
                a.pend_site[e] = (unsigned long long)(lat_off + site);
                a.pend_val[e] = s;
              } else {
                atomicOr(err, kErrListFull);  // reported, never written past the end
              }
            } else {
              L[site] = s;
            }
            const int crd[3] = {x, y, z};
            const int dim[3] = {nx, ny, nz};
            long long img[NDIM];
            if (s) {
#pragma unroll
              for (int k = 0; k < NDIM; ++k)
                img[k] = nearest_image(crd[k], dim[k], unpack_area(aps),
                                       kEarlyCs ? cs_s[k] : __ldcg(pt.rcs + rs * NDIM + k));
              add_delta<NDIM>(pt, rs, 1, dps, img, 1);
              push_s = rs;
            }
            if (t) {
#pragma unroll
              for (int k = 0; k < NDIM; ++k)
                img[k] = nearest_image(crd[k], dim[k], unpack_area(apt),
                                       kEarlyCs ? cs_t[k] : __ldcg(pt.rcs + rt * NDIM + k));
              add_delta<NDIM>(pt, rt, -1, dpt, img, -1);
              push_t = rt;
            }
          }
        }
      }
      n_acc += __popc(__ballot_sync(kFull, accepted));
      // the changed rows onto the block's dirty list: one shared-memory
      // atomic per warp and batch
      const unsigned bs = __ballot_sync(kFull, push_s >= 0);
      const unsigned bt = __ballot_sync(kFull, push_t >= 0);
      if (bs | bt) {  // warp-uniform
        const unsigned npush = (unsigned)(__popc(bs) + __popc(bt));
        unsigned at = 0;
        if (lane == 0) at = atomicAdd(pt.cnt, npush);
        at = __shfl_sync(kFull, at, 0);
        // The host sizes the lists for two rows per attempt; a list that
        // would still overflow is reported, never written past its end.
        if ((long long)at + npush > a.list_cap) {
          if (lane == 0) atomicOr(err, kErrListFull);
        } else {
          if (push_s >= 0) pt.list[at + __popc(bs & lanemask_lt())] = (uint32_t)push_s;
          if (push_t >= 0)
            pt.list[at + __popc(bs) + __popc(bt & lanemask_lt())] = (uint32_t)push_t;
        }
      }
    }
    n_eval += nb;
    __syncwarp();  // the tile buffers are rewritten by the next tile
  };

  // Tiles per row and per layer of replica r's slot (cx, cy).
  auto tile_grid = [&](const int r, const int cx, const int cy, int& tnx, int& tny) {
    tnx = (class_count(__ldg(&a.reps[r].nx), cx) + G::CX - 1) / G::CX;
    tny = (class_count(__ldg(&a.reps[r].ny), cy) + G::CY - 1) / G::CY;
  };
  // A tile by its index within the replica's slot.
  auto run_tile = [&](const PhaseTables<NDIM>& pt, const int r, const int local,
                      const int cx, const int cy, const int cz,
                      const unsigned long long tick, const unsigned long long phase) {
    int tnx, tny;
    tile_grid(r, cx, cy, tnx, tny);
    const int tx = local % tnx, rest = local / tnx;
    const int ty = rest % tny, tz = rest / tny;
    run_tile_at(pt, r, tx, ty, tz, cx, cy, cz, tick, phase);
  };

  // The block's tiles of one phase.  3D: warp w starts with tile w, then
  // claims the next unclaimed one from a shared counter, so the phase ends
  // within one tile on every warp (a 256^3 slot gives a block ~54 tiles of
  // 20 warps: 2.7 rounds).  Counter claim_phase % 2 serves this phase; the
  // other one was last used before the previous barrier and is cleared for
  // the next phase.  2D: warp-strided (2D blocks hold a whole number of
  // rounds on the large lattices, and the claim costs the 2D kernel a spill).
  unsigned claim_phase = 0;
  auto claimed_tiles = [&](int count, auto&& body) {
    unsigned* ctr = &s_next[claim_phase & 1u];
    if (tid == 0) s_next[(claim_phase + 1u) & 1u] = 0u;
    ++claim_phase;
    for (int k = warp; k < count;) {
      body(k);
      unsigned v = 0;
      if (lane == 0) v = atomicAdd(ctr, 1u);
      k = wpb + (int)__shfl_sync(kFull, v, 0);
    }
  };

  if (!a.block_local) {
    // Grid dispatch: the tiles of a slot, over all replicas, are dealt out
    // to every warp of the grid; one grid barrier ends each phase.
    int step = 0;
    for (int m = 0; m < a.mcs; ++m) {
      const unsigned long long tick = s_tick0 + (unsigned long long)m;
      for (int si = 0; si < a.nslot_active; ++si, ++step) {
        const int cur = step & 1, prv = cur ^ 1;
        const PhaseTables<NDIM> pt = tables(cur);
        if (step > 0) replay_phase(prv);
        const int slot = a.slots[si];
        const int cx = slot % 3, cy = (slot / 3) % 3, cz = slot / 9;
        const unsigned long long phase = tick * NSLOTS + (unsigned long long)slot;
        const int* pre = a.task_prefix + slot * (a.nrep + 1);
        const int ntiles = __ldg(pre + a.nrep);
        // One lattice: each block takes one contiguous run of the slot's
        // tiles (rows of tiles in raster order), the same band in every
        // phase, so the band's lines and most of its halo stay with this
        // SM's side of L2.  Batches: tiles dealt round-robin over all warps
        // (the light edge tiles of ragged replicas would unbalance bands).
        if constexpr (ONE) {
          const int per_b = ntiles / (int)gridDim.x, extra = ntiles % (int)gridDim.x;
          const int tb0 = (int)blockIdx.x * per_b + min((int)blockIdx.x, extra);
          const int tb1 = tb0 + per_b + ((int)blockIdx.x < extra ? 1 : 0);
          if constexpr (NDIM == 3) {
            claimed_tiles(tb1 - tb0,
                          [&](int k) { run_tile(pt, 0, tb0 + k, cx, cy, cz, tick, phase); });
          } else {
            // tile coordinates stepped by the warp stride, not divided out
            // per tile
            int tnx, tny;
            tile_grid(0, cx, cy, tnx, tny);
            int task = tb0 + warp;
            int tx = task % tnx, ty = (task / tnx) % tny;
            for (; task < tb1; task += wpb) {
              run_tile_at(pt, 0, tx, ty, 0, cx, cy, cz, tick, phase);
              tx += wpb;
              while (tx >= tnx) {
                tx -= tnx;
                ++ty;
              }
            }
          }
        } else {
          for (int task = (int)blockIdx.x * wpb + warp; task < ntiles;
               task += (int)gridDim.x * wpb) {
            const int i = find_task_replica(pre, a.nrep, task);
            const int r = a.rep_map ? __ldg(a.rep_map + i) : i;
            run_tile(pt, r, task - __ldg(pre + i), cx, cy, cz, tick, phase);
          }
        }
        // The replayed list is consumed; every attempt of the slot is done
        // once all blocks pass the barrier.
        __syncthreads();
        if (tid == 0) s_cnt[prv] = 0;
        if (!grid_barrier(a.ctl, ++episode, &s_ok)) return;
        if (EXT && a.act_on) {  // the slot's copies land before the next slot reads
          apply_pending(tick);
          __syncthreads();
          if (tid == 0) s_pend = 0;
          if (!grid_barrier(a.ctl, ++episode, &s_ok)) return;
        }
      }
    }
    // Final replay: the last phase's deltas into the copy it read, so that
    // both copies agree when the kernel ends.
    if (step > 0) replay_phase((step - 1) & 1);
  } else if constexpr (!ONE) {
    // Replica dispatch: a block claims whole replicas (largest first) and
    // runs all their MCS with block barriers between phases; a replica's
    // lattice and tables then stay in this SM's share of L2.  The one grid
    // barrier makes every block read the starting tick before block 0 can
    // advance it.
    if (!grid_barrier(a.ctl, ++episode, &s_ok)) return;
    for (;;) {
      if (tid == 0) s_claim = (int)atomicAdd(&a.ctl[kCtlQueue], 1u);
      __syncthreads();
      const int qi = s_claim;
      if (qi >= a.queue_len) break;  // block-uniform
      const int r = __ldg(a.rep_order + qi);
      int step = 0;
      for (int m = 0; m < a.mcs; ++m) {
        const unsigned long long tick = s_tick0 + (unsigned long long)m;
        for (int si = 0; si < a.nslot_active; ++si, ++step) {
          const int cur = step & 1, prv = cur ^ 1;
          const PhaseTables<NDIM> pt = tables(cur);
          if (step > 0) replay_phase(prv);
          const int slot = a.slots[si];
          const int cx = slot % 3, cy = (slot / 3) % 3, cz = slot / 9;
          const unsigned long long phase = tick * NSLOTS + (unsigned long long)slot;
          const int* pre = a.task_prefix + slot * (a.nrep + 1);
          const int ntiles = __ldg(pre + r + 1) - __ldg(pre + r);
          if constexpr (NDIM == 3) {
            claimed_tiles(ntiles, [&](int k) { run_tile(pt, r, k, cx, cy, cz, tick, phase); });
          } else {
            for (int local = warp; local < ntiles; local += wpb)
              run_tile(pt, r, local, cx, cy, cz, tick, phase);
          }
          __syncthreads();
          if (tid == 0) s_cnt[prv] = 0;
          if (EXT && a.act_on) {
            apply_pending(tick);
            __syncthreads();
            if (tid == 0) s_pend = 0;
          }
          __syncthreads();
        }
      }
      if (step > 0) replay_phase((step - 1) & 1);
      __syncthreads();
      if (tid < 2) s_cnt[tid] = 0;
      __syncthreads();
    }
  }

  if (lane == 0 && cnt_rep >= 0) {
    if (n_eval) atomicAdd(&a.counters[2 * cnt_rep], n_eval);
    if (n_acc) atomicAdd(&a.counters[2 * cnt_rep + 1], n_acc);
  }
  if (SCORE) flush_scores(a, sc, sc_rep, sc_tick);
  if (a.tick_ptr && a.tick_advance && blockIdx.x == 0 && tid == 0 && a.mcs > 0)
    *a.tick_ptr = s_tick0 + (unsigned long long)a.mcs;
}

// ---- table recount ---------------------------------------------------------

template <int NDIM>
__global__ void __launch_bounds__(kInitThreads)
    init_pass1(const uint32_t* __restrict__ lat,
               const DevReplica* __restrict__ reps, int nrep, long long total,
               unsigned long long* first, int* ctype, uint32_t* ctl) {
  int* err = reinterpret_cast<int*>(&ctl[kCtlErr]);
  const int lane = threadIdx.x & 31;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
       g < total; g += (long long)gridDim.x * blockDim.x) {
    const int r = find_site_replica(reps, nrep, g);
    const long long local = g - __ldg(&reps[r].lat_off);
    const uint32_t v = lat[g];
    const uint32_t id = v & 0xFFFFFFu;
    const int ty = (int)(v >> 24);
    const bool bad = id > (uint32_t)__ldg(&reps[r].ncells);
    if (bad) atomicOr(err, kErrBadId);
    if (ty >= kMaxTypes) atomicOr(err, kErrBadType);
    if (id == 0 && ty != 0) atomicOr(err, kErrMediumType);
    const long long row = bad ? -1 : __ldg(&reps[r].cell_off) + id;
    // Lanes of one cell (neighbouring sites usually share one) check their
    // types against the lowest such lane, which holds the lowest site index
    // and alone updates the row: one CAS and one min per cell and warp.
    const unsigned mask = __activemask();
    const unsigned peers = __match_any_sync(mask, (unsigned long long)row);
    const int leader = __ffs(peers) - 1;
    const int lty = __shfl_sync(mask, ty, leader);
    if (bad) continue;
    if (ty != lty) atomicOr(err, kErrTypeConflict);
    if (lane == leader) {
      const int old = atomicCAS(&ctype[row], -1, ty);
      if (old != -1 && old != ty) atomicOr(err, kErrTypeConflict);
      atomicMin(&first[row], (unsigned long long)local);
    }
  }
}

// Every site of a cell adds 1 to its area, its number of foreign Moore
// neighbours to its perimeter, and its coordinates (periodic image nearest
// the cell's first site in raster order) to its centroid sums.
template <int NDIM>
__global__ void __launch_bounds__(kInitThreads)
    init_pass2(const uint32_t* __restrict__ lat,
               const DevReplica* __restrict__ reps, int nrep, long long total,
               const unsigned long long* __restrict__ first,
               unsigned long long* ap, long long* cs) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
       g < total; g += (long long)gridDim.x * blockDim.x) {
    const int r = find_site_replica(reps, nrep, g);
    const DevReplica R = reps[r];
    const uint32_t v = lat[g];
    const uint32_t id = v & 0xFFFFFFu;
    if (id == 0 || id > (uint32_t)R.ncells) continue;
    const long long local = g - R.lat_off;
    const int x = (int)(local % R.nx);
    const int y = (int)((local / R.nx) % R.ny);
    const int z = (int)(local / ((long long)R.nx * R.ny));
    const uint32_t* L = lat + R.lat_off;
    int foreign = 0;
#pragma unroll
    for (int dz = (NDIM == 3 ? -1 : 0); dz <= (NDIM == 3 ? 1 : 0); ++dz)
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          if (!dz && !dy && !dx) continue;
          int xx = x + dx, yy = y + dy, zz = z + dz;
          xx = xx < 0 ? xx + R.nx : (xx >= R.nx ? xx - R.nx : xx);
          yy = yy < 0 ? yy + R.ny : (yy >= R.ny ? yy - R.ny : yy);
          zz = zz < 0 ? zz + R.nz : (zz >= R.nz ? zz - R.nz : zz);
          foreign += L[((long long)zz * R.ny + yy) * R.nx + xx] != v;
        }
    const long long row = R.cell_off + id;
    atomicAdd(ap + row, pack_delta(1, foreign));
    const long long f = (long long)first[row];
    const int anchor[3] = {(int)(f % R.nx), (int)((f / R.nx) % R.ny),
                           (int)(f / ((long long)R.nx * R.ny))};
    const int crd[3] = {x, y, z};
    const int dim[3] = {R.nx, R.ny, R.nz};
#pragma unroll
    for (int k = 0; k < NDIM; ++k)
      atomicAdd(reinterpret_cast<unsigned long long*>(&cs[row * NDIM + k]),
                (unsigned long long)nearest_image(crd[k], dim[k], 1, anchor[k]));
  }
}

// Failure-detection probe: every block waits at a barrier episode that
// needs twice the blocks the grid has, so the bounded wait runs out and the
// error word records kErrTimeout.  No memory beyond ctl[] is touched.
__global__ void barrier_probe(uint32_t* ctl, unsigned long long timeout_ns) {
  __shared__ int s_ok;
  grid_barrier(ctl, 2u, &s_ok, timeout_ns);
}

template <int NDIM, int V>
const void* sweep_fn_v(bool perim, bool scores, bool act, bool one = false) {
  if (one && !scores && !act)
    return perim ? (const void*)sweep_kernel<NDIM, true, V, false, false, true>
                 : (const void*)sweep_kernel<NDIM, false, V, false, false, true>;
  if constexpr (V == 0) {
    if (act)
      return perim ? (const void*)sweep_kernel<NDIM, true, 0, false, true>
                   : (const void*)sweep_kernel<NDIM, false, 0, false, true>;
  }
  if constexpr (NDIM == 2) {
    if (scores)
      return perim ? (const void*)sweep_kernel<NDIM, true, V, true>
                   : (const void*)sweep_kernel<NDIM, false, V, true>;
  }
  return perim ? (const void*)sweep_kernel<NDIM, true, V, false>
               : (const void*)sweep_kernel<NDIM, false, V, false>;
}

// Score launches exist for 2D lattices (the differentiable ensembles), act
// launches for variant 0 without scores (the engine sees to both).
const void* sweep_fn(int ndim, bool perim, int variant, bool scores, bool act, bool one = false) {
  if (act) variant = 0;
  if (ndim == 2) {
    switch (variant) {
      case 1: return sweep_fn_v<2, 1>(perim, scores, false, one);
      case 2: return sweep_fn_v<2, 2>(perim, scores, false, one);
      case 3: return sweep_fn_v<2, 3>(perim, scores, false, one);
      default: return sweep_fn_v<2, 0>(perim, act ? false : scores, act, one);
    }
  }
  switch (variant) {
    case 1: return sweep_fn_v<3, 1>(perim, false, false, one);
    case 2: return sweep_fn_v<3, 2>(perim, false, false, one);
    case 3: return sweep_fn_v<3, 3>(perim, false, false, one);
    default: return sweep_fn_v<3, 0>(perim, false, act, one);
  }
}

// ---- likelihood-ratio backward ---------------------------------------------
struct Checkpoints {
  int n;
  int t[kMaxCheckpoints];
  // Baseline over replicas beyond this launch's (replicas sharded over
  // processes): sum of O[.][c] and replica count of all shards.
  int use_total;
  int nrep_total;
  float total[kMaxCheckpoints];
};

// grad[k] = sum_r sum_c dL/dO[r][c] (O[r][c] - b[r][c])
//                     * sum_{t < checkpoints[c]} scores[r][t][k]
// with the leave-one-out baseline b[r][c] = mean of O[.][c] over the other
// replicas (0 for a single replica), so that each replica's term is an
// unbiased estimate of dE[O]/dtheta scaled by dL/dO[r][c].  With use_total
// the other replicas are those of every shard (total / nrep_total).
// One block per parameter k; threads stride over replicas, each walking its
// replica's scores once in time order while passing the checkpoints.
__global__ void lr_backward_kernel(const float* __restrict__ scores,
                                   const float* __restrict__ dl_do,
                                   const float* __restrict__ obs, const Checkpoints cp,
                                   int nrep, int len, float* grad) {
  const int ncheck = cp.n;
  const int k = blockIdx.x;
  __shared__ float s_mean[kMaxCheckpoints];  // sum over replicas
  __shared__ float s_red[32];
  for (int c = threadIdx.x; c < ncheck; c += blockDim.x) {
    float m = 0.0f;
    if (cp.use_total) {
      m = cp.total[c];
    } else {
      for (int r = 0; r < nrep; ++r) m += obs[(long long)r * ncheck + c];
    }
    s_mean[c] = m;
  }
  const int nall = cp.use_total ? cp.nrep_total : nrep;
  __syncthreads();
  float acc = 0.0f;
  for (int r = threadIdx.x; r < nrep; r += blockDim.x) {
    float cum = 0.0f;
    int t = 0;
    for (int c = 0; c < ncheck; ++c) {
      const int upto = min(cp.t[c], len);
      for (; t < upto; ++t) cum += scores[((long long)r * len + t) * kScoreMax + k];
      const long long rc = (long long)r * ncheck + c;
      const float o = obs[rc];
      const float dev = nall > 1 ? o - (s_mean[c] - o) / (float)(nall - 1) : o;
      acc += dl_do[rc] * dev * cum;
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (int)(blockDim.x >> 5) ? s_red[threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if (threadIdx.x == 0) grad[k] = v;
  }
}

// ---- 3D persistence ----------------------------------------------------------
__device__ __forceinline__ int find_row_replica(const DevReplica* reps, int nrep, long long row) {
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&reps[mid].cell_off) <= row)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Initial preferred directions: uniform on the sphere, by rejection from the
// cube [-1, 1)^3 with Philox draws of counter (cell, 0xFFFFFFF0 - try,
// stream, 0xFFFFFFFF) (outside the sweep's phases), normalised in double.
// The reference draws normalised Gaussians from std::random_device
// (src/cpm.cu:226-248).
__global__ void init_prefdir_kernel(double* prefdir, const DevReplica* __restrict__ reps,
                                    int nrep, long long rows, unsigned long long seed,
                                    unsigned stream0) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
       row += (long long)gridDim.x * blockDim.x) {
    const int r = find_row_replica(reps, nrep, row);
    const uint32_t cell = (uint32_t)(row - __ldg(&reps[r].cell_off));
    double d[3] = {1.0, 0.0, 0.0};
    for (uint32_t tr = 0; tr < 64; ++tr) {
      uint32_t c0 = cell, c1 = 0xFFFFFFF0u - tr, c2 = stream0 + (uint32_t)r, c3 = 0xFFFFFFFFu;
      philox4x32_10(c0, c1, c2, c3, k0, k1);
      const double x = (double)(c0 >> 8) * 0x1p-23 - 1.0;
      const double y = (double)(c1 >> 8) * 0x1p-23 - 1.0;
      const double z = (double)(c2 >> 8) * 0x1p-23 - 1.0;
      const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
      if (r2 > 0.0 && r2 <= 1.0) {
        const double l = __dsqrt_rn(r2);
        d[0] = __ddiv_rn(x, l);
        d[1] = __ddiv_rn(y, l);
        d[2] = __ddiv_rn(z, l);
        break;
      }
    }
    prefdir[3 * row + 0] = d[0];
    prefdir[3 * row + 1] = d[1];
    prefdir[3 * row + 2] = d[2];
  }
}

// Mean coordinate of a cell on one axis, in [0, n): exact sum / area.
__device__ __forceinline__ double mean_coord(long long sum, long long area, int n) {
  double m = __ddiv_rn((double)sum, (double)area);
  m = __dsub_rn(m, __dmul_rn((double)n, floor(__ddiv_rn(m, (double)n))));
  return m;
}

// hist slots [H][rows][3] all set to the cells' current mean coordinates
// (the reference fills its history at every push, src/cpm.cu:578-583).
__global__ void persist_fill_kernel(double* hist, int H, const unsigned long long* __restrict__ ap,
                                    const long long* __restrict__ cs,
                                    const DevReplica* __restrict__ reps, int nrep, long long rows) {
  for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
       row += (long long)gridDim.x * blockDim.x) {
    const int r = find_row_replica(reps, nrep, row);
    const long long area = unpack_area(__ldg(ap + row));
    const int dims[3] = {__ldg(&reps[r].nx), __ldg(&reps[r].ny), __ldg(&reps[r].nz)};
    for (int k = 0; k < 3; ++k) {
      const double m = area > 0 ? mean_coord(__ldg(cs + 3 * row + k), area, dims[k]) : 0.0;
      for (int h = 0; h < H; ++h) hist[((long long)h * rows + row) * 3 + k] = m;
    }
  }
}

// After a run: the current mean goes into history slot `slot`; the mean of
// slot (slot + 1) % H (H runs ago, the oldest) gives the displacement d.
// As src/kernels.cu:159-212: d is divided by its length taken before the
// per-axis wrap into (-n/2, n/2], then the preferred direction becomes
// normalize(d (1 - p) + pref p) with p the cell type's diffusion; cells with
// no displacement (or no sites) keep theirs.  Double precision throughout.
__global__ void persist_update_kernel(double* prefdir, double* hist, int H, int slot,
                                      const unsigned long long* __restrict__ ap,
                                      const long long* __restrict__ cs,
                                      const int* __restrict__ ctype,
                                      const DevParams* __restrict__ params,
                                      const DevReplica* __restrict__ reps, int nrep,
                                      long long rows) {
  for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
       row += (long long)gridDim.x * blockDim.x) {
    const int r = find_row_replica(reps, nrep, row);
    const long long cell = row - __ldg(&reps[r].cell_off);
    const long long area = unpack_area(__ldg(ap + row));
    const int dims[3] = {__ldg(&reps[r].nx), __ldg(&reps[r].ny), __ldg(&reps[r].nz)};
    double cur[3], d[3];
    for (int k = 0; k < 3; ++k) {
      cur[k] = area > 0 ? mean_coord(__ldg(cs + 3 * row + k), area, dims[k]) : 0.0;
      hist[((long long)slot * rows + row) * 3 + k] = cur[k];
    }
    const int prev_slot = (slot + 1) % H;
    for (int k = 0; k < 3; ++k)
      d[k] = __dsub_rn(cur[k], hist[((long long)prev_slot * rows + row) * 3 + k]);
    if (cell == 0 || area <= 0) continue;
    const double len = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])),
                                            __dmul_rn(d[2], d[2])));
    if (len == 0.0) continue;
    const int ty = __ldg(ctype + row);
    if (ty < 0 || ty >= kMaxTypes) continue;
    const double p = (double)__ldg(&params[__ldg(&reps[r].pset)].persist_diff[ty]);
    double np[3];
    for (int k = 0; k < 3; ++k) {
      double v = d[k];
      if (v > (double)(dims[k] / 2)) v = __dsub_rn(v, (double)dims[k]);
      if (v < (double)(-(dims[k] / 2))) v = __dadd_rn(v, (double)dims[k]);
      v = __ddiv_rn(v, len);
      np[k] = __dadd_rn(__dmul_rn(v, __dsub_rn(1.0, p)), __dmul_rn(prefdir[3 * row + k], p));
    }
    const double l2 = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(np[0], np[0]), __dmul_rn(np[1], np[1])),
                                           __dmul_rn(np[2], np[2])));
    if (l2 == 0.0) continue;
    for (int k = 0; k < 3; ++k) prefdir[3 * row + k] = __ddiv_rn(np[k], l2);
  }
}

// ---- sorting order parameter -------------------------------------------------
// Per replica: number of Moore neighbour pairs (each pair once) of two
// different non-medium cells, and how many of them join cells of different
// types.  counts[2 r] = all such pairs, counts[2 r + 1] = heterotypic ones.
__global__ void observe_heterotypic_kernel(const uint32_t* __restrict__ lat,
                                           const DevReplica* __restrict__ reps, int nrep,
                                           long long total,
                                           unsigned long long* counts) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int r = find_site_replica(reps, nrep, g);
    const DevReplica R = reps[r];
    const long long local = g - R.lat_off;
    const int x = (int)(local % R.nx), y = (int)((local / R.nx) % R.ny);
    const uint32_t v = lat[g];
    unsigned pairs = 0, hetero = 0;
    if (v & 0xFFFFFFu) {
      // forward half of the Moore neighbourhood: (0,1), (1,-1), (1,0), (1,1)
      const int dys[4] = {0, 1, 1, 1}, dxs[4] = {1, -1, 0, 1};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        int xx = x + dxs[k], yy = y + dys[k];
        xx = xx < 0 ? xx + R.nx : (xx >= R.nx ? xx - R.nx : xx);
        yy = yy >= R.ny ? yy - R.ny : yy;
        const uint32_t w = lat[R.lat_off + (long long)yy * R.nx + xx];
        if ((w & 0xFFFFFFu) && w != v) {
          ++pairs;
          hetero += (w >> 24) != (v >> 24);
        }
      }
    }
    if (pairs) {
      atomicAdd(&counts[2 * r], (unsigned long long)pairs);
      if (hetero) atomicAdd(&counts[2 * r + 1], (unsigned long long)hetero);
    }
  }
}

// ---- periodic Voronoi seeding -------------------------------------------------
// One thread per site.  Buckets are scanned ring by ring (Chebyshev distance
// r in bucket units, wrapped; a bucket met twice through the wrap changes
// nothing) until the best squared distance is below the squared lower bound
// r * min(w) of every bucket not yet scanned, so the answer is the exact
// brute-force nearest point with ties to the lowest index.
__device__ __forceinline__ double min_image(double a, double b, int n) {
  double d = fabs(__dsub_rn(a, b));
  const double e = __dsub_rn((double)n, d);
  return e < d ? e : d;
}

__global__ void voronoi_kernel(uint32_t* lat, VoronoiGrid vg, const double* __restrict__ pts,
                               const int* __restrict__ idx, const uint32_t* __restrict__ values,
                               const int* __restrict__ start) {
  const long long sites = (long long)vg.n[0] * vg.n[1] * vg.n[2];
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < sites;
       s += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(s % vg.n[0]), y = (int)((s / vg.n[0]) % vg.n[1]),
              z = (int)(s / ((long long)vg.n[0] * vg.n[1]));
    const double c[3] = {(double)x, (double)y, (double)z};
    int b[3];
    for (int a = 0; a < 3; ++a) {
      b[a] = (int)floor(__ddiv_rn(c[a], vg.w[a]));
      b[a] = b[a] < 0 ? 0 : (b[a] >= vg.g[a] ? vg.g[a] - 1 : b[a]);
    }
    double best = 1e300;
    int best_k = 0x7FFFFFFF;
    uint32_t best_v = 0;
    const int rz_max = vg.ndim == 3 ? 1 : 0;
    for (int r = 0; r <= vg.rmax; ++r) {
      for (int dz = -r * rz_max; dz <= r * rz_max; ++dz)
        for (int dy = -r; dy <= r; ++dy)
          for (int dx = -r; dx <= r; ++dx) {
            const int ax = dx < 0 ? -dx : dx, ay = dy < 0 ? -dy : dy, az = dz < 0 ? -dz : dz;
            const int cheb = ax > ay ? (ax > az ? ax : az) : (ay > az ? ay : az);
            if (cheb != r) continue;  // the shell of ring r only
            int bx = (b[0] + dx) % vg.g[0], by = (b[1] + dy) % vg.g[1],
                bz = (b[2] + dz) % vg.g[2];
            bx += bx < 0 ? vg.g[0] : 0;
            by += by < 0 ? vg.g[1] : 0;
            bz += bz < 0 ? vg.g[2] : 0;
            const int bucket = (bz * vg.g[1] + by) * vg.g[0] + bx;
            const int k1 = __ldg(start + bucket + 1);
            for (int k = __ldg(start + bucket); k < k1; ++k) {
              const double ddx = min_image(c[0], __ldg(pts + 3 * k), vg.n[0]);
              const double ddy = min_image(c[1], __ldg(pts + 3 * k + 1), vg.n[1]);
              double d2 = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy));
              if (vg.ndim == 3) {
                const double ddz = min_image(c[2], __ldg(pts + 3 * k + 2), vg.n[2]);
                d2 = __dadd_rn(d2, __dmul_rn(ddz, ddz));
              }
              const int kk = __ldg(idx + k);
              if (d2 < best || (d2 == best && kk < best_k)) {
                best = d2;
                best_k = kk;
              }
            }
          }
      // every bucket not scanned yet lies at periodic Chebyshev distance
      // >= r + 1, so its points are at least r * min(w) away; the margin
      // covers the rounding of the bucket indices
      const double lb = __dsub_rn(__dmul_rn((double)r, vg.lb_scale), 1e-6);
      if (best_k != 0x7FFFFFFF && lb > 0.0 && best < __dmul_rn(lb, lb)) break;
    }
    if (best_k != 0x7FFFFFFF) best_v = __ldg(values + best_k);
    lat[s] = best_v;
  }
}

// ---- boundary counts per type pair ------------------------------------------
// A block takes tiles of kBoundaryTile sites of one replica, histograms the
// pairs in shared memory and adds the non-zero bins to global memory.
template <int NDIM>
__global__ void observe_boundaries_kernel(const uint32_t* __restrict__ lat,
                                          const DevReplica* __restrict__ reps, int nrep,
                                          const long long* __restrict__ tile_start,
                                          long long ntiles, int T,
                                          unsigned long long* counts) {
  extern __shared__ unsigned int hist[];  // T * T
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int lo = 0, hi = nrep - 1;  // the replica owning tile t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(tile_start + mid) <= t) lo = mid; else hi = mid - 1;
    }
    const int r = lo;
    const DevReplica R = reps[r];
    const long long sites = (long long)R.nx * R.ny * R.nz;
    const long long first = (t - __ldg(tile_start + r)) * kBoundaryTile;
    for (int i = threadIdx.x; i < T * T; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (long long local = first + threadIdx.x;
         local < sites && local < first + kBoundaryTile; local += blockDim.x) {
      const int x = (int)(local % R.nx), y = (int)((local / R.nx) % R.ny),
                z = (int)(local / ((long long)R.nx * R.ny));
      const uint32_t v = lat[R.lat_off + local];
      const int tv = (int)(v >> 24);
      // forward half of the neighbourhood: offsets after (0,0,0) in
      // (dz, dy, dx) row-major order
      for (int m = (NDIM == 3 ? 14 : 5); m < (NDIM == 3 ? 27 : 9); ++m) {
        const int ox = m % 3 - 1, oy = (m / 3) % 3 - 1, oz = NDIM == 3 ? m / 9 - 1 : 0;
        int xx = x + ox, yy = y + oy, zz = z + oz;
        xx = xx < 0 ? xx + R.nx : (xx >= R.nx ? xx - R.nx : xx);
        yy = yy < 0 ? yy + R.ny : (yy >= R.ny ? yy - R.ny : yy);
        zz = zz < 0 ? zz + R.nz : (zz >= R.nz ? zz - R.nz : zz);
        const uint32_t w = lat[R.lat_off + ((long long)zz * R.ny + yy) * R.nx + xx];
        if (w == v) continue;
        const int tw = (int)(w >> 24);
        if (tv >= T || tw >= T) continue;
        const int a = tv < tw ? tv : tw, bb = tv < tw ? tw : tv;
        atomicAdd(&hist[a * T + bb], 1u);
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < T * T; i += blockDim.x)
      if (hist[i]) atomicAdd(&counts[(long long)r * T * T + i], (unsigned long long)hist[i]);
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_voronoi(uint32_t* lat, const VoronoiGrid& vg, const double* pts,
                           const int* idx, const uint32_t* values, const int* start,
                           cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long sites = (long long)vg.n[0] * vg.n[1] * vg.n[2];
  const int grid = (int)std::max(1LL, std::min<long long>((sites + 255) / 256, (long long)sms * 16));
  voronoi_kernel<<<grid, 256, 0, s>>>(lat, vg, pts, idx, values, start);
  return cudaGetLastError();
}

cudaError_t launch_observe_boundaries(int ndim, const uint32_t* lat, const DevReplica* reps,
                                      int nrep, const long long* tile_start, long long ntiles,
                                      int T, unsigned long long* counts, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = (int)std::max(1LL, std::min<long long>(ntiles, (long long)sms * 8));
  const size_t shm = sizeof(unsigned int) * T * T;
  if (ndim == 2)
    observe_boundaries_kernel<2><<<grid, 256, shm, s>>>(lat, reps, nrep, tile_start, ntiles, T,
                                                        counts);
  else
    observe_boundaries_kernel<3><<<grid, 256, shm, s>>>(lat, reps, nrep, tile_start, ntiles, T,
                                                        counts);
  return cudaGetLastError();
}

cudaError_t launch_lr_backward(const float* scores, const float* dl_do,
                               const float* obs, const int* checkpoints, int nrep,
                               int len, int nparam, int ncheck, const float* obs_total,
                               int nrep_total, float* grad, cudaStream_t s) {
  if (ncheck < 1 || ncheck > kMaxCheckpoints || nparam < 1 || nparam > kScoreMax)
    return cudaErrorInvalidValue;
  Checkpoints cp;
  cp.n = ncheck;
  cp.use_total = obs_total ? 1 : 0;
  cp.nrep_total = nrep_total;
  for (int c = 0; c < ncheck; ++c) {
    cp.t[c] = checkpoints[c];
    cp.total[c] = obs_total ? obs_total[c] : 0.0f;
  }
  lr_backward_kernel<<<nparam, 256, 0, s>>>(scores, dl_do, obs, cp, nrep, len, grad);
  return cudaGetLastError();
}

namespace {
int rows_grid(long long rows) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (rows + 255) / 256;
  return (int)std::max(1LL, std::min<long long>(want, (long long)sms * 8));
}
}  // namespace

cudaError_t launch_init_prefdir(double* prefdir, const DevReplica* reps, int nrep,
                                long long rows, unsigned long long seed, unsigned stream0,
                                cudaStream_t s) {
  init_prefdir_kernel<<<rows_grid(rows), 256, 0, s>>>(prefdir, reps, nrep, rows, seed, stream0);
  return cudaGetLastError();
}

cudaError_t launch_persist_fill(double* hist, int H, const unsigned long long* ap,
                                const long long* cs, const DevReplica* reps, int nrep,
                                long long rows, cudaStream_t s) {
  persist_fill_kernel<<<rows_grid(rows), 256, 0, s>>>(hist, H, ap, cs, reps, nrep, rows);
  return cudaGetLastError();
}

cudaError_t launch_persist_update(double* prefdir, double* hist, int H, int slot,
                                  const unsigned long long* ap, const long long* cs,
                                  const int* ctype, const DevParams* params,
                                  const DevReplica* reps, int nrep, long long rows,
                                  cudaStream_t s) {
  persist_update_kernel<<<rows_grid(rows), 256, 0, s>>>(prefdir, hist, H, slot, ap, cs, ctype,
                                                        params, reps, nrep, rows);
  return cudaGetLastError();
}

cudaError_t launch_observe_heterotypic(const uint32_t* lat, const DevReplica* reps,
                                       int nrep, long long total_sites,
                                       unsigned long long* counts, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (total_sites + 255) / 256;
  const int grid = (int)std::max(1LL, std::min<long long>(want, (long long)sms * 8));
  observe_heterotypic_kernel<<<grid, 256, 0, s>>>(lat, reps, nrep, total_sites, counts);
  return cudaGetLastError();
}

SweepShape sweep_shape(int ndim, int variant, bool scores) {
  if (ndim == 2 && scores) {
    switch (variant) {
      case 1: return shape_of<2, 1, true>();
      case 2: return shape_of<2, 2, true>();
      case 3: return shape_of<2, 3, true>();
      default: return shape_of<2, 0, true>();
    }
  }
  if (ndim == 2) {
    switch (variant) {
      case 1: return shape_of<2, 1>();
      case 2: return shape_of<2, 2>();
      case 3: return shape_of<2, 3>();
      default: return shape_of<2, 0>();
    }
  }
  switch (variant) {
    case 1: return shape_of<3, 1>();
    case 2: return shape_of<3, 2>();
    case 3: return shape_of<3, 3>();
    default: return shape_of<3, 0>();
  }
}

int sweep_max_blocks_per_sm(int ndim, bool perim, int variant, bool scores) {
  const SweepShape sh = sweep_shape(ndim, variant, scores);
  const void* fn = sweep_fn(ndim, perim, variant, scores, false);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sh.smem) != cudaSuccess)
    return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, 32 * sh.warps, sh.smem) !=
      cudaSuccess)
    return 0;
  return n;
}

cudaError_t launch_sweep(int ndim, bool perim, int variant, const SweepArgs& a,
                         int grid, cudaStream_t s, bool scores) {
  const bool ext = a.act_on || a.prefdir;
  if (ext) variant = 0;  // the extended-term kernels are built for variant 0
  const SweepShape sh = sweep_shape(ndim, variant, scores && !ext);
  // single-lattice grid launches have kernels of their own (tile bands, the
  // replica index a constant)
  const bool one = a.nrep == 1 && a.rep_map == nullptr && !a.block_local && !scores && !ext;
  const void* fn = sweep_fn(ndim, perim, variant, scores && !ext, ext, one);
  if (scores || ext || one) {  // these kernels get their shared-memory attribute on first use
    const cudaError_t e = cudaFuncSetAttribute(
        fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
    if (e != cudaSuccess) return e;
  }
  void* args[] = {const_cast<SweepArgs*>(&a)};
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(32 * sh.warps), args, sh.smem, s);
}

cudaError_t launch_barrier_probe(uint32_t* ctl, unsigned long long timeout_ns,
                                 cudaStream_t s) {
  void* args[] = {&ctl, &timeout_ns};
  return cudaLaunchCooperativeKernel((const void*)barrier_probe, dim3(2), dim3(32),
                                     args, 0, s);
}

cudaError_t launch_init(int ndim, const uint32_t* lat, const DevReplica* reps,
                        int nrep, long long total_sites, unsigned long long* ap,
                        long long* cs, unsigned long long* first, int* ctype,
                        uint32_t* ctl, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long want = (total_sites + kInitThreads - 1) / kInitThreads;
  const int grid = (int)(want < (long long)sms * 8 ? (want > 0 ? want : 1)
                                                   : (long long)sms * 8);
  if (ndim == 2) {
    init_pass1<2><<<grid, kInitThreads, 0, s>>>(lat, reps, nrep, total_sites,
                                                 first, ctype, ctl);
    init_pass2<2><<<grid, kInitThreads, 0, s>>>(lat, reps, nrep, total_sites,
                                                 first, ap, cs);
  } else {
    init_pass1<3><<<grid, kInitThreads, 0, s>>>(lat, reps, nrep, total_sites,
                                                 first, ctype, ctl);
    init_pass2<3><<<grid, kInitThreads, 0, s>>>(lat, reps, nrep, total_sites,
                                                 first, ap, cs);
  }
  return cudaGetLastError();
}

}  // namespace gpucpm
