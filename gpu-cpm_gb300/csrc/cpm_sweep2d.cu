// cpm_sweep2d.cu — the 2D sweep of a single lattice with TMA-staged,
// row-major warp tiles.
//
//   sweep2d_kernel<PERIM, CY>  the checkerboard Metropolis sweep of one 2D
//                              lattice whose width is a multiple of 4 sites
//                              (the tissue workloads); same schedule, same
//                              random stream and the same FP32 operation order
//                              as sweep_kernel (cpm_kernels.cu), so its
//                              results are bit-identical.  Replaces
//                              copyAttempt (src/kernels2d.cu:44-583) for
//                              these lattices.
//
// What differs from sweep_kernel is how a warp tile reaches shared memory and
// how the passes read it:
//  * A tile of 32 x CY targets of one slot spans 64 x 2CY lattice sites; it is
//    staged with its halo as a row-major box of 72 x (2CY + 1) words starting
//    at lattice column 64 tx - 4 (a multiple of 4, so every staged row starts
//    on a 16-byte boundary).  Interior tiles are copied by one
//    cp.async.bulk.tensor.2d issued by lane 0 and completed on a per-warp
//    mbarrier; tiles on the periodic seam (the copy engine cannot wrap) load
//    the same box with 16-byte vector loads, one wrapped coordinate per
//    vector.  Either way the staging costs the warp a handful of
//    instructions per tile instead of one load and one store per site.
//  * Target column c of the tile sits at staged column 2c + 4 + parity, so a
//    lane reads a target's row of three sites with two 8-byte loads: a
//    3 x 3 neighbourhood is six ld.shared.v2 instead of nine scalar loads, and
//    32 lanes read 256 consecutive bytes (two wavefronts, no conflict).
//  * Parameters of the one replica are loaded once per launch.
//
// Coherence.  Lattice words are written with generic stores and read back by
// the copy engine (async proxy) in later phases: every warp's issuing lane
// executes fence.proxy.async.global once per phase, after the grid barrier
// (which orders every SM's writes) and before the phase's first copy.  Within
// a phase every site a tile's attempts read is either one of its own targets
// or a site of another class, which no attempt of the phase writes, so a copy
// never races with a store it depends on (a copied box also holds columns of
// neighbouring tiles' targets, which the tile never reads).
//
// Work split.  Block b of G sweeps tiles b, b + G, b + 2G, ... of a slot
// (row-major, each row of tiles rotated by its row index), the same tiles in
// every phase, so that every block's share samples the whole lattice, holds
// its share of the tiles across the periodic seam in x (loaded without the
// copy engine), and blocks finish a phase close together; its warps claim
// those tiles one at a time from a shared counter, so that the phase ends
// within about one tile on every warp although tiles differ in how many
// attempts they evaluate.
//
// Cluster mode (CLU).  A small lattice is swept by one thread-block cluster
// of G blocks instead of the whole grid.  Block r keeps lattice rows
// [r H, r H + H) in its own shared memory for the whole launch, together
// with one halo row above and one below (copies of the neighbouring blocks'
// boundary rows), every row padded with 4 periodic copies of columns on
// each side.  Tiles are read in place from that strip: no staging.  A block
// writes its targets (always its own rows) in place, keeps its dirty lists in
// shared memory, and after a phase in which it changed one of its two
// boundary rows it stores that row into the neighbour's halo (distributed
// shared memory).  Phases end at the cluster's hardware barrier
// (barrier.cluster, release / acquire at cluster scope) instead of the grid
// barrier in global memory.  The cell tables stay in global memory with the
// same double buffering.  A halo row is read only in phases of the other row
// class, so it never changes while it is read.
#include <cooperative_groups.h>
#include <cuda.h>  // CUtensorMap (the map itself is encoded on the host)

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "cpm_rowtile.cuh"
#include "cpm_sweep_common.cuh"

namespace gpucpm {
namespace {

template <int CY>
struct RowTile {
  static constexpr int SR = 2 * CY + 1;  // staged rows
  static constexpr int WORDS = SR * kPitch;
  static constexpr int NT = 32 * CY;     // targets
  static constexpr unsigned BYTES = WORDS * 4u;
};

// Per-warp shared memory.  The tile leads and the struct is 128-byte
// aligned, as the copy engine's destination must be.
template <int CY>
struct alignas(128) Warp2Smem {
  uint32_t tile[RowTile<CY>::WORDS];
  unsigned long long bar;  // mbarrier of the tile copy
  uint2 qb[RowTile<CY>::NT];
  uint16_t qa[RowTile<CY>::NT];
};

// Per-warp shared memory of the cluster sweep (tiles are read in place).
template <int CY>
struct alignas(16) WarpCluSmem {
  uint2 qb[RowTile<CY>::NT];
  uint16_t qa[RowTile<CY>::NT];
};

template <int CY>
constexpr int row_tile_warps(int cap) {
  const int w = (int)(kSweepSmemMax / sizeof(Warp2Smem<CY>));
  return w < cap ? w : cap;
}

// Target (qx, qy) and its Moore neighbours in (dy, dx) lexicographic order,
// from a tile of row pitch `pitch` words.
template <int PAR>
__device__ __forceinline__ uint32_t nbhd(const uint32_t* tile, int pitch, int qx, int qy,
                                         uint32_t* nb) {
  uint32_t t;
  row3<PAR>(tile + 2 * qy * pitch, 0, qx, nb[0], nb[1], nb[2]);
  row3<PAR>(tile + (2 * qy + 1) * pitch, 0, qx, nb[3], t, nb[4]);
  row3<PAR>(tile + (2 * qy + 2) * pitch, 0, qx, nb[5], nb[6], nb[7]);
  return t;
}

// staged index of target (qx, qy) and offset of neighbour k
template <int PAR>
__device__ __forceinline__ int center_idx(int pitch, int qx, int qy) {
  return (2 * qy + 1) * pitch + 2 * qx + 4 + PAR;
}
__device__ __forceinline__ int nb_off(int pitch, int k) {
  const int m = k + (k >= 4);
  return (m / 3 - 1) * pitch + (m % 3 - 1);
}

// Warps per block of the cluster sweep by tile height: one one-row tile per
// warp covers the 1,024 targets a block of a 16-block cluster has per phase
// on 256^2 (32 x 2 tiles: 16 warps, 32 x 4: 8); taller tiles need fewer
// warps, which then get more registers.  One more warp replays the dirty
// list while the others work their tiles.
__host__ __device__ constexpr int cluster_warps(int cy) {
  return (cy == 1 ? 31 : (cy >= 4 ? 8 : 16)) + 1;  // + the replay warp (1,024 threads at most)
}

template <bool PERIM, int CY, bool CLU = false>
__global__ void __launch_bounds__(32 * (CLU ? cluster_warps(CY) : kMaxSweepWarps), 1)
    sweep2d_kernel(const __grid_constant__ SweepArgs a, const __grid_constant__ CUtensorMap tmap,
                   const int use_tma, const int strip_rows) {
  using RT = RowTile<CY>;
  constexpr unsigned long long NSLOTS = 9;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_ok;
  __shared__ unsigned s_cnt[2];
  __shared__ unsigned long long s_tick0;
  __shared__ unsigned s_next[2];  // next unclaimed tile of the band (by phase parity)
  __shared__ uint32_t s_halo[2];  // (cluster mode) halo rows holding copies of the own edge rows

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wpb = blockDim.x >> 5;
  // (cluster mode) this block's strip of rows leads the dynamic shared
  // memory: strip_rows + 2 rows (halo above, own rows, halo below) of
  // sp = nx + 8 words, lattice column x at word 4 + x of its row
  using WS = std::conditional_t<CLU, WarpCluSmem<CY>, Warp2Smem<CY>>;
  const int sp = CLU ? __ldg(&a.reps[0].nx) + 8 : 0;
  const int strip_words = CLU ? ((strip_rows + 2) * sp + 31) & ~31 : 0;
  uint32_t* const strip = reinterpret_cast<uint32_t*>(smem_raw);
  WS& ws = reinterpret_cast<WS*>(smem_raw + 4 * (size_t)strip_words)[warp];
  // (cluster mode) the block's two dirty lists follow the warp areas
  uint32_t* const slist = reinterpret_cast<uint32_t*>(
      smem_raw + 4 * (size_t)strip_words + sizeof(WS) * (size_t)wpb);
  uint32_t tile_s = 0, bar_s = 0;
  if constexpr (!CLU) {
    tile_s = smem_addr(ws.tile);
    bar_s = smem_addr(&ws.bar);
  }
  const uint32_t k0 = (uint32_t)a.seed, k1 = (uint32_t)(a.seed >> 32);
  int* err = reinterpret_cast<int*>(&a.ctl[kCtlErr]);
  auto blist = [&](int b) {
    return CLU ? slist + (long long)b * a.list_cap
               : a.dlist + (2LL * blockIdx.x + b) * a.list_cap;
  };
  unsigned episode = 0;
  unsigned long long n_eval = 0, n_acc = 0;  // warp-uniform
  uint32_t bar_parity = 0;
  bool fill_ok = true;  // warp-uniform: false once a tile copy timed out
  if (tid < 2) s_cnt[tid] = 0;
  if (tid < 2) s_next[tid] = 0;
  if (tid == 0) s_tick0 = a.tick_ptr ? __ldcg(a.tick_ptr) : a.tick0;
  if (!CLU && lane == 0) {
    mbar_init(bar_s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();

  // The one replica's constants.
  const DevParams* P = a.params + __ldg(&a.reps[0].pset);
  const unsigned fixed_mask = __ldg(&P->fixed_mask);
  const bool stick_on = __ldg(&P->stick_on) != 0;
  const bool chemo_on = __ldg(&P->chemo_on) != 0;
  const bool perim_on = PERIM && __ldg(&P->perim_on) != 0;
  const float T = __ldg(&P->temperature);
  const int nx = __ldg(&a.reps[0].nx), ny = __ldg(&a.reps[0].ny);
  const int ncells = __ldg(&a.reps[0].ncells);
  const long long lat_off = __ldg(&a.reps[0].lat_off);
  const long long cell_off = __ldg(&a.reps[0].cell_off);
  uint32_t* L = a.lat + lat_off;

  // Cluster mode: load this block's rows and its two halo rows (the rows
  // above and below, periodic) with their padding columns, then meet the
  // other blocks so that no block starts before every strip is in place.
  cooperative_groups::cluster_group cluster = cooperative_groups::this_cluster();
  const int crank = CLU ? (int)cluster.block_rank() : 0;
  const int row0 = crank * strip_rows;
  const int row1 = CLU ? min(ny, row0 + strip_rows) : 0;
  const int nown = CLU ? max(0, row1 - row0) : 0;  // own rows (0: an idle block)
  if constexpr (CLU) {
    const int vpr = sp / 4;  // vectors per strip row
    const int nvec = nown > 0 ? (nown + 2) * vpr : 0;
    for (int v = tid; v < nvec; v += blockDim.x) {
      const int r = v / vpr, k = v - r * vpr;
      int gy = row0 - 1 + r;
      gy = gy < 0 ? gy + ny : (gy >= ny ? gy - ny : gy);
      int gx = 4 * k - 4;
      gx = gx < 0 ? gx + nx : (gx >= nx ? gx - nx : gx);
      reinterpret_cast<uint4*>(strip)[v] =
          __ldcg(reinterpret_cast<const uint4*>(L + (long long)gy * nx + gx));
    }
    if (tid < 2 && nown > 0) {
      // the first own row is the bottom halo of the block above, the last
      // one the top halo of the block below
      const int gy = tid == 0 ? (row0 == 0 ? ny - 1 : row0 - 1) : (row1 == ny ? 0 : row1);
      const int nrank = gy / strip_rows;
      const int nrows = min(ny, (nrank + 1) * strip_rows) - nrank * strip_rows;
      const uint32_t local = smem_addr(strip + (tid == 0 ? nrows + 1 : 0) * sp);
      uint32_t remote;
      asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(nrank));
      s_halo[tid] = remote;
    }
    cluster.sync();
  }

  // word x of a copy of an own row at shared::cluster address `row`
  auto halo_store = [&](uint32_t row, int x, uint32_t v) {
    auto st = [](uint32_t addr, uint32_t val) {
      asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(val) : "memory");
    };
    st(row + 4u * (4 + x), v);
    if (x < 4) st(row + 4u * (4 + x + nx), v);
    if (x >= nx - 4) st(row + 4u * (x - nx + 4), v);
  };

  auto tables = [&](int cur) {
    PhaseTables<2> pt;
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
  auto replay_phase = [&](int prv) {
    const unsigned n = min(s_cnt[prv], (unsigned)a.list_cap);  // see kErrListFull
    replay<2, CLU>(blist(prv), n, prv ? a.dap[1] : a.dap[0], prv ? a.dcs[1] : a.dcs[0],
                   prv ? a.ap[1] : a.ap[0], prv ? a.cs[1] : a.cs[0]);
  };

  // Stage tile (tx, ty) of slot (cx, cy): 72 x SR words from lattice column
  // 64 tx - 4 and row yorig.
  auto stage = [&](int X0, int yorig) {
    if constexpr (!CLU) {  // (cluster mode reads its tiles in place)
      const bool interior =
          use_tma && X0 >= 0 && X0 + kPitch <= nx && yorig >= 0 && yorig + RT::SR <= ny;
      if (interior) {
        if (lane == 0) tma_load_tile(tile_s, bar_s, &tmap, X0, yorig, RT::BYTES);
        fill_ok = mbar_wait_bounded(bar_s, bar_parity, err) && fill_ok;
        bar_parity ^= 1u;
        fill_ok = __all_sync(kFull, fill_ok);
      } else {
        for (int v = lane; v < RT::SR * kVecPerRow; v += 32) {
          const int row = v / kVecPerRow, col = v - row * kVecPerRow;
          int gy = yorig + row;
          gy = gy < 0 ? gy + ny : (gy >= ny ? gy - ny : gy);
          int gx = X0 + 4 * col;
          gx = gx < 0 ? gx + nx : (gx >= nx ? gx - nx : gx);
          const uint4 val = __ldcg(reinterpret_cast<const uint4*>(L + (long long)gy * nx + gx));
          *reinterpret_cast<uint4*>(ws.tile + row * kPitch + 4 * col) = val;
        }
        __syncwarp();
      }
    }
  };

  // One warp tile, column parity PAR (= cx).
  // Tile (tx, target rows j0 ...) of slot (cx, cy); rows at and beyond jend
  // belong to another tile row (the slot's end, or another block's strip in
  // cluster mode).
  auto run_tile = [&](auto par, const PhaseTables<2>& pt, const int tx, const int j0,
                      const int jend,
                      const int cy, const unsigned long long phase) {
    constexpr int PAR = decltype(par)::value;
    const int ncx = nx >> 1;
    const int i0 = tx * 32;
    const int cntx = min(32, ncx - i0), cnty = min(CY, jend - j0);
    const int X0 = 2 * i0 - 4;
    const int yorig = class_coord(ny, cy, j0) - 1;
    // the tile's box (staged, or in place in the strip) and its row pitch
    const uint32_t* tb;
    int pitch;
    if constexpr (CLU) {
      tb = strip + (yorig - row0 + 1) * sp + 2 * i0;
      pitch = sp;
    } else {
      stage(X0, yorig);
      if (!fill_ok) return;  // a copy timed out: the phase's barrier reports it
      tb = ws.tile;
      pitch = kPitch;
    }

    // ---- pass 1: boundary test ---------------------------------------
    // (cluster mode: every row's test first, its loads free to overlap,
    // then the list; the grid sweeps, with more warps to hide latency, are
    // faster row by row)
    auto boundary = [&](int qy) {
      bool bnd = false;
      if (lane < cntx && qy < cnty) {
        uint32_t nb[8];
        const uint32_t t = nbhd<PAR>(tb, pitch, lane, qy, nb);
#pragma unroll
        for (int k = 0; k < 8; ++k) bnd |= nb[k] != t;
      }
      return bnd;
    };
    unsigned bmask = 0;  // (cluster mode) bit qy: the lane's target of row qy is a boundary site
    if constexpr (CLU) {
#pragma unroll
      for (int qy = 0; qy < CY; ++qy) bmask |= (unsigned)boundary(qy) << qy;
    }
    int na = 0;
#pragma unroll
    for (int qy = 0; qy < CY; ++qy) {
      const bool bnd = CLU ? ((bmask >> qy) & 1u) != 0 : boundary(qy);
      const unsigned ball = __ballot_sync(kFull, bnd);
      if (bnd) ws.qa[na + __popc(ball & lanemask_lt())] = (uint16_t)(qy * 32 + lane);
      na += __popc(ball);
    }
    __syncwarp();

    // ---- pass 2: random draw and source pick -------------------------
    // Two batches per round where there are two, their draws computed side
    // by side (two independent Philox chains per lane); entries keep their
    // order, so the result is that of one batch at a time.
    int nbq = 0;
    auto counters = [&](int j, uint32_t (&c)[4]) {
      const int q = ws.qa[j];
      const int qx = q & 31, qy = q >> 5;
      const int x = 2 * (i0 + qx) + PAR;
      const int y = class_coord(ny, cy, j0 + qy);
      const long long site = (long long)y * nx + x;
      c[0] = (uint32_t)site;
      c[1] = (uint32_t)phase;
      c[2] = a.stream0;
      c[3] = (uint32_t)(phase >> 32);
      return q;
    };
    auto pick = [&](int q, const uint32_t (&c)[4], uint2& entry) {
      const int qx = q & 31, qy = q >> 5;
      const int kdir = (int)__umulhi(c[0], 8u);
      const int ci = center_idx<PAR>(pitch, qx, qy);
      const uint32_t tv = tb[ci], sv = tb[ci + nb_off(pitch, kdir)];
      bool keep = sv != tv;
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
      entry = make_uint2((uint32_t)q | ((uint32_t)kdir << 16) | (medium << 24), c[1]);
      return keep;
    };
    auto push = [&](bool keep, const uint2& entry) {
      const unsigned ball = __ballot_sync(kFull, keep);
      if (keep) ws.qb[nbq + __popc(ball & lanemask_lt())] = entry;
      nbq += __popc(ball);
    };
    int base = 0;
    for (; base + 32 < na; base += 64) {  // two batches, the second maybe partial
      const int ja = base + lane, jb = min(base + 32 + lane, na - 1);
      uint32_t ca[4], cb[4];
      const int qa_ = counters(ja, ca), qb_ = counters(jb, cb);
      philox4x32_10(ca[0], ca[1], ca[2], ca[3], k0, k1);
      philox4x32_10(cb[0], cb[1], cb[2], cb[3], k0, k1);
      uint2 ea, eb;
      const bool keep_a = pick(qa_, ca, ea);
      const bool keep_b = pick(qb_, cb, eb) && base + 32 + lane < na;
      push(keep_a, ea);
      push(keep_b, eb);
    }
    if (base < na) {  // one last batch of at most 32
      const int j = base + lane;
      bool keep = false;
      uint2 entry = make_uint2(0u, 0u);
      if (j < na) {
        uint32_t c[4];
        const int q = counters(j, c);
        philox4x32_10(c[0], c[1], c[2], c[3], k0, k1);
        keep = pick(q, c, entry);
      }
      push(keep, entry);
    }
    __syncwarp();

    // ---- pass 3: dH, Metropolis test, commit -------------------------
    for (int base = 0; base < nbq; base += 32) {
      const int j = base + lane;
      bool accepted = false;
      long long push_s = -1, push_t = -1;  // table rows this lane changed
      if (j < nbq) {
        const uint2 entry = ws.qb[j];
        const int q = (int)(entry.x & 0xFFFFu), kdir = (int)((entry.x >> 16) & 0xFFu);
        const int qx = q & 31, qy = q >> 5;
        uint32_t nb[8];
        const uint32_t t = nbhd<PAR>(tb, pitch, qx, qy, nb);
        const uint32_t s =
            (entry.x >> 24) ? 0u : tb[center_idx<PAR>(pitch, qx, qy) + nb_off(pitch, kdir)];
        const uint32_t is = s & 0xFFFFFFu, it = t & 0xFFFFFFu;
        if (is > (uint32_t)ncells || it > (uint32_t)ncells) {
          atomicOr(err, kErrBadId);
        } else {
          const int ts = (int)(s >> 24) & (kMaxTypes - 1);
          const int tt = (int)(t >> 24) & (kMaxTypes - 1);
          const long long rs = cell_off + is, rt = cell_off + it;
          const unsigned long long aps = s ? __ldcg(pt.rap + rs) : 0ull;
          const unsigned long long apt = t ? __ldcg(pt.rap + rt) : 0ull;
          // centroid sums, needed only on acceptance, fetched with the row
          // so that an accepted attempt waits on one L2 round trip
          long long cs_s[2], cs_t[2];
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            cs_s[k] = s ? __ldcg(pt.rcs + rs * 2 + k) : 0;
            cs_t[k] = t ? __ldcg(pt.rcs + rt * 2 + k) : 0;
          }
          float e_old = 0.0f, e_new = 0.0f;
          int cnt_s = 0, cnt_t = 0;
          const float* Jt = P->J + tt * kMaxTypes;
          const float* Js = P->J + ts * kMaxTypes;
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const uint32_t v = nb[k];
            const int tn = (int)(v >> 24) & (kMaxTypes - 1);
            if (v != t) e_old = __fadd_rn(e_old, __ldg(Jt + tn));
            if (v != s) e_new = __fadd_rn(e_new, __ldg(Js + tn));
            cnt_s += v == s;
            cnt_t += v == t;
          }
          if (stick_on) {
            // stickiness of the old configuration, summed in neighbour order
            // and added to its adhesion as one term
            float e_st = 0.0f;
            const float* St = P->stick + tt * kMaxTypes;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const uint32_t v = nb[k];
              const int tn = (int)(v >> 24) & (kMaxTypes - 1);
              if (v != t) e_st = __fadd_rn(e_st, __ldg(St + tn));
            }
            e_old = __fadd_rn(e_old, e_st);
          }
          float dH = __fsub_rn(e_new, e_old);
          const int x = 2 * (i0 + qx) + PAR;
          const int y = class_coord(ny, cy, j0 + qy);
          {
            // chemotaxis first, as in the reference's sum; lambda of the
            // source type, of the target type for a medium source
            float chemo = 0.0f;
            if (chemo_on) {
              const float lam = __ldg(&P->chemo[ts ? ts : tt]);
              if (lam != 0.0f)
                chemo = __fmul_rn(-lam, chemo_dot<2>(a.field + 2 * lat_off,
                                                     (long long)nx * ny, x, y, 0, kdir, nx,
                                                     ny, 1));
            }
            dH = __fadd_rn(chemo, dH);
          }
          const int dps = 8 - 2 * cnt_s;
          const int dpt = 2 * cnt_t - 8;
          if (perim_on) {
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
            const long long qv = 1 + 2LL * (unpack_area(aps) - __ldg(&P->tgt_area[ts]));
            dH = __fmaf_rn(__ldg(&P->lam_area[ts]), __ll2float_rn(qv), dH);
          }
          if (t) {
            const long long qv = 1 - 2LL * (unpack_area(apt) - __ldg(&P->tgt_area[tt]));
            dH = __fmaf_rn(__ldg(&P->lam_area[tt]), __ll2float_rn(qv), dH);
          }
          bool ok;
          if (dH < 0.0f) {
            ok = true;
          } else if (!(T > 0.0f)) {
            ok = false;
          } else {
            const float u = __fmul_rn(__uint2float_rn((entry.y >> 8) | 1u), 0x1p-24f);
            ok = u < exp_neg(__fdiv_rn(-dH, T));
          }
          if (ok) {
            accepted = true;
            if constexpr (CLU) {
              // targets lie in this block's rows; the padding copies too
              uint32_t* row = strip + (y - row0 + 1) * sp + 4;
              row[x] = s;
              if (x < 4) row[x + nx] = s;
              if (x >= nx - 4) row[x - nx] = s;
              // an edge row also into its copy in the neighbour's halo
              if (y == row0) halo_store(s_halo[0], x, s);
              if (y == row1 - 1) halo_store(s_halo[1], x, s);
            } else
              L[(long long)y * nx + x] = s;
            const int crd[2] = {x, y};
            const int dim[2] = {nx, ny};
            long long img[2];
            if (s) {
#pragma unroll
              for (int k = 0; k < 2; ++k)
                img[k] = nearest_image(crd[k], dim[k], unpack_area(aps), cs_s[k]);
              add_delta<2>(pt, rs, 1, dps, img, 1);
              push_s = rs;
            }
            if (t) {
#pragma unroll
              for (int k = 0; k < 2; ++k)
                img[k] = nearest_image(crd[k], dim[k], unpack_area(apt), cs_t[k]);
              add_delta<2>(pt, rt, -1, dpt, img, -1);
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
        if ((long long)at + npush > a.list_cap) {
          if (lane == 0) atomicOr(err, kErrListFull);
        } else {
          if (push_s >= 0) pt.list[at + __popc(bs & lanemask_lt())] = (uint32_t)push_s;
          if (push_t >= 0)
            pt.list[at + __popc(bs) + __popc(bt & lanemask_lt())] = (uint32_t)push_t;
        }
      }
    }
    n_eval += nbq;
    __syncwarp();  // the tile buffers are rewritten by the next tile
  };

  int step = 0;
  for (int m = 0; m < a.mcs; ++m) {
    const unsigned long long tick = s_tick0 + (unsigned long long)m;
    for (int si = 0; si < a.nslot_active; ++si, ++step) {
      const int cur = step & 1, prv = cur ^ 1;
      const PhaseTables<2> pt = tables(cur);
      // (cluster mode: the block's last warp replays while the others work
      // their tiles; the replay touches only the copy this phase does not
      // read, through atomics that commute with the phase's own)
      const int tile_warps = CLU ? wpb - 1 : wpb;
      if (step > 0) {
        if (!CLU) {
          replay_phase(prv);
        } else if (warp == wpb - 1) {
          const unsigned n = min(s_cnt[prv], (unsigned)a.list_cap);
          replay_lanes<2, true, (CY == 1 ? 1 : 4)>(blist(prv), n, prv ? a.dap[1] : a.dap[0],
                                prv ? a.dcs[1] : a.dcs[0], prv ? a.ap[1] : a.ap[0],
                                prv ? a.cs[1] : a.cs[0], lane, 32);
        }
      }
      const int slot = a.slots[si];
      const int cx = slot % 3, cy = (slot / 3) % 3;
      const unsigned long long phase = tick * NSLOTS + (unsigned long long)slot;
      // tiles of the slot: 32 target columns by CY target rows
      const int tnx = ((nx >> 1) + 31) / 32;
      const int tny = (class_count(ny, cy) + CY - 1) / CY;
      const int ntiles = tnx * tny;
      // each block sweeps every gridDim.x-th tile (tb1 - tb0 of them), the
      // same in every phase; its warps take them in turn.  In cluster mode
      // a block sweeps the band of tile rows whose targets lie in its rows.
      const int ncy = class_count(ny, cy);
      int tb0, tb1, jlo = 0, jhi = 0;
      if constexpr (CLU) {
        if (cy < 2) {
          jlo = (row0 - cy + 1) / 2;
          jhi = min(ncy, (row1 - cy + 1) / 2);
        } else if ((ny - 1) >= row0 && (ny - 1) < row1) {
          jhi = 1;
        }
        tb0 = 0;
        tb1 = jhi > jlo ? tnx * ((jhi - jlo + CY - 1) / CY) : 0;
      } else {
        const int per_b = ntiles / (int)gridDim.x, extra = ntiles % (int)gridDim.x;
        tb0 = (int)blockIdx.x * per_b + min((int)blockIdx.x, extra);
        tb1 = tb0 + per_b + ((int)blockIdx.x < extra ? 1 : 0);
      }
      // copies of this phase must see every SM's stores of the last one
      if (!CLU && lane == 0 && use_tma) asm volatile("fence.proxy.async.global;" ::: "memory");
      // warp w starts with the block's tile w, then claims the next unclaimed
      // one; counter step % 2 serves this phase, the other one (last used
      // before the previous barrier) is cleared for the next phase
      unsigned* ctr = &s_next[step & 1];
      if (tid == 0) s_next[(step + 1) & 1] = 0u;
      for (int k = warp; warp < tile_warps && k < tb1 - tb0;) {
        const int task = CLU ? tb0 + k : (int)blockIdx.x + k * (int)gridDim.x;
        const int ty = task / tnx;
        // (grid mode) tile row ty is taken rotated by ty tiles, so that a
        // block's tiles, every gridDim.x-th, fall in every column of tiles
        // and each block gets its share of the seam columns
        int tx = task - ty * tnx;
        if (!CLU) tx = (tx + ty) % tnx;
        const int j0 = CLU ? jlo + ty * CY : ty * CY, jend = CLU ? jhi : ncy;
        if (cx)
          run_tile(std::integral_constant<int, 1>{}, pt, tx, j0, jend, cy, phase);
        else
          run_tile(std::integral_constant<int, 0>{}, pt, tx, j0, jend, cy, phase);
        unsigned v = 0;
        if (lane == 0) v = atomicAdd(ctr, 1u);
        k = tile_warps + (int)__shfl_sync(kFull, v, 0);
      }
      __syncthreads();
      if (tid == 0) s_cnt[prv] = 0;
      if constexpr (CLU) {
        // the hardware barrier of the cluster's blocks (all co-scheduled, as
        // the threads of a block are for __syncthreads), with release and
        // acquire at cluster scope for the strips and the global tables
        cluster.sync();
      } else {
        if (!grid_barrier(a.ctl, ++episode, &s_ok)) return;
      }
    }
  }
  if (step > 0) replay_phase((step - 1) & 1);

  if (lane == 0) {
    if (n_eval) atomicAdd(&a.counters[0], n_eval);
    if (n_acc) atomicAdd(&a.counters[1], n_acc);
  }
  if (a.tick_ptr && a.tick_advance && blockIdx.x == 0 && tid == 0 && a.mcs > 0)
    *a.tick_ptr = s_tick0 + (unsigned long long)a.mcs;
  if constexpr (CLU) {
    // this block's rows back to the lattice in global memory; no block
    // leaves while another may still read its shared memory
    const int nvr = nx / 4, nvec = nown * nvr;
    uint4* dst = reinterpret_cast<uint4*>(L + (long long)row0 * nx);
    const uint4* src = reinterpret_cast<const uint4*>(strip);
    __syncthreads();
    for (int v = tid; v < nvec; v += blockDim.x) {
      const int r = v / nvr, k = v - r * nvr;
      dst[v] = src[(r + 1) * (sp / 4) + 1 + k];
    }
    cluster.sync();
  }
}

template <int CY>
const void* sweep2d_fn(bool perim) {
  return perim ? (const void*)sweep2d_kernel<true, CY> : (const void*)sweep2d_kernel<false, CY>;
}

const void* sweep2d_fn_v(bool perim, int variant) {
  switch (variant) {
    case 1: return sweep2d_fn<8>(perim);
    case 2: return sweep2d_fn<16>(perim);
    case 3: return sweep2d_fn<1>(perim);
    default: return sweep2d_fn<6>(perim);
  }
}

template <int CY>
SweepShape row_shape(int warps_cap) {
  SweepShape s;
  s.variant = 0;
  s.cx = 32;
  s.cy = CY;
  s.cz = 1;
  s.warps = row_tile_warps<CY>(warps_cap);
  s.smem = sizeof(Warp2Smem<CY>) * (size_t)s.warps;
  return s;
}

}  // namespace

int row_tile_rows(int variant) {
  switch (variant) {
    case 1: return 2 * 8 + 1;
    case 2: return 2 * 16 + 1;
    case 3: return 2 * 1 + 1;
    default: return 2 * 6 + 1;
  }
}

bool row_tiles_fit(int nx, int ny) {
  // vector loads need rows on 16-byte boundaries; one periodic wrap per
  // staged coordinate needs the lattice wider than a staged row and taller
  // than two staged boxes
  return nx % 4 == 0 && nx >= kPitch && ny >= 2 * row_tile_rows(2);
}

cudaError_t launch_sweep2d(bool perim, int variant, const SweepArgs& a, const void* tmap,
                           int use_tma, int grid, int warps_cap, cudaStream_t s) {
  SweepShape sh;
  switch (variant) {
    case 1: sh = row_shape<8>(warps_cap); break;
    case 2: sh = row_shape<16>(warps_cap); break;
    case 3: sh = row_shape<1>(warps_cap); break;
    default: sh = row_shape<6>(warps_cap); break;
  }
  const void* fn = sweep2d_fn_v(perim, variant);
  cudaError_t e =
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
  if (e != cudaSuccess) return e;
  alignas(64) CUtensorMap map;
  std::memcpy(&map, tmap, sizeof map);
  int tma = use_tma ? 1 : 0, strip_rows = 0;
  void* args[] = {const_cast<SweepArgs*>(&a), &map, &tma, &strip_rows};
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(32 * sh.warps), args, sh.smem, s);
}

// Cluster mode.  Blocks of cluster_warps(CY) warps; each block's shared memory
// holds its strip of H rows, the warp areas and its two dirty lists.
namespace {

// Tile rows and warps of the cluster sweep's variants (v0..v3): taller
// tiles fill the compacted batches better, one-row tiles give every warp of
// a block a tile on the smallest strips.
constexpr int kClusterCY[4] = {2, 4, 8, 1};
constexpr int kClusterW[4] = {cluster_warps(2), cluster_warps(4), cluster_warps(8),
                              cluster_warps(1)};

template <int CY>
const void* cluster_fn_cy(bool perim) {
  return perim ? (const void*)sweep2d_kernel<true, CY, true>
               : (const void*)sweep2d_kernel<false, CY, true>;
}
const void* cluster_fn(bool perim, int v) {
  switch (v) {
    case 0: return cluster_fn_cy<2>(perim);
    case 1: return cluster_fn_cy<4>(perim);
    case 2: return cluster_fn_cy<8>(perim);
    default: return cluster_fn_cy<1>(perim);
  }
}
size_t warp_area(int v) {
  switch (v) {
    case 0: return sizeof(WarpCluSmem<2>);
    case 1: return sizeof(WarpCluSmem<4>);
    case 2: return sizeof(WarpCluSmem<8>);
    default: return sizeof(WarpCluSmem<1>);
  }
}

long long cluster_list_cap(int nx, int H) {
  // two rows per target of the block's tiles in one phase: at most H / 2 + 1
  // target rows of one class per strip, tiles rounded up by at most 7 rows,
  // 32 targets per row of a tile column
  return 2LL * 32 * (((nx >> 1) + 31) / 32) * (H / 2 + 1 + 7);
}

size_t cluster_smem(int nx, int H, int v) {
  // own rows and two halo rows, each padded by 4 columns on both sides
  const size_t strip = (size_t)(((long long)(H + 2) * (nx + 8) + 31) & ~31LL) * 4;
  return strip + warp_area(v) * (size_t)kClusterW[v] + 2 * 4 * (size_t)cluster_list_cap(nx, H);
}

cudaLaunchConfig_t cluster_config(int G, int v, size_t smem, cudaStream_t s,
                                  cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(G);
  cfg.blockDim = dim3(32 * kClusterW[v]);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

cudaError_t cluster_attributes(bool perim, int v, size_t smem) {
  const void* fn = cluster_fn(perim, v);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}
}  // namespace

bool cluster_sweep_plan(int nx, int ny, int* G, int* H, long long* list_cap) {
  if (!row_tiles_fit(nx, ny)) return false;
  for (int g : {16, 8}) {
    const int h = (ny + g - 1) / g;
    bool fits = true;
    for (int v = 0; v < 4 && fits; ++v) {
      const size_t smem = cluster_smem(nx, h, v);
      if (smem > (size_t)kSweepSmemMax - 1024) {
        fits = false;
        break;
      }
      for (bool perim : {false, true}) {
        if (cluster_attributes(perim, v, smem) != cudaSuccess) {
          fits = false;
          break;
        }
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t cfg = cluster_config(g, v, smem, nullptr, attr);
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, cluster_fn(perim, v), &cfg) != cudaSuccess ||
            n < 1) {
          fits = false;
          break;
        }
      }
    }
    cudaGetLastError();  // (a refused size is not an error of the engine)
    if (!fits) continue;
    *G = g;
    *H = h;
    *list_cap = cluster_list_cap(nx, h);
    return true;
  }
  return false;
}

int cluster_tile_rows(int variant) {
  return kClusterCY[variant >= 0 && variant < 4 ? variant : 3];
}

cudaError_t launch_sweep2d_cluster(bool perim, int variant, const SweepArgs& a, const void* tmap,
                                   int nx, int G, int H, cudaStream_t s) {
  const int v = variant >= 0 && variant < 4 ? variant : 3;
  const size_t smem = cluster_smem(nx, H, v);
  cudaError_t e = cluster_attributes(perim, v, smem);
  if (e != cudaSuccess) return e;
  alignas(64) CUtensorMap map;
  std::memcpy(&map, tmap, sizeof map);
  int tma = 0, strip_rows = H;
  void* args[] = {const_cast<SweepArgs*>(&a), &map, &tma, &strip_rows};
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config(G, v, smem, s, attr);
  return cudaLaunchKernelExC(&cfg, cluster_fn(perim, v), args);
}

}  // namespace gpucpm
