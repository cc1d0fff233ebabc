// cpm_sweep3d.cu — the 3D sweep of a single lattice with TMA-staged,
// row-major warp tiles.
//
//   sweep3d_kernel<PERIM, CY, CZ>  the checkerboard Metropolis sweep of one
//                              3D lattice (26-neighbourhood) whose width is a
//                              multiple of 4 sites (the 256^3 tissue); same
//                              schedule, random stream and FP32 operation
//                              order as sweep_kernel<3, ...> (cpm_kernels.cu),
//                              so its results are bit-identical.  Replaces
//                              copyAttempt3d (src/kernels3d.cu:51-594) for
//                              these lattices.
//
// The layout is the one of the 2D row-tile sweep (cpm_sweep2d.cu), one
// dimension up: a tile of 32 x CY x CZ targets of one slot is staged with
// its halo as a box of 72 x (2CY + 1) x (2CZ + 1) words from lattice column
// 64 tx - 4.  Interior tiles are copied by one cp.async.bulk.tensor.3d
// issued by lane 0; tiles on the periodic seam use 16-byte vector loads.  A
// target's 3 x 3 x 3 block is read as nine staged rows of three sites, two
// 8-byte loads each, and consumed row by row, so the 26 neighbour values
// never need to be live at once.  Coherence and the work split (bands of
// tiles per block, claimed by warps from a shared counter) are those of the
// 2D row-tile sweep.
#include <cuda.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "cpm_rowtile.cuh"
#include "cpm_sweep_common.cuh"

namespace gpucpm {
namespace {

template <int CY, int CZ>
struct BoxTile {
  static constexpr int SY = 2 * CY + 1;  // staged rows per plane
  static constexpr int SZ = 2 * CZ + 1;  // staged planes
  static constexpr int WORDS = SZ * SY * kPitch;
  static constexpr int NT = 32 * CY * CZ;  // targets
  static constexpr unsigned BYTES = WORDS * 4u;
};

template <int CY, int CZ>
struct alignas(128) Warp3Smem {
  uint32_t tile[BoxTile<CY, CZ>::WORDS];
  unsigned long long bar;  // mbarrier of the tile copy
  uint2 qb[BoxTile<CY, CZ>::NT];
  uint16_t qa[BoxTile<CY, CZ>::NT];
};

template <int CY, int CZ>
constexpr int box_tile_warps(int cap) {
  const int w = (int)(kSweepSmemMax / sizeof(Warp3Smem<CY, CZ>));
  return w < cap ? w : cap;
}

// staged index of target (qx, qy, qz), column parity PAR
template <int SY, int PAR>
__device__ __forceinline__ int center3(int qx, int qy, int qz) {
  return ((2 * qz + 1) * SY + 2 * qy + 1) * kPitch + 2 * qx + 4 + PAR;
}
// offset of neighbour k ((dz, dy, dx) lexicographic, centre excluded)
template <int SY>
__device__ __forceinline__ int nb_off3(int k) {
  const int m = k + (k >= 13);
  return ((m / 9 - 1) * SY + (m / 3) % 3 - 1) * kPitch + (m % 3 - 1);
}

template <bool PERIM, int CY, int CZ>
__global__ void __launch_bounds__(32 * kMaxSweepWarps3d, 1)
    sweep3d_kernel(const __grid_constant__ SweepArgs a, const __grid_constant__ CUtensorMap tmap,
                   const int use_tma) {
  using BT = BoxTile<CY, CZ>;
  constexpr int SY = BT::SY;
  constexpr unsigned long long NSLOTS = 27;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_ok;
  __shared__ unsigned s_cnt[2];
  __shared__ unsigned long long s_tick0;
  __shared__ unsigned s_next[2];  // next unclaimed tile of the band (by phase parity)

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wpb = blockDim.x >> 5;
  Warp3Smem<CY, CZ>& ws = reinterpret_cast<Warp3Smem<CY, CZ>*>(smem_raw)[warp];
  const uint32_t tile_s = smem_addr(ws.tile), bar_s = smem_addr(&ws.bar);
  const uint32_t k0 = (uint32_t)a.seed, k1 = (uint32_t)(a.seed >> 32);
  int* err = reinterpret_cast<int*>(&a.ctl[kCtlErr]);
  auto blist = [&](int b) { return a.dlist + (2LL * blockIdx.x + b) * a.list_cap; };
  unsigned episode = 0;
  unsigned long long n_eval = 0, n_acc = 0;  // warp-uniform
  uint32_t bar_parity = 0;
  bool fill_ok = true;  // warp-uniform: false once a tile copy timed out
  if (tid < 2) s_cnt[tid] = 0;
  if (tid < 2) s_next[tid] = 0;
  if (tid == 0) s_tick0 = a.tick_ptr ? __ldcg(a.tick_ptr) : a.tick0;
  if (lane == 0) {
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
  const int nx = __ldg(&a.reps[0].nx), ny = __ldg(&a.reps[0].ny), nz = __ldg(&a.reps[0].nz);
  const int ncells = __ldg(&a.reps[0].ncells);
  const long long lat_off = __ldg(&a.reps[0].lat_off);
  const long long cell_off = __ldg(&a.reps[0].cell_off);
  const long long plane = (long long)nx * ny;
  uint32_t* L = a.lat + lat_off;

  auto tables = [&](int cur) {
    PhaseTables<3> pt;
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
    replay<3>(blist(prv), n, prv ? a.dap[1] : a.dap[0], prv ? a.dcs[1] : a.dcs[0],
              prv ? a.ap[1] : a.ap[0], prv ? a.cs[1] : a.cs[0]);
  };

  // Stage the box whose first site is (X0, yorig, zorig).
  auto stage = [&](int X0, int yorig, int zorig) {
    const bool interior = use_tma && X0 >= 0 && X0 + kPitch <= nx && yorig >= 0 &&
                          yorig + SY <= ny && zorig >= 0 && zorig + BT::SZ <= nz;
    if (interior) {
      if (lane == 0) tma_load_tile3(tile_s, bar_s, &tmap, X0, yorig, zorig, BT::BYTES);
      fill_ok = mbar_wait_bounded(bar_s, bar_parity, err) && fill_ok;
      bar_parity ^= 1u;
      fill_ok = __all_sync(kFull, fill_ok);
    } else {
      for (int v = lane; v < BT::SZ * SY * kVecPerRow; v += 32) {
        const int row = v / kVecPerRow, col = v - row * kVecPerRow;  // row = pz * SY + py
        const int pz = row / SY, py = row - pz * SY;
        int gz = zorig + pz;
        gz = gz < 0 ? gz + nz : (gz >= nz ? gz - nz : gz);
        int gy = yorig + py;
        gy = gy < 0 ? gy + ny : (gy >= ny ? gy - ny : gy);
        int gx = X0 + 4 * col;
        gx = gx < 0 ? gx + nx : (gx >= nx ? gx - nx : gx);
        const uint4 val = __ldcg(
            reinterpret_cast<const uint4*>(L + (long long)gz * plane + (long long)gy * nx + gx));
        *reinterpret_cast<uint4*>(ws.tile + row * kPitch + 4 * col) = val;
      }
      __syncwarp();
    }
  };

  auto run_tile = [&](auto par, const PhaseTables<3>& pt, const int tx, const int ty,
                      const int tz, const int cy, const int cz,
                      const unsigned long long phase) {
    constexpr int PAR = decltype(par)::value;
    const int ncx = nx >> 1, ncy = class_count(ny, cy), ncz = class_count(nz, cz);
    const int i0 = tx * 32, j0 = ty * CY, l0 = tz * CZ;
    const int cntx = min(32, ncx - i0), cnty = min(CY, ncy - j0), cntz = min(CZ, ncz - l0);
    stage(2 * i0 - 4, class_coord(ny, cy, j0) - 1, class_coord(nz, cz, l0) - 1);
    if (!fill_ok) return;  // a copy timed out: the phase's barrier reports it

    // ---- pass 1: boundary test ---------------------------------------
    int na = 0;
#pragma unroll
    for (int it = 0; it < CY * CZ; ++it) {
      const int qy = it % CY, qz = it / CY;
      bool bnd = false;
      if (lane < cntx && qy < cnty && qz < cntz) {
        const uint32_t t = ws.tile[center3<SY, PAR>(lane, qy, qz)];
#pragma unroll
        for (int dz = 0; dz < 3; ++dz)
#pragma unroll
          for (int dy = 0; dy < 3; ++dy) {
            uint32_t l, c, r;
            row3<PAR>(ws.tile, (2 * qz + dz) * SY + 2 * qy + dy, lane, l, c, r);
            bnd |= (l != t) | (c != t) | (r != t);
          }
      }
      const unsigned ball = __ballot_sync(kFull, bnd);
      if (bnd) ws.qa[na + __popc(ball & lanemask_lt())] = (uint16_t)(it * 32 + lane);
      na += __popc(ball);
    }
    __syncwarp();

    // ---- pass 2: random draw and source pick -------------------------
    int nbq = 0;
    for (int base = 0; base < na; base += 32) {
      const int j = base + lane;
      bool keep = false;
      uint2 entry = make_uint2(0u, 0u);
      if (j < na) {
        const int q = ws.qa[j];
        const int qx = q & 31, qy = (q >> 5) % CY, qz = (q >> 5) / CY;
        const int x = 2 * (i0 + qx) + PAR;
        const int y = class_coord(ny, cy, j0 + qy);
        const int z = class_coord(nz, cz, l0 + qz);
        const long long site = (long long)z * plane + (long long)y * nx + x;
        uint32_t c0 = (uint32_t)site, c1 = (uint32_t)phase, c2 = a.stream0,
                 c3 = (uint32_t)(phase >> 32);
        philox4x32_10(c0, c1, c2, c3, k0, k1);
        const int kdir = (int)__umulhi(c0, 26u);
        const int c = center3<SY, PAR>(qx, qy, qz);
        const uint32_t tv = ws.tile[c], sv = ws.tile[c + nb_off3<SY>(kdir)];
        keep = sv != tv;
        uint32_t medium = 0;  // 1: the source is replaced by the medium
        if (fixed_mask && keep) {
          // a target of a fixed type never changes; a source of a fixed type
          // proposes the medium instead (src/kernels3d.cu:251-261)
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
      if (keep) ws.qb[nbq + __popc(ball & lanemask_lt())] = entry;
      nbq += __popc(ball);
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
        const int qx = q & 31, qy = (q >> 5) % CY, qz = (q >> 5) / CY;
        const int c = center3<SY, PAR>(qx, qy, qz);
        const uint32_t t = ws.tile[c];
        const uint32_t s = (entry.x >> 24) ? 0u : ws.tile[c + nb_off3<SY>(kdir)];
        const uint32_t is = s & 0xFFFFFFu, it = t & 0xFFFFFFu;
        if (is > (uint32_t)ncells || it > (uint32_t)ncells) {
          atomicOr(err, kErrBadId);
        } else {
          const int ts = (int)(s >> 24) & (kMaxTypes - 1);
          const int tt = (int)(t >> 24) & (kMaxTypes - 1);
          const long long rs = cell_off + is, rt = cell_off + it;
          const unsigned long long aps = s ? __ldcg(pt.rap + rs) : 0ull;
          const unsigned long long apt = t ? __ldcg(pt.rap + rt) : 0ull;
          // adhesion (and the old configuration's stickiness) summed in
          // neighbour order, the 3 x 3 x 3 block read row by row
          float e_old = 0.0f, e_new = 0.0f, e_st = 0.0f;
          int cnt_s = 0, cnt_t = 0;
          const float* Jt = P->J + tt * kMaxTypes;
          const float* Js = P->J + ts * kMaxTypes;
          const float* St = P->stick + tt * kMaxTypes;
          auto visit = [&](const uint32_t v) {
            const int tn = (int)(v >> 24) & (kMaxTypes - 1);
            if (v != t) e_old = __fadd_rn(e_old, __ldg(Jt + tn));
            if (v != s) e_new = __fadd_rn(e_new, __ldg(Js + tn));
            if (stick_on && v != t) e_st = __fadd_rn(e_st, __ldg(St + tn));
            cnt_s += v == s;
            cnt_t += v == t;
          };
#pragma unroll
          for (int dz = 0; dz < 3; ++dz)
#pragma unroll
            for (int dy = 0; dy < 3; ++dy) {
              uint32_t l, cc, r;
              row3<PAR>(ws.tile, (2 * qz + dz) * SY + 2 * qy + dy, qx, l, cc, r);
              visit(l);
              if (dz != 1 || dy != 1) visit(cc);  // (the centre is the target)
              visit(r);
            }
          if (stick_on) e_old = __fadd_rn(e_old, e_st);
          float dH = __fsub_rn(e_new, e_old);
          const int x = 2 * (i0 + qx) + PAR;
          const int y = class_coord(ny, cy, j0 + qy);
          const int z = class_coord(nz, cz, l0 + qz);
          {
            // chemotaxis first, as in the reference's sum; lambda of the
            // source type, of the target type for a medium source
            float chemo = 0.0f;
            if (chemo_on) {
              const float lam = __ldg(&P->chemo[ts ? ts : tt]);
              if (lam != 0.0f)
                chemo = __fmul_rn(-lam, chemo_dot<3>(a.field + 3 * lat_off, plane * nz, x, y,
                                                     z, kdir, nx, ny, nz));
            }
            dH = __fadd_rn(chemo, dH);
          }
          const int dps = 26 - 2 * cnt_s;
          const int dpt = 2 * cnt_t - 26;
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
            L[(long long)z * plane + (long long)y * nx + x] = s;
            const int crd[3] = {x, y, z};
            const int dim[3] = {nx, ny, nz};
            long long img[3];
            if (s) {
#pragma unroll
              for (int d = 0; d < 3; ++d)
                img[d] = nearest_image(crd[d], dim[d], unpack_area(aps),
                                       __ldcg(pt.rcs + rs * 3 + d));
              add_delta<3>(pt, rs, 1, dps, img, 1);
              push_s = rs;
            }
            if (t) {
#pragma unroll
              for (int d = 0; d < 3; ++d)
                img[d] = nearest_image(crd[d], dim[d], unpack_area(apt),
                                       __ldcg(pt.rcs + rt * 3 + d));
              add_delta<3>(pt, rt, -1, dpt, img, -1);
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
      const PhaseTables<3> pt = tables(cur);
      if (step > 0) replay_phase(prv);
      const int slot = a.slots[si];
      const int cx = slot % 3, cy = (slot / 3) % 3, cz = slot / 9;
      const unsigned long long phase = tick * NSLOTS + (unsigned long long)slot;
      const int tnx = ((nx >> 1) + 31) / 32;
      const int tny = (class_count(ny, cy) + CY - 1) / CY;
      const int tnz = (class_count(nz, cz) + CZ - 1) / CZ;
      const int ntiles = tnx * tny * tnz;
      // block b of G sweeps tiles b, b + G, b + 2G, ... of the slot, the
      // same in every phase, each row of tiles along x taken rotated by its
      // row index: every block's share samples the lattice and holds as many
      // boxes across the periodic seam in x (the first and last tile of a
      // row, loaded without the copy engine) as the others, whatever the
      // number of tiles per row.  Its warps claim the block's tiles from a
      // counter.
      if (lane == 0 && use_tma) asm volatile("fence.proxy.async.global;" ::: "memory");
      unsigned* ctr = &s_next[step & 1];
      if (tid == 0) s_next[(step + 1) & 1] = 0u;
      for (int k = warp;;) {
        const int task = (int)blockIdx.x + k * (int)gridDim.x;
        if (task >= ntiles) break;
        const int rest = task / tnx;
        const int tx = (task % tnx + rest) % tnx;
        const int ty = rest % tny, tz = rest / tny;
        if (cx)
          run_tile(std::integral_constant<int, 1>{}, pt, tx, ty, tz, cy, cz, phase);
        else
          run_tile(std::integral_constant<int, 0>{}, pt, tx, ty, tz, cy, cz, phase);
        unsigned v = 0;
        if (lane == 0) v = atomicAdd(ctr, 1u);
        k = wpb + (int)__shfl_sync(kFull, v, 0);
      }
      __syncthreads();
      if (tid == 0) s_cnt[prv] = 0;
      if (!grid_barrier(a.ctl, ++episode, &s_ok)) return;
    }
  }
  if (step > 0) replay_phase((step - 1) & 1);

  if (lane == 0) {
    if (n_eval) atomicAdd(&a.counters[0], n_eval);
    if (n_acc) atomicAdd(&a.counters[1], n_acc);
  }
  if (a.tick_ptr && a.tick_advance && blockIdx.x == 0 && tid == 0 && a.mcs > 0)
    *a.tick_ptr = s_tick0 + (unsigned long long)a.mcs;
}

template <int CY, int CZ>
const void* sweep3d_fn(bool perim) {
  return perim ? (const void*)sweep3d_kernel<true, CY, CZ>
               : (const void*)sweep3d_kernel<false, CY, CZ>;
}

template <int CY, int CZ>
SweepShape box_shape(int warps_cap) {
  SweepShape s;
  s.variant = 0;
  s.cx = 32;
  s.cy = CY;
  s.cz = CZ;
  s.warps = box_tile_warps<CY, CZ>(warps_cap);
  s.smem = sizeof(Warp3Smem<CY, CZ>) * (size_t)s.warps;
  return s;
}

}  // namespace

// Tile variants of the 3D row-tile sweep, as sweep_kernel<3, ...>'s:
// v0 32 x 2 x 2, v1 32 x 4 x 2, v2 32 x 4 x 4, v3 32 x 1 x 1 targets.
void box_tile_extent(int variant, int* rows, int* planes) {
  static const int cy[4] = {2, 4, 4, 1}, cz[4] = {2, 2, 4, 1};
  const int v = variant >= 0 && variant < 4 ? variant : 0;
  *rows = 2 * cy[v] + 1;
  *planes = 2 * cz[v] + 1;
}

bool box_tiles_fit(int nx, int ny, int nz) {
  // 16-byte rows; one periodic wrap per staged coordinate (lattice wider
  // than a staged row, taller and deeper than two of the largest boxes)
  return nx % 4 == 0 && nx >= kPitch && ny >= 18 && nz >= 18;
}

cudaError_t launch_sweep3d(bool perim, int variant, const SweepArgs& a, const void* tmap,
                           int use_tma, int grid, int warps_cap, cudaStream_t s) {
  SweepShape sh;
  const void* fn;
  switch (variant) {
    case 1: sh = box_shape<4, 2>(warps_cap); fn = sweep3d_fn<4, 2>(perim); break;
    case 2: sh = box_shape<4, 4>(warps_cap); fn = sweep3d_fn<4, 4>(perim); break;
    case 3: sh = box_shape<1, 1>(warps_cap); fn = sweep3d_fn<1, 1>(perim); break;
    default: sh = box_shape<2, 2>(warps_cap); fn = sweep3d_fn<2, 2>(perim); break;
  }
  cudaError_t e =
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
  if (e != cudaSuccess) return e;
  alignas(64) CUtensorMap map;
  std::memcpy(&map, tmap, sizeof map);
  int tma = use_tma ? 1 : 0;
  void* args[] = {const_cast<SweepArgs*>(&a), &map, &tma};
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(32 * sh.warps), args, sh.smem, s);
}

}  // namespace gpucpm
