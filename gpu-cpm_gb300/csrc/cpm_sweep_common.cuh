// cpm_sweep_common.cuh — device pieces shared by the sweep kernels
// (cpm_kernels.cu: every dimensionality, batches, scores, act; cpm_sweep2d.cu:
// 2D single lattices with TMA-staged row-major tiles): lane masks, source
// coordinates and chemotaxis, the double-buffered cell tables and their
// delta replay.
#pragma once

#include <cstdint>

#include "cpm_device.cuh"

namespace gpucpm {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Chemotaxis: unit copy direction (target minus source) dotted with the
// field at the source site, every step rounded as written (the oracle
// repeats it).  As in the reference, the direction is the raw difference of
// the wrapped coordinates in 2D (src/kernels2d.cu:302-309) and the nearest
// image in 3D (src/kernels3d.cu:275-299).  F: the replica's field, `sites`
// values per component.
__device__ __forceinline__ int wrap_coord(int v, int n) {
  return v < 0 ? v + n : (v >= n ? v - n : v);
}

// Coordinates of the source of an attempt: neighbour `kdir` (the order of
// Stage::nb_offset) of the target (x, y, z), wrapped.
template <int NDIM>
__device__ __forceinline__ void source_coords(int kdir, int x, int y, int z, int nx, int ny,
                                              int nz, int& sx, int& sy, int& sz) {
  int ox, oy, oz;
  if (NDIM == 2) {
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
  sx = wrap_coord(x + ox, nx);
  sy = wrap_coord(y + oy, ny);
  sz = NDIM == 3 ? wrap_coord(z + oz, nz) : 0;
}

// Unit copy direction (target minus source) of neighbour kdir: the raw
// difference of the wrapped coordinates in 2D (src/kernels2d.cu:302-309),
// the nearest image in 3D (src/kernels3d.cu:275-299); FP32, rounded as
// written (the oracle repeats it).  Also returns the source coordinates.
template <int NDIM>
__device__ __forceinline__ void unit_dir(int kdir, int x, int y, int z, int nx, int ny, int nz,
                                         float& ux, float& uy, float& uz, int& sx, int& sy,
                                         int& sz) {
  source_coords<NDIM>(kdir, x, y, z, nx, ny, nz, sx, sy, sz);
  int dx = x - sx, dy = y - sy, dz = z - sz;
  if (NDIM == 3) {
    if (dx > nx / 2) dx -= nx;
    if (dx < -(nx / 2)) dx += nx;
    if (dy > ny / 2) dy -= ny;
    if (dy < -(ny / 2)) dy += ny;
    if (dz > nz / 2) dz -= nz;
    if (dz < -(nz / 2)) dz += nz;
  }
  const float fx = (float)dx, fy = (float)dy, fz = (float)dz;
  float s2 = __fmul_rn(fx, fx);
  s2 = __fmaf_rn(fy, fy, s2);
  if (NDIM == 3) s2 = __fmaf_rn(fz, fz, s2);
  const float len = __fsqrt_rn(s2);
  ux = __fdiv_rn(fx, len);
  uy = __fdiv_rn(fy, len);
  uz = NDIM == 3 ? __fdiv_rn(fz, len) : 0.0f;
}

template <int NDIM>
__device__ __forceinline__ float chemo_dot(const float* F, long long sites, int x, int y,
                                           int z, int kdir, int nx, int ny, int nz) {
  float ux, uy, uz;
  int sx, sy, sz;
  unit_dir<NDIM>(kdir, x, y, z, nx, ny, nz, ux, uy, uz, sx, sy, sz);
  const long long site = ((long long)sz * ny + sy) * nx + sx;
  float c = __fmul_rn(ux, __ldg(F + site));
  c = __fmaf_rn(uy, __ldg(F + sites + site), c);
  if (NDIM == 3) c = __fmaf_rn(uz, __ldg(F + 2 * sites + site), c);
  return c;
}

// Per-phase view of the double-buffered tables.
template <int NDIM>
struct PhaseTables {
  const unsigned long long* rap;  // read copy (tables at phase start)
  const long long* rcs;
  unsigned long long* wap;        // other copy: receives this phase's deltas
  long long* wcs;
  unsigned long long* dap;        // this phase's deltas (replayed next phase)
  long long* dcs;
  uint32_t* list;                 // this block's dirty list for the phase
  unsigned* cnt;                  // its length (shared memory)
};

// One accepted copy's change of one table row: added to the other table
// copy and to the phase delta table.  Reductions only (no value comes
// back), so the accepting warp does not wait on L2.  The row goes on the
// block's dirty list separately (warp-aggregated, duplicates allowed).
template <int NDIM>
__device__ __forceinline__ void add_delta(const PhaseTables<NDIM>& pt,
                                          long long row, int darea, int dperim,
                                          const long long* img, long long sign) {
  const unsigned long long pd = pack_delta(darea, dperim);
  atomicAdd(pt.wap + row, pd);
  atomicAdd(pt.dap + row, pd);
#pragma unroll
  for (int k = 0; k < NDIM; ++k) {
    const unsigned long long v = (unsigned long long)(sign * img[k]);
    atomicAdd(reinterpret_cast<unsigned long long*>(pt.wcs + row * NDIM + k), v);
    atomicAdd(reinterpret_cast<unsigned long long*>(pt.dcs + row * NDIM + k), v);
  }
}

// Replays the deltas of the rows on a block's dirty list into `ap`/`cs`,
// strided over the block's threads.  A row can be on several lists (or
// twice on one); taking its delta with an exchange hands it to exactly one
// of them and leaves the delta table zeroed for the phase after next.  All
// exchanges of a row are issued before any add, so a row costs one round
// trip to L2.  SMEM_LIST: the list lives in shared memory (cluster sweep).
// replay_lanes takes entries first, first + stride, ... (one warp's lanes),
// U of them per round with all their exchanges in flight together (a single
// replay warp then waits on one round trip per U x 32 entries).
template <int NDIM, bool SMEM_LIST = false, int U = 1>
__device__ __forceinline__ void replay_lanes(const uint32_t* list, unsigned n,
                                             unsigned long long* dap, long long* dcs,
                                             unsigned long long* ap, long long* cs,
                                             unsigned first, unsigned stride) {
  for (unsigned j0 = first; j0 < n; j0 += U * stride) {
    uint32_t row[U];
    unsigned long long d[U], dc[U][NDIM];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const unsigned j = j0 + (unsigned)u * stride;
      row[u] = 0u;
      d[u] = 0ull;
#pragma unroll
      for (int k = 0; k < NDIM; ++k) dc[u][k] = 0ull;
      if (j < n) {
        row[u] = SMEM_LIST ? list[j] : __ldcg(list + j);
        d[u] = atomicExch(dap + row[u], 0ull);
#pragma unroll
        for (int k = 0; k < NDIM; ++k)
          dc[u][k] = atomicExch(
              reinterpret_cast<unsigned long long*>(dcs + (long long)row[u] * NDIM + k), 0ull);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (d[u]) atomicAdd(ap + row[u], d[u]);
#pragma unroll
      for (int k = 0; k < NDIM; ++k)
        if (dc[u][k])
          atomicAdd(reinterpret_cast<unsigned long long*>(cs + (long long)row[u] * NDIM + k),
                    dc[u][k]);
    }
  }
}
template <int NDIM, bool SMEM_LIST = false>
__device__ __forceinline__ void replay(const uint32_t* list, unsigned n,
                                       unsigned long long* dap, long long* dcs,
                                       unsigned long long* ap, long long* cs) {
  replay_lanes<NDIM, SMEM_LIST>(list, n, dap, dcs, ap, cs, threadIdx.x, blockDim.x);
}

}  // namespace
}  // namespace gpucpm
