// cpm_rowtile.cuh — device pieces of the row-tile sweeps (cpm_sweep2d.cu,
// cpm_sweep3d.cu): the staged row layout, the per-warp mbarrier and the
// tensor-map copies that fill a tile, and the 8-byte neighbourhood reads.
//
// A staged row holds 72 lattice words from a column that is a multiple of 4,
// so every row starts on a 16-byte boundary (the copy engine's rule for a
// tile's first coordinate, and the vector loads' alignment).  A warp tile of
// 32 targets along x spans 64 lattice columns; target column c of parity P
// sits at staged column 2c + 4 + P.
#pragma once

#include <cuda.h>  // CUtensorMap

#include <cstdint>

#include "cpm_device.cuh"

namespace gpucpm {
namespace {

constexpr int kPitch = 72;              // words per staged row
constexpr int kVecPerRow = kPitch / 4;  // 16-byte vectors per staged row

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Lane 0: arm the warp's barrier for one tile and start the copy of the box
// whose first lattice site is (x, y) or (x, y, z).  The shared-memory proxy
// fence orders the warp's earlier generic reads and writes of the tile
// buffer before the copy engine's writes into it.  x must be a multiple of 4
// (16-byte start), which the tile origins guarantee.
__device__ __forceinline__ void tma_load_tile(uint32_t dst, uint32_t bar, const CUtensorMap* map,
                                              int x, int y, unsigned bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_tile3(uint32_t dst, uint32_t bar, const CUtensorMap* map,
                                               int x, int y, int z, unsigned bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// Waits for the copy that completes phase `parity` of the barrier, bounded
// by the sweep's barrier timeout; false (and kErrTimeout) if it ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_timer_ns();
  for (unsigned spins = 1;; ++spins) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((spins & 63u) == 0 && global_timer_ns() - t0 > kBarrierTimeoutNs) {
      atomicOr(err, kErrTimeout);
      return false;
    }
  }
}

// The three sites of staged row `row` around target column qx of parity PAR
// (left, centre, right), from two 8-byte loads.
template <int PAR>
__device__ __forceinline__ void row3(const uint32_t* tile, int row, int qx, uint32_t& l,
                                     uint32_t& c, uint32_t& r) {
  const uint32_t* p = tile + row * kPitch + 2 * qx + 2 + 2 * PAR;
  const uint2 A = *reinterpret_cast<const uint2*>(p);
  const uint2 B = *reinterpret_cast<const uint2*>(p + 2);
  if (PAR) {
    l = A.x;
    c = A.y;
    r = B.x;
  } else {
    l = A.y;
    c = B.x;
    r = B.y;
  }
}

}  // namespace
}  // namespace gpucpm
