// cpm_device.cuh — device helpers of the sweep: Philox4x32-10, the FP32
// exp used by the Metropolis test, the checkerboard class arithmetic and a
// bounded grid barrier.
#pragma once

#include <cstdint>
#include "cpm_internal.h"

namespace gpucpm {

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): ten rounds of two
// 32x32->64 multiplies with the key bumped by the Weyl constants between
// rounds.  Replaces the reference's per-thread FP64 Park-Miller LCG
// (src/random.cu:5-12), whose stream depends on thread order.
__device__ __forceinline__ void philox4x32_10(uint32_t& c0, uint32_t& c1,
                                              uint32_t& c2, uint32_t& c3,
                                              uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
}

// exp(x) for x <= 0, FP32, every step explicitly rounded so that the host
// oracle reproduces it bit for bit.  Cody-Waite reduction x = k ln2 + r with
// ln2 split into its FP32 rounding plus remainder, exp(r) by the degree-7
// Taylor polynomial (coefficients 1/n!) in Horner form, then 2^k by building
// the exponent field.  Returns 0 below -20, where exp(x) < 2^-24 is smaller
// than every uniform the sweep draws.
__device__ __forceinline__ float exp_neg(float x) {
  if (x < -20.0f) return 0.0f;
  const float kf = rintf(__fmul_rn(x, 0x1.715476p+0f));
  float r = __fmaf_rn(-kf, 0x1.62e430p-1f, x);
  r = __fmaf_rn(-kf, -0x1.05c610p-29f, r);
  float p = 0x1.a01a02p-13f;
  p = __fmaf_rn(p, r, 0x1.6c16c2p-10f);
  p = __fmaf_rn(p, r, 0x1.111112p-7f);
  p = __fmaf_rn(p, r, 0x1.555556p-5f);
  p = __fmaf_rn(p, r, 0x1.555556p-3f);
  p = __fmaf_rn(p, r, 0x1.000000p-1f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  const int k = (int)kf;
  return __fmul_rn(p, __int_as_float((k + 127) << 23));
}

// log2(v) for v >= 1 in FP32 (act model): v = m 2^e with m in
// [1/sqrt(2), sqrt(2)); log2(m) = (2 / ln 2) atanh(z), z = (m - 1)/(m + 1),
// |z| <= 0.1716, by the odd series z + z^3/3 + ... + z^11/11 in Horner form.
// About 1 ulp from the exact value; the oracle repeats it step for step.
__device__ __forceinline__ float log2_pos(float v) {
  const unsigned b = __float_as_uint(v);
  int e = (int)((b >> 23) & 0xFFu) - 127;
  float m = __uint_as_float((b & 0x7FFFFFu) | (127u << 23));
  if (m > 1.41421356f) {
    m = __fmul_rn(m, 0.5f);
    e += 1;
  }
  const float z = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float z2 = __fmul_rn(z, z);
  float p = __fdiv_rn(1.0f, 11.0f);
  p = __fmaf_rn(p, z2, __fdiv_rn(1.0f, 9.0f));
  p = __fmaf_rn(p, z2, __fdiv_rn(1.0f, 7.0f));
  p = __fmaf_rn(p, z2, 0.2f);
  p = __fmaf_rn(p, z2, __fdiv_rn(1.0f, 3.0f));
  p = __fmaf_rn(p, z2, 1.0f);
  return __fadd_rn((float)e, __fmul_rn(__fmul_rn(z, p), 2.8853900817779268f));
}

// 2^y in FP32 for y in [-126, 127] (act model): y = k + f, |f| <= 1/2;
// 2^f = e^r with r = f ln 2 (ln 2 in two parts), by the Taylor series to
// degree 7; 2^k applied through the exponent field.
__device__ __forceinline__ float exp2_own(float y) {
  const float kf = rintf(y);
  const float f = __fsub_rn(y, kf);
  const float r = __fmaf_rn(f, 0x1.62e430p-1f, __fmul_rn(f, -0x1.05c610p-29f));
  float p = __fdiv_rn(1.0f, 5040.0f);
  p = __fmaf_rn(p, r, __fdiv_rn(1.0f, 720.0f));
  p = __fmaf_rn(p, r, __fdiv_rn(1.0f, 120.0f));
  p = __fmaf_rn(p, r, __fdiv_rn(1.0f, 24.0f));
  p = __fmaf_rn(p, r, __fdiv_rn(1.0f, 6.0f));
  p = __fmaf_rn(p, r, 0.5f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  const int k = (int)kf;
  return __fmul_rn(p, __int_as_float((k + 127) << 23));
}

// Checkerboard classes along one axis of length n: class 0 holds the even
// coordinates below n - (n & 1), class 1 the odd ones, class 2 the last
// coordinate of an odd axis.  An axis of length 1 (z in 2D) has one class.
__device__ __forceinline__ int class_count(int n, int c) {
  if (n == 1) return c == 0 ? 1 : 0;
  return c < 2 ? (n >> 1) : (n & 1);
}
__device__ __forceinline__ int class_coord(int n, int c, int i) {
  if (n == 1) return 0;
  return c < 2 ? 2 * i + c : n - 1;
}

// Periodic image of coordinate xc nearest to the running mean S / a of a
// cell (a >= 1): the rule of the reference's centroid CAS loops
// (src/kernels.cu:63-119), applied to exact int64 sums.
__device__ __forceinline__ long long nearest_image(int xc, int n, long long a,
                                                   long long S) {
  const long long d = (long long)xc * a - S;
  const long long na = (long long)n * a;
  if (2 * d > na) return (long long)xc - n;
  if (2 * d < -na) return (long long)xc + n;
  return xc;
}

__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];"
               : "=r"(v)
               : "l"(p)
               : "memory");
  return v;
}

__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v)
               : "memory");
}

// Grid-wide barrier of a cooperative launch (all blocks co-resident).  The
// arrival counter ctl[kCtlBarrier] is zeroed before the launch and only
// grows.  At the e-th barrier (e = 1, 2, ...) each block adds 1 to it with a
// release reduction and polls it with acquire loads, with backoff, until it
// reaches gridDim.x * e.
// The wait is bounded: after `timeout_ns` the block sets kErrTimeout and
// every block returns false at its next barrier, so a lost block ends the
// kernel with an error status instead of a hang.  Block-uniform result.
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;

__device__ __forceinline__ bool grid_barrier(
    uint32_t* ctl, unsigned episode, int* s_ok,
    unsigned long long timeout_ns = kBarrierTimeoutNs) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned target = gridDim.x * episode;
    // arrival: a release reduction (nothing comes back), then acquire polls
    // of the counter itself until every block of this episode has arrived
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&ctl[kCtlBarrier]) : "memory");
    const unsigned long long t0 = global_timer_ns();
    unsigned spins = 0, nap = 32;
    while (ld_acquire_gpu(&ctl[kCtlBarrier]) < target) {
      if ((++spins & 15u) == 0) {
        if (ld_acquire_gpu(&ctl[kCtlErr]) & kErrTimeout) {
          ok = 0;
          break;
        }
        if (global_timer_ns() - t0 > timeout_ns) {
          atomicOr((int*)&ctl[kCtlErr], kErrTimeout);
          ok = 0;
          break;
        }
      }
      if (spins > 64) {  // (polls are L2 round trips: most waits end before)
        __nanosleep(nap);
        if (nap < 128) nap <<= 1;
      }
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

}  // namespace gpucpm
