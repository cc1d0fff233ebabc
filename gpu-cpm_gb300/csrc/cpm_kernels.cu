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
//
// Sweep schedule.  Sites are coloured by their class on every axis (even /
// odd / last coordinate of an odd axis); one phase ("slot") is one colour,
// and one MCS runs every non-empty slot in lexicographic (cz, cy, cx) order.
// All targets of a slot are >= 2 apart on each axis, so an attempt never
// reads a site another attempt of the same slot may write; the cell tables
// are read as they stood when the slot began and the integer deltas of the
// slot are folded in after a grid barrier.  The result is independent of
// thread, block and replica order, which is what makes the CPU oracle
// (oracle/cpm_oracle.cpp) reproduce it bit for bit.
//
// Work decomposition.  A warp owns a segment of 32 consecutive targets of
// one target row of one replica; a block task is kWarpsPerBlock segments of
// one replica, so the block stages that replica's J / lambda / target tables
// in shared memory once per task switch.  Block tasks of a slot are
// flattened over replicas (prefix table per slot) and dealt out
// grid-stride, which balances ragged batches by work, not by replica.
//
// Memory.  Mutable data (lattice, tables, deltas, dirty lists) is read with
// ld.global.cg so that no SM serves a stale L1 line after a barrier; the
// per-replica parameters are read-only for the kernel's lifetime.
#include <cstdint>

#include "cpm_device.cuh"

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

template <int NDIM>
__device__ __forceinline__ void add_delta(const SweepArgs& a, long long row,
                                          int darea, int dperim,
                                          const long long* img, int sign,
                                          uint32_t* dlist, uint32_t* dcount) {
  atomicAdd(&a.dap[row].x, darea);
  atomicAdd(&a.dap[row].y, dperim);
#pragma unroll
  for (int k = 0; k < NDIM; ++k)
    atomicAdd(reinterpret_cast<unsigned long long*>(&a.dcs[row * NDIM + k]),
              (unsigned long long)(sign * img[k]));
  if (atomicExch(&a.dflag[row], 1u) == 0u) {
    const uint32_t pos = atomicAdd(dcount, 1u);
    dlist[pos] = (uint32_t)row;
  }
}

template <int NDIM, bool PERIM>
__global__ void __launch_bounds__(kSweepThreads)
    sweep_kernel(const SweepArgs a) {
  constexpr int NB = NDIM == 2 ? 8 : 26;
  constexpr unsigned long long NSLOTS = NDIM == 2 ? 9 : 27;
  __shared__ DevParams sp;
  __shared__ int s_ok;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t k0 = (uint32_t)a.seed, k1 = (uint32_t)(a.seed >> 32);
  const unsigned nblk = gridDim.x;
  int* err = reinterpret_cast<int*>(&a.ctl[kCtlErr]);
  int cur_rep = -1;
  unsigned episode = 0;
  int step = 0;

  for (int m = 0; m < a.mcs; ++m) {
    const unsigned long long tick = a.tick0 + (unsigned long long)m;
    for (int si = 0; si < a.nslot_active; ++si) {
      const int slot = a.slots[si];
      const int cx = slot % 3, cy = (slot / 3) % 3, cz = slot / 9;
      const unsigned long long phase = tick * NSLOTS + (unsigned long long)slot;
      const int* pre = a.task_prefix + slot * (a.nrep + 1);
      const int ntasks = __ldg(pre + a.nrep);
      const int lst = step & 1;
      uint32_t* dcount = &a.ctl[kCtlDirty0 + lst];
      uint32_t* dlist = a.dlist + (long long)lst * a.rows;

      for (int task = blockIdx.x; task < ntasks; task += gridDim.x) {
        const int r = find_task_replica(pre, a.nrep, task);
        if (r != cur_rep) {  // block-uniform
          __syncthreads();
          const int* src = reinterpret_cast<const int*>(a.params + r);
          int* dst = reinterpret_cast<int*>(&sp);
          for (int i = threadIdx.x; i < (int)(sizeof(DevParams) / 4);
               i += blockDim.x)
            dst[i] = __ldg(src + i);
          __syncthreads();
          cur_rep = r;
        }
        const int nx = __ldg(&a.reps[r].nx), ny = __ldg(&a.reps[r].ny),
                  nz = __ldg(&a.reps[r].nz), ncells = __ldg(&a.reps[r].ncells);
        const long long lat_off = __ldg(&a.reps[r].lat_off);
        const long long cell_off = __ldg(&a.reps[r].cell_off);
        const int ncx = class_count(nx, cx), ncy = class_count(ny, cy),
                  ncz = class_count(nz, cz);
        const int spr = (ncx + 31) >> 5;
        const long long nseg = (long long)ncy * ncz * spr;
        const long long seg =
            (long long)(task - __ldg(pre + r)) * kWarpsPerBlock + warp;
        if (seg >= nseg) continue;  // warp-uniform

        const int row = (int)(seg / spr);
        const int i = (int)(seg - (long long)row * spr) * 32 + lane;
        const bool valid = i < ncx;
        const int x = class_coord(nx, cx, valid ? i : ncx - 1);
        const int y = class_coord(ny, cy, row % ncy);
        const int z = class_coord(nz, cz, row / ncy);
        uint32_t* L = a.lat + lat_off;

        // Neighbourhood in (dz, dy, dx) lexicographic order, centre skipped.
        const int xs[3] = {x == 0 ? nx - 1 : x - 1, x, x == nx - 1 ? 0 : x + 1};
        const int ys[3] = {y == 0 ? ny - 1 : y - 1, y, y == ny - 1 ? 0 : y + 1};
        int zs[3] = {0, 0, 0};
        if (NDIM == 3) {
          zs[0] = z == 0 ? nz - 1 : z - 1;
          zs[1] = z;
          zs[2] = z == nz - 1 ? 0 : z + 1;
        }
        uint32_t nb[NB];
        {
          int k = 0;
#pragma unroll
          for (int dz = (NDIM == 3 ? 0 : 1); dz < (NDIM == 3 ? 3 : 2); ++dz)
#pragma unroll
            for (int dy = 0; dy < 3; ++dy)
#pragma unroll
              for (int dx = 0; dx < 3; ++dx) {
                if (dz == 1 && dy == 1 && dx == 1) continue;
                nb[k++] = __ldcg(
                    L + ((long long)zs[dz] * ny + ys[dy]) * nx + xs[dx]);
              }
        }
        const long long site = ((long long)z * ny + y) * nx + x;
        const uint32_t t = __ldcg(L + site);
        bool boundary = false;
#pragma unroll
        for (int k = 0; k < NB; ++k) boundary |= nb[k] != t;

        bool evaluated = false, accepted = false;
        if (valid && boundary) {
          uint32_t c0 = (uint32_t)site, c1 = (uint32_t)phase,
                   c2 = a.stream0 + (uint32_t)r, c3 = (uint32_t)(phase >> 32);
          philox4x32_10(c0, c1, c2, c3, k0, k1);
          const int kdir = (int)__umulhi(c0, (unsigned)NB);
          uint32_t s = nb[0];
#pragma unroll
          for (int k = 1; k < NB; ++k)
            if (k == kdir) s = nb[k];
          const uint32_t is = s & 0xFFFFFFu, it = t & 0xFFFFFFu;
          if (s != t && (is > (uint32_t)ncells || it > (uint32_t)ncells)) {
            atomicOr(err, kErrBadId);
          } else if (s != t) {
            evaluated = true;
            const int ts = (int)(s >> 24) & (kMaxTypes - 1);
            const int tt = (int)(t >> 24) & (kMaxTypes - 1);
            float e_old = 0.0f, e_new = 0.0f;
            int cnt_s = 0, cnt_t = 0;
#pragma unroll
            for (int k = 0; k < NB; ++k) {
              const int tn = (int)(nb[k] >> 24) & (kMaxTypes - 1);
              if (nb[k] != t) e_old = __fadd_rn(e_old, sp.J[tt * kMaxTypes + tn]);
              if (nb[k] != s) e_new = __fadd_rn(e_new, sp.J[ts * kMaxTypes + tn]);
              cnt_s += nb[k] == s;
              cnt_t += nb[k] == t;
            }
            float dH = __fsub_rn(e_new, e_old);
            const int dps = NB - 2 * cnt_s;
            const int dpt = 2 * cnt_t - NB;
            const long long rs = cell_off + is, rt = cell_off + it;
            const int2 aps = s ? __ldcg(a.ap + rs) : make_int2(0, 0);
            const int2 apt = t ? __ldcg(a.ap + rt) : make_int2(0, 0);
            if (PERIM && sp.perim_on) {
              if (s) {
                const long long q =
                    (long long)dps * (2LL * (aps.y - sp.tgt_perim[ts]) + dps);
                dH = __fmaf_rn(sp.lam_perim[ts], __ll2float_rn(q), dH);
              }
              if (t) {
                const long long q =
                    (long long)dpt * (2LL * (apt.y - sp.tgt_perim[tt]) + dpt);
                dH = __fmaf_rn(sp.lam_perim[tt], __ll2float_rn(q), dH);
              }
            }
            if (s) {
              const long long q = 1 + 2LL * (aps.x - sp.tgt_area[ts]);
              dH = __fmaf_rn(sp.lam_area[ts], __ll2float_rn(q), dH);
            }
            if (t) {
              const long long q = 1 - 2LL * (apt.x - sp.tgt_area[tt]);
              dH = __fmaf_rn(sp.lam_area[tt], __ll2float_rn(q), dH);
            }
            const float T = sp.temperature;
            bool ok;
            if (dH < 0.0f) {
              ok = true;
            } else if (!(T > 0.0f)) {
              ok = false;
            } else {
              const float u = __fmul_rn(__uint2float_rn((c1 >> 8) | 1u), 0x1p-24f);
              ok = u < exp_neg(__fdiv_rn(-dH, T));
            }
            if (ok) {
              accepted = true;
              L[site] = s;
              const int crd[3] = {x, y, z};
              const int dim[3] = {nx, ny, nz};
              long long img[NDIM];
              if (s) {
#pragma unroll
                for (int k = 0; k < NDIM; ++k)
                  img[k] = nearest_image(crd[k], dim[k], aps.x,
                                         __ldcg(a.cs + rs * NDIM + k));
                add_delta<NDIM>(a, rs, 1, dps, img, 1, dlist, dcount);
              }
              if (t) {
#pragma unroll
                for (int k = 0; k < NDIM; ++k)
                  img[k] = nearest_image(crd[k], dim[k], apt.x,
                                         __ldcg(a.cs + rt * NDIM + k));
                add_delta<NDIM>(a, rt, -1, dpt, img, -1, dlist, dcount);
              }
            }
          }
        }
        const unsigned be = __ballot_sync(0xffffffffu, evaluated);
        const unsigned ba = __ballot_sync(0xffffffffu, accepted);
        if (lane == 0 && be) {
          atomicAdd(&a.counters[2 * r], (unsigned long long)__popc(be));
          if (ba) atomicAdd(&a.counters[2 * r + 1], (unsigned long long)__popc(ba));
        }
      }

      // All attempts of the slot have read the tables: fold the deltas.
      if (!grid_barrier(a.ctl, nblk * ++episode, &s_ok)) return;
      const uint32_t n = __ldcg(dcount);
      for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n;
           j += gridDim.x * blockDim.x) {
        const uint32_t row = __ldcg(dlist + j);
        const int2 d = __ldcg(a.dap + row);
        const int2 v = __ldcg(a.ap + row);
        a.ap[row] = make_int2(v.x + d.x, v.y + d.y);
        a.dap[row] = make_int2(0, 0);
#pragma unroll
        for (int k = 0; k < NDIM; ++k) {
          const long long idx = (long long)row * NDIM + k;
          a.cs[idx] = __ldcg(a.cs + idx) + __ldcg(a.dcs + idx);
          a.dcs[idx] = 0;
        }
        a.dflag[row] = 0u;
      }
      if (blockIdx.x == 0 && threadIdx.x == 0)
        a.ctl[kCtlDirty0 + (lst ^ 1)] = 0u;
      if (!grid_barrier(a.ctl, nblk * ++episode, &s_ok)) return;
      ++step;
    }
  }
}

// ---- table recount ---------------------------------------------------------

template <int NDIM>
__global__ void __launch_bounds__(kInitThreads)
    init_pass1(const uint32_t* __restrict__ lat,
               const DevReplica* __restrict__ reps, int nrep, long long total,
               unsigned long long* first, int* ctype, uint32_t* ctl) {
  int* err = reinterpret_cast<int*>(&ctl[kCtlErr]);
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
       g < total; g += (long long)gridDim.x * blockDim.x) {
    const int r = find_site_replica(reps, nrep, g);
    const long long local = g - __ldg(&reps[r].lat_off);
    const uint32_t v = lat[g];
    const uint32_t id = v & 0xFFFFFFu;
    const int ty = (int)(v >> 24);
    if (id > (uint32_t)__ldg(&reps[r].ncells)) {
      atomicOr(err, kErrBadId);
      continue;
    }
    if (ty >= kMaxTypes) atomicOr(err, kErrBadType);
    if (id == 0 && ty != 0) atomicOr(err, kErrMediumType);
    const long long row = __ldg(&reps[r].cell_off) + id;
    const int old = atomicCAS(&ctype[row], -1, ty);
    if (old != -1 && old != ty) atomicOr(err, kErrTypeConflict);
    atomicMin(&first[row], (unsigned long long)local);
  }
}

// Every site of a cell adds 1 to its area, its number of foreign Moore
// neighbours to its perimeter, and its coordinates (periodic image nearest
// the cell's first site in raster order) to its centroid sums.
template <int NDIM>
__global__ void __launch_bounds__(kInitThreads)
    init_pass2(const uint32_t* __restrict__ lat,
               const DevReplica* __restrict__ reps, int nrep, long long total,
               const unsigned long long* __restrict__ first, int2* ap,
               long long* cs) {
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
    atomicAdd(&ap[row].x, 1);
    atomicAdd(&ap[row].y, foreign);
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

// Failure-detection probe: every block waits at a barrier that needs one
// block more than the grid has, so the bounded wait runs out and the error
// word records kErrTimeout.  No memory beyond ctl[] is touched.
__global__ void barrier_probe(uint32_t* ctl, unsigned long long timeout_ns) {
  __shared__ int s_ok;
  grid_barrier(ctl, gridDim.x + 1, &s_ok, timeout_ns);
}

const void* sweep_fn(int ndim, bool perim) {
  if (ndim == 2)
    return perim ? (const void*)sweep_kernel<2, true>
                 : (const void*)sweep_kernel<2, false>;
  return perim ? (const void*)sweep_kernel<3, true>
               : (const void*)sweep_kernel<3, false>;
}

}  // namespace

int sweep_max_blocks_per_sm(int ndim, bool perim) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_fn(ndim, perim),
                                                    kSweepThreads, 0) !=
      cudaSuccess)
    return 0;
  return n;
}

cudaError_t launch_sweep(int ndim, bool perim, const SweepArgs& a, int grid,
                         cudaStream_t s) {
  void* args[] = {const_cast<SweepArgs*>(&a)};
  return cudaLaunchCooperativeKernel(sweep_fn(ndim, perim), dim3(grid),
                                     dim3(kSweepThreads), args, 0, s);
}

cudaError_t launch_barrier_probe(uint32_t* ctl, unsigned long long timeout_ns,
                                 cudaStream_t s) {
  void* args[] = {&ctl, &timeout_ns};
  return cudaLaunchCooperativeKernel((const void*)barrier_probe, dim3(2), dim3(32),
                                     args, 0, s);
}

cudaError_t launch_init(int ndim, const uint32_t* lat, const DevReplica* reps,
                        int nrep, long long total_sites, int2* ap,
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
