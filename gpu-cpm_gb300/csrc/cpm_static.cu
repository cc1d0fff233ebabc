// cpm_static.cu — cpm_sweep_static: the sweep on caller-owned device buffers
// with no allocation at all.
//
// Some callers cannot allocate device memory: code running inside a
// framework that owns the GPU's memory pool, a loop that must not allocate
// once it has started, or a host that only hands this library fixed
// buffers.  For them this entry point takes the lattice and the cell tables
// as device pointers and takes every other buffer the sweep needs (second
// table copy, phase deltas, dirty flags and lists, barrier words, replica
// descriptor, parameters) from one array compiled into the library, g_work
// below.  The sweep itself is the same kernel cpm_run launches, so the
// result is bit-identical to a handle's run with the same seed, stream id
// and tick.
//
// The array is a file-scope __device__ variable: its address on a device is
// looked up with cudaGetSymbolAddress the first time the entry point runs
// on that device (with that device current) and cached for the life of the
// process.  cudaDeviceReset destroys the context that holds the array, so
// the cached address is stale afterwards: a process that resets a device
// must not call this entry point on it again.  The array's contents persist
// between calls, so every call first clears the parts the sweep requires to
// start at zero.  All calls share it, so calls must not overlap on the GPU.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/gpucpm.h"
#include "cpm_internal.h"

namespace gpucpm {
namespace {

constexpr long long kMaxRows = CPM_STATIC_MAX_CELLS + 1;
constexpr long long kListEntries = 1LL << 20;  // all dirty lists of a launch
constexpr int kMaxDevices = 64;

// Byte offsets of the regions of g_work (each 256-byte aligned).
constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t kOffAp0 = 0;
constexpr size_t kOffAp1 = kOffAp0 + align256(8 * kMaxRows);
constexpr size_t kOffCs0 = kOffAp1 + align256(8 * kMaxRows);
constexpr size_t kOffCs1 = kOffCs0 + align256(8 * 3 * kMaxRows);
constexpr size_t kOffDap0 = kOffCs1 + align256(8 * 3 * kMaxRows);
constexpr size_t kOffDap1 = kOffDap0 + align256(8 * kMaxRows);
constexpr size_t kOffDcs0 = kOffDap1 + align256(8 * kMaxRows);
constexpr size_t kOffDcs1 = kOffDcs0 + align256(8 * 3 * kMaxRows);
constexpr size_t kOffFirst = kOffDcs1 + align256(8 * 3 * kMaxRows);
constexpr size_t kOffCtype = kOffFirst + align256(8 * kMaxRows);
constexpr size_t kOffList = kOffCtype + align256(4 * kMaxRows);
constexpr size_t kOffCtl = kOffList + align256(4 * kListEntries);
constexpr size_t kOffCounters = kOffCtl + align256(4 * kCtlWords);
constexpr size_t kOffRep = kOffCounters + align256(16);
constexpr size_t kOffParams = kOffRep + align256(sizeof(DevReplica));
constexpr size_t kOffPrefix = kOffParams + align256(sizeof(DevParams));
constexpr size_t kWorkBytes = kOffPrefix + align256(4 * 27 * 2);

static __device__ __align__(256) unsigned char g_work[kWorkBytes];

std::mutex g_mu;
unsigned char* g_work_addr[kMaxDevices];

// Device address of g_work on the current device, looked up once per device.
cudaError_t work_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_work_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_work);
    if (e != cudaSuccess) return e;
    g_work_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_work_addr[dev];
  return cudaSuccess;
}

__global__ void pack_tables(const int32_t* __restrict__ area,
                            const int32_t* __restrict__ perim,
                            unsigned long long* ap0, unsigned long long* ap1,
                            long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long w =
        (unsigned long long)(uint32_t)area[i] |
        ((unsigned long long)(uint32_t)perim[i] << 32);
    ap0[i] = w;
    ap1[i] = w;
  }
}

__global__ void unpack_tables(const unsigned long long* __restrict__ ap,
                              int32_t* area, int32_t* perim, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    area[i] = unpack_area(ap[i]);
    perim[i] = unpack_perim(ap[i]);
  }
}

int fail(int code, const char* msg) {
  set_thread_error(msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  char buf[256];
  snprintf(buf, sizeof buf, "cpm_sweep_static: %s: %s", what, cudaGetErrorString(e));
  set_thread_error(buf);
  return CPM_ERR_CUDA;
}

#define STATIC_CUDA(call)                          \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

int class_count_host(int n, int c) {
  if (n == 1) return c == 0 ? 1 : 0;
  return c < 2 ? (n >> 1) : (n & 1);
}

}  // namespace
}  // namespace gpucpm

using namespace gpucpm;

extern "C" int cpm_sweep_static(int dimensionality, int nx, int ny, int nz,
                                int number_of_cells, uint32_t* lattice,
                                int32_t* area, int32_t* perimeter,
                                int64_t* centroid_sums, int recount,
                                const cpm_static_params* params, uint64_t seed,
                                uint32_t stream_id, uint64_t tick, int mcs,
                                void* stream, uint64_t* counters_out) {
  const int ndim = dimensionality;
  if (ndim != 2 && ndim != 3)
    return fail(CPM_ERR_INVALID, "cpm_sweep_static: dimensionality must be 2 or 3");
  if (ndim == 2) nz = 1;
  if (nx < 3 || ny < 3 || (ndim == 3 && nz < 3))
    return fail(CPM_ERR_INVALID, "cpm_sweep_static: every side must be at least 3");
  const long long sites = (long long)nx * ny * nz;
  if (sites > CPM_STATIC_MAX_SITES)
    return fail(CPM_ERR_INVALID,
                "cpm_sweep_static: lattice larger than CPM_STATIC_MAX_SITES (2^18 sites)");
  if (number_of_cells < 0 || number_of_cells > CPM_STATIC_MAX_CELLS)
    return fail(CPM_ERR_INVALID,
                "cpm_sweep_static: number_of_cells outside [0, CPM_STATIC_MAX_CELLS]");
  if (!lattice || !area || !perimeter || !centroid_sums || !params)
    return fail(CPM_ERR_INVALID, "cpm_sweep_static: NULL buffer or params");
  if (mcs < 0) return fail(CPM_ERR_INVALID, "cpm_sweep_static: mcs must be >= 0");
  for (int k = 0; k < kMaxTypes; ++k)
    if (params->chemotaxis[k] != 0.0f || params->act_lambda[k] != 0.0f ||
        params->persistence_lambda[k] != 0.0f)
      return fail(CPM_ERR_UNSUPPORTED,
                  "cpm_sweep_static: chemotaxis, act and persistence need a handle engine");
  // Non-finite energies would make every Metropolis decision meaningless;
  // refused as the handle setters refuse them.
  if (!std::isfinite(params->temperature))
    return fail(CPM_ERR_INVALID, "cpm_sweep_static: temperature must be finite");
  for (int k = 0; k < kMaxTypes; ++k)
    if (!std::isfinite(params->lambda_area[k]) || !std::isfinite(params->lambda_perimeter[k]))
      return fail(CPM_ERR_INVALID, "cpm_sweep_static: lambdas must be finite");
  for (int k = 0; k < kMaxTypes * kMaxTypes; ++k)
    if (!std::isfinite(params->J[k]) || !std::isfinite(params->stickiness[k]))
      return fail(CPM_ERR_INVALID, "cpm_sweep_static: adhesion and stickiness must be finite");
  const long long rows = (long long)number_of_cells + 1;
  cudaStream_t s = (cudaStream_t)stream;

  // Launch geometry, as the engine computes it for a single replica with
  // tile variant 0.
  const SweepShape sh = sweep_shape(ndim, 0);
  const int tcx = sh.cx, tcy = sh.cy, tcz = sh.cz;
  int prefix[27 * 2] = {0};
  SweepArgs a;
  std::memset(&a, 0, sizeof a);
  long long max_tiles = 1;
  for (int slot = 0; slot < 27; ++slot) {
    const int cx = slot % 3, cy = (slot / 3) % 3, cz = slot / 9;
    long long tiles = 0;
    if (!(ndim == 2 && cz != 0)) {
      const long long ncx = class_count_host(nx, cx), ncy = class_count_host(ny, cy),
                      ncz = class_count_host(nz, cz);
      if (ncx && ncy && ncz)
        tiles = ((ncx + tcx - 1) / tcx) * ((ncy + tcy - 1) / tcy) * ((ncz + tcz - 1) / tcz);
    }
    prefix[slot * 2 + 1] = (int)tiles;
    if (tiles > 0) a.slots[a.nslot_active++] = slot;
    if (tiles > max_tiles) max_tiles = tiles;
  }
  int dev = 0, sms = 0;
  STATIC_CUDA(cudaGetDevice(&dev));
  STATIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const bool perim_on = [&] {
    for (int k = 0; k < kMaxTypes; ++k)
      if (params->lambda_perimeter[k] != 0.0f) return true;
    return false;
  }();
  const int per_sm = sweep_max_blocks_per_sm(ndim, perim_on, 0);
  if (per_sm < 1) return fail(CPM_ERR_CUDA, "cpm_sweep_static: cannot place the sweep kernel");
  const long long blocks_needed = (max_tiles + sh.warps - 1) / sh.warps;
  const int grid = (int)std::max(1LL, std::min<long long>((long long)per_sm * sms, blocks_needed));
  // Dirty-list space of one block and phase: two table rows per target of
  // the tiles it sweeps.  The single-lattice sweep gives each block one
  // contiguous band of at most ceil(tiles / grid) tiles, and a tile holds at
  // most min(tile extent, class size) targets along each axis, so narrow
  // lattices (nx far below the tile width) do not pay for empty tile columns.
  // Over every shape within CPM_STATIC_MAX_SITES the lists of a launch then
  // need at most 516,096 entries (2D, 66 x 3890) and 337,920 (3D,
  // 66 x 642 x 6) on 152 SMs, within kListEntries.
  const long long eff_tile = (long long)std::min(tcx, std::max(1, class_count_host(nx, 0))) *
                             std::min(tcy, std::max(1, class_count_host(ny, 0))) *
                             std::min(tcz, std::max(1, class_count_host(nz, 0)));
  const long long list_cap = 2LL * eff_tile * ((max_tiles + grid - 1) / grid);
  if (list_cap * 2 * grid > kListEntries)
    return fail(CPM_ERR_INVALID,
                "cpm_sweep_static: lattice shape needs more dirty-list space than the "
                "fixed working array holds");

  unsigned char* w = nullptr;
  STATIC_CUDA(work_address(&w));
  auto* ap0 = reinterpret_cast<unsigned long long*>(w + kOffAp0);
  auto* ap1 = reinterpret_cast<unsigned long long*>(w + kOffAp1);
  auto* cs0 = reinterpret_cast<long long*>(w + kOffCs0);
  auto* cs1 = reinterpret_cast<long long*>(w + kOffCs1);
  auto* ctl = reinterpret_cast<uint32_t*>(w + kOffCtl);
  auto* counters = reinterpret_cast<unsigned long long*>(w + kOffCounters);
  auto* rep = reinterpret_cast<DevReplica*>(w + kOffRep);
  auto* dparams = reinterpret_cast<DevParams*>(w + kOffParams);
  auto* dprefix = reinterpret_cast<int*>(w + kOffPrefix);

  // Everything the sweep expects to start at zero (the array keeps the last
  // call's contents, and a failed call may have left deltas behind).
  // (deltas of both phases: kOffDap0 .. kOffFirst)
  STATIC_CUDA(cudaMemsetAsync(w + kOffDap0, 0, kOffFirst - kOffDap0, s));
  STATIC_CUDA(cudaMemsetAsync(ctl, 0, 4 * kCtlWords, s));
  STATIC_CUDA(cudaMemsetAsync(counters, 0, 16, s));

  DevReplica R;
  R.nx = nx;
  R.ny = ny;
  R.nz = nz;
  R.ncells = number_of_cells;
  R.lat_off = 0;
  R.cell_off = 0;
  R.pset = 0;
  R.pad = 0;
  DevParams P;
  std::memset(&P, 0, sizeof P);
  std::memcpy(P.J, params->J, sizeof P.J);
  std::memcpy(P.lam_area, params->lambda_area, sizeof P.lam_area);
  std::memcpy(P.tgt_area, params->target_area, sizeof P.tgt_area);
  std::memcpy(P.lam_perim, params->lambda_perimeter, sizeof P.lam_perim);
  std::memcpy(P.tgt_perim, params->target_perimeter, sizeof P.tgt_perim);
  P.temperature = params->temperature;
  P.perim_on = perim_on ? 1 : 0;
  std::memcpy(P.stick, params->stickiness, sizeof P.stick);
  for (int k = 0; k < kMaxTypes * kMaxTypes; ++k)
    if (P.stick[k] != 0.0f) P.stick_on = 1;
  for (int k = 0; k < kMaxTypes; ++k)
    if (params->fixed[k]) P.fixed_mask |= 1u << k;
  STATIC_CUDA(cudaMemcpyAsync(rep, &R, sizeof R, cudaMemcpyHostToDevice, s));
  STATIC_CUDA(cudaMemcpyAsync(dparams, &P, sizeof P, cudaMemcpyHostToDevice, s));
  STATIC_CUDA(cudaMemcpyAsync(dprefix, prefix, sizeof prefix, cudaMemcpyHostToDevice, s));

  const int pack_grid = (int)std::min<long long>((rows + 255) / 256, 1024);
  if (recount) {
    STATIC_CUDA(cudaMemsetAsync(ap0, 0, 8 * rows, s));
    STATIC_CUDA(cudaMemsetAsync(cs0, 0, 8 * ndim * rows, s));
    STATIC_CUDA(cudaMemsetAsync(w + kOffFirst, 0xFF, 8 * rows, s));
    STATIC_CUDA(cudaMemsetAsync(w + kOffCtype, 0xFF, 4 * rows, s));
    STATIC_CUDA(launch_init(ndim, lattice, rep, 1, sites, ap0,
                            cs0, reinterpret_cast<unsigned long long*>(w + kOffFirst),
                            reinterpret_cast<int*>(w + kOffCtype), ctl, s));
    uint32_t word = 0;
    STATIC_CUDA(cudaMemcpyAsync(&word, ctl + kCtlErr, 4, cudaMemcpyDeviceToHost, s));
    STATIC_CUDA(cudaStreamSynchronize(s));
    if (word)
      return fail(CPM_ERR_INVALID,
                  "cpm_sweep_static: the lattice holds an id above number_of_cells, a type "
                  ">= 32, a typed medium site or one id with two types");
    STATIC_CUDA(cudaMemcpyAsync(ap1, ap0, 8 * rows, cudaMemcpyDeviceToDevice, s));
  } else {
    pack_tables<<<pack_grid, 256, 0, s>>>(area, perimeter, ap0, ap1, rows);
    STATIC_CUDA(cudaGetLastError());
    STATIC_CUDA(cudaMemcpyAsync(cs0, centroid_sums, 8 * ndim * rows,
                                cudaMemcpyDeviceToDevice, s));
  }
  STATIC_CUDA(cudaMemcpyAsync(cs1, cs0, 8 * ndim * rows, cudaMemcpyDeviceToDevice, s));

  if (mcs > 0) {
    a.lat = lattice;
    a.ap[0] = ap0;
    a.ap[1] = ap1;
    a.cs[0] = cs0;
    a.cs[1] = cs1;
    a.dap[0] = reinterpret_cast<unsigned long long*>(w + kOffDap0);
    a.dap[1] = reinterpret_cast<unsigned long long*>(w + kOffDap1);
    a.dcs[0] = reinterpret_cast<long long*>(w + kOffDcs0);
    a.dcs[1] = reinterpret_cast<long long*>(w + kOffDcs1);
    a.dlist = reinterpret_cast<uint32_t*>(w + kOffList);
    a.ctl = ctl;
    a.counters = counters;
    a.reps = rep;
    a.params = dparams;
    a.task_prefix = dprefix;
    a.list_cap = list_cap;
    a.tick0 = tick;
    a.seed = seed;
    a.nrep = 1;
    a.mcs = mcs;
    a.stream0 = stream_id;
    STATIC_CUDA(launch_sweep(ndim, perim_on, 0, a, grid, s));
  }

  unpack_tables<<<pack_grid, 256, 0, s>>>(ap0, area, perimeter, rows);
  STATIC_CUDA(cudaGetLastError());
  STATIC_CUDA(cudaMemcpyAsync(centroid_sums, cs0, 8 * ndim * rows,
                              cudaMemcpyDeviceToDevice, s));
  uint32_t word = 0;
  unsigned long long c[2] = {0, 0};
  STATIC_CUDA(cudaMemcpyAsync(&word, ctl + kCtlErr, 4, cudaMemcpyDeviceToHost, s));
  STATIC_CUDA(cudaMemcpyAsync(c, counters, 16, cudaMemcpyDeviceToHost, s));
  STATIC_CUDA(cudaStreamSynchronize(s));
  if (counters_out) {
    counters_out[0] = c[0];
    counters_out[1] = c[1];
  }
  if (word & kErrTimeout)
    return fail(CPM_ERR_TIMEOUT, "cpm_sweep_static: a grid barrier of the sweep timed out");
  if (word & kErrListFull)
    return fail(CPM_ERR_CUDA, "cpm_sweep_static: a dirty list was too small (internal error)");
  if (word)
    return fail(CPM_ERR_INVALID, "cpm_sweep_static: the sweep met an id above number_of_cells");
  return CPM_OK;
}
