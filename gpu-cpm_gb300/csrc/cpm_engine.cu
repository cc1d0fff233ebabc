// cpm_engine.cu — host runtime of the GB300 Cellular Potts engine and the
// C-ABI of include/gpucpm.h.
//
// Replaces the reference's host class Cpm (src/cpm.h:78-151, src/cpm.cu):
// allocation (src/cpm.cu:176-261), parameter setters (:57-158), addCell
// (:160-174), the launch schedule of run() (:291-517), host<->device copies
// (:531-597) and centroid readback (:68-110).  Differences by design:
//   * one CUDA stream per handle instead of the legacy default stream;
//   * one cooperative persistent launch per run() covers every MCS, slot and
//     replica (the reference relaunches per inner_iterations and grid-syncs
//     per attempt); hybrid-dispatch batches make two;
//   * parameters live in device records shared by replicas (copy on write)
//     and uploaded once per run when changed (the reference re-uploads its
//     __constant__ struct in every setter, src/kernels.cu:50-53);
//   * every call returns a status and keeps a message (the reference prints
//     CUDA errors and carries on, src/cpm.cu:52-56).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/gpucpm.h"
#include "cpm_internal.h"

using namespace gpucpm;

namespace {

thread_local std::string g_create_error;

constexpr int kMaxMcsPerLaunch = 1 << 16;

}  // namespace

void gpucpm::set_thread_error(const char* message) { g_create_error = message; }

struct cpm_handle {
  int ndim = 2;
  int nrep = 0;
  int device = 0;
  std::vector<DevReplica> reps;
  // Parameter records shared by replicas (reps[r].pset), copied on the first
  // write that addresses one replica only; records no replica uses are
  // dropped at upload.  A batch whose replicas share their parameters
  // uploads one record.
  std::vector<DevParams> psets;
  std::vector<int> pset_refs;  // replicas using each record
  bool params_dirty = true;
  bool reps_dirty = false;  // some reps[r].pset changed since the last upload
  int params_cap = 0;       // records d_params holds
  long long total_sites = 0;
  long long rows = 0;

  uint32_t* h_lat = nullptr;  // pinned, all replicas back to back
  // chemotaxis field (allocated on first use): host doubles as the
  // reference keeps them, device floats; layout of SweepArgs::field
  std::vector<double> h_field;
  float* d_field = nullptr;
  // act model (allocated on first use): MCS of the last copy into each site,
  // and the per-block lists of copies deferred to the end of their phase
  std::vector<uint32_t> h_act;
  uint32_t* d_act = nullptr;
  unsigned long long* d_pend_site = nullptr;
  uint32_t* d_pend_val = nullptr;
  long long pend_entries = 0;  // capacity of the pending arrays (all blocks)
  bool act_active = false;     // some replica's record has an act lambda
  // 3D persistence (allocated on first use): preferred direction per table
  // row, and the ring of the cells' mean coordinates after the last runs
  double* d_prefdir = nullptr;  // [rows][3]
  double* d_hist = nullptr;     // [hist_size][rows][3]
  int hist_size = 1;            // the reference's `history` (Cpm constructor)
  int hist_slot = 0;            // slot the next run's means go to
  bool persist_active = false;  // 3D and some record has a persistence lambda
  uint32_t* d_lat = nullptr;
  unsigned long long* d_ap[2] = {nullptr, nullptr};  // packed (area, perimeter)
  long long* d_cs[2] = {nullptr, nullptr};
  unsigned long long* d_dap[2] = {nullptr, nullptr};
  long long* d_dcs[2] = {nullptr, nullptr};
  uint32_t* d_dlist = nullptr;
  uint32_t* d_ctl = nullptr;
  unsigned long long* d_counters = nullptr;
  unsigned long long* d_first = nullptr;
  int* d_ctype = nullptr;
  DevReplica* d_reps = nullptr;
  DevParams* d_params = nullptr;
  int* d_task_prefix = nullptr;
  int* d_hyb_prefix = nullptr;  // [variant][27][nrep + 1] (hybrid grid part)
  int* d_rep_order = nullptr;  // replicas by decreasing site count

  cudaStream_t stream = nullptr;      // stream work is enqueued on
  cudaStream_t own_stream = nullptr;  // created with the handle
  // One launch configuration per tile variant; `variant` is the one runs use
  // (0 until cpm_autotune picks another).
  struct Config {
    SweepShape shape;
    int grid = 1;                  // grid dispatch
    long long list_cap = 0;
    int grid_local = 1;            // replica dispatch
    long long list_cap_local = 0;
    std::vector<int> task_prefix;  // [27][nrep + 1] warp tiles per slot
    std::vector<int> active_slots;
    // hybrid dispatch: the first hyb_ng replicas of rep_order run in grid
    // dispatch (hyb_prefix: [27][hyb_ng + 1], in rep_order), the rest in
    // replica dispatch, a whole number of rounds
    int hyb_ng = 0;
    std::vector<int> hyb_prefix;
  } cfg[kTileVariants];
  int variant = 0;
  int dispatch = CPM_DISPATCH_GRID;  // CPM_DISPATCH_*
  // Single lattices whose width is a multiple of 4 run the row-tile sweeps
  // (cpm_sweep2d.cu, cpm_sweep3d.cu).  fill: CPM_FILL_PARITY = the parity-split sweep_kernel,
  // CPM_FILL_VECTOR = row tiles staged with 16-byte loads, CPM_FILL_TMA = row
  // tiles whose interior tiles are copied by the tensor-map engine (the
  // default where the maps could be encoded).
  int fill = CPM_FILL_PARITY;
  bool row_ok = false, tma_ok = false;
  // CPM_FILL_CLUSTER: small 2D lattices swept by one thread-block cluster of
  // cl_G blocks, cl_H rows each, dirty lists of cl_cap entries per block
  bool cluster_ok = false;
  int cl_G = 0, cl_H = 0;
  long long cl_cap = 0;
  struct alignas(64) TileMap {
    unsigned char bytes[128];  // CUtensorMap of the lattice, box of one variant
  } tmap[kTileVariants];
  std::vector<unsigned long long> attempts;  // per replica, host-counted

  // Graph-captured run (cpm_run_graph): the captured launch reads and
  // advances the device copy of the tick.
  unsigned long long* d_tick = nullptr;
  bool d_tick_stale = true;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_mcs = 0, graph_variant = -1, graph_dispatch = -1, graph_fill = -1;
  int graph_launches = 1;  // sweep kernels per replay (2 for hybrid)
  cudaStream_t graph_stream = nullptr;

  uint64_t seed = 0;
  uint32_t stream_id = 0;
  uint64_t tick = 0;
  bool pushed = false;
  int added_cells = 0;
  uint64_t launches = 0;
  std::string err;

  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(CPM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
};

namespace {

#define CPM_CUDA(h, call)                                   \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return (h)->cuda_fail(e_, #call); \
  } while (0)

// Entry points that touch the GPU make the handle's device current first:
// the library carries its own CUDA runtime, whose current device is not the
// one a caller (torch, another library) selected.
#define CPM_BIND(h)                                   \
  do {                                                \
    if (!(h)) return CPM_ERR_INVALID;                 \
    CPM_CUDA((h), cudaSetDevice((h)->device));        \
  } while (0)

int class_count_h(int n, int c) {
  if (n == 1) return c == 0 ? 1 : 0;
  return c < 2 ? (n >> 1) : (n & 1);
}

void free_all(cpm_handle* h) {
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFreeHost(h->h_lat);
  cudaFree(h->d_field);
  cudaFree(h->d_act);
  cudaFree(h->d_pend_site);
  cudaFree(h->d_pend_val);
  cudaFree(h->d_prefdir);
  cudaFree(h->d_hist);
  cudaFree(h->d_lat);
  for (int b = 0; b < 2; ++b) {
    cudaFree(h->d_ap[b]);
    cudaFree(h->d_cs[b]);
    cudaFree(h->d_dap[b]);
    cudaFree(h->d_dcs[b]);
  }
  cudaFree(h->d_dlist);
  cudaFree(h->d_ctl);
  cudaFree(h->d_counters);
  cudaFree(h->d_first);
  cudaFree(h->d_ctype);
  cudaFree(h->d_reps);
  cudaFree(h->d_params);
  cudaFree(h->d_task_prefix);
  cudaFree(h->d_hyb_prefix);
  cudaFree(h->d_rep_order);
  cudaFree(h->d_tick);
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
}

// Tensor maps of a single lattice for the row-tile sweeps: the lattice as a
// ny x nx (nz x ny x nx) array of 32-bit words, one box of 72 x (2 CY + 1)
// (x (2 CZ + 1)) words per tile variant.  cuTensorMapEncodeTiled is reached through the runtime's driver
// entry point, so the library does not link the driver library itself.
// False (and no maps) when the entry point or the encoding is unavailable.
bool encode_tile_maps(cpm_handle* h) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!encode) return false;
  const DevReplica& R = h->reps[0];
  for (int v = 0; v < kTileVariants; ++v) {
    const cuuint64_t dims[3] = {(cuuint64_t)R.nx, (cuuint64_t)R.ny, (cuuint64_t)R.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)R.nx * 4, (cuuint64_t)R.nx * R.ny * 4};
    cuuint32_t box[3] = {72u, (cuuint32_t)row_tile_rows(v), 1u};
    if (h->ndim == 3) {
      int rows = 0, planes = 0;
      box_tile_extent(v, &rows, &planes);
      box[1] = (cuuint32_t)rows;
      box[2] = (cuuint32_t)planes;
    }
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    if (encode(reinterpret_cast<CUtensorMap*>(h->tmap[v].bytes), CU_TENSOR_MAP_DATA_TYPE_UINT32,
               (cuuint32_t)h->ndim, h->d_lat + R.lat_off, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

void default_params(DevParams& p, float T) {
  std::memset(&p, 0, sizeof p);
  p.temperature = T;
}

bool perim_on(const DevParams& p) {
  for (int k = 0; k < kMaxTypes; ++k)
    if (p.lam_perim[k] != 0.0f) return true;
  return false;
}

int build_engine(int n, int ndim, const int* nx, const int* ny, const int* nz,
                 const int* ncells, float T, cpm_handle** out) {
  if (!out) {
    g_create_error = "out pointer is NULL";
    return CPM_ERR_INVALID;
  }
  *out = nullptr;
  if (n < 1 || (ndim != 2 && ndim != 3)) {
    g_create_error = "need n >= 1 replicas and dimensionality 2 or 3";
    return CPM_ERR_INVALID;
  }
  cpm_handle* h = new (std::nothrow) cpm_handle();
  if (!h) {
    g_create_error = "host allocation failed";
    return CPM_ERR_ALLOC;
  }
  h->ndim = ndim;
  h->nrep = n;
  long long sites = 0, rows = 0;
  for (int r = 0; r < n; ++r) {
    DevReplica R;
    R.nx = nx[r];
    R.ny = ny[r];
    R.nz = ndim == 3 ? nz[r] : 1;
    R.ncells = ncells[r];
    if (R.nx < 3 || R.ny < 3 || (ndim == 3 && R.nz < 3)) {
      g_create_error = "every side must be at least 3";
      delete h;
      return CPM_ERR_INVALID;
    }
    if (ndim == 2 && nz && nz[r] != 1) {
      g_create_error = "nz must be 1 for a 2D lattice";
      delete h;
      return CPM_ERR_INVALID;
    }
    const long long ns = (long long)R.nx * R.ny * R.nz;
    if (ns >= (1LL << 31)) {
      g_create_error = "a replica may hold at most 2^31-1 sites";
      delete h;
      return CPM_ERR_INVALID;
    }
    if (R.ncells < 0 || R.ncells > 0xFFFFFF) {
      g_create_error = "number_of_cells must be in [0, 2^24-1]";
      delete h;
      return CPM_ERR_INVALID;
    }
    R.lat_off = sites;
    R.cell_off = rows;
    sites += ns;
    rows += (long long)R.ncells + 1;
    h->reps.push_back(R);
  }
  if (rows >= (1LL << 31)) {
    g_create_error = "too many cells in total (table rows >= 2^31)";
    delete h;
    return CPM_ERR_INVALID;
  }
  h->total_sites = sites;
  h->rows = rows;
  h->psets.resize(1);
  default_params(h->psets[0], T);
  h->pset_refs.assign(1, n);
  for (auto& R : h->reps) R.pset = 0;
  h->attempts.assign(n, 0);

  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  h->stream = h->own_stream;
  auto al = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes ? bytes : 1);
  };
  al((void**)&h->d_lat, sizeof(uint32_t) * sites);
  for (int b = 0; b < 2; ++b) {
    al((void**)&h->d_ap[b], sizeof(unsigned long long) * rows);
    al((void**)&h->d_cs[b], sizeof(long long) * rows * ndim);
    al((void**)&h->d_dap[b], sizeof(unsigned long long) * rows);
    al((void**)&h->d_dcs[b], sizeof(long long) * rows * ndim);
  }
  al((void**)&h->d_ctl, sizeof(uint32_t) * kCtlWords);
  al((void**)&h->d_counters, sizeof(unsigned long long) * 2 * n);
  al((void**)&h->d_first, sizeof(unsigned long long) * rows);
  al((void**)&h->d_ctype, sizeof(int) * rows);
  al((void**)&h->d_reps, sizeof(DevReplica) * n);
  al((void**)&h->d_params, sizeof(DevParams));
  h->params_cap = 1;
  al((void**)&h->d_task_prefix, sizeof(int) * kTileVariants * 27 * (n + 1));
  al((void**)&h->d_hyb_prefix, sizeof(int) * kTileVariants * 27 * (n + 1));
  al((void**)&h->d_rep_order, sizeof(int) * n);
  al((void**)&h->d_tick, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&h->h_lat, sizeof(uint32_t) * (sites ? sites : 1));
  if (e != cudaSuccess) {
    g_create_error = std::string("device/pinned allocation failed: ") + cudaGetErrorString(e);
    free_all(h);
    delete h;
    return e == cudaErrorMemoryAllocation ? CPM_ERR_ALLOC : CPM_ERR_CUDA;
  }
  std::memset(h->h_lat, 0, sizeof(uint32_t) * sites);
  if (n == 1 && (ndim == 2 ? row_tiles_fit(nx[0], ny[0]) : box_tiles_fit(nx[0], ny[0], nz[0]))) {
    h->row_ok = true;
    h->tma_ok = encode_tile_maps(h);
    h->fill = h->tma_ok ? CPM_FILL_TMA : CPM_FILL_VECTOR;
    if (ndim == 2)
      h->cluster_ok = cluster_sweep_plan(nx[0], ny[0], &h->cl_G, &h->cl_H, &h->cl_cap);
  }

  // One launch configuration per tile variant: warp tiles per slot and
  // replica (prefix over replicas), grid, dirty-list capacity.
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  long long dlist_entries = 1;
  long long max_rows = 1, max_sites = 1;
  for (const DevReplica& R : h->reps) {
    max_rows = std::max(max_rows, (long long)R.ncells + 1);
    max_sites = std::max(max_sites, (long long)R.nx * R.ny * R.nz);
  }
  std::vector<int> order(n);
  for (int r = 0; r < n; ++r) order[r] = r;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const DevReplica &X = h->reps[x], &Y = h->reps[y];
    return (long long)X.nx * X.ny * X.nz > (long long)Y.nx * Y.ny * Y.nz;
  });
  for (int v = 0; v < kTileVariants; ++v) {
    cpm_handle::Config& c = h->cfg[v];
    c.shape = sweep_shape(ndim, v);
    c.task_prefix.assign(27 * (n + 1), 0);
    long long max_tasks = 1;
    for (int slot = 0; slot < 27; ++slot) {
      const int cx = slot % 3, cy = (slot / 3) % 3, cz = slot / 9;
      long long acc = 0;
      for (int r = 0; r < n; ++r) {
        c.task_prefix[slot * (n + 1) + r] = (int)acc;
        const DevReplica& R = h->reps[r];
        if (ndim == 2 && cz != 0) continue;
        const long long ncx = class_count_h(R.nx, cx), ncy = class_count_h(R.ny, cy),
                        ncz = class_count_h(R.nz, cz);
        if (!ncx || !ncy || !ncz) continue;
        acc += ((ncx + c.shape.cx - 1) / c.shape.cx) * ((ncy + c.shape.cy - 1) / c.shape.cy) *
               ((ncz + c.shape.cz - 1) / c.shape.cz);
      }
      if (acc >= (1LL << 31)) {
        g_create_error = "batch too large for one launch";
        free_all(h);
        delete h;
        return CPM_ERR_INVALID;
      }
      c.task_prefix[slot * (n + 1) + n] = (int)acc;
      if (acc > 0) c.active_slots.push_back(slot);
      max_tasks = std::max(max_tasks, acc);
    }
    const int per_sm = std::min(sweep_max_blocks_per_sm(ndim, true, v),
                                sweep_max_blocks_per_sm(ndim, false, v));
    if (per_sm < 1 || sms < 1) {
      g_create_error = "cannot place the sweep kernel on this device";
      free_all(h);
      delete h;
      return CPM_ERR_CUDA;
    }
    // One block per SM (fewer if the largest slot has fewer warp tiles).
    const long long blocks_needed = (max_tasks + c.shape.warps - 1) / c.shape.warps;
    c.grid = (int)std::max(1LL, std::min<long long>((long long)per_sm * sms, blocks_needed));
    // Per-block dirty lists (two per block, for the running and the previous
    // phase): a warp works at most ceil(tiles / warps) tiles per slot, each
    // attempt touching at most two table rows.
    const long long warps = (long long)c.grid * c.shape.warps;
    const long long nt = (long long)c.shape.cx * c.shape.cy * c.shape.cz;
    c.list_cap = 2LL * nt * c.shape.warps * ((max_tasks + warps - 1) / warps);
    if (ndim == 2) {  // score launches run fewer warps per block (more tiles each)
      const int sw = sweep_shape(ndim, v, true).warps;
      const long long swarps = (long long)c.grid * sw;
      c.list_cap = std::max(c.list_cap, 2LL * nt * sw * ((max_tasks + swarps - 1) / swarps));
    }
    if (n == 1 && (ndim == 2 ? row_tiles_fit(nx[0], ny[0])
                             : box_tiles_fit(nx[0], ny[0], nz[0]))) {
      // the row-tile sweeps of the one lattice: tiles of 32 x ry (x rz)
      // targets, dealt to the blocks one at a time; a block gets at most
      // ceil(tiles / grid) of them
      int rows = 0, planes = 3;
      if (ndim == 2)
        rows = row_tile_rows(v);
      else
        box_tile_extent(v, &rows, &planes);
      const long long ry = rows / 2, rz = planes / 2;
      const long long tnx = ((nx[0] / 2) + 31) / 32;
      const long long tiles = tnx * (((ny[0] + 1) / 2 + ry - 1) / ry) *
                              (ndim == 3 ? (((nz[0] + 1) / 2 + rz - 1) / rz) : 1);
      const long long per_block = (tiles + c.grid - 1) / c.grid;
      c.list_cap = std::max(c.list_cap, 2LL * per_block * 32 * ry * rz);
    }
    dlist_entries = std::max(dlist_entries, c.list_cap * 2 * c.grid);
    // Replica dispatch: one block per replica at a time; its dirty list takes
    // up to two rows per attempt of the replica's largest slot.
    long long max_rep_tiles = 1;
    for (int slot = 0; slot < 27; ++slot)
      for (int r = 0; r < n; ++r)
        max_rep_tiles = std::max<long long>(
            max_rep_tiles, c.task_prefix[slot * (n + 1) + r + 1] - c.task_prefix[slot * (n + 1) + r]);
    c.grid_local = std::min(per_sm * sms, n);
    c.list_cap_local = n > 1 ? 2LL * nt * max_rep_tiles : 0;  // batches only
    dlist_entries = std::max(dlist_entries, c.list_cap_local * 2 * c.grid_local);
    // Hybrid split: replica dispatch gets whole rounds of the smallest
    // replicas, grid dispatch the rest.
    c.hyb_ng = n - (n / c.grid_local) * c.grid_local;
    const int ng = c.hyb_ng;
    c.hyb_prefix.assign(27 * (ng + 1), 0);
    for (int slot = 0; slot < 27; ++slot) {
      int acc = 0;
      for (int i = 0; i < ng; ++i) {
        c.hyb_prefix[slot * (ng + 1) + i] = acc;
        const int r = order[i];
        acc += c.task_prefix[slot * (n + 1) + r + 1] - c.task_prefix[slot * (n + 1) + r];
      }
      c.hyb_prefix[slot * (ng + 1) + ng] = acc;
    }
  }
  // act runs defer one copy per attempt at most: half a dirty list's entries
  h->pend_entries = dlist_entries / 4 + 1;
  e = cudaMalloc((void**)&h->d_dlist, sizeof(uint32_t) * dlist_entries);
  if (e != cudaSuccess) {
    g_create_error = std::string("dirty-list allocation failed: ") + cudaGetErrorString(e);
    free_all(h);
    delete h;
    return e == cudaErrorMemoryAllocation ? CPM_ERR_ALLOC : CPM_ERR_CUDA;
  }

  // Replica dispatch by default when there are replicas for every block and
  // no replica is much larger than a block's fair share of the sites, hybrid
  // when those replicas do not fill whole rounds (the autotuner can change
  // the choice).
  h->dispatch = (n >= h->cfg[0].grid_local && n >= sms &&
                 max_sites * (long long)h->cfg[0].grid_local <= 2 * sites)
                    ? (h->cfg[0].hyb_ng > 0 ? CPM_DISPATCH_HYBRID : CPM_DISPATCH_REPLICA)
                    : CPM_DISPATCH_GRID;
  e = cudaMemcpyAsync(h->d_reps, h->reps.data(), sizeof(DevReplica) * n,
                      cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->d_rep_order, order.data(), sizeof(int) * n,
                        cudaMemcpyHostToDevice, h->stream);
  for (int v = 0; v < kTileVariants && e == cudaSuccess; ++v) {
    e = cudaMemcpyAsync(h->d_task_prefix + (size_t)v * 27 * (n + 1),
                        h->cfg[v].task_prefix.data(), sizeof(int) * 27 * (n + 1),
                        cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->d_hyb_prefix + (size_t)v * 27 * (n + 1),
                          h->cfg[v].hyb_prefix.data(),
                          sizeof(int) * h->cfg[v].hyb_prefix.size(), cudaMemcpyHostToDevice,
                          h->stream);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(h->d_ctl, 0, sizeof(uint32_t) * kCtlWords, h->stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * 2 * n, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    g_create_error = std::string("initial upload failed: ") + cudaGetErrorString(e);
    free_all(h);
    delete h;
    return CPM_ERR_CUDA;
  }
  *out = h;
  return CPM_OK;
}

int check_replica(cpm_handle* h, int r) {
  if (!h) return CPM_ERR_INVALID;
  if (r < 0 || r >= h->nrep)
    return h->fail(CPM_ERR_INVALID, "replica %d out of range [0, %d)", r, h->nrep);
  return CPM_OK;
}

int check_type(cpm_handle* h, int t) {
  if (t < 0 || t >= kMaxTypes)
    return h->fail(CPM_ERR_INVALID, "cell type %d out of range [0, %d)", t, kMaxTypes);
  return CPM_OK;
}

template <class F>
int for_replicas(cpm_handle* h, int r, F&& f) {
  if (!h) return CPM_ERR_INVALID;
  if (r == -1) {
    for (size_t i = 0; i < h->psets.size(); ++i)
      if (h->pset_refs[i] > 0) f(h->psets[i]);
  } else {
    if (int rc = check_replica(h, r)) return rc;
    int p = h->reps[r].pset;
    if (h->pset_refs[p] > 1) {  // shared: give replica r its own copy
      h->psets.push_back(h->psets[p]);
      h->pset_refs.push_back(1);
      --h->pset_refs[p];
      p = (int)h->psets.size() - 1;
      h->reps[r].pset = p;
      h->reps_dirty = true;
    }
    f(h->psets[p]);
  }
  h->params_dirty = true;
  return CPM_OK;
}

int set_temperature(cpm_handle* h, int r, float T) {
  if (!h) return CPM_ERR_INVALID;
  if (!std::isfinite(T)) return h->fail(CPM_ERR_INVALID, "temperature must be finite");
  return for_replicas(h, r, [&](DevParams& p) { p.temperature = T; });
}

int set_area(cpm_handle* h, int r, int type, int target, float lambda) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  return for_replicas(h, r, [&](DevParams& p) {
    p.tgt_area[type] = target;
    p.lam_area[type] = lambda;
  });
}

int set_perimeter(cpm_handle* h, int r, int type, int target, float lambda) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  return for_replicas(h, r, [&](DevParams& p) {
    p.tgt_perim[type] = target;
    p.lam_perim[type] = lambda;
    p.perim_on = perim_on(p) ? 1 : 0;
  });
}

int set_fixed(cpm_handle* h, int r, int type, int fixed) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  return for_replicas(h, r, [&](DevParams& p) {
    if (fixed)
      p.fixed_mask |= 1u << type;
    else
      p.fixed_mask &= ~(1u << type);
  });
}

int set_stickiness(cpm_handle* h, int r, int type, int other, float S) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  if (int rc = check_type(h, other)) return rc;
  if (!std::isfinite(S)) return h->fail(CPM_ERR_INVALID, "stickiness must be finite");
  return for_replicas(h, r, [&](DevParams& p) { p.stick[type * kMaxTypes + other] = S; });
}

int set_adhesion(cpm_handle* h, int r, int type, int other, float J, int sym) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  if (int rc = check_type(h, other)) return rc;
  return for_replicas(h, r, [&](DevParams& p) {
    p.J[type * kMaxTypes + other] = J;
    if (sym) p.J[other * kMaxTypes + type] = J;
  });
}

int read_error_word(cpm_handle* h, uint32_t* word) {
  CPM_CUDA(h, cudaMemcpyAsync(word, h->d_ctl + kCtlErr, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, h->stream));
  CPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CPM_OK;
}

// Persistence buffers on first use: directions drawn from (seed, stream),
// history filled from the current tables when they exist.
int ensure_persist(cpm_handle* h) {
  if (!h->d_prefdir) {
    CPM_CUDA(h, cudaMalloc((void**)&h->d_prefdir, sizeof(double) * 3 * h->rows));
    CPM_CUDA(h, launch_init_prefdir(h->d_prefdir, h->d_reps, h->nrep, h->rows, h->seed,
                                    h->stream_id, h->stream));
  }
  if (!h->d_hist) {
    CPM_CUDA(h, cudaMalloc((void**)&h->d_hist, sizeof(double) * 3 * h->rows * h->hist_size));
    CPM_CUDA(h, cudaMemsetAsync(h->d_hist, 0, sizeof(double) * 3 * h->rows * h->hist_size,
                                h->stream));
    h->hist_slot = 0;
    if (h->pushed)
      CPM_CUDA(h, launch_persist_fill(h->d_hist, h->hist_size, h->d_ap[0], h->d_cs[0], h->d_reps,
                                      h->nrep, h->rows, h->stream));
  }
  return CPM_OK;
}

// After a run of a persistence engine: the cells' means into the history,
// and the preferred directions updated (src/cpm.cu:486-510).
int persist_after_run(cpm_handle* h) {
  if (!h->persist_active) return CPM_OK;
  CPM_CUDA(h, launch_persist_update(h->d_prefdir, h->d_hist, h->hist_size, h->hist_slot,
                                    h->d_ap[0], h->d_cs[0], h->d_ctype, h->d_params, h->d_reps,
                                    h->nrep, h->rows, h->stream));
  h->launches += 1;
  h->hist_slot = (h->hist_slot + 1) % h->hist_size;
  return CPM_OK;
}

// The act lattice (zeros) and the pending lists, on first use.
int ensure_act(cpm_handle* h) {
  if (!h->d_act) {
    const size_t n = (size_t)h->total_sites;
    try {
      h->h_act.assign(n, 0u);
    } catch (...) {
      return h->fail(CPM_ERR_ALLOC, "host act lattice allocation failed");
    }
    CPM_CUDA(h, cudaMalloc((void**)&h->d_act, sizeof(uint32_t) * (n ? n : 1)));
    CPM_CUDA(h, cudaMemsetAsync(h->d_act, 0, sizeof(uint32_t) * (n ? n : 1), h->stream));
  }
  if (!h->d_pend_site) {
    CPM_CUDA(h, cudaMalloc((void**)&h->d_pend_site,
                           sizeof(unsigned long long) * h->pend_entries));
    CPM_CUDA(h, cudaMalloc((void**)&h->d_pend_val, sizeof(uint32_t) * h->pend_entries));
  }
  return CPM_OK;
}

int upload_params(cpm_handle* h) {
  if (!h->params_dirty && !h->reps_dirty) return CPM_OK;
  // Drop records no replica uses and renumber the rest.
  const int n0 = (int)h->psets.size();
  std::vector<int> remap(n0, -1);
  int m = 0;
  for (int i = 0; i < n0; ++i) {
    if (h->pset_refs[i] <= 0) continue;
    remap[i] = m;
    if (m != i) {
      h->psets[m] = h->psets[i];
      h->pset_refs[m] = h->pset_refs[i];
    }
    ++m;
  }
  if (m != n0) {
    h->psets.resize(m);
    h->pset_refs.resize(m);
    for (auto& R : h->reps) R.pset = remap[R.pset];
    h->reps_dirty = true;
  }
  for (auto& p : h->psets) {
    p.perim_on = perim_on(p) ? 1 : 0;
    p.stick_on = 0;
    for (int k = 0; k < kMaxTypes * kMaxTypes; ++k)
      if (p.stick[k] != 0.0f) p.stick_on = 1;
    p.chemo_on = 0;
    for (int k = 0; k < kMaxTypes; ++k)
      if (p.chemo[k] != 0.0f) p.chemo_on = 1;
    if (p.chemo_on && !h->d_field)
      return h->fail(CPM_ERR_STATE, "chemotaxis is set but the engine has no field "
                                    "(create it with the field flag or call cpm_host_field_r)");
    p.act_on = 0;
    for (int k = 0; k < kMaxTypes; ++k)
      if (p.act_lambda[k] != 0.0f) p.act_on = 1;
    p.persist_on = 0;
    for (int k = 0; k < kMaxTypes; ++k)
      if (p.persist_lambda[k] != 0.0f) p.persist_on = 1;
  }
  bool persist = false;
  for (const auto& p : h->psets) persist = persist || (h->ndim == 3 && p.persist_on);
  if (persist) {
    if (int rc = ensure_persist(h)) return rc;
  }
  if (persist != h->persist_active) {
    h->persist_active = persist;
    if (h->graph_exec) {
      cudaGraphExecDestroy(h->graph_exec);
      h->graph_exec = nullptr;
    }
  }
  bool act = false;
  for (const auto& p : h->psets) act = act || p.act_on;
  if (act) {
    if (int rc = ensure_act(h)) return rc;
  }
  if (act != h->act_active) {  // another kernel, other arguments
    h->act_active = act;
    if (h->graph_exec) {
      cudaGraphExecDestroy(h->graph_exec);
      h->graph_exec = nullptr;
    }
  }
  if (m > h->params_cap) {
    CPM_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->d_params);
    h->d_params = nullptr;
    h->params_cap = 0;
    CPM_CUDA(h, cudaMalloc((void**)&h->d_params, sizeof(DevParams) * m));
    h->params_cap = m;
    if (h->graph_exec) {  // it holds the old address
      cudaGraphExecDestroy(h->graph_exec);
      h->graph_exec = nullptr;
    }
  }
  CPM_CUDA(h, cudaMemcpyAsync(h->d_params, h->psets.data(), sizeof(DevParams) * m,
                              cudaMemcpyHostToDevice, h->stream));
  if (h->reps_dirty)
    CPM_CUDA(h, cudaMemcpyAsync(h->d_reps, h->reps.data(), sizeof(DevReplica) * h->nrep,
                                cudaMemcpyHostToDevice, h->stream));
  CPM_CUDA(h, cudaStreamSynchronize(h->stream));  // the host copies may change next
  h->params_dirty = false;
  h->reps_dirty = false;
  return CPM_OK;
}

bool any_perimeter(const cpm_handle* h) {
  for (size_t i = 0; i < h->psets.size(); ++i)
    if (h->pset_refs[i] > 0 && perim_on(h->psets[i])) return true;
  return false;
}

// Kernel arguments of a sweep with tile variant v and dispatch d (tick0 /
// mcs filled in by the caller).
SweepArgs sweep_args(const cpm_handle* h, int v, int d) {
  if (h->act_active || h->persist_active) v = 0;  // extended-term kernels: variant 0
  SweepArgs a;
  std::memset(&a, 0, sizeof a);
  a.lat = h->d_lat;
  for (int b = 0; b < 2; ++b) {
    a.ap[b] = h->d_ap[b];
    a.cs[b] = h->d_cs[b];
    a.dap[b] = h->d_dap[b];
    a.dcs[b] = h->d_dcs[b];
  }
  const cpm_handle::Config& c = h->cfg[v];
  a.dlist = h->d_dlist;
  a.block_local = d == CPM_DISPATCH_REPLICA ? 1 : 0;
  a.field = h->d_field;
  a.act = h->d_act;
  a.act_on = h->act_active ? 1 : 0;
  a.prefdir = h->persist_active ? h->d_prefdir : nullptr;
  a.pend_site = h->d_pend_site;
  a.pend_val = h->d_pend_val;
  a.pend_cap = (d == CPM_DISPATCH_REPLICA ? c.list_cap_local : c.list_cap) / 2;
  a.list_cap = a.block_local ? c.list_cap_local : c.list_cap;
  a.rep_order = h->d_rep_order;
  a.queue_len = h->nrep;
  a.rep_map = nullptr;
  a.tick_advance = 1;
  a.ctl = h->d_ctl;
  a.counters = h->d_counters;
  a.reps = h->d_reps;
  a.params = h->d_params;
  a.task_prefix = h->d_task_prefix + (size_t)v * 27 * (h->nrep + 1);
  a.seed = h->seed;
  a.nrep = h->nrep;
  a.stream0 = h->stream_id;
  a.nslot_active = (int)c.active_slots.size();
  for (int i = 0; i < a.nslot_active; ++i) a.slots[i] = c.active_slots[i];
  return a;
}

int grid_of(const cpm_handle* h, int v, int d) {
  if (h->act_active || h->persist_active) v = 0;
  return d == CPM_DISPATCH_REPLICA ? h->cfg[v].grid_local : h->cfg[v].grid;
}

// The launches of one sweep run (`a` from sweep_args with dispatch `d`,
// times filled in): one launch for GRID and REPLICA, two for HYBRID (grid
// dispatch over the first hyb_ng replicas of rep_order, then replica
// dispatch over the rest).  Each launch starts with its barrier words
// cleared.  Returns the number of launches through *nlaunch.
cudaError_t enqueue_sweep(const cpm_handle* h, int v, int d, const SweepArgs& a, bool perim,
                          bool scores, int* nlaunch) {
  if (h->act_active || h->persist_active) v = 0;
  const cpm_handle::Config& c = h->cfg[v];
  *nlaunch = 0;
  auto one = [&](const SweepArgs& x, int grid) {
    cudaError_t e = cudaMemsetAsync(h->d_ctl, 0, sizeof(uint32_t) * kCtlErr, h->stream);
    const bool row = h->fill != CPM_FILL_PARITY && h->row_ok && !scores && !h->act_active &&
                     !h->persist_active && x.nrep == 1 && x.rep_map == nullptr &&
                     !x.block_local;
    if (e == cudaSuccess && row && h->fill == CPM_FILL_CLUSTER) {
      SweepArgs xc = x;
      xc.list_cap = h->cl_cap;
      e = launch_sweep2d_cluster(perim, v, xc, h->tmap[3].bytes, h->reps[0].nx, h->cl_G,
                                 h->cl_H, h->stream);
    } else if (e == cudaSuccess && row)
      e = (h->ndim == 2 ? launch_sweep2d : launch_sweep3d)(
          perim, v, x, h->tmap[v].bytes, h->fill == CPM_FILL_TMA ? 1 : 0, grid, c.shape.warps,
          h->stream);
    else if (e == cudaSuccess)
      e = launch_sweep(h->ndim, perim, v, x, grid, h->stream, scores);
    if (e == cudaSuccess) ++*nlaunch;
    return e;
  };
  if (d != CPM_DISPATCH_HYBRID) return one(a, grid_of(h, v, d));
  const int ng = c.hyb_ng;
  if (ng > 0) {  // grid dispatch over the largest replicas
    SweepArgs g = a;
    g.block_local = 0;
    g.list_cap = c.list_cap;
    g.pend_cap = c.list_cap / 2;
    g.nrep = ng;
    g.task_prefix = h->d_hyb_prefix + (size_t)v * 27 * (h->nrep + 1);
    g.rep_map = h->d_rep_order;
    g.tick_advance = ng < h->nrep ? 0 : 1;
    if (cudaError_t e = one(g, c.grid)) return e;
  }
  if (ng < h->nrep) {  // replica dispatch over the rest, whole rounds
    SweepArgs q = a;
    q.block_local = 1;
    q.list_cap = c.list_cap_local;
    q.pend_cap = c.list_cap_local / 2;
    q.rep_order = h->d_rep_order + ng;
    q.queue_len = h->nrep - ng;
    if (cudaError_t e = one(q, c.grid_local)) return e;
  }
  return cudaSuccess;
}

void count_attempts(cpm_handle* h, int mcs) {
  for (int r = 0; r < h->nrep; ++r) {
    const DevReplica& R = h->reps[r];
    h->attempts[r] += (unsigned long long)R.nx * R.ny * R.nz * (unsigned long long)mcs;
  }
}

std::string describe_errors(uint32_t w) {
  std::string s;
  auto add = [&](const char* m) {
    if (!s.empty()) s += "; ";
    s += m;
  };
  if (w & kErrBadId) add("a site holds an id above number_of_cells");
  if (w & kErrBadType) add("a site holds a type >= 32");
  if (w & kErrMediumType) add("a site holds id 0 with a non-zero type");
  if (w & kErrTypeConflict) add("one cell id appears with two different types");
  if (w & kErrTimeout) add("a grid barrier of the sweep timed out");
  if (w & kErrListFull) add("a dirty list of the sweep was too small (internal error)");
  return s;
}

}  // namespace

extern "C" {

int cpm_create(int dimension, int dimensionality, int number_of_cells,
               float temperature, int flags, cpm_handle** out) {
  if (flags & ~(CPM_FLAG_FIELD | CPM_FLAG_ACT)) {
    g_create_error = "unknown flags (CPM_FLAG_FIELD and CPM_FLAG_ACT are the flags)";
    if (out) *out = nullptr;
    return CPM_ERR_UNSUPPORTED;
  }
  const int nz = dimensionality == 3 ? dimension : 1;
  const int rc = build_engine(1, dimensionality, &dimension, &dimension, &nz,
                              &number_of_cells, temperature, out);
  if (rc == CPM_OK && (flags & CPM_FLAG_FIELD)) {
    if (int rc2 = cpm_host_field_r(*out, 0, nullptr, nullptr)) {
      g_create_error = cpm_last_error(*out);
      cpm_destroy(*out);
      *out = nullptr;
      return rc2;
    }
  }
  if (rc == CPM_OK && (flags & CPM_FLAG_ACT)) {
    if (int rc2 = cpm_host_act_r(*out, 0, nullptr, nullptr)) {
      g_create_error = cpm_last_error(*out);
      cpm_destroy(*out);
      *out = nullptr;
      return rc2;
    }
  }
  return rc;
}

int cpm_create_box(int nx, int ny, int nz, int dimensionality,
                   int number_of_cells, float temperature, cpm_handle** out) {
  return build_engine(1, dimensionality, &nx, &ny, &nz, &number_of_cells,
                      temperature, out);
}

int cpm_create_batch(int n, int dimensionality, const int* nx, const int* ny,
                     const int* nz, const int* ncells, cpm_handle** out) {
  if (!nx || !ny || !ncells || (dimensionality == 3 && !nz)) {
    g_create_error = "nx, ny, ncells (and nz in 3D) must be non-NULL";
    if (out) *out = nullptr;
    return CPM_ERR_INVALID;
  }
  return build_engine(n, dimensionality, nx, ny, nz, ncells, 1.0f, out);
}

int cpm_destroy(cpm_handle* h) {
  if (!h) return CPM_OK;
  cudaSetDevice(h->device);
  free_all(h);
  delete h;
  return CPM_OK;
}

int cpm_set_device(int device) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    g_create_error = std::string("cudaSetDevice failed: ") + cudaGetErrorString(e);
    return CPM_ERR_CUDA;
  }
  return CPM_OK;
}

const char* cpm_last_error(const cpm_handle* h) {
  return h ? h->err.c_str() : g_create_error.c_str();
}

int cpm_set_temperature(cpm_handle* h, float T) { return set_temperature(h, -1, T); }
int cpm_set_temperature_r(cpm_handle* h, int r, float T) { return set_temperature(h, r < 0 ? -2 : r, T); }
int cpm_set_area(cpm_handle* h, int type, int target, float lambda) {
  return set_area(h, -1, type, target, lambda);
}
int cpm_set_area_r(cpm_handle* h, int r, int type, int target, float lambda) {
  return set_area(h, r < 0 ? -2 : r, type, target, lambda);
}
int cpm_set_perimeter(cpm_handle* h, int type, int target, float lambda) {
  return set_perimeter(h, -1, type, target, lambda);
}
int cpm_set_perimeter_r(cpm_handle* h, int r, int type, int target, float lambda) {
  return set_perimeter(h, r < 0 ? -2 : r, type, target, lambda);
}
int cpm_set_fixed(cpm_handle* h, int type, int fixed) { return set_fixed(h, -1, type, fixed); }
int cpm_set_fixed_r(cpm_handle* h, int r, int type, int fixed) {
  return set_fixed(h, r < 0 ? -2 : r, type, fixed);
}
int cpm_set_stickiness(cpm_handle* h, int type, int other, float S) {
  return set_stickiness(h, -1, type, other, S);
}
int cpm_set_stickiness_r(cpm_handle* h, int r, int type, int other, float S) {
  return set_stickiness(h, r < 0 ? -2 : r, type, other, S);
}
int cpm_set_adhesion(cpm_handle* h, int type, int other, float J, int symmetric) {
  return set_adhesion(h, -1, type, other, J, symmetric);
}
int cpm_set_adhesion_r(cpm_handle* h, int r, int type, int other, float J, int symmetric) {
  return set_adhesion(h, r < 0 ? -2 : r, type, other, J, symmetric);
}

int cpm_add_cell(cpm_handle* h, int type, int x, int y, int z) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  const DevReplica& R = h->reps[0];
  if (h->ndim == 2) z = 0;
  if (x < 0 || x >= R.nx || y < 0 || y >= R.ny || z < 0 || z >= R.nz)
    return h->fail(CPM_ERR_INVALID, "add_cell position (%d, %d, %d) outside the lattice", x, y, z);
  if (h->added_cells >= R.ncells)
    return h->fail(CPM_ERR_INVALID, "add_cell would exceed number_of_cells = %d", R.ncells);
  h->added_cells += 1;
  h->h_lat[R.lat_off + ((long long)z * R.ny + y) * R.nx + x] =
      (uint32_t)h->added_cells | ((uint32_t)type << 24);
  return CPM_OK;
}

int cpm_host_field_r(cpm_handle* h, int r, double** ptr, int64_t* nvalues) {
  if (int rc = check_replica(h, r)) return rc;
  CPM_BIND(h);
  if (!h->d_field) {
    const size_t n = (size_t)h->total_sites * h->ndim;
    try {
      h->h_field.assign(n, 0.0);
    } catch (...) {
      return h->fail(CPM_ERR_ALLOC, "host field allocation failed");
    }
    CPM_CUDA(h, cudaMalloc((void**)&h->d_field, sizeof(float) * (n ? n : 1)));
    CPM_CUDA(h, cudaMemsetAsync(h->d_field, 0, sizeof(float) * (n ? n : 1), h->stream));
    if (h->graph_exec) {  // captured without a field
      cudaGraphExecDestroy(h->graph_exec);
      h->graph_exec = nullptr;
    }
  }
  const DevReplica& R = h->reps[r];
  if (ptr) *ptr = h->h_field.data() + (size_t)h->ndim * R.lat_off;
  if (nvalues) *nvalues = (int64_t)h->ndim * R.nx * R.ny * R.nz;
  return CPM_OK;
}

namespace {
int set_act(cpm_handle* h, int r, int type, int max_act, float lambda) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  if (!std::isfinite(lambda)) return h->fail(CPM_ERR_INVALID, "lambda must be finite");
  if (max_act < 0) return h->fail(CPM_ERR_INVALID, "max_act must be >= 0");
  return for_replicas(h, r, [&](DevParams& p) {
    p.act_max[type] = max_act;
    p.act_lambda[type] = lambda;
  });
}

int set_persistence(cpm_handle* h, int r, int type, int time, float diffusion, float lambda) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  if (!std::isfinite(lambda) || !std::isfinite(diffusion))
    return h->fail(CPM_ERR_INVALID, "lambda and diffusion must be finite");
  return for_replicas(h, r, [&](DevParams& p) {
    p.persist_lambda[type] = lambda;
    p.persist_diff[type] = diffusion;
    p.persist_time[type] = time;
  });
}

int set_chemotaxis(cpm_handle* h, int r, int type, float lambda) {
  if (!h) return CPM_ERR_INVALID;
  if (int rc = check_type(h, type)) return rc;
  if (!std::isfinite(lambda)) return h->fail(CPM_ERR_INVALID, "lambda must be finite");
  return for_replicas(h, r, [&](DevParams& p) { p.chemo[type] = lambda; });
}
}  // namespace
int cpm_host_act_r(cpm_handle* h, int r, uint32_t** ptr, int64_t* nsites) {
  if (int rc = check_replica(h, r)) return rc;
  CPM_BIND(h);
  if (int rc = ensure_act(h)) return rc;
  const DevReplica& R = h->reps[r];
  if (ptr) *ptr = h->h_act.data() + R.lat_off;
  if (nsites) *nsites = (int64_t)R.nx * R.ny * R.nz;
  return CPM_OK;
}
int cpm_has_act(const cpm_handle* h, int* has) {
  if (!h || !has) return CPM_ERR_INVALID;
  *has = h->d_act ? 1 : 0;
  return CPM_OK;
}
int cpm_set_act(cpm_handle* h, int type, int max_act, float lambda) {
  return set_act(h, -1, type, max_act, lambda);
}
int cpm_set_act_r(cpm_handle* h, int r, int type, int max_act, float lambda) {
  return set_act(h, r < 0 ? -2 : r, type, max_act, lambda);
}
int cpm_set_chemotaxis(cpm_handle* h, int type, float lambda) {
  return set_chemotaxis(h, -1, type, lambda);
}
int cpm_set_chemotaxis_r(cpm_handle* h, int r, int type, float lambda) {
  return set_chemotaxis(h, r < 0 ? -2 : r, type, lambda);
}
int cpm_set_persistence(cpm_handle* h, int type, int time, float diffusion, float lambda) {
  return set_persistence(h, -1, type, time, diffusion, lambda);
}
int cpm_set_persistence_r(cpm_handle* h, int r, int type, int time, float diffusion,
                          float lambda) {
  return set_persistence(h, r < 0 ? -2 : r, type, time, diffusion, lambda);
}

int cpm_set_history(cpm_handle* h, int history) {
  if (!h) return CPM_ERR_INVALID;
  if (history < 1) return h->fail(CPM_ERR_INVALID, "history must be >= 1");
  if (history == h->hist_size) return CPM_OK;
  CPM_BIND(h);
  h->hist_size = history;
  if (h->d_hist) {  // reallocated and refilled from the current tables
    CPM_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->d_hist);
    h->d_hist = nullptr;
    return ensure_persist(h);
  }
  return CPM_OK;
}

int cpm_has_persistence(const cpm_handle* h, int* has, int* history) {
  if (!h) return CPM_ERR_INVALID;
  if (has) *has = (h->d_prefdir && h->d_hist) ? 1 : 0;
  if (history) *history = h->hist_size;
  return CPM_OK;
}

namespace {
// Copies of replica r's rows of the persistence state; `to_host` picks the
// direction.  History slots in the caller's buffer run oldest first.
int persistence_copy(cpm_handle* h, int r, double* prefdir, double* history, bool to_host) {
  if (int rc = check_replica(h, r)) return rc;
  CPM_BIND(h);
  if (!to_host && h->ndim == 3 && h->pushed) {  // restoring: allocate first
    if (int rc = ensure_persist(h)) return rc;
  }
  if (!h->d_prefdir || !h->d_hist)
    return h->fail(CPM_ERR_STATE, "the engine has no persistence state");
  const DevReplica& R = h->reps[r];
  const size_t n = (size_t)(R.ncells + 1) * 3;
  const auto kind = to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice;
  auto copy = [&](double* dev, double* host) {
    return to_host ? cudaMemcpyAsync(host, dev, n * sizeof(double), kind, h->stream)
                   : cudaMemcpyAsync(dev, host, n * sizeof(double), kind, h->stream);
  };
  if (prefdir) CPM_CUDA(h, copy(h->d_prefdir + R.cell_off * 3, prefdir));
  if (history)
    for (int k = 0; k < h->hist_size; ++k) {
      const int slot = (h->hist_slot + k) % h->hist_size;
      CPM_CUDA(h, copy(h->d_hist + ((size_t)slot * h->rows + R.cell_off) * 3, history + k * n));
    }
  CPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CPM_OK;
}
}  // namespace

int cpm_get_persistence_r(cpm_handle* h, int r, double* prefdir, double* history) {
  return persistence_copy(h, r, prefdir, history, true);
}
int cpm_set_persistence_state_r(cpm_handle* h, int r, const double* prefdir,
                                const double* history) {
  return persistence_copy(h, r, const_cast<double*>(prefdir), const_cast<double*>(history),
                          false);
}

int cpm_host_lattice_r(cpm_handle* h, int r, uint32_t** ptr, int64_t* nsites) {
  if (int rc = check_replica(h, r)) return rc;
  const DevReplica& R = h->reps[r];
  if (ptr) *ptr = h->h_lat + R.lat_off;
  if (nsites) *nsites = (int64_t)R.nx * R.ny * R.nz;
  return CPM_OK;
}
int cpm_host_lattice(cpm_handle* h, uint32_t** ptr, int64_t* nsites) {
  return cpm_host_lattice_r(h, 0, ptr, nsites);
}

int cpm_device_lattice_r(cpm_handle* h, int r, uint32_t** dptr) {
  if (int rc = check_replica(h, r)) return rc;
  if (dptr) *dptr = h->d_lat + h->reps[r].lat_off;
  return CPM_OK;
}

namespace {
// Tables of every replica recomputed from the device lattice.
int recount_tables(cpm_handle* h) {
  h->pushed = false;
  for (int b = 0; b < 2; ++b) {
    CPM_CUDA(h, cudaMemsetAsync(h->d_ap[b], 0, sizeof(unsigned long long) * h->rows, h->stream));
    CPM_CUDA(h, cudaMemsetAsync(h->d_cs[b], 0, sizeof(long long) * h->rows * h->ndim, h->stream));
    CPM_CUDA(h, cudaMemsetAsync(h->d_dap[b], 0, sizeof(unsigned long long) * h->rows, h->stream));
    CPM_CUDA(h, cudaMemsetAsync(h->d_dcs[b], 0, sizeof(long long) * h->rows * h->ndim, h->stream));
  }
  CPM_CUDA(h, cudaMemsetAsync(h->d_first, 0xFF, sizeof(unsigned long long) * h->rows, h->stream));
  CPM_CUDA(h, cudaMemsetAsync(h->d_ctype, 0xFF, sizeof(int) * h->rows, h->stream));
  CPM_CUDA(h, cudaMemsetAsync(h->d_ctl, 0, sizeof(uint32_t) * kCtlWords, h->stream));
  CPM_CUDA(h, launch_init(h->ndim, h->d_lat, h->d_reps, h->nrep, h->total_sites,
                          h->d_ap[0], h->d_cs[0], h->d_first, h->d_ctype, h->d_ctl,
                          h->stream));
  h->launches += 2;
  // Both table copies start equal (the sweep keeps them equal between runs).
  CPM_CUDA(h, cudaMemcpyAsync(h->d_ap[1], h->d_ap[0], sizeof(unsigned long long) * h->rows,
                              cudaMemcpyDeviceToDevice, h->stream));
  CPM_CUDA(h, cudaMemcpyAsync(h->d_cs[1], h->d_cs[0], sizeof(long long) * h->rows * h->ndim,
                              cudaMemcpyDeviceToDevice, h->stream));
  uint32_t w = 0;
  if (int rc = read_error_word(h, &w)) return rc;
  if (w) {
    CPM_CUDA(h, cudaMemsetAsync(h->d_ctl, 0, sizeof(uint32_t) * kCtlWords, h->stream));
    return h->fail(CPM_ERR_INVALID, "the lattice was rejected: %s",
                   describe_errors(w).c_str());
  }
  h->pushed = true;
  return CPM_OK;
}
}  // namespace

int cpm_push(cpm_handle* h) {
  CPM_BIND(h);
  h->pushed = false;
  CPM_CUDA(h, cudaMemcpyAsync(h->d_lat, h->h_lat, sizeof(uint32_t) * h->total_sites,
                              cudaMemcpyHostToDevice, h->stream));
  if (h->d_act)  // act stamps go along (src/cpm.cu:547-549)
    CPM_CUDA(h, cudaMemcpyAsync(h->d_act, h->h_act.data(), sizeof(uint32_t) * h->total_sites,
                                cudaMemcpyHostToDevice, h->stream));
  if (h->d_field) {  // the field goes along, as in Cpm::moveCellIdsToGpu
    std::vector<float> f(h->h_field.begin(), h->h_field.end());
    CPM_CUDA(h, cudaMemcpyAsync(h->d_field, f.data(), sizeof(float) * f.size(),
                                cudaMemcpyHostToDevice, h->stream));
    CPM_CUDA(h, cudaStreamSynchronize(h->stream));  // `f` lives on this frame
  }
  if (int rc = recount_tables(h)) return rc;
  if (h->d_hist) {  // every history slot holds the pushed means (src/cpm.cu:578-583)
    CPM_CUDA(h, launch_persist_fill(h->d_hist, h->hist_size, h->d_ap[0], h->d_cs[0], h->d_reps,
                                    h->nrep, h->rows, h->stream));
    h->hist_slot = 0;
  }
  return CPM_OK;
}

int cpm_recount(cpm_handle* h) {
  CPM_BIND(h);
  return recount_tables(h);
}

int cpm_set_centroid_sums_r(cpm_handle* h, int r, const int64_t* centroid_sums) {
  if (int rc = check_replica(h, r)) return rc;
  CPM_BIND(h);
  if (!centroid_sums) return h->fail(CPM_ERR_INVALID, "centroid_sums is NULL");
  if (!h->pushed) return h->fail(CPM_ERR_STATE, "set centroid sums after a successful push");
  const DevReplica& R = h->reps[r];
  const size_t bytes = sizeof(long long) * ((size_t)R.ncells + 1) * h->ndim;
  for (int b = 0; b < 2; ++b)
    CPM_CUDA(h, cudaMemcpyAsync(h->d_cs[b] + R.cell_off * h->ndim, centroid_sums, bytes,
                                cudaMemcpyHostToDevice, h->stream));
  CPM_CUDA(h, cudaStreamSynchronize(h->stream));  // the caller's buffer may go
  return CPM_OK;
}

int cpm_get_params_r(const cpm_handle* h, int r, cpm_static_params* out) {
  if (!h || !out || r < 0 || r >= h->nrep) return CPM_ERR_INVALID;
  const DevParams& p = h->psets[h->reps[r].pset];
  std::memcpy(out->J, p.J, sizeof out->J);
  std::memcpy(out->lambda_area, p.lam_area, sizeof out->lambda_area);
  std::memcpy(out->target_area, p.tgt_area, sizeof out->target_area);
  std::memcpy(out->lambda_perimeter, p.lam_perim, sizeof out->lambda_perimeter);
  std::memcpy(out->target_perimeter, p.tgt_perim, sizeof out->target_perimeter);
  out->temperature = p.temperature;
  std::memcpy(out->stickiness, p.stick, sizeof out->stickiness);
  for (int k = 0; k < kMaxTypes; ++k) out->fixed[k] = (p.fixed_mask >> k) & 1u;
  std::memcpy(out->chemotaxis, p.chemo, sizeof out->chemotaxis);
  std::memcpy(out->act_lambda, p.act_lambda, sizeof out->act_lambda);
  std::memcpy(out->act_max, p.act_max, sizeof out->act_max);
  std::memcpy(out->persistence_lambda, p.persist_lambda, sizeof out->persistence_lambda);
  std::memcpy(out->persistence_diffusion, p.persist_diff, sizeof out->persistence_diffusion);
  std::memcpy(out->persistence_time, p.persist_time, sizeof out->persistence_time);
  return CPM_OK;
}

namespace {
int set_params(cpm_handle* h, int r, const cpm_static_params* in) {
  if (!h) return CPM_ERR_INVALID;
  if (!in) return h->fail(CPM_ERR_INVALID, "params is NULL");
  if (!std::isfinite(in->temperature))
    return h->fail(CPM_ERR_INVALID, "temperature must be finite");
  for (int k = 0; k < kMaxTypes; ++k) {
    if (!std::isfinite(in->chemotaxis[k]) || !std::isfinite(in->act_lambda[k]) ||
        !std::isfinite(in->persistence_lambda[k]) || !std::isfinite(in->persistence_diffusion[k]))
      return h->fail(CPM_ERR_INVALID, "lambdas and diffusion must be finite");
    if (in->act_max[k] < 0) return h->fail(CPM_ERR_INVALID, "act_max must be >= 0");
  }
  auto fill = [&](DevParams& p) {
    std::memcpy(p.J, in->J, sizeof p.J);
    std::memcpy(p.lam_area, in->lambda_area, sizeof p.lam_area);
    std::memcpy(p.tgt_area, in->target_area, sizeof p.tgt_area);
    std::memcpy(p.lam_perim, in->lambda_perimeter, sizeof p.lam_perim);
    std::memcpy(p.tgt_perim, in->target_perimeter, sizeof p.tgt_perim);
    p.temperature = in->temperature;
    std::memcpy(p.stick, in->stickiness, sizeof p.stick);
    p.fixed_mask = 0;
    for (int k = 0; k < kMaxTypes; ++k)
      if (in->fixed[k]) p.fixed_mask |= 1u << k;
    std::memcpy(p.chemo, in->chemotaxis, sizeof p.chemo);
    std::memcpy(p.act_lambda, in->act_lambda, sizeof p.act_lambda);
    std::memcpy(p.act_max, in->act_max, sizeof p.act_max);
    std::memcpy(p.persist_lambda, in->persistence_lambda, sizeof p.persist_lambda);
    std::memcpy(p.persist_diff, in->persistence_diffusion, sizeof p.persist_diff);
    std::memcpy(p.persist_time, in->persistence_time, sizeof p.persist_time);
  };
  if (r == -1) {  // every field of every replica: one shared record
    DevParams p;
    default_params(p, in->temperature);
    fill(p);
    h->psets.assign(1, p);
    h->pset_refs.assign(1, h->nrep);
    for (auto& R : h->reps) R.pset = 0;
    h->reps_dirty = true;
    h->params_dirty = true;
    return CPM_OK;
  }
  return for_replicas(h, r, fill);
}
}  // namespace

int cpm_set_params(cpm_handle* h, const cpm_static_params* in) { return set_params(h, -1, in); }
int cpm_set_params_r(cpm_handle* h, int r, const cpm_static_params* in) {
  return set_params(h, r < 0 ? -2 : r, in);
}

int cpm_get_param_index(const cpm_handle* h, int* out) {
  if (!h || !out) return CPM_ERR_INVALID;
  for (int r = 0; r < h->nrep; ++r) out[r] = h->reps[r].pset;
  return CPM_OK;
}

int cpm_get_device(const cpm_handle* h, int* device) {
  if (!h || !device) return CPM_ERR_INVALID;
  *device = h->device;
  return CPM_OK;
}

int cpm_get_seed(const cpm_handle* h, uint64_t* seed, uint32_t* stream_id) {
  if (!h) return CPM_ERR_INVALID;
  if (seed) *seed = h->seed;
  if (stream_id) *stream_id = h->stream_id;
  return CPM_OK;
}

int cpm_pull(cpm_handle* h) {
  CPM_BIND(h);
  CPM_CUDA(h, cudaMemcpyAsync(h->h_lat, h->d_lat, sizeof(uint32_t) * h->total_sites,
                              cudaMemcpyDeviceToHost, h->stream));
  if (h->d_act)  // and the act stamps (src/cpm.cu:534-536)
    CPM_CUDA(h, cudaMemcpyAsync(h->h_act.data(), h->d_act, sizeof(uint32_t) * h->total_sites,
                                cudaMemcpyDeviceToHost, h->stream));
  CPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CPM_OK;
}

int cpm_run(cpm_handle* h, int mcs) {
  CPM_BIND(h);
  if (mcs < 0) return h->fail(CPM_ERR_INVALID, "mcs must be >= 0");
  if (!h->pushed) return h->fail(CPM_ERR_STATE, "run() before a successful push_to_gpu()");
  if (mcs == 0) return CPM_OK;
  if (int rc = upload_params(h)) return rc;
  const bool any_perim = any_perimeter(h);
  SweepArgs a = sweep_args(h, h->variant, h->dispatch);
  int left = mcs;
  while (left > 0) {
    const int chunk = std::min(left, kMaxMcsPerLaunch);
    a.tick0 = h->tick;
    a.mcs = chunk;
    // Barrier counter and release flag start at zero in every launch; the
    // sticky error word is left alone until cpm_synchronize reads it.
    int nl = 0;
    CPM_CUDA(h, enqueue_sweep(h, h->variant, h->dispatch, a, any_perim, false, &nl));
    h->launches += nl;
    h->tick += (uint64_t)chunk;
    left -= chunk;
  }
  h->d_tick_stale = true;
  count_attempts(h, mcs);
  return persist_after_run(h);
}

int cpm_run_graph(cpm_handle* h, int mcs) {
  CPM_BIND(h);
  if (mcs <= 0 || mcs > kMaxMcsPerLaunch)
    return h->fail(CPM_ERR_INVALID, "mcs must be in [1, %d] for a graph run", kMaxMcsPerLaunch);
  if (!h->pushed) return h->fail(CPM_ERR_STATE, "run before a successful push_to_gpu()");
  if (h->stream == nullptr)
    return h->fail(CPM_ERR_STATE, "graph runs need a non-default stream");
  if (int rc = upload_params(h)) return rc;
  if (!h->graph_exec || h->graph_mcs != mcs || h->graph_variant != h->variant ||
      h->graph_dispatch != h->dispatch || h->graph_fill != h->fill ||
      h->graph_stream != h->stream) {
    if (h->graph_exec) {
      cudaGraphExecDestroy(h->graph_exec);
      h->graph_exec = nullptr;
    }
    // Capture: reset the barrier words, then the persistent sweep reading
    // its start time from (and advancing) the device tick.
    SweepArgs a = sweep_args(h, h->variant, h->dispatch);
    a.tick_ptr = h->d_tick;
    a.mcs = mcs;
    cudaGraph_t g = nullptr;
    CPM_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int nl = 0;
    cudaError_t e2 = enqueue_sweep(h, h->variant, h->dispatch, a, any_perimeter(h), false, &nl);
    cudaError_t e3 = cudaStreamEndCapture(h->stream, &g);
    if (e2 != cudaSuccess) return h->cuda_fail(e2, "capture of the sweep launch");
    if (e3 != cudaSuccess) return h->cuda_fail(e3, "cudaStreamEndCapture");
    cudaError_t e4 = cudaGraphInstantiate(&h->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e4 != cudaSuccess) return h->cuda_fail(e4, "cudaGraphInstantiate");
    h->graph_mcs = mcs;
    h->graph_launches = nl;
    h->graph_variant = h->variant;
    h->graph_dispatch = h->dispatch;
    h->graph_fill = h->fill;
    h->graph_stream = h->stream;
  }
  if (h->d_tick_stale) {
    const unsigned long long t = h->tick;
    CPM_CUDA(h, cudaMemcpyAsync(h->d_tick, &t, sizeof t, cudaMemcpyHostToDevice, h->stream));
    CPM_CUDA(h, cudaStreamSynchronize(h->stream));  // `t` lives on this frame
    h->d_tick_stale = false;
  }
  CPM_CUDA(h, cudaGraphLaunch(h->graph_exec, h->stream));
  h->launches += h->graph_launches;
  h->tick += (uint64_t)mcs;
  count_attempts(h, mcs);
  return persist_after_run(h);  // a launch of its own: its slot changes per run
}

int cpm_autotune(cpm_handle* h, int probe_mcs, int* chosen, float* ms_per_mcs) {
  CPM_BIND(h);
  if (!h->pushed) return h->fail(CPM_ERR_STATE, "autotune before a successful push_to_gpu()");
  if (probe_mcs < 1) probe_mcs = 2;
  if (int rc = upload_params(h)) return rc;
  // Work on a saved copy of the state: every variant runs the same MCS from
  // the same start, and the state (lattice, tables, counters, tick) is put
  // back afterwards.  The sweep's result does not depend on the variant, so
  // only the time differs.
  const size_t lat_b = sizeof(uint32_t) * h->total_sites;
  const size_t ap_b = sizeof(unsigned long long) * h->rows;
  const size_t cs_b = sizeof(long long) * h->rows * h->ndim;
  const size_t cnt_b = sizeof(unsigned long long) * 2 * h->nrep;
  const size_t act_b = h->d_act ? lat_b : 0;  // act stamps, when kept
  char* save = nullptr;
  CPM_CUDA(h, cudaMalloc(&save, lat_b + ap_b + cs_b + cnt_b + act_b));
  auto copy = [&](bool to_save) -> cudaError_t {
    char* p = save;
    void* dst[5] = {p, p + lat_b, p + lat_b + ap_b, p + lat_b + ap_b + cs_b,
                    p + lat_b + ap_b + cs_b + cnt_b};
    void* src[5] = {h->d_lat, h->d_ap[0], h->d_cs[0], h->d_counters, h->d_act};
    const size_t n[5] = {lat_b, ap_b, cs_b, cnt_b, act_b};
    for (int i = 0; i < 5; ++i) {
      if (!n[i]) continue;
      cudaError_t e = to_save ? cudaMemcpyAsync(dst[i], src[i], n[i], cudaMemcpyDeviceToDevice, h->stream)
                              : cudaMemcpyAsync(src[i], dst[i], n[i], cudaMemcpyDeviceToDevice, h->stream);
      if (e != cudaSuccess) return e;
    }
    if (!to_save) {
      cudaError_t e = cudaMemcpyAsync(h->d_ap[1], h->d_ap[0], ap_b, cudaMemcpyDeviceToDevice, h->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_cs[1], h->d_cs[0], cs_b, cudaMemcpyDeviceToDevice, h->stream);
      return e;
    }
    return cudaSuccess;
  };
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaError_t e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  if (e == cudaSuccess) e = copy(true);
  const uint64_t tick = h->tick;
  float best = -1.0f;
  int best_v = h->variant, best_d = h->dispatch;
  const bool any_perim = any_perimeter(h);
  // Every (tile variant, dispatch) pair, replica dispatch only for batches,
  // timed in three rounds (the fastest run counts): a variant's first launch
  // also loads its module, and clocks may still be rising.
  // (hybrid only where it splits the batch into two non-empty parts)
  std::vector<std::pair<int, int>> pairs;
  for (int d = 0; d < (h->nrep > 1 ? 3 : 1); ++d)
    for (int v = 0; v < kTileVariants; ++v)
      if (d != CPM_DISPATCH_HYBRID || (h->cfg[v].hyb_ng > 0 && h->cfg[v].hyb_ng < h->nrep))
        pairs.emplace_back(v, d);
  // A lattice that one thread-block cluster can hold is also tried in the
  // cluster sweep (every one of its tile heights), unless the caller chose
  // the parity-split sweep.
  const int row_fill = h->fill == CPM_FILL_CLUSTER ? (h->tma_ok ? CPM_FILL_TMA : CPM_FILL_VECTOR)
                                                   : h->fill;
  const bool try_cluster = h->cluster_ok && h->fill != CPM_FILL_PARITY;
  if (try_cluster)
    for (int v = 0; v < kTileVariants; ++v) pairs.emplace_back(v, -1);
  int best_fill = row_fill;
  const int npairs = (int)pairs.size();
  for (int i = 0; i < 3 * npairs && e == cudaSuccess; ++i) {
    const int v = pairs[i % npairs].first;
    const bool cl = pairs[i % npairs].second < 0;
    const int d = cl ? CPM_DISPATCH_GRID : pairs[i % npairs].second;
    h->fill = cl ? CPM_FILL_CLUSTER : row_fill;
    SweepArgs a = sweep_args(h, v, d);
    a.tick0 = tick;
    a.mcs = probe_mcs;
    e = copy(false);
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], h->stream);
    int nl = 0;
    if (e == cudaSuccess) e = enqueue_sweep(h, v, d, a, any_perim, false, &nl);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], h->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
    h->launches += nl;
    if (e == cudaSuccess && (best < 0.0f || ms < best)) {
      best = ms;
      best_v = v;
      best_d = d;
      best_fill = h->fill;
    }
  }
  h->fill = best_fill;
  if (e == cudaSuccess) e = copy(false);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(save);
  if (ev[0]) cudaEventDestroy(ev[0]);
  if (ev[1]) cudaEventDestroy(ev[1]);
  if (e != cudaSuccess) return h->cuda_fail(e, "autotune");
  uint32_t w = 0;
  if (int rc = read_error_word(h, &w)) return rc;
  if (w) return h->fail(CPM_ERR_TIMEOUT, "autotune: %s", describe_errors(w).c_str());
  h->variant = best_v;
  h->dispatch = best_d;
  h->tick = tick;
  if (chosen) *chosen = best_v;
  if (ms_per_mcs) *ms_per_mcs = best / (float)probe_mcs;
  return CPM_OK;
}

static_assert(sizeof(cpm_score_spec) == sizeof(ScoreSpec), "score spec layout");
static_assert(CPM_SCORE_MAX == kScoreMax, "score width");

int cpm_run_scores(cpm_handle* h, int mcs, float* d_scores, uint64_t score_base,
                   int score_len, const cpm_score_spec* spec) {
  CPM_BIND(h);
  if (h->ndim != 2) return h->fail(CPM_ERR_UNSUPPORTED, "scores are computed for 2D engines");
  if (mcs < 0 || !d_scores || !spec || score_len < 0)
    return h->fail(CPM_ERR_INVALID, "cpm_run_scores: bad arguments");
  if (!h->pushed) return h->fail(CPM_ERR_STATE, "run before a successful push_to_gpu()");
  ScoreSpec sp;
  std::memcpy(&sp, spec, sizeof sp);
  if (sp.n_pairs < 0 || sp.n_pairs > kScorePairsMax ||
      sp.n_pairs + (sp.lambda_area ? 1 : 0) + (sp.lambda_perim ? 1 : 0) +
              (sp.temperature ? 1 : 0) > kScoreMax)
    return h->fail(CPM_ERR_INVALID, "cpm_run_scores: too many score parameters");
  for (int k = 0; k < sp.n_pairs; ++k)
    if (sp.pair_a[k] < 0 || sp.pair_a[k] >= kScoreTypes || sp.pair_b[k] < 0 ||
        sp.pair_b[k] >= kScoreTypes)
      return h->fail(CPM_ERR_INVALID, "cpm_run_scores: score types must be < %d", kScoreTypes);
  if (mcs == 0) return CPM_OK;
  if (int rc = upload_params(h)) return rc;
  if (h->act_active || h->persist_active)
    return h->fail(CPM_ERR_UNSUPPORTED, "cpm_run_scores: scores of runs with the act or "
                                        "persistence term are not supported");
  SweepArgs a = sweep_args(h, h->variant, h->dispatch);
  a.scores = d_scores;
  a.score_base = score_base;
  a.score_len = score_len;
  a.score_spec = sp;
  int left = mcs;
  while (left > 0) {
    const int chunk = std::min(left, kMaxMcsPerLaunch);
    a.tick0 = h->tick;
    a.mcs = chunk;
    int nl = 0;
    CPM_CUDA(h, enqueue_sweep(h, h->variant, h->dispatch, a, any_perimeter(h), true, &nl));
    h->launches += nl;
    h->tick += (uint64_t)chunk;
    left -= chunk;
  }
  h->d_tick_stale = true;
  count_attempts(h, mcs);
  return CPM_OK;
}

int cpm_observe_heterotypic(cpm_handle* h, float* out_host) {
  CPM_BIND(h);
  if (h->ndim != 2) return h->fail(CPM_ERR_UNSUPPORTED, "2D engines only");
  if (!out_host) return h->fail(CPM_ERR_INVALID, "out_host is NULL");
  unsigned long long* counts = nullptr;
  CPM_CUDA(h, cudaMallocAsync((void**)&counts, sizeof(unsigned long long) * 2 * h->nrep,
                              h->stream));
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * 2 * h->nrep, h->stream);
  if (e == cudaSuccess)
    e = launch_observe_heterotypic(h->d_lat, h->d_reps, h->nrep, h->total_sites, counts,
                                   h->stream);
  h->launches += 1;
  std::vector<unsigned long long> c(2 * h->nrep);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c.data(), counts, sizeof(unsigned long long) * 2 * h->nrep,
                        cudaMemcpyDeviceToHost, h->stream);
  cudaFreeAsync(counts, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "cpm_observe_heterotypic");
  for (int r = 0; r < h->nrep; ++r)
    out_host[r] = c[2 * r] ? (float)((double)c[2 * r + 1] / (double)c[2 * r]) : 0.0f;
  return CPM_OK;
}

int cpm_seed_voronoi_r(cpm_handle* h, int r, int npoints, const double* points,
                       const uint32_t* values) {
  if (int rc = check_replica(h, r)) return rc;
  CPM_BIND(h);
  if (npoints < 1 || !points || !values)
    return h->fail(CPM_ERR_INVALID, "cpm_seed_voronoi_r: need npoints >= 1, points, values");
  const DevReplica& R = h->reps[r];
  const int nd = h->ndim;
  const int n[3] = {R.nx, R.ny, R.nz};
  for (int k = 0; k < npoints; ++k) {
    for (int a = 0; a < nd; ++a) {
      const double p = points[(size_t)k * nd + a];
      if (!(p >= 0.0 && p < (double)n[a]))
        return h->fail(CPM_ERR_INVALID, "cpm_seed_voronoi_r: point %d lies outside [0, n)", k);
    }
    const uint32_t v = values[k], id = v & 0xFFFFFFu, ty = v >> 24;
    if ((int)id > R.ncells || ty >= (uint32_t)kMaxTypes || (id == 0 && ty != 0))
      return h->fail(CPM_ERR_INVALID,
                     "cpm_seed_voronoi_r: value %d is not id <= ncells | type < 32 << 24 "
                     "(id 0 with type 0)", k);
  }
  // Bucket grid with about two points per bucket.
  VoronoiGrid vg;
  vg.ndim = nd;
  const double sites = (double)n[0] * n[1] * n[2];
  const double side = std::pow(2.0 * sites / npoints, 1.0 / nd);
  long long G = 1;
  double wmin = 1e300;
  vg.rmax = 0;
  for (int a = 0; a < 3; ++a) {
    vg.n[a] = n[a];
    int g = a < nd ? (int)std::lround((double)n[a] / side) : 1;
    g = std::max(1, std::min(g, n[a]));
    vg.g[a] = g;
    vg.w[a] = (double)n[a] / g;
    if (a < nd) wmin = std::min(wmin, vg.w[a]);
    vg.rmax = std::max(vg.rmax, g / 2 + 1);
    G *= g;
  }
  vg.lb_scale = wmin;
  if (G > (1LL << 30))
    return h->fail(CPM_ERR_INVALID, "cpm_seed_voronoi_r: too many buckets");
  // Counting sort of the points by bucket (host; O(npoints)).
  std::vector<int> bucket_of(npoints), start(G + 1, 0);
  for (int k = 0; k < npoints; ++k) {
    long long b = 0;
    for (int a = nd - 1; a >= 0; --a) {
      int ba = (int)std::floor(points[(size_t)k * nd + a] / vg.w[a]);
      ba = std::max(0, std::min(ba, vg.g[a] - 1));
      b = b * vg.g[a] + ba;
    }
    bucket_of[k] = (int)b;
    ++start[b + 1];
  }
  for (long long b = 0; b < G; ++b) start[b + 1] += start[b];
  // Work bound.  A site's search ends within about (d + 1) sqrt(ndim)
  // max(w) / min(w) + 1 rings, d the Chebyshev distance (in buckets, wrapped)
  // from its bucket to the nearest occupied one; d comes from a breadth-first
  // search over the bucket grid.  Point sets clustered so much that the
  // search would run for seconds are refused instead of launched.
  {
    std::vector<int> dist(G, -1), frontier, next;
    for (long long b = 0; b < G; ++b)
      if (start[b + 1] > start[b]) {
        dist[b] = 0;
        frontier.push_back((int)b);
      }
    for (int d = 1; !frontier.empty(); ++d) {
      next.clear();
      for (int b : frontier) {
        const int bx = b % vg.g[0], by = (b / vg.g[0]) % vg.g[1], bz = b / (vg.g[0] * vg.g[1]);
        for (int dz = (nd == 3 ? -1 : 0); dz <= (nd == 3 ? 1 : 0); ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const int x2 = (bx + dx + vg.g[0]) % vg.g[0], y2 = (by + dy + vg.g[1]) % vg.g[1],
                        z2 = (bz + dz + vg.g[2]) % vg.g[2];
              const int b2 = (z2 * vg.g[1] + y2) * vg.g[0] + x2;
              if (dist[b2] < 0) {
                dist[b2] = d;
                next.push_back(b2);
              }
            }
      }
      frontier.swap(next);
    }
    double wmax = 0.0;
    for (int a = 0; a < nd; ++a) wmax = std::max(wmax, vg.w[a]);
    const double per_bucket_sites = sites / (double)G;
    const double per_bucket_points = (double)npoints / (double)G;
    double work = 0.0;  // estimated distance evaluations
    for (long long b = 0; b < G; ++b) {
      const double rings =
          std::min((double)vg.rmax, (dist[b] + 1) * std::sqrt((double)nd) * wmax / wmin + 1.0);
      work += per_bucket_sites * std::pow(2.0 * rings + 1.0, nd) * std::max(1.0, per_bucket_points);
    }
    if (work > 5e11)
      return h->fail(CPM_ERR_INVALID,
                     "cpm_seed_voronoi_r: the points are too unevenly spread for the bucketed "
                     "search (about %.3g distance evaluations); spread them more evenly or "
                     "label the lattice on the host", work);
  }
  std::vector<double> pts((size_t)npoints * 3, 0.0);
  std::vector<int> idx(npoints), fill(start.begin(), start.end() - 1);
  for (int k = 0; k < npoints; ++k) {
    const int slot = fill[bucket_of[k]]++;
    for (int a = 0; a < nd; ++a) pts[(size_t)slot * 3 + a] = points[(size_t)k * nd + a];
    idx[slot] = k;
  }
  double* d_pts = nullptr;
  int *d_idx = nullptr, *d_start = nullptr;
  uint32_t* d_val = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d_pts, sizeof(double) * pts.size(), h->stream);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_idx, sizeof(int) * npoints, h->stream);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_val, sizeof(uint32_t) * npoints, h->stream);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_start, sizeof(int) * (G + 1), h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_pts, pts.data(), sizeof(double) * pts.size(), cudaMemcpyHostToDevice,
                        h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_idx, idx.data(), sizeof(int) * npoints, cudaMemcpyHostToDevice,
                        h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_val, values, sizeof(uint32_t) * npoints, cudaMemcpyHostToDevice,
                        h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_start, start.data(), sizeof(int) * (G + 1), cudaMemcpyHostToDevice,
                        h->stream);
  if (e == cudaSuccess)
    e = launch_voronoi(h->d_lat + R.lat_off, vg, d_pts, d_idx, d_val, d_start, h->stream);
  h->launches += 1;
  cudaFreeAsync(d_pts, h->stream);
  cudaFreeAsync(d_idx, h->stream);
  cudaFreeAsync(d_val, h->stream);
  cudaFreeAsync(d_start, h->stream);
  // the host vectors are read by the copies: wait before they go
  const cudaError_t e2 = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "cpm_seed_voronoi_r");
  if (e2 != cudaSuccess) return h->cuda_fail(e2, "cpm_seed_voronoi_r");
  h->pushed = false;  // the tables no longer describe the lattice
  return CPM_OK;
}

int cpm_observe_boundaries(cpm_handle* h, int ntypes, uint64_t* out_host) {
  CPM_BIND(h);
  if (ntypes < 1 || ntypes > kMaxTypes)
    return h->fail(CPM_ERR_INVALID, "ntypes must be in [1, %d]", kMaxTypes);
  if (!out_host) return h->fail(CPM_ERR_INVALID, "out_host is NULL");
  std::vector<long long> tile_start(h->nrep + 1, 0);
  for (int r = 0; r < h->nrep; ++r) {
    const DevReplica& R = h->reps[r];
    const long long sites = (long long)R.nx * R.ny * R.nz;
    tile_start[r + 1] = tile_start[r] + (sites + kBoundaryTile - 1) / kBoundaryTile;
  }
  const long long ntiles = tile_start[h->nrep];
  const size_t nc = (size_t)h->nrep * ntypes * ntypes;
  unsigned long long* counts = nullptr;
  long long* d_ts = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&counts, sizeof(unsigned long long) * nc, h->stream);
  if (e == cudaSuccess)
    e = cudaMallocAsync((void**)&d_ts, sizeof(long long) * (h->nrep + 1), h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * nc, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_ts, tile_start.data(), sizeof(long long) * (h->nrep + 1),
                        cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess)
    e = launch_observe_boundaries(h->ndim, h->d_lat, h->d_reps, h->nrep, d_ts, ntiles, ntypes,
                                  counts, h->stream);
  h->launches += 1;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out_host, counts, sizeof(unsigned long long) * nc,
                        cudaMemcpyDeviceToHost, h->stream);
  cudaFreeAsync(counts, h->stream);
  cudaFreeAsync(d_ts, h->stream);
  const cudaError_t e2 = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "cpm_observe_boundaries");
  if (e2 != cudaSuccess) return h->cuda_fail(e2, "cpm_observe_boundaries");
  return CPM_OK;
}

int cpm_lr_backward(const float* scores, const float* dl_do, const float* obs,
                    const int* checkpoints, int nrep, int len, int nparam, int ncheck,
                    const float* obs_total, int nrep_total, float* grad, void* stream) {
  if (!scores || !dl_do || !obs || !checkpoints || !grad || nrep < 1 || len < 0 ||
      nparam < 1 || nparam > kScoreMax || ncheck < 1 || ncheck > kMaxCheckpoints ||
      (obs_total && nrep_total < nrep)) {
    g_create_error = "cpm_lr_backward: bad arguments";
    return CPM_ERR_INVALID;
  }
  cudaError_t e = launch_lr_backward(scores, dl_do, obs, checkpoints, nrep, len, nparam,
                                     ncheck, obs_total, nrep_total, grad,
                                     (cudaStream_t)stream);
  if (e != cudaSuccess) {
    g_create_error = std::string("cpm_lr_backward: ") + cudaGetErrorString(e);
    return CPM_ERR_CUDA;
  }
  return CPM_OK;
}

int cpm_set_variant(cpm_handle* h, int variant) {
  if (!h) return CPM_ERR_INVALID;
  if (variant < 0 || variant >= kTileVariants)
    return h->fail(CPM_ERR_INVALID, "tile variant %d out of range [0, %d)", variant, kTileVariants);
  h->variant = variant;
  return CPM_OK;
}

int cpm_set_fill(cpm_handle* h, int fill) {
  if (!h) return CPM_ERR_INVALID;
  if (fill != CPM_FILL_PARITY && fill != CPM_FILL_VECTOR && fill != CPM_FILL_TMA &&
      fill != CPM_FILL_CLUSTER)
    return h->fail(CPM_ERR_INVALID, "fill %d is not parity (0), vector (1), tma (2) or "
                                    "cluster (3)", fill);
  if (fill == CPM_FILL_CLUSTER && !h->cluster_ok)
    return h->fail(CPM_ERR_UNSUPPORTED, "no thread-block cluster holds this lattice (one 2D "
                                        "lattice that fits row tiles and ~190 KB of rows per "
                                        "block of a 16- or 8-block cluster)");
  if (fill != CPM_FILL_PARITY && !h->row_ok)
    return h->fail(CPM_ERR_UNSUPPORTED, "row tiles need one lattice with nx a multiple of 4 "
                                        "and nx >= 72; in 2D ny >= 66, in 3D ny, nz >= 18");
  if (fill == CPM_FILL_TMA && !h->tma_ok)
    return h->fail(CPM_ERR_UNSUPPORTED, "the tensor maps of this lattice could not be encoded");
  h->fill = fill;
  return CPM_OK;
}

int cpm_get_fill(const cpm_handle* h, int* fill) {
  if (!h || !fill) return CPM_ERR_INVALID;
  *fill = h->fill;
  return CPM_OK;
}

int cpm_set_dispatch(cpm_handle* h, int dispatch) {
  if (!h) return CPM_ERR_INVALID;
  if (dispatch != CPM_DISPATCH_GRID && dispatch != CPM_DISPATCH_REPLICA &&
      dispatch != CPM_DISPATCH_HYBRID)
    return h->fail(CPM_ERR_INVALID, "dispatch %d is not grid (0), replica (1) or hybrid (2)",
                   dispatch);
  if (dispatch != CPM_DISPATCH_GRID && h->nrep < 2)
    return h->fail(CPM_ERR_UNSUPPORTED, "replica and hybrid dispatch need a batch of two or "
                                        "more replicas");
  h->dispatch = dispatch;
  return CPM_OK;
}

int cpm_synchronize(cpm_handle* h) {
  CPM_BIND(h);
  uint32_t w = 0;
  if (int rc = read_error_word(h, &w)) return rc;
  if (w) {
    CPM_CUDA(h, cudaMemsetAsync(h->d_ctl + kCtlErr, 0, sizeof(uint32_t), h->stream));
    CPM_CUDA(h, cudaStreamSynchronize(h->stream));
    h->pushed = false;  // the lattice and tables may disagree now
    return h->fail((w & kErrTimeout) ? CPM_ERR_TIMEOUT : CPM_ERR_INVALID,
                   "sweep failed: %s", describe_errors(w).c_str());
  }
  return CPM_OK;
}

int cpm_set_stream(cpm_handle* h, void* stream) {
  CPM_BIND(h);
  cudaStream_t next = stream ? (cudaStream_t)stream : h->own_stream;
  if (next != h->stream) {
    // Work already queued on the old stream must finish before the new one
    // touches the same buffers.
    CPM_CUDA(h, cudaStreamSynchronize(h->stream));
    h->stream = next;
  }
  return CPM_OK;
}

int cpm_set_seed(cpm_handle* h, uint64_t seed, uint32_t stream_id) {
  if (!h) return CPM_ERR_INVALID;
  h->seed = seed;
  h->stream_id = stream_id;
  return CPM_OK;
}

int cpm_get_tick(const cpm_handle* h, uint64_t* tick) {
  if (!h || !tick) return CPM_ERR_INVALID;
  *tick = h->tick;
  return CPM_OK;
}

int cpm_set_tick(cpm_handle* h, uint64_t tick) {
  if (!h) return CPM_ERR_INVALID;
  h->tick = tick;
  h->d_tick_stale = true;
  return CPM_OK;
}

int cpm_get_tables_r(cpm_handle* h, int r, int32_t* area, int32_t* perimeter,
                     int64_t* centroid_sums) {
  if (int rc = check_replica(h, r)) return rc;
  CPM_BIND(h);
  const DevReplica& R = h->reps[r];
  const long long n1 = (long long)R.ncells + 1;
  if (area || perimeter) {
    std::vector<unsigned long long> ap(n1);
    CPM_CUDA(h, cudaMemcpyAsync(ap.data(), h->d_ap[0] + R.cell_off,
                                sizeof(unsigned long long) * n1, cudaMemcpyDeviceToHost,
                                h->stream));
    CPM_CUDA(h, cudaStreamSynchronize(h->stream));
    for (long long c = 0; c < n1; ++c) {
      if (area) area[c] = unpack_area(ap[c]);
      if (perimeter) perimeter[c] = unpack_perim(ap[c]);
    }
  }
  if (centroid_sums) {
    CPM_CUDA(h, cudaMemcpyAsync(centroid_sums, h->d_cs[0] + R.cell_off * h->ndim,
                                sizeof(long long) * n1 * h->ndim,
                                cudaMemcpyDeviceToHost, h->stream));
    CPM_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return CPM_OK;
}

int cpm_get_centroids(cpm_handle* h, double* out, int capacity, int* n_out) {
  CPM_BIND(h);
  const int n = h->added_cells;
  if (n_out) *n_out = n;
  if (!out || capacity <= 0 || n == 0) return CPM_OK;
  const DevReplica& R = h->reps[0];
  const int d = h->ndim;
  const int m = std::min(n, capacity);
  std::vector<unsigned long long> ap(m);
  std::vector<long long> cs((size_t)m * d);
  CPM_CUDA(h, cudaMemcpyAsync(ap.data(), h->d_ap[0] + R.cell_off + 1,
                              sizeof(unsigned long long) * m, cudaMemcpyDeviceToHost,
                              h->stream));
  CPM_CUDA(h, cudaMemcpyAsync(cs.data(), h->d_cs[0] + (R.cell_off + 1) * d,
                              sizeof(long long) * m * d, cudaMemcpyDeviceToHost, h->stream));
  CPM_CUDA(h, cudaStreamSynchronize(h->stream));
  const int dims[3] = {R.nx, R.ny, R.nz};
  for (int c = 0; c < m; ++c)
    for (int k = 0; k < d; ++k) {
      double v = (double)cs[(size_t)c * d + k] / (double)unpack_area(ap[c]);
      if (std::isfinite(v)) v -= dims[k] * std::floor(v / dims[k]);
      out[(size_t)c * d + k] = v;
    }
  return CPM_OK;
}

int cpm_get_counters_r(cpm_handle* h, int r, cpm_counters* out) {
  if (!out || !h) return CPM_ERR_INVALID;
  if (r < -1 || r >= h->nrep)
    return h->fail(CPM_ERR_INVALID, "replica %d out of range", r);
  CPM_BIND(h);
  std::vector<unsigned long long> c(2 * h->nrep);
  CPM_CUDA(h, cudaMemcpyAsync(c.data(), h->d_counters, sizeof(unsigned long long) * 2 * h->nrep,
                              cudaMemcpyDeviceToHost, h->stream));
  CPM_CUDA(h, cudaStreamSynchronize(h->stream));
  out->attempts = out->evaluated = out->accepted = 0;
  for (int q = 0; q < h->nrep; ++q) {
    if (r >= 0 && q != r) continue;
    out->attempts += h->attempts[q];
    out->evaluated += c[2 * q];
    out->accepted += c[2 * q + 1];
  }
  return CPM_OK;
}

int cpm_get_counters(cpm_handle* h, cpm_counters* out) {
  return cpm_get_counters_r(h, -1, out);
}

int cpm_reset_counters(cpm_handle* h) {
  CPM_BIND(h);
  CPM_CUDA(h, cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * 2 * h->nrep,
                              h->stream));
  std::fill(h->attempts.begin(), h->attempts.end(), 0ull);
  return CPM_OK;
}

int cpm_info(const cpm_handle* h, int* n_replicas, int* dimensionality,
             int* sweep_grid, uint64_t* kernel_launches) {
  if (!h) return CPM_ERR_INVALID;
  if (n_replicas) *n_replicas = h->nrep;
  if (dimensionality) *dimensionality = h->ndim;
  if (sweep_grid) *sweep_grid = grid_of(h, h->variant, h->dispatch);
  if (kernel_launches) *kernel_launches = h->launches;
  return CPM_OK;
}

int cpm_sweep_config(const cpm_handle* h, int* variant, int* tile_x, int* tile_y,
                     int* tile_z, int* warps_per_block, int* grid, int* dispatch) {
  if (!h) return CPM_ERR_INVALID;
  const cpm_handle::Config& c = h->cfg[h->variant];
  if (variant) *variant = h->variant;
  if (tile_x) *tile_x = c.shape.cx;
  if (tile_y) *tile_y = c.shape.cy;
  if (tile_z) *tile_z = c.shape.cz;
  if (warps_per_block) *warps_per_block = c.shape.warps;
  if (grid) *grid = grid_of(h, h->variant, h->dispatch);
  if (dispatch) *dispatch = h->dispatch;
  if (h->fill == CPM_FILL_CLUSTER) {  // one cluster, its own tile heights
    if (tile_y) *tile_y = cluster_tile_rows(h->variant);
    if (tile_z) *tile_z = 1;
    if (grid) *grid = h->cl_G;
  }
  return CPM_OK;
}

int cpm_debug_barrier_timeout(uint64_t timeout_ns, int* status) {
  if (!status) return CPM_ERR_INVALID;
  *status = 0;
  uint32_t* ctl = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&ctl, sizeof(uint32_t) * kCtlWords);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * kCtlWords, s);
  if (e == cudaSuccess) e = launch_barrier_probe(ctl, timeout_ns, s);
  uint32_t w = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&w, ctl + kCtlErr, sizeof w, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(ctl);
  if (s) cudaStreamDestroy(s);
  if (e != cudaSuccess) {
    g_create_error = std::string("barrier probe failed: ") + cudaGetErrorString(e);
    return CPM_ERR_CUDA;
  }
  *status = (w & kErrTimeout) ? CPM_ERR_TIMEOUT : CPM_OK;
  return CPM_OK;
}

}  // extern "C"
