// cpm_internal.h — structures shared by the host engine (cpm_engine.cu) and
// the sm_103a kernels (cpm_kernels.cu).  Not part of the public C-ABI.
//
// Device memory layout of one engine (a batch of R replicas; a plain
// gpucpm.Cpm is a batch of one):
//   lat    : uint32 [sum_r sites_r]      replica r at reps[r].lat_off,
//                                        row-major (z*ny + y)*nx + x
//   ap[2]  : uint64 [rows]               packed (area | perimeter << 32) of
//                                        replica r's id c at row
//                                        reps[r].cell_off + c; two copies
//   cs[2]  : int64  [rows * ndim]        exact centroid coordinate sums,
//                                        two copies
//   dap[2], dcs[2]                       deltas of one phase (two phases in
//                                        flight alternate)
//   dlist  : uint32 [grid * 2 * list_cap] two dirty lists per sweep block:
//                                        rows changed in a phase (a row may
//                                        appear more than once)
//   ctl    : uint32 [64]                 barrier counter / release flag,
//                                        replica queue, sticky error bits
//   (optional) field (chemotaxis, float), act stamps (uint32 per site),
//   prefdir [rows][3] and the persistence ring [history][rows][3] (double)
// Table double buffering: phase k reads copy k % 2 and adds its deltas both
// into the other copy and into dap/dcs[k % 2]; phase k + 1 replays those
// deltas into copy k % 2, which missed them (each delta is taken with an
// exchange, so a row listed twice is replayed once).  So every phase reads
// tables as they stood when it began, with one grid barrier per phase.  The
// tables are
// small next to the lattice (4096^2 at 100 sites per cell: 67 MB of lattice,
// 4 MB per table copy) and stay L2-resident through a run.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gpucpm {

constexpr int kMaxTypes = 32;
// Warps per sweep block (one block per SM): 24 at 80 registers in 2D; 20 at
// 96 registers in 3D and in score launches, whose attempts would spill at 80.
constexpr int kMaxSweepWarps = 24;
constexpr int kMaxSweepWarps3d = 20;
template <int NDIM, bool SCORE = false>
constexpr int max_sweep_warps() {
  return (NDIM == 3 || SCORE) ? kMaxSweepWarps3d : kMaxSweepWarps;
}
constexpr int kSweepSmemMax = 227 * 1024;  // usable shared memory per block
constexpr int kInitThreads = 256;

// Warp tile: CX x CY x CZ targets of one slot, staged with their one-site
// halo in the warp's own shared memory.  Four compiled variants per
// dimensionality; the autotuner (cpm_autotune) picks one per engine.  The
// sweep's result does not depend on the variant.
//   2D  v0 32 x 6 (66 x 13 sites)   v1 32 x 8      v2 32 x 16     v3 32 x 1
//   3D  v0 32 x 2 x 2 (66 x 5 x 5)  v1 32 x 4 x 2  v2 32 x 4 x 4  v3 32 x 1 x 1
// v3 is for lattices too small to give every warp of the GPU a wide tile
// (256^2 has 85 tiles of 32 x 6 per slot): one row of targets per warp cuts
// the serial chain of a phase to one iteration of each pass.
constexpr int kTileVariants = 4;
template <int NDIM, int V>
struct TileGeom;
template <>
struct TileGeom<2, 0> {
  static constexpr int CX = 32, CY = 6, CZ = 1;
};
template <>
struct TileGeom<2, 1> {
  static constexpr int CX = 32, CY = 8, CZ = 1;
};
template <>
struct TileGeom<2, 2> {
  static constexpr int CX = 32, CY = 16, CZ = 1;
};
template <>
struct TileGeom<2, 3> {
  static constexpr int CX = 32, CY = 1, CZ = 1;
};
template <>
struct TileGeom<3, 0> {
  static constexpr int CX = 32, CY = 2, CZ = 2;
};
template <>
struct TileGeom<3, 1> {
  static constexpr int CX = 32, CY = 4, CZ = 2;
};
template <>
struct TileGeom<3, 2> {
  static constexpr int CX = 32, CY = 4, CZ = 4;
};
template <>
struct TileGeom<3, 3> {
  static constexpr int CX = 32, CY = 1, CZ = 1;
};

// Launch shape of one sweep configuration.
struct SweepShape {
  int variant;      // tile variant
  int cx, cy, cz;   // its tile extent in targets
  int warps;        // warps per block (tiles in flight per block)
  size_t smem;      // dynamic shared memory per block
};
SweepShape sweep_shape(int ndim, int variant, bool scores = false);

// ctl[] word indices (the barrier counter has a 128-byte line of its own)
constexpr int kCtlBarrier = 0;
constexpr int kCtlQueue = 40;  // next replica to claim (replica dispatch)
constexpr int kCtlErr = 48;  // words [0, kCtlErr) are zeroed before a launch
constexpr int kCtlWords = 64;

// error bits in ctl[kCtlErr]
constexpr int kErrTimeout = 1;      // a grid barrier waited too long
constexpr int kErrBadId = 2;        // site id above the replica's ncells
constexpr int kErrBadType = 4;      // type >= kMaxTypes
constexpr int kErrMediumType = 8;   // id 0 with a non-zero type
constexpr int kErrTypeConflict = 16;  // one id with two types
constexpr int kErrListFull = 32;      // a dirty list would overflow (not written)

// Per-replica parameters, kept in global memory (read through the
// read-only cache; a replica's few hundred used bytes stay L1-resident).
struct DevParams {
  float J[kMaxTypes * kMaxTypes];      // J[own type][neighbour type]
  // stickiness S[own type][neighbour type]: added to the adhesion of the
  // configuration before the copy only (src/kernels2d.cu:399-400)
  float stick[kMaxTypes * kMaxTypes];
  float lam_area[kMaxTypes];
  int tgt_area[kMaxTypes];
  float lam_perim[kMaxTypes];
  int tgt_perim[kMaxTypes];
  float temperature;
  int perim_on;         // any lam_perim != 0
  unsigned fixed_mask;  // bit t: cells of type t never move (src/kernels2d.cu:280-290)
  int stick_on;         // any stickiness != 0
  // chemotaxis lambda per type: dH -= lambda (d . field at the source), d the
  // unit copy direction (src/kernels2d.cu:302-334, src/kernels3d.cu:275-324)
  float chemo[kMaxTypes];
  int chemo_on;         // any chemo != 0
  // act model (src/kernels2d.cu:312-473): lambda and max_act per type
  int act_on;           // any act_lambda != 0
  // persistence (3D, src/kernels3d.cu:327-343, src/kernels.cu:159-212):
  // lambda and diffusion per type
  int persist_on;       // any persist_lambda != 0
  int pad;
  float act_lambda[kMaxTypes];
  int act_max[kMaxTypes];
  float persist_lambda[kMaxTypes];
  float persist_diff[kMaxTypes];
  int persist_time[kMaxTypes];  // stored for get/set only (not read by any kernel)
};

struct DevReplica {
  int nx, ny, nz, ncells;
  long long lat_off;   // first site of the replica in lat[]
  long long cell_off;  // table row of the replica's id 0
  int pset;            // its parameter record in params[] (shared by replicas)
  int pad;
};

// (area, perimeter) packed in one 64-bit word: area in the low 32 bits (it
// never goes below zero), perimeter in the high 32 bits.  A signed 64-bit
// addition of pack_delta(da, dp) updates both fields exactly.
__host__ __device__ inline unsigned long long pack_delta(int da, int dp) {
  return (unsigned long long)((long long)dp * 4294967296LL + (long long)da);
}
__host__ __device__ inline int unpack_area(unsigned long long w) {
  return (int)(uint32_t)w;
}
__host__ __device__ inline int unpack_perim(unsigned long long w) {
  return (int)(uint32_t)(w >> 32);
}

// Likelihood-ratio scores: up to kScoreMax parameters per replica and MCS,
// in the order (J pairs..., lambda_area, lambda_perim, T).  J pair k is the
// symmetric adhesion of types (pair_a[k], pair_b[k]); only types <
// kScoreTypes enter the derivative.  lambda_area (lambda_perim) is one value
// shared by every cell type's area (perimeter) lambda, each type keeping its
// own target.
constexpr int kScoreMax = 8;
constexpr int kScorePairsMax = 6;
constexpr int kScoreRegs = kScorePairsMax + 3;  // pairs, lambda_area, lambda_perim, T
constexpr int kScoreTypes = 4;
constexpr int kMaxCheckpoints = 64;  // observation times of one backward
struct ScoreSpec {
  int n_pairs;
  int pair_a[kScorePairsMax];
  int pair_b[kScorePairsMax];
  int lambda_area;   // 1: include d/d lambda_area
  int lambda_perim;  // 1: include d/d lambda_perim
  int temperature;   // 1: include d/dT
};

// Arguments of the persistent sweep kernel.
struct SweepArgs {
  uint32_t* lat;
  unsigned long long* ap[2];
  long long* cs[2];
  unsigned long long* dap[2];
  long long* dcs[2];
  uint32_t* dlist;
  uint32_t* ctl;
  unsigned long long* counters;  // [nrep][2]: evaluated, accepted
  const DevReplica* reps;
  const DevParams* params;
  const int* task_prefix;  // [27][nrep + 1] warp tiles per slot, prefix
  long long list_cap;      // entries of one dirty list of one block
  // Dispatch: 0 = the tiles of every slot over all replicas go to all warps
  // of the grid, one grid barrier per phase; 1 = each block claims whole
  // replicas in rep_order and runs all their phases with block barriers.
  int block_local;
  const int* rep_order;  // replicas by decreasing site count (replica dispatch:
                         // the queue, queue_len entries)
  int queue_len;         // replica dispatch: replicas to claim
  // Grid dispatch over a subset of the replicas (hybrid runs): task_prefix
  // and nrep describe the subset, and rep_map[i] is subset member i's
  // replica (null: the subset is every replica, in order).
  const int* rep_map;
  // chemotaxis field, float: replica r's component k of site i at
  // field[ndim * lat_off + k * sites_r + i] (null when no field exists)
  const float* field;
  // Act model: act[i] = the MCS of the last copy into site i.  With act_on
  // (some record has an act lambda) every accepted copy is deferred: it goes
  // to the block's pending list (site, value) and is written, with its act
  // stamp, after the phase's barrier, so that an attempt's reads around its
  // source (other targets of the slot) see the phase's starting state.
  uint32_t* act;
  int act_on;
  // (3D persistence) preferred direction of each table row, [rows][3]
  const double* prefdir;
  unsigned long long* pend_site;
  uint32_t* pend_val;
  long long pend_cap;  // entries of one block's pending list
  // Monte Carlo time of the first MCS: tick0, or *tick_ptr when tick_ptr is
  // set (graph replays); in the latter case block 0 advances *tick_ptr by
  // mcs when the launch ends.
  unsigned long long* tick_ptr;
  int tick_advance;  // 0: leave *tick_ptr to a later launch of the same run
  unsigned long long tick0;
  // Score output (score launches only): scores[(r * score_len + tick -
  // score_base) * kScoreMax + k] receives replica r's summed score of
  // parameter k over the attempts of MCS `tick`.
  float* scores;
  unsigned long long score_base;
  int score_len;
  ScoreSpec score_spec;
  unsigned long long seed;
  int nrep;
  int mcs;
  unsigned int stream0;
  int nslot_active;
  int slots[27];
};

// Message returned by cpm_last_error(NULL) for calls without a handle.
void set_thread_error(const char* message);

// Launchers (cpm_kernels.cu).  Each returns the cudaError_t of its launch.
cudaError_t launch_sweep(int ndim, bool perim, int variant, const SweepArgs& a,
                         int grid, cudaStream_t s, bool scores = false);
// The row-tile sweep of one 2D lattice (cpm_sweep2d.cu): tmap points to the
// 128-byte CUtensorMap of the variant's box (72 x row_tile_rows(variant)
// words); use_tma = 0 stages every tile with vector loads.  At most
// warps_cap warps per block.
cudaError_t launch_sweep2d(bool perim, int variant, const SweepArgs& a, const void* tmap,
                           int use_tma, int grid, int warps_cap, cudaStream_t s);
bool row_tiles_fit(int nx, int ny);
int row_tile_rows(int variant);
// Cluster mode of the 2D row-tile sweep (small single lattices): plan (G
// blocks of one cluster, H rows per block, dirty-list entries per block)
// and launch.  The plan is false where no cluster of that shape fits.
bool cluster_sweep_plan(int nx, int ny, int* G, int* H, long long* list_cap);
cudaError_t launch_sweep2d_cluster(bool perim, int variant, const SweepArgs& a, const void* tmap,
                                   int nx, int G, int H, cudaStream_t s);
// Target rows per tile of the cluster sweep's variants.
int cluster_tile_rows(int variant);
// The 3D row-tile sweep (cpm_sweep3d.cu): boxes of 72 x rows x planes words.
cudaError_t launch_sweep3d(bool perim, int variant, const SweepArgs& a, const void* tmap,
                           int use_tma, int grid, int warps_cap, cudaStream_t s);
bool box_tiles_fit(int nx, int ny, int nz);
void box_tile_extent(int variant, int* rows, int* planes);
int sweep_max_blocks_per_sm(int ndim, bool perim, int variant, bool scores = false);
// checkpoints: host array of ncheck (<= kMaxCheckpoints) MCS counts.
cudaError_t launch_lr_backward(const float* scores, const float* dl_do,
                               const float* obs, const int* checkpoints, int nrep,
                               int len, int nparam, int ncheck, const float* obs_total,
                               int nrep_total, float* grad, cudaStream_t s);
// 3D persistence: initial preferred directions, history fill (push), and
// the update after a run (slot: the history slot that receives this run).
cudaError_t launch_init_prefdir(double* prefdir, const DevReplica* reps, int nrep,
                                long long rows, unsigned long long seed, unsigned stream0,
                                cudaStream_t s);
cudaError_t launch_persist_fill(double* hist, int H, const unsigned long long* ap,
                                const long long* cs, const DevReplica* reps, int nrep,
                                long long rows, cudaStream_t s);
cudaError_t launch_persist_update(double* prefdir, double* hist, int H, int slot,
                                  const unsigned long long* ap, const long long* cs,
                                  const int* ctype, const DevParams* params,
                                  const DevReplica* reps, int nrep, long long rows,
                                  cudaStream_t s);
cudaError_t launch_observe_heterotypic(const uint32_t* lat, const DevReplica* reps,
                                       int nrep, long long total_sites,
                                       unsigned long long* counts, cudaStream_t s);
// Periodic Voronoi seeding of one lattice region (nx*ny*nz sites at `lat`):
// every site takes values[k] of its nearest point (min-image Euclidean
// distance in double, ties to the lowest k).  Points are binned in a
// g[0]*g[1]*g[2] bucket grid of widths w[] (bucket-major order: pts[k*3+a],
// idx[k] their original index, start[b]..start[b+1] bucket b's points).
struct VoronoiGrid {
  int n[3];         // lattice sides (n[2] = 1 in 2D)
  int g[3];         // buckets per axis
  double w[3];      // bucket widths n / g
  double lb_scale;  // min(w): ring r bounds unscanned points at r * min(w)
  int ndim;
  int rmax;         // rings to scan at most (covers every bucket)
};
cudaError_t launch_voronoi(uint32_t* lat, const VoronoiGrid& vg, const double* pts,
                           const int* idx, const uint32_t* values, const int* start,
                           cudaStream_t s);
// Boundary counts per replica and unordered type pair: Moore pairs (each
// once) of sites with different values, counts[r*T*T + a*T + b] for a <= b
// (types >= T are skipped).  tile_start: per replica the first of its tiles
// of kBoundaryTile sites (nrep+1 entries).
constexpr int kBoundaryTile = 4096;
cudaError_t launch_observe_boundaries(int ndim, const uint32_t* lat, const DevReplica* reps,
                                      int nrep, const long long* tile_start,
                                      long long ntiles, int T, unsigned long long* counts,
                                      cudaStream_t s);
cudaError_t launch_barrier_probe(uint32_t* ctl, unsigned long long timeout_ns,
                                 cudaStream_t s);
cudaError_t launch_init(int ndim, const uint32_t* lat, const DevReplica* reps,
                        int nrep, long long total_sites, unsigned long long* ap,
                        long long* cs, unsigned long long* first, int* ctype,
                        uint32_t* ctl, cudaStream_t s);

}  // namespace gpucpm
