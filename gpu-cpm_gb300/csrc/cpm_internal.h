// cpm_internal.h — structures shared by the host engine (cpm_engine.cu) and
// the sm_103a kernels (cpm_kernels.cu).  Not part of the public C-ABI.
//
// Device memory layout of one engine (a batch of R replicas; a plain
// gpucpm.Cpm is a batch of one):
//   lat  : uint32  [sum_r sites_r]        replica r at reps[r].lat_off,
//                                         row-major (z*ny + y)*nx + x
//   ap   : int2    [sum_r (ncells_r+1)]   (area, perimeter), replica r's id
//                                         c at row reps[r].cell_off + c
//   cs   : int64   [rows * ndim]          exact centroid coordinate sums
//   dap, dcs                              deltas of the running phase
//   dflag: uint32  [rows]                 row is on the phase's dirty list
//   dlist: uint32  [2 * rows]             two alternating dirty lists
//   ctl  : uint32  [8]                    barrier counter, 2 dirty counts,
//                                         sticky error bits
// The tables are small next to the lattice (4096^2 at 100 sites per cell:
// 67 MB of lattice, 4 MB of tables) and stay L2-resident through a run.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gpucpm {

constexpr int kMaxTypes = 32;
constexpr int kWarpsPerBlock = 8;
constexpr int kSweepThreads = 32 * kWarpsPerBlock;
constexpr int kInitThreads = 256;

// ctl[] word indices
constexpr int kCtlBarrier = 0;
constexpr int kCtlDirty0 = 1;  // dirty counts at kCtlDirty0 + (step & 1)
constexpr int kCtlErr = 3;
constexpr int kCtlWords = 8;

// error bits in ctl[kCtlErr]
constexpr int kErrTimeout = 1;      // a grid barrier waited too long
constexpr int kErrBadId = 2;        // site id above the replica's ncells
constexpr int kErrBadType = 4;      // type >= kMaxTypes
constexpr int kErrMediumType = 8;   // id 0 with a non-zero type
constexpr int kErrTypeConflict = 16;  // one id with two types

// Per-replica parameters, kept in global memory and staged into shared
// memory by each block for the replica it is working on.
struct DevParams {
  float J[kMaxTypes * kMaxTypes];  // J[own type][neighbour type]
  float lam_area[kMaxTypes];
  int tgt_area[kMaxTypes];
  float lam_perim[kMaxTypes];
  int tgt_perim[kMaxTypes];
  float temperature;
  int perim_on;  // any lam_perim != 0
  int pad[2];
};

struct DevReplica {
  int nx, ny, nz, ncells;
  long long lat_off;   // first site of the replica in lat[]
  long long cell_off;  // table row of the replica's id 0
};

// Arguments of the persistent sweep kernel.
struct SweepArgs {
  uint32_t* lat;
  int2* ap;
  long long* cs;
  int2* dap;
  long long* dcs;
  uint32_t* dflag;
  uint32_t* dlist;
  uint32_t* ctl;
  unsigned long long* counters;  // [nrep][2]: evaluated, accepted
  const DevReplica* reps;
  const DevParams* params;
  const int* task_prefix;  // [27][nrep + 1] block tasks per slot, prefix
  long long rows;          // total table rows (dirty list capacity)
  unsigned long long tick0;
  unsigned long long seed;
  int nrep;
  int mcs;
  unsigned int stream0;
  int nslot_active;
  int slots[27];
};

// Launchers (cpm_kernels.cu).  Each returns the cudaError_t of its launch.
cudaError_t launch_sweep(int ndim, bool perim, const SweepArgs& a, int grid,
                         cudaStream_t s);
int sweep_max_blocks_per_sm(int ndim, bool perim);
cudaError_t launch_barrier_probe(uint32_t* ctl, unsigned long long timeout_ns,
                                 cudaStream_t s);
cudaError_t launch_init(int ndim, const uint32_t* lat, const DevReplica* reps,
                        int nrep, long long total_sites, int2* ap,
                        long long* cs, unsigned long long* first, int* ctype,
                        uint32_t* ctl, cudaStream_t s);

}  // namespace gpucpm
