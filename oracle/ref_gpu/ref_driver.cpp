// ref_driver.cpp — host driver of the reference's own CUDA kernels.
//
// TEST INFRASTRUCTURE ONLY: used by the statistical-parity tests and by
// bench.py to run and time shabaz/gpu-cpm's sweep on the same GPU.  The
// device code is the reference's, unchanged: oracle/ref_gpu/build.py
// compiles src/kernels.cu (which includes kernels2d.cu, kernels3d.cu and
// random.cu) with the reference's own nvcc flags (setup.py:79-86: fast math,
// maxrregcount 40) for sm_103a instead of sm_70 into oracle/_ref/*.cubin.
// This file replaces only the reference's host class Cpm, whose sources do
// not travel: it loads the cubin through the CUDA driver API and repeats
// the host steps of
//   Cpm::Cpm                  src/cpm.cu:176-261   (buffers)
//   Cpm::moveCellIdsToGpu     src/cpm.cu:541-597   (H2D, table init kernel)
//   Cpm::run                  src/cpm.cu:291-517   (argument block, grid
//                                                   D/tpb/ppt, cooperative
//                                                   launch per
//                                                   inner_iterations)
//   Cpm::retreiveCellIdsFromGpu src/cpm.cu:531-540
// The seed of a run is passed in (the reference draws it from
// std::random_device, src/cpm.cu:347-350) so that runs can be repeated.
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// Layout of the reference's __constant__ Settings (src/settings.h:4-31),
// restated field for field: the kernels read it by these offsets.
constexpr int kNumTypes = 20;
struct TypeSettings {
  double persistenceLambda;
  double persistenceDiffusion;
  int persistenceTime;
  double areaLambda;
  int areaTarget;
  double actLambda;
  int actMax;
  double perimeterLambda;
  int perimeterTarget;
  short adhesion[kNumTypes];
  short stickiness[kNumTypes];
  int fixed;
  double chemotaxis;
};
struct Settings {
  TypeSettings types[kNumTypes];
  int temperature;
};
static_assert(sizeof(TypeSettings) == 160, "reference TypeSettings layout");
static_assert(sizeof(Settings) == 3208, "reference Settings layout");

struct State {
  CUcontext ctx = nullptr;
  CUmodule mod = nullptr;
  CUdeviceptr settings_sym = 0;
  size_t settings_size = 0;
  Settings settings;
  int dim = 0, ndim = 2, ncells = 0;
  long long sites = 0;
  CUdeviceptr cellIds = 0, areas = 0, writeAreas = 0, circumferences = 0,
              centroids = 0, analytics = 0, acts = 0, field = 0;
  int mcs = 0;
  std::string err;
} g;

int fail(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  g.err = std::string(what) + ": " + (s ? s : "?");
  return (int)r ? (int)r : 1;
}

#define DRV(call)                          \
  do {                                     \
    CUresult r_ = (call);                  \
    if (r_ != CUDA_SUCCESS) return fail(#call, r_); \
  } while (0)

// Mangled name of copyAttempt<b0..b5> / copyAttempt3d<b0..b6>
// (src/kernels2d.cu:44-55, src/kernels3d.cu:49-61), Itanium ABI.
std::string kernel_name(int ndim, const int* toggles) {
  std::string s = ndim == 2 ? "_Z11copyAttemptI" : "_Z13copyAttempt3dI";
  const int n = ndim == 2 ? 6 : 7;
  for (int i = 0; i < n; ++i) s += toggles[i] ? "Lb1E" : "Lb0E";
  s += ndim == 2 ? "EvPjS0_S0_S0_PyiiS0_iS0_iiiiibbbbPdS2_ibii"
                 : "EvPjS0_S0_S0_PyiiS0_iS0_iiiiibbbbPdS2_ibiii";
  return s;
}

int upload_settings() {
  DRV(cuCtxSetCurrent(g.ctx));
  DRV(cuMemcpyHtoD(g.settings_sym, &g.settings, sizeof(Settings)));
  return 0;
}

void free_buffers() {
  CUdeviceptr* bufs[] = {&g.cellIds, &g.areas, &g.writeAreas, &g.circumferences,
                         &g.centroids, &g.analytics, &g.acts, &g.field};
  for (CUdeviceptr* b : bufs)
    if (*b) {
      cuMemFree(*b);
      *b = 0;
    }
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g.err.c_str(); }

// Load the reference cubin on device `device` (primary context).
int ref_open(const char* cubin_path, int device) {
  DRV(cuInit(0));
  CUdevice dev;
  DRV(cuDeviceGet(&dev, device));
  DRV(cuDevicePrimaryCtxRetain(&g.ctx, dev));
  DRV(cuCtxSetCurrent(g.ctx));
  if (g.mod) {
    cuModuleUnload(g.mod);
    g.mod = nullptr;
  }
  DRV(cuModuleLoad(&g.mod, cubin_path));
  DRV(cuModuleGetGlobal(&g.settings_sym, &g.settings_size, g.mod, "constantSettings"));
  if (g.settings_size != sizeof(Settings)) {
    g.err = "constantSettings size differs from the restated Settings layout";
    return 1;
  }
  return 0;
}

// Cpm::Cpm (src/cpm.cu:176-261) for the buffers the copy-attempt kernels use.
int ref_create(int dimension, int dimensionality, int ncells, int temperature) {
  DRV(cuCtxSetCurrent(g.ctx));
  free_buffers();
  g.dim = dimension;
  g.ndim = dimensionality;
  g.ncells = ncells;
  g.sites = dimensionality == 2 ? (long long)dimension * dimension
                                : (long long)dimension * dimension * dimension;
  g.mcs = 0;
  std::memset(&g.settings, 0, sizeof g.settings);
  g.settings.temperature = temperature;
  DRV(cuMemAlloc(&g.cellIds, 4 * g.sites));
  DRV(cuMemAlloc(&g.areas, 4 * (ncells + 1)));
  DRV(cuMemAlloc(&g.writeAreas, 4 * (ncells + 1)));
  DRV(cuMemAlloc(&g.circumferences, 4 * (ncells + 1)));
  DRV(cuMemAlloc(&g.centroids, 8 * dimensionality * (ncells + 1)));
  DRV(cuMemAlloc(&g.analytics, 16));
  DRV(cuMemAlloc(&g.acts, 16));
  return upload_settings();
}

// Cpm::setArea / setPerimeter / setAdhesion / setTemperature
// (src/cpm.cu:57-60,119-143).
int ref_set_area(int type, int target, double lambda) {
  g.settings.types[type].areaTarget = target;
  g.settings.types[type].areaLambda = lambda;
  return upload_settings();
}
int ref_set_perimeter(int type, int target, double lambda) {
  g.settings.types[type].perimeterTarget = target;
  g.settings.types[type].perimeterLambda = lambda;
  return upload_settings();
}
int ref_set_adhesion(int type, int other, int J) {
  g.settings.types[type].adhesion[other] = (short)J;
  g.settings.types[other].adhesion[type] = (short)J;
  return upload_settings();
}
int ref_set_stickiness(int type, int other, int S) {  // Cpm::setStickiness, src/cpm.cu:145-148
  g.settings.types[type].stickiness[other] = (short)S;
  return upload_settings();
}
int ref_set_chemotaxis(int type, double lambda) {  // Cpm::setChemotaxis, src/cpm.cu:155-158
  g.settings.types[type].chemotaxis = lambda;
  return upload_settings();
}
// The field Cpm::moveCellIdsToGpu copies along (src/cpm.cu:542-544): doubles,
// component-major [ndim][sites].
int ref_set_field(const double* host) {
  DRV(cuCtxSetCurrent(g.ctx));
  if (!g.field) DRV(cuMemAlloc(&g.field, 8 * g.ndim * g.sites));
  DRV(cuMemcpyHtoD(g.field, host, 8 * g.ndim * g.sites));
  return 0;
}
int ref_set_fixed(int type, int fixed) {  // Cpm::setFixed, src/cpm.cu:150-153
  g.settings.types[type].fixed = fixed;
  return upload_settings();
}
int ref_set_temperature(int T) {
  g.settings.temperature = T;
  return upload_settings();
}

// Cpm::moveCellIdsToGpu (src/cpm.cu:541-597): lattice H2D, tables zeroed,
// calculateAreasAndCircumferences{,3d} with the reference's launch shape.
int ref_push(const uint32_t* lattice) {
  DRV(cuCtxSetCurrent(g.ctx));
  DRV(cuMemcpyHtoD(g.cellIds, lattice, 4 * g.sites));
  DRV(cuMemsetD8(g.areas, 0, 4 * (g.ncells + 1)));
  DRV(cuMemsetD8(g.writeAreas, 0, 4 * (g.ncells + 1)));
  DRV(cuMemsetD8(g.circumferences, 0, 4 * (g.ncells + 1)));
  DRV(cuMemsetD8(g.centroids, 0, 8 * g.ndim * (g.ncells + 1)));
  CUfunction f;
  DRV(cuModuleGetFunction(&f, g.mod, g.ndim == 2 ? "_Z31calculateAreasAndCircumferencesPjS_S_S_Pyi"
                                                : "_Z33calculateAreasAndCircumferences3dPjS_S_S_Pyi"));
  void* args[] = {&g.cellIds, &g.areas, &g.writeAreas, &g.circumferences, &g.centroids, &g.dim};
  const int tpb = g.dim > 1024 ? 1024 : g.dim;
  const int extra = g.dim / 1024 > 1 ? g.dim / 1024 : 1;
  if (g.ndim == 2)
    DRV(cuLaunchKernel(f, g.dim, extra, 1, tpb, 1, 1, 0, 0, args, nullptr));
  else
    DRV(cuLaunchKernel(f, g.dim, g.dim, extra, tpb, 1, 1, 0, 0, args, nullptr));
  DRV(cuCtxSynchronize());
  return 0;
}

// Cpm::run (src/cpm.cu:291-517), cooperative path.  `perimeter` and `fixed`
// select the toggle variants as partial_dispatch=1 would (any perimeter
// lambda != 0, any fixed type, src/cpm.cu:308-320); act, persistence and
// chemotaxis toggles are off.
int ref_run(int cell_sync, int block_sync, int global_sync, int threads_per_block,
            int positions_per_thread, int positions_per_checkerboard,
            int updates_per_checkerboard_switch, int updates_per_barrier, int iterations,
            int inner_iterations, int shared, int perimeter, int centroid_tracking,
            int seed, int fixed, int chemotaxis) {
  DRV(cuCtxSetCurrent(g.ctx));
  int toggles[7] = {shared ? 1 : 0, 0, perimeter ? 1 : 0, 0, chemotaxis ? 1 : 0,
                    fixed ? 1 : 0, centroid_tracking ? 1 : 0};
  CUfunction f;
  const std::string name = kernel_name(g.ndim, toggles);
  DRV(cuModuleGetFunction(&f, g.mod, name.c_str()));
  int sharedDim = g.ndim == 2 ? 64 : 32;
  CUdeviceptr field = g.field, prefDirs = 0;
  bool bsync = block_sync, gsync = global_sync, csync = cell_sync, inside = false;
  bool globalCheckerboard = false;
  int gX = 0, gY = 0, gZ = 0;
  int inner = inner_iterations, ppt = positions_per_thread, ppc = positions_per_checkerboard,
      upcs = updates_per_checkerboard_switch, upb = updates_per_barrier;
  const int blocks = g.dim / threads_per_block / positions_per_thread;
  const unsigned smem = shared ? (g.ndim == 2 ? 64 * 64 * 4 : 32 * 32 * 32 * 4) : 0;
  for (int m = 0; m < iterations / inner_iterations; ++m) {
    void* args[26] = {&g.cellIds, &g.areas, &g.writeAreas, &g.circumferences,
                      &g.centroids, &g.dim, &seed, &g.acts, &g.mcs, &g.analytics,
                      &inner, &ppt, &ppc, &upcs, &upb, &bsync, &gsync, &csync,
                      &inside, &field, &prefDirs, &sharedDim, &globalCheckerboard,
                      &gX, &gY, &gZ};
    if (g.ndim == 2)
      DRV(cuLaunchCooperativeKernel(f, blocks, blocks, 1, threads_per_block,
                                    threads_per_block, 1, smem, 0, args));
    else
      DRV(cuLaunchCooperativeKernel(f, blocks, blocks, blocks, threads_per_block,
                                    threads_per_block, threads_per_block, smem, 0, args));
    g.mcs += inner_iterations;
  }
  return 0;
}

int ref_synchronize() {
  DRV(cuCtxSetCurrent(g.ctx));
  DRV(cuCtxSynchronize());
  return 0;
}

int ref_pull(uint32_t* lattice) {
  DRV(cuCtxSetCurrent(g.ctx));
  DRV(cuMemcpyDtoH(lattice, g.cellIds, 4 * g.sites));
  return 0;
}

int ref_tables(uint32_t* areas, uint32_t* circumferences) {
  DRV(cuCtxSetCurrent(g.ctx));
  if (areas) DRV(cuMemcpyDtoH(areas, g.areas, 4 * (g.ncells + 1)));
  if (circumferences) DRV(cuMemcpyDtoH(circumferences, g.circumferences, 4 * (g.ncells + 1)));
  return 0;
}

// Largest cooperative grid (blocks per SM x SMs) of a kernel variant.
int ref_max_coop_blocks(int threads_per_block, int shared, int perimeter, int* out) {
  DRV(cuCtxSetCurrent(g.ctx));
  int toggles[7] = {shared ? 1 : 0, 0, perimeter ? 1 : 0, 0, 0, 0, 0};
  CUfunction f;
  DRV(cuModuleGetFunction(&f, g.mod, kernel_name(g.ndim, toggles).c_str()));
  const int threads = g.ndim == 2 ? threads_per_block * threads_per_block
                                  : threads_per_block * threads_per_block * threads_per_block;
  const unsigned smem = shared ? (g.ndim == 2 ? 64 * 64 * 4 : 32 * 32 * 32 * 4) : 0;
  int per_sm = 0, sms = 0;
  DRV(cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, threads, smem));
  CUdevice dev;
  DRV(cuCtxGetDevice(&dev));
  DRV(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev));
  *out = per_sm * sms;
  return 0;
}

}  // extern "C"
