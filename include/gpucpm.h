/*
 * gpucpm.h — C-ABI of the GB300 Cellular Potts engine (libgpucpm_gb300.so).
 *
 * The reference (shabaz/gpu-cpm) has no C-ABI: its boundary is the CPython
 * type `gpucpm.Cpm` (src/python_wrapper.cpp) wrapping the C++ class `Cpm`
 * (src/cpm.h:78-151, src/cpm.cu).  Every entry point below replaces one
 * method of that type / class; the citation names the reference code it
 * stands in for.  The Python module `gpucpm` shipped with this library binds
 * these symbols with ctypes and reproduces the reference's method set.
 *
 * Conventions
 *   - Plain C types only.  Every function returns an int status (CPM_OK = 0).
 *   - A handle is single-threaded: callers serialise calls on one handle.
 *   - Lattice sites hold `id | (type << 24)` (src/cpm.cu:163,171); id 0 with
 *     type 0 is the medium.  Layout is row-major: index = (z*ny + y)*nx + x.
 *   - Work is enqueued on the handle's own CUDA stream; cpm_run() returns
 *     before the sweep finishes (as Cpm::run does for 2D, src/cpm.cu:291).
 *     cpm_synchronize() waits and reports any device-side error.
 */
#ifndef GPUCPM_H_
#define GPUCPM_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define CPM_OK 0
#define CPM_ERR_INVALID 1     /* bad argument or bad lattice contents      */
#define CPM_ERR_CUDA 2        /* a CUDA runtime call failed                 */
#define CPM_ERR_ALLOC 3       /* host or device allocation failed          */
#define CPM_ERR_STATE 4       /* call out of order (e.g. run before push)  */
#define CPM_ERR_TIMEOUT 5     /* a bounded grid barrier gave up            */
#define CPM_ERR_UNSUPPORTED 6 /* feature outside this engine's scope       */

/* Largest number of cell types with parameters (the reference has 20,
 * src/settings.h:4; this engine accepts up to 32). */
#define CPM_MAX_TYPES 32

typedef struct cpm_handle cpm_handle;
typedef struct cpm_static_params cpm_static_params; /* defined below */

/* Counters of one run, summed over all replicas (see cpm_get_counters). */
typedef struct {
    uint64_t attempts;  /* copy attempts made (one per site per MCS)       */
    uint64_t evaluated; /* attempts whose source id differs from target's  */
    uint64_t accepted;  /* attempts that copied the source id              */
} cpm_counters;

/* ---- lifetime --------------------------------------------------------- */

/* Replaces Cpm::Cpm (src/cpm.cu:176-261) as reached through PyCpm_init
 * (src/python_wrapper.cpp:27-41).  Argument order follows the Python
 * constructor (dimension, dimensionality, number_of_cells, temperature).
 * `flags`: CPM_FLAG_FIELD allocates the chemotaxis field (has_field),
 * CPM_FLAG_ACT the act stamps (has_act).  Allocates the device lattice and
 * the cell tables for ids 0..number_of_cells on the current CUDA device. */
#define CPM_FLAG_FIELD 1
#define CPM_FLAG_ACT 2
int cpm_create(int dimension, int dimensionality, int number_of_cells,
               float temperature, int flags, cpm_handle** out);

/* Same as cpm_create for a non-cubic box nx*ny(*nz); nz must be 1 in 2D.
 * No counterpart in the reference (square/cubic only, src/cpm.cu:182-184). */
int cpm_create_box(int nx, int ny, int nz, int dimensionality,
                   int number_of_cells, float temperature, cpm_handle** out);

/* Batched engine: `n` independent replicas (2D or 3D) with their own box
 * sizes, cell counts and parameters, advanced together by one persistent
 * launch.  nx/ny/nz/ncells are arrays of length n.  Replica r is addressed
 * with the *_r entry points below.  No counterpart in the reference. */
int cpm_create_batch(int n, int dimensionality, const int* nx, const int* ny,
                     const int* nz, const int* ncells, cpm_handle** out);

/* Replaces Cpm::~Cpm (src/cpm.cu:263-285). */
int cpm_destroy(cpm_handle* h);

/* Select the CUDA device later cpm_create* calls of this thread allocate
 * on (the reference always uses device 0, src/cpm.cu:366).  A handle keeps
 * the device it was created on for all its later calls. */
int cpm_set_device(int device);

/* Human-readable description of the last error on this handle (or of the
 * last failed cpm_create* when h is NULL).  Never returns NULL. */
const char* cpm_last_error(const cpm_handle* h);

/* ---- parameters (src/cpm.cu:57-158, kwargs of PyCpm_setConstraints,
 *      src/python_wrapper.cpp:55-129).  Applied to every replica; the *_r
 *      forms address one replica of a batch. ----------------------------- */

/* Replaces Cpm::setTemperature (src/cpm.cu:57-60).  The reference stores an
 * int (src/settings.h:30); this engine uses float. */
int cpm_set_temperature(cpm_handle* h, float temperature);
int cpm_set_temperature_r(cpm_handle* h, int replica, float temperature);

/* Replaces Cpm::setArea (src/cpm.cu:125-129). */
int cpm_set_area(cpm_handle* h, int type, int target, float lambda);
int cpm_set_area_r(cpm_handle* h, int replica, int type, int target,
                   float lambda);

/* Replaces Cpm::setPerimeter (src/cpm.cu:119-123). */
int cpm_set_perimeter(cpm_handle* h, int type, int target, float lambda);
int cpm_set_perimeter_r(cpm_handle* h, int replica, int type, int target,
                        float lambda);

/* Replaces Cpm::setAdhesion (src/cpm.cu:137-143).  J is float here (the
 * reference stores short, src/settings.h:20).  symmetric != 0 also sets
 * J[other][type]. */
int cpm_set_adhesion(cpm_handle* h, int type, int other, float J,
                     int symmetric);
int cpm_set_adhesion_r(cpm_handle* h, int replica, int type, int other,
                       float J, int symmetric);

/* Replaces Cpm::setAct (src/cpm.cu:131-135).  An attempt adds
 * -lambda / max_act * (A_source - A_target) to dH (src/kernels2d.cu:312-473,
 * src/kernels3d.cu:301-470), lambda and max_act of the target type (of the
 * source type for a medium target).  A_site is the geometric mean of
 * max(max_act + act - mcs, 0) over the site and its neighbours of the same
 * cell (0 for the medium), act being the MCS of the last copy into a site;
 * here computed as exp2 of the mean log2 with this library's own FP32 log2 /
 * exp2.  Copies of runs with an act lambda are written at the end of their
 * phase, so that every attempt reads the phase's starting state; such runs
 * use tile variant 0 and cannot accumulate scores. */
int cpm_set_act(cpm_handle* h, int type, int max_act, float lambda);
int cpm_set_act_r(cpm_handle* h, int replica, int type, int max_act, float lambda);

/* Replaces Cpm::getActData (src/cpm.cu:523-525) behind get_act_state
 * (src/python_wrapper.cpp:310-326): replica r's act stamps (the MCS of the
 * last copy into each site, row-major), allocated with zeros on the first
 * call (or at cpm_create with CPM_FLAG_ACT) and pushed / pulled with the
 * lattice.  cpm_has_act tells whether they exist. */
int cpm_host_act_r(cpm_handle* h, int replica, uint32_t** ptr, int64_t* nsites);
int cpm_has_act(const cpm_handle* h, int* has);

/* Replaces Cpm::setChemotaxis (src/cpm.cu:155-158): lambda of a type.  An
 * attempt adds -lambda * (d . F) to dH, with d the unit copy direction
 * (source to target) and F the field at the source site; lambda is the
 * source type's, or the target type's when the source is the medium
 * (src/kernels2d.cu:302-334, src/kernels3d.cu:275-324).  Needs a field.
 * As in the reference, d is the raw difference of the wrapped coordinates
 * in 2D (so it points the other way across the lattice seam) and the
 * nearest-image difference in 3D. */
int cpm_set_chemotaxis(cpm_handle* h, int type, float lambda);
int cpm_set_chemotaxis_r(cpm_handle* h, int replica, int type, float lambda);

/* Replaces Cpm::setPersistence (src/cpm.cu:112-116), 3D only as in the
 * reference (its 2D kernels have no such term).  An attempt adds
 * -lambda * (d . p) to dH, d the unit copy direction (nearest image) and p
 * the preferred direction of the source cell (of the target when the source
 * is the medium); lambda is the source type's (the target's when the source
 * is the medium), src/kernels3d.cu:327-343.  After every cpm_run /
 * cpm_run_graph call (one launch of the reference's run loop,
 * src/cpm.cu:486-510) each cell's mean coordinate goes into a ring of
 * `history` slots and p <- normalize(d' (1 - diffusion) + p diffusion), d'
 * the displacement since the oldest slot divided by its length before the
 * per-axis wrap (src/kernels.cu:159-212).  `time` is stored and read back
 * only: the reference uses it in a host update that its run loop no longer
 * calls (src/cpm.cu:599-648).  Preferred directions start uniform on the
 * sphere, drawn from (seed, stream id) on first use. */
int cpm_set_persistence(cpm_handle* h, int type, int time, float diffusion, float lambda);
int cpm_set_persistence_r(cpm_handle* h, int replica, int type, int time, float diffusion,
                          float lambda);

/* The reference's `history` constructor argument (src/python_wrapper.cpp:
 * 27-41): slots of the mean-coordinate ring, >= 1 (default 1, with which the
 * displacement is always zero and p never changes, as in the reference).
 * Changing it refills the ring from the current tables. */
int cpm_set_history(cpm_handle* h, int history);

/* Persistence state of replica r for checkpoints: prefdir[(ncells+1)*3] and
 * the ring history[history][(ncells+1)*3], oldest slot first (double).
 * Either pointer may be NULL.  The getter fails with CPM_ERR_STATE when the
 * engine has no persistence state yet (cpm_has_persistence); the setter
 * creates it on a pushed 3D engine. */
int cpm_get_persistence_r(cpm_handle* h, int replica, double* prefdir, double* history);
int cpm_set_persistence_state_r(cpm_handle* h, int replica, const double* prefdir,
                                const double* history);
int cpm_has_persistence(const cpm_handle* h, int* has, int* history);

/* Replaces Cpm::setFixed (src/cpm.cu:150-153).  Cells of a fixed type never
 * move: an attempt whose target belongs to one does nothing, and one whose
 * source belongs to one proposes the medium instead (src/kernels2d.cu:
 * 280-290, src/kernels3d.cu:251-261).  fixed != 0 sets, 0 clears. */
int cpm_set_fixed(cpm_handle* h, int type, int fixed);
int cpm_set_fixed_r(cpm_handle* h, int replica, int type, int fixed);

/* Replaces Cpm::setStickiness (src/cpm.cu:145-148): S[type][other], added
 * to the adhesion energy of the configuration before the copy only
 * (src/kernels2d.cu:399-400).  Not symmetric, as in the reference.  float
 * here (the reference stores short, src/settings.h:22). */
int cpm_set_stickiness(cpm_handle* h, int type, int other, float S);
int cpm_set_stickiness_r(cpm_handle* h, int replica, int type, int other,
                         float S);

/* ---- lattice ---------------------------------------------------------- */

/* Replaces Cpm::addCell (src/cpm.cu:160-174): the next id (1, 2, ...) of
 * `type` is written at (x, y[, z]) of the host lattice.  z is ignored in 2D.
 * Cells added this way are the ones cpm_get_centroids reports. */
int cpm_add_cell(cpm_handle* h, int type, int x, int y, int z);

/* Replaces Cpm::getCellIds (src/cpm.cu:519-521) behind get_state
 * (src/python_wrapper.cpp:292-308): the host lattice buffer of replica 0
 * (pinned memory owned by the handle; valid until cpm_destroy). */
int cpm_host_lattice(cpm_handle* h, uint32_t** ptr, int64_t* nsites);
int cpm_host_lattice_r(cpm_handle* h, int replica, uint32_t** ptr,
                       int64_t* nsites);

/* Replaces Cpm::getField (src/cpm.cu:527-529) behind get_field
 * (src/python_wrapper.cpp:274-290): the host chemotaxis field of replica r,
 * `dimensionality` components of one value per site ([k][z][y][x] doubles,
 * component k = x, y, z), allocated with zeros on the first call.  Pushed
 * with the lattice (as float); the sweep never writes it. */
int cpm_host_field_r(cpm_handle* h, int replica, double** ptr, int64_t* nvalues);

/* Device lattice of a replica (row-major uint32), for zero-copy readers. */
int cpm_device_lattice_r(cpm_handle* h, int replica, uint32_t** dptr);

/* Replaces Cpm::moveCellIdsToGpu (src/cpm.cu:541-597): copies every host
 * lattice to the device and recomputes area, perimeter and centroid sums of
 * every cell.  Fails with CPM_ERR_INVALID (and leaves the tables unusable)
 * if a site holds an id above number_of_cells, a type >= CPM_MAX_TYPES, a
 * non-zero type on id 0, or one id with two types.  Synchronous. */
int cpm_push(cpm_handle* h);

/* Replaces Cpm::retreiveCellIdsFromGpu (src/cpm.cu:531-540): copies every
 * device lattice back into the host buffers.  Synchronous. */
int cpm_pull(cpm_handle* h);

/* ---- state I/O and resume (no counterpart in the reference, whose state
 *      lives only in H2D / D2H round trips, src/cpm.cu:531-597) ---------- */

/* cpm_push without the host copy: revalidates every device lattice and
 * recomputes the tables from it, for callers that changed the lattice in
 * place on the device (e.g. through a view of cpm_device_lattice_r).
 * Synchronous. */
int cpm_recount(cpm_handle* h);

/* Replace replica r's centroid sums (as cpm_get_tables_r returned them) on
 * the device.  Area and perimeter are exact functions of the lattice, which
 * push / recount recompute; centroid sums also record which periodic image
 * each site joined as, so an exact resume restores them after the push.
 * Needs a successful push.  Synchronous. */
int cpm_set_centroid_sums_r(cpm_handle* h, int replica, const int64_t* centroid_sums);

/* A replica's parameters as one record (the layout of cpm_static_params
 * below): read, write for one replica, or write for every replica. */
int cpm_get_params_r(const cpm_handle* h, int replica, cpm_static_params* out);
int cpm_set_params_r(cpm_handle* h, int replica, const cpm_static_params* in);
int cpm_set_params(cpm_handle* h, const cpm_static_params* in);

/* out[r] (n_replicas ints) = the parameter record replica r uses; replicas
 * with equal values share all parameters (so a checkpoint stores each
 * record once). */
int cpm_get_param_index(const cpm_handle* h, int* out);

/* The Philox key and stream id set by cpm_set_seed / the CUDA device the
 * handle lives on. */
int cpm_get_seed(const cpm_handle* h, uint64_t* seed, uint32_t* stream_id);
int cpm_get_device(const cpm_handle* h, int* device);

/* ---- sweeps ----------------------------------------------------------- */

/* Replaces Cpm::run (src/cpm.cu:291-517): `mcs` Monte Carlo steps of the
 * checkerboard Metropolis sweep on every replica.  One MCS makes one copy
 * attempt per lattice site.  Asynchronous; the launch geometry knobs of the
 * reference's run() have no meaning here (the engine sizes its own grid). */
int cpm_run(cpm_handle* h, int mcs);

/* Same as cpm_run as one CUDA-graph launch: the first call with a given
 * `mcs` (or after cpm_autotune / cpm_set_variant / cpm_set_dispatch /
 * cpm_set_stream) captures
 * the run (barrier reset + the persistent sweep) into a graph; every call
 * replays it.  The captured sweep reads its start time from device memory
 * and advances it, so replays continue the Monte Carlo time like cpm_run.
 * Needs a non-default stream (the handle's own stream qualifies).  No
 * counterpart in the reference.  1 <= mcs <= 65536. */
int cpm_run_graph(cpm_handle* h, int mcs);

/* Dispatch of a sweep launch over the replicas of a batch:
 *   CPM_DISPATCH_GRID     the tiles of a slot, over all replicas, go to all
 *                         warps of the grid; one grid barrier per phase
 *                         (one large lattice, or a few);
 *   CPM_DISPATCH_REPLICA  each block claims whole replicas, largest first,
 *                         and runs all their phases with block barriers, so
 *                         a replica's lattice and tables stay near one SM
 *                         (many small replicas).
 *   CPM_DISPATCH_HYBRID   two launches per run: GRID over the largest
 *                         replicas, then REPLICA over the others, as many
 *                         as make whole rounds of one replica per block
 *                         (512 equal replicas on 152 SMs: GRID over 56,
 *                         REPLICA over 456, instead of a last REPLICA round
 *                         that leaves 96 blocks idle).
 * Results do not depend on the dispatch.  A batch starts with REPLICA when
 * it has a replica for every block and none is much larger than a block's
 * share of the sites (HYBRID when they do not fill whole rounds), else
 * GRID. */
#define CPM_DISPATCH_GRID 0
#define CPM_DISPATCH_REPLICA 1
#define CPM_DISPATCH_HYBRID 2

/* Project autotuner: times `probe_mcs` MCS of every compiled tile variant
 * (warp tile shape and warps per block), under each dispatch for a batch
 * (grid, replica, and hybrid where it splits the batch into two parts),
 * three times each (the fastest run counts: a first launch also loads its
 * module; a GPU coming out of idle should be warmed up first),
 * on a saved copy of the current state, restores the state, and makes the
 * fastest pair the one later runs use.  The sweep's result does not depend
 * on either choice.  *chosen (may be NULL) receives the variant,
 * *ms_per_mcs (may be NULL) its time per MCS.  No counterpart in the
 * reference, whose geometry is passed per run() call
 * (src/python_wrapper.cpp:182-227). */
int cpm_autotune(cpm_handle* h, int probe_mcs, int* chosen, float* ms_per_mcs);

/* Select a tile variant (0 to 3) or a dispatch explicitly / describe the
 * current launch: warp tile extent in targets, warps per block, grid size
 * and dispatch. */
int cpm_set_variant(cpm_handle* h, int variant);
int cpm_set_dispatch(cpm_handle* h, int dispatch);
int cpm_sweep_config(const cpm_handle* h, int* variant, int* tile_x,
                     int* tile_y, int* tile_z, int* warps_per_block,
                     int* grid, int* dispatch);

/* How warp tiles reach shared memory in the sweep of one lattice.  No
 * counterpart in the reference (its tile load is src/kernels2d.cu:109-176).
 *   CPM_FILL_PARITY  the general sweep: scalar loads, even and odd columns
 *                    in separate halves of the tile
 *   CPM_FILL_VECTOR  row-major tiles from 16-byte vector loads
 *   CPM_FILL_TMA     row-major tiles, interior tiles copied by the tensor
 *                    memory accelerator (cp.async.bulk.tensor), tiles on the
 *                    periodic seam from vector loads
 *   CPM_FILL_CLUSTER (small 2D lattices) one thread-block cluster of 16 (or 8)
 *                    blocks holds the lattice in its shared memory, one
 *                    strip of rows per block with copies of its neighbours'
 *                    edge rows, for a whole run; tiles are read in place
 *                    and the phases end at a barrier inside the cluster.
 *                    cpm_autotune tries it wherever it fits and keeps it
 *                    when it is faster.
 * Row-major tiles need a single lattice with nx a multiple of 4 and
 * nx >= 72 (in 2D ny >= 66, in 3D ny >= 18 and nz >= 18); such lattices start
 * in CPM_FILL_TMA (CPM_FILL_VECTOR where the tensor maps cannot be encoded),
 * all others in CPM_FILL_PARITY.
 * The result does not depend on the fill: it selects the kernel only
 * (CPM_ERR_UNSUPPORTED for a fill the lattice cannot use). */
#define CPM_FILL_PARITY 0
#define CPM_FILL_VECTOR 1
#define CPM_FILL_TMA 2
#define CPM_FILL_CLUSTER 3
int cpm_set_fill(cpm_handle* h, int fill);
int cpm_get_fill(const cpm_handle* h, int* fill);

/* Replaces Cpm::synchronize (src/cpm.cu:653-655).  Waits for the handle's
 * stream and reports device-side errors (CPM_ERR_TIMEOUT, CPM_ERR_CUDA). */
int cpm_synchronize(cpm_handle* h);

/* Enqueue the handle's work on `stream` (a cudaStream_t of the same device,
 * owned by the caller, e.g. a torch.cuda.Stream) instead of its own stream;
 * NULL switches back to the handle's own stream.  The reference always uses
 * the legacy default stream. */
int cpm_set_stream(cpm_handle* h, void* stream);

/* Random stream: the sweep draws Philox4x32-10 numbers keyed by `seed` with
 * counter (site, phase, stream_id).  Replica r of a batch uses stream
 * stream_id + r.  Default seed 0, stream 0.  (The reference reseeds from
 * std::random_device on every run, src/cpm.cu:347-350.) */
int cpm_set_seed(cpm_handle* h, uint64_t seed, uint32_t stream_id);

/* Monte Carlo time: number of MCS run since creation (Cpm::_mcs,
 * src/cpm.cu:484).  Together with the lattice and the seed it is a complete
 * resume point. */
int cpm_get_tick(const cpm_handle* h, uint64_t* tick);
int cpm_set_tick(cpm_handle* h, uint64_t tick);

/* ---- readback --------------------------------------------------------- */

/* Replaces Cpm::get2dCentroids / get3dCentroids (src/cpm.cu:68-110): mean
 * coordinate of cells 1..n_added (the cells made by cpm_add_cell) of replica
 * 0, `dimensionality` doubles per cell, each in [0, side).  `out` holds
 * `capacity` cells; *n_out receives n_added.  Synchronous. */
int cpm_get_centroids(cpm_handle* h, double* out, int capacity, int* n_out);

/* Cell tables of one replica for ids 0..number_of_cells: area, perimeter
 * (number of (site, Moore neighbour) pairs with the site in the cell and the
 * neighbour not), and the exact int64 coordinate sums, `dimensionality` per
 * cell (periodic images chosen nearest the cell's running mean).  Any
 * pointer may be NULL.  Synchronous.  No counterpart in the reference. */
int cpm_get_tables_r(cpm_handle* h, int replica, int32_t* area,
                     int32_t* perimeter, int64_t* centroid_sums);

/* Attempt / evaluation / acceptance counts accumulated since the last
 * cpm_reset_counters (summed over replicas, or of one replica). */
int cpm_get_counters(cpm_handle* h, cpm_counters* out);
int cpm_get_counters_r(cpm_handle* h, int replica, cpm_counters* out);
int cpm_reset_counters(cpm_handle* h);

/* Engine information: number of replicas, dimensionality, CUDA grid size of
 * the sweep launch, and the number of kernel launches enqueued so far. */
int cpm_info(const cpm_handle* h, int* n_replicas, int* dimensionality,
             int* sweep_grid, uint64_t* kernel_launches);

/* ---- likelihood-ratio gradients (no counterpart in the reference) ------- */

/* Parameters the scores differentiate, in this order: J of symmetric type
 * pairs (pair_a[k], pair_b[k]) for k < n_pairs (types < 4); then, each if
 * enabled, one lambda_area shared by all cell types, one lambda_perim shared
 * by all cell types (every type keeps its own area / perimeter target), and
 * the temperature.  At most CPM_SCORE_MAX parameters. */
#define CPM_SCORE_MAX 8
typedef struct {
    int n_pairs;
    int pair_a[6];
    int pair_b[6];
    int lambda_area;
    int lambda_perim;
    int temperature;
} cpm_score_spec;

/* cpm_run that also accumulates, per replica and MCS, the likelihood-ratio
 * score sum_attempts d log P(decision | theta) / d theta of every attempt
 * with dH > 0 (P(accept) = exp(-dH/T)); attempts with dH <= 0 are accepted
 * with probability 1 and score 0.  The lattice evolves exactly as under
 * cpm_run.  d_scores (device, float) is [n_replicas][score_len][CPM_SCORE_MAX];
 * the MCS with tick t adds into row t - score_base (rows outside
 * [0, score_len) are skipped).  2D engines only.  Asynchronous. */
int cpm_run_scores(cpm_handle* h, int mcs, float* d_scores, uint64_t score_base,
                   int score_len, const cpm_score_spec* spec);

/* Sorting order parameter of every replica: the fraction of Moore neighbour
 * pairs of two different non-medium cells that join cells of different
 * types.  out_host receives n_replicas floats.  2D engines only.
 * Synchronous. */
int cpm_observe_heterotypic(cpm_handle* h, float* out_host);

/* No counterpart in the reference (its examples draw cell boundaries with
 * skimage on the host).  Boundary lengths of every replica's device lattice
 * by unordered type pair: out_host[r*ntypes*ntypes + a*ntypes + b], a <= b,
 * counts the Moore neighbour pairs (each pair once; 8 neighbours in 2D, 26
 * in 3D) whose two sites hold different values and have types a and b
 * (pairs with a type >= ntypes are skipped; entries with a > b stay 0).
 * The sum over 1 <= a <= b is the number of cell-cell contacts, over
 * 1 <= a < b the heterotypic ones (cpm_observe_heterotypic's ratio). */
int cpm_observe_boundaries(cpm_handle* h, int ntypes, uint64_t* out_host);

/* No counterpart in the reference (its examples paint squares on the host).
 * Fills replica r's DEVICE lattice with a periodic Voronoi tiling of
 * `npoints` points (host arrays): points[k*dimensionality + a] in [0, n_a)
 * (x first), values[k] = id | type << 24 given to the sites whose nearest
 * point (min-image Euclidean distance in double) is k, ties to the lowest
 * k, so the result is the brute-force answer bit for bit.  Points are
 * bucketed on the host and searched ring by ring on the device; point sets
 * clustered so much that the search would run for seconds are refused
 * (CPM_ERR_INVALID) before anything is launched.  The tables
 * are stale afterwards: cpm_recount (or cpm_pull, edit, cpm_push) must
 * come before the next run. */
int cpm_seed_voronoi_r(cpm_handle* h, int replica, int npoints, const double* points,
                       const uint32_t* values);

/* Backward of the likelihood-ratio estimator, on the GPU:
 *   grad[k] = sum_r sum_c dl_do[r][c] (obs[r][c] - b[r][c])
 *                     * sum_{t < checkpoints[c]} scores[r][t][k]
 * with the leave-one-out baseline b[r][c] = mean of obs[.][c] over the
 * other replicas (0 when R = 1).  For a loss L = mean_r f(obs[r]) this is
 * an unbiased estimate of dE[f]/dtheta.  When the replicas are sharded over
 * processes, obs_total (host, [ncheck]: sum of obs[.][c] over every shard)
 * and nrep_total (replicas of every shard) make the baseline global; NULL
 * and 0 use this launch's replicas only.  scores, dl_do, obs and
 * grad are device pointers ([R][len][CPM_SCORE_MAX], [R][ncheck], [R][ncheck],
 * [nparam]); checkpoints is a host array of ncheck (<= 64) MCS counts.
 * Enqueued on `stream` (NULL: default stream). */
int cpm_lr_backward(const float* scores, const float* dl_do, const float* obs,
                    const int* checkpoints, int nrep, int len, int nparam,
                    int ncheck, const float* obs_total, int nrep_total,
                    float* grad, void* stream);

/* ---- sweep without allocation ------------------------------------------ */

/* Size limits of cpm_sweep_static (its working memory is a fixed array). */
#define CPM_STATIC_MAX_SITES (1 << 18)
#define CPM_STATIC_MAX_CELLS 16383

/* One replica's parameters (cpm_get_params_r / cpm_set_params_r) and the
 * parameters of cpm_sweep_static, in the conventions of the setters above:
 * J[a * CPM_MAX_TYPES + b] is the adhesion a site of type a feels from a
 * neighbour of type b; index 0 of the per-type arrays is the medium. */
struct cpm_static_params {
    float J[CPM_MAX_TYPES * CPM_MAX_TYPES];
    float lambda_area[CPM_MAX_TYPES];
    int target_area[CPM_MAX_TYPES];
    float lambda_perimeter[CPM_MAX_TYPES];
    int target_perimeter[CPM_MAX_TYPES];
    float temperature;
    float stickiness[CPM_MAX_TYPES * CPM_MAX_TYPES]; /* as cpm_set_stickiness */
    int fixed[CPM_MAX_TYPES];                        /* as cpm_set_fixed */
    /* handle engines only: cpm_sweep_static refuses non-zero lambdas here */
    float chemotaxis[CPM_MAX_TYPES];                 /* as cpm_set_chemotaxis */
    float act_lambda[CPM_MAX_TYPES];                 /* as cpm_set_act */
    int act_max[CPM_MAX_TYPES];
    float persistence_lambda[CPM_MAX_TYPES];         /* as cpm_set_persistence */
    float persistence_diffusion[CPM_MAX_TYPES];
    int persistence_time[CPM_MAX_TYPES];
};

/* No counterpart in the reference.  Runs `mcs` Monte Carlo steps of the same
 * sweep as cpm_run on one lattice that lives entirely in caller-owned device
 * memory, and allocates nothing: no cudaMalloc, no cudaFree, no handle.  It
 * is meant for callers that cannot allocate device memory themselves: code
 * running inside a framework that owns the device memory pool, a pre-sized
 * real-time or embedded loop that must not allocate after start-up, or a
 * host that hands this library fixed buffers only.
 *
 * Buffers (device pointers, all in/out): lattice[nx*ny*nz] (id | type << 24,
 * row-major), area[n+1], perimeter[n+1], centroid_sums[(n+1)*dimensionality]
 * with n = number_of_cells.  With recount != 0 the tables are first
 * recomputed from the lattice (their input contents are ignored); with
 * recount == 0 they must describe the lattice, e.g. as left by an earlier
 * call.  Random stream and time as in cpm_set_seed / cpm_set_tick: the
 * result equals a handle's cpm_run from tick `tick` with the same seed and
 * stream id.
 *
 * Working memory is one fixed array compiled into the library (about 6.5 MB,
 * held on every GPU that loads the library until the process exits), which
 * bounds the sizes: nx*ny*nz <= CPM_STATIC_MAX_SITES and number_of_cells <=
 * CPM_STATIC_MAX_CELLS; larger requests fail with CPM_ERR_INVALID before any
 * GPU work.  Every shape within those limits fits the array's dirty-list
 * space, narrow ones (nx far below 64) included.  A non-finite temperature,
 * lambda, adhesion or stickiness fails with CPM_ERR_INVALID.  The call is
 * synchronous and cannot be captured into a CUDA graph: do not call it while
 * its stream, or a stream in global capture mode, is being captured.  The
 * first call on a device looks the array's address up on that device (make
 * that call before any graph capture on the device) and keeps it for the
 * life of the process; after cudaDeviceReset on that device the kept address is stale,
 * so do not call this entry point on a device the process has reset.  Every
 * call shares the one array: calls must not overlap on the GPU (two host
 * threads calling at once on different streams would race).  The call works
 * on `stream` (NULL: the default stream) and waits for that stream before it
 * returns, with the status of the sweep; counters_out, if not NULL,
 * receives {evaluated, accepted} of this call. */
int cpm_sweep_static(int dimensionality, int nx, int ny, int nz,
                     int number_of_cells, uint32_t* lattice, int32_t* area,
                     int32_t* perimeter, int64_t* centroid_sums, int recount,
                     const cpm_static_params* params, uint64_t seed,
                     uint32_t stream_id, uint64_t tick, int mcs, void* stream,
                     uint64_t* counters_out);

/* ---- diagnostics ------------------------------------------------------ */

/* Failure-detection self-test: launches a two-block cooperative kernel whose
 * grid barrier can never complete and whose wait limit is `timeout_ns`, and
 * stores in *status the status that limit produced (CPM_ERR_TIMEOUT when the
 * bounded wait ran out, as it must).  Touches no engine state.  No
 * counterpart in the reference, whose grid.sync() waits without a limit
 * (src/kernels2d.cu:175,193). */
int cpm_debug_barrier_timeout(uint64_t timeout_ns, int* status);

#ifdef __cplusplus
}
#endif

#endif /* GPUCPM_H_ */
