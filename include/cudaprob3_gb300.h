/*
 * cudaprob3_gb300.h -- C ABI of the GB300 Barger propagator (libcp3gb300.so).
 *
 * Plain pointers and sizes only.  Each entry point names the reference interface it
 * replaces (CUDAProb3++ "linear" fork: AtmosCudaPropagatorSingle / BeamCudaPropagatorSingle,
 * which derive from AtmosCpuPropagator<double> / BeamCpuPropagator<double> and
 * Propagator<double>).  The C++ facade cudaprob3_gb300.hpp wraps this ABI in classes with the
 * reference's names and turns non-zero statuses into std::runtime_error.
 *
 * Handles are independent: every parameter lives in the handle (host) and in per-handle
 * device buffers, never in process-global or __constant__ state, so two handles may compute
 * concurrently on different streams.  A single handle is not thread-safe.
 *
 * Result layouts (device and the bulk-copy calls):
 *   atmospheric  [9][n_cosines][n_energies]    (channel t = a*3+b is P(a -> b))
 *   beam         [9][n_energies]
 * FP64 handles hold doubles, MIXED handles hold floats.
 */
#ifndef CUDAPROB3_GB300_H
#define CUDAPROB3_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cp3_propagator cp3_propagator;

/* Status codes.  The reference throws std::runtime_error (input errors) or prints and calls
 * exit(1) (CUDA errors, hpc_helpers.cuh:71-78); here every call returns one of these and
 * cp3_last_error() holds the message. */
enum cp3_status {
    CP3_OK = 0,
    CP3_ERR_BAD_SIZE = 1,      /* vector size differs from the handle's grid / empty model */
    CP3_ERR_NOT_SET = 2,       /* a required setter was not called (e.g. production height) */
    CP3_ERR_LAYER_LIMIT = 3,   /* a trajectory crosses more shells than CP3_MAX_SHELLS */
    CP3_ERR_CUDA = 4,          /* CUDA runtime error (message has the CUDA error string) */
    CP3_ERR_OOM = 5,           /* device allocation failed */
    CP3_ERR_BAD_ARGUMENT = 6,  /* invalid enum / pointer / device id */
    CP3_ERR_INDEX = 7,         /* getProbability index out of range */
    CP3_ERR_ORDER = 8,         /* radii not monotone ("radii order messed up") */
    CP3_ERR_FILE = 9,          /* density model file missing or malformed */
    CP3_ERR_UNSUPPORTED = 10   /* feature not available for this handle kind / precision */
};

/* Arithmetic of a handle. */
enum cp3_precision {
    CP3_FP64 = 0,  /* plain FP64 throughout: the drop-in for the reference's FP64 kernels */
    CP3_MIXED = 1  /* FP32 transition matrices, layer products and probabilities; FP64
                      eigen-decomposition; double-float phase reduction */
};

/* NeutrinoType (types.hpp:29). */
enum cp3_neutrino { CP3_NEUTRINO = 0, CP3_ANTINEUTRINO = 1 };

/* Most shells one trajectory may cross (the reference's compile-time MaxNLayers()==10,
 * constants.hpp:46, is a runtime check against this value here). */
#define CP3_MAX_SHELLS 128

/* ---- lifetime ------------------------------------------------------------------------ */

/* AtmosCudaPropagatorSingle(int id, int n_cosines, int n_energies)
 * (atmoscudapropagator.cuh:52, atmoscudapropagator.cu:30-57). */
int cp3_atmos_create(int device, int n_cosines, int n_energies, int precision,
                     cp3_propagator** out);

/* BeamCudaPropagatorSingle(int id, int n_energies, int n_threads)
 * (beamcudapropagator.cuh:52, beamcudapropagator.cu:29-54). */
int cp3_beam_create(int device, int n_energies, int precision, cp3_propagator** out);

/* ~AtmosCudaPropagatorSingle / ~BeamCudaPropagatorSingle (atmoscudapropagator.cu:64-67). */
int cp3_destroy(cp3_propagator* h);

/* Message of the last failed call on h (h == NULL: last failed create on this thread). */
const char* cp3_last_error(const cp3_propagator* h);

/* Queries: kind (0 atmospheric, 1 beam), precision, grid sizes. */
int cp3_get_info(const cp3_propagator* h, int* kind, int* precision, int* n_cosines,
                 int* n_energies);

/* ---- setters (Propagator / AtmosCpuPropagator / BeamCpuPropagator) ----------------------- */

/* Propagator::setEnergyList (propagator.hpp:213-218) + device copy
 * (atmoscudapropagator.cu:181-186).  n must equal the handle's n_energies.  GeV.  The list is
 * copied into the handle's pinned staging buffer before the call returns (the caller's array
 * may be reused at once) and uploaded asynchronously on the handle's own stream, after the
 * handle's last compute; a compute on another stream waits for the upload. */
int cp3_set_energies(cp3_propagator* h, const double* energies, int n);

/* AtmosCpuPropagator::setCosineList (atmoscpupropagator.hpp:368-381) + device copy
 * (atmoscudapropagator.cu:188-191).  Recomputes the per-cosine shell counts. */
int cp3_set_cosines(cp3_propagator* h, const double* cosines, int n);

/* Propagator::setMNSMatrix (propagator.hpp:148-183): radians; knutype < 0 flips dcp. */
int cp3_set_mns(cp3_propagator* h, double theta12, double theta13, double theta23, double dcp,
                int knutype);

/* Propagator::setNeutrinoMasses (propagator.hpp:188-209): eV^2, dm23sq = m3^2 - m2^2. */
int cp3_set_masses(cp3_propagator* h, double dm12sq, double dm23sq);

/* AtmosCpuPropagator::setDensity(radii, rhos, yps) (atmoscpupropagator.hpp:116-170) and its
 * device copy (atmoscudapropagator.cu:121-140).  Radii in km, ascending or descending,
 * including the r = 0 row; rho in g/cm^3; ye = Z/A. */
int cp3_set_layers(cp3_propagator* h, const double* radii, const double* rho, const double* ye,
                   int n);

/* AtmosCpuPropagator::setDensity(radii, a, b, c, yps) (atmoscpupropagator.hpp:181-242):
 * rho(r) = a r^2 + b r + c per shell, averaged along each trajectory segment
 * (physics::getDensityOfLayerPoly, physics.hpp:651-739). */
int cp3_set_layers_poly(cp3_propagator* h, const double* radii, const double* a,
                        const double* b, const double* c, const double* ye, int n);

/* AtmosCpuPropagator::setDensityFromFile (atmoscpupropagator.hpp:250-344): 3-column
 * (r rho ye) or 5-column (r a b c ye) text, '#' comments.  Two-column files (r rho), which
 * the reference rejects with std::terminate, are accepted with ye from default_ye_core for
 * r <= 3480 km and default_ye_mantle outside. */
int cp3_set_density_file(cp3_propagator* h, const char* path, double default_ye_core,
                         double default_ye_mantle);

/* AtmosCpuPropagator::setChemicalComposition (atmoscpupropagator.hpp:481-491,
 * atmoscudapropagator.cu:207-220): n must equal the number of model rows. */
int cp3_set_chemical_composition(cp3_propagator* h, const double* ye, int n);

/* AtmosCpuPropagator::getNlayerBoundaries (atmoscpupropagator.hpp:85): *n = the number of
 * rows of the density model (its layer boundaries, the r = 0 row included), one more than
 * its layers.  The reference sets the count only in setDensityFromFile
 * (atmoscpupropagator.hpp:343) and returns an uninitialised value after the other density
 * setters; here every density setter sets it.  CP3_ERR_NOT_SET before a density model,
 * CP3_ERR_UNSUPPORTED on a beam handle. */
int cp3_get_n_layer_boundaries(cp3_propagator* h, int* n);

/* AtmosCpuPropagator::setProductionHeight (atmoscpupropagator.hpp:386-393): km; the cosine
 * list must be set first ("must set cosine list before production height"). */
int cp3_set_production_height(cp3_propagator* h, double height_km);

/* BeamCpuPropagator::setDensity(rho) / setPathLength(L) (beamcpupropagator.hpp:84-91;
 * device copies beamcudapropagator.cu:83-101).  g/cm^3 (Ye = 0.5 implied) and km. */
int cp3_set_beam_density(cp3_propagator* h, double rho);
int cp3_set_beam_path_length(cp3_propagator* h, double path_km);

/* ---- production-height averaging (physics.hpp:997-1067) ---------------------------------- */

/* AtmosCpuPropagator::SetNumberOfProductionHeightBinsForAveraging +
 * setProductionHeightList (atmoscpupropagator.hpp:85-110, 395-427).  The reference's
 * switch never turns averaging on (:97-99); here n_bins >= 1 turns it on explicitly and
 * n_bins == 0 turns it off.  prob: [2][3][n_energies][n_cosines][n_bins];
 * edges_km: n_bins + 1 entries.  n_bins <= 20. */
int cp3_set_production_height_averaging(cp3_propagator* h, int n_bins, const double* prob,
                                        const double* edges_km);

/* ---- compute ----------------------------------------------------------------------------- */

/* calculateProbabilities(NeutrinoType) (atmoscudapropagator.cu:202-205, 266-310;
 * beamcudapropagator.cu:103-106, 162-186): launch and wait. */
int cp3_calculate(cp3_propagator* h, int neutrino_type);

/* Launch on `stream` (a cudaStream_t; NULL = the handle's own stream) and return.  Later
 * result reads and cp3_synchronize order themselves after this stream. */
int cp3_calculate_async(cp3_propagator* h, int neutrino_type, void* stream);

/* Computation plus the whole result copied to host memory dst (the device layout,
 * 9 * n_cosines * n_energies values of the handle's precision), asynchronous on `stream`.
 * The cosine rows are computed in n_chunks pieces (<= 0: the default, 4 pieces of at least
 * 32 MB each, fewer for smaller results).  Each piece's copy goes on the handle's copy
 * stream once the piece is computed, so copies overlap computation; dst must be page-locked
 * for that.  `stream` waits for the last copy.  A later computation of the same row pieces
 * waits only for each piece's own copy, so a call on another stream can compute while this
 * one's download is still running.  (Atmospheric handles; a beam handle's single copy
 * follows its kernel on `stream`.)  Replaces calculateProbabilities followed by the full
 * download of the first getProbability (atmoscudapropagator.cu:222-235). */
int cp3_calculate_to_host_async(cp3_propagator* h, int neutrino_type, void* dst, int n_chunks,
                                void* stream);

/* waitForCompletion (atmoscudapropagator.cu:313-316). */
int cp3_synchronize(cp3_propagator* h);

/* ---- results ----------------------------------------------------------------------------- */

/* AtmosCudaPropagatorSingle::getProbability(ic, ie, t) (atmoscudapropagator.cu:222-235).
 * The first call after a compute copies the whole result to the host. */
int cp3_get_probability(cp3_propagator* h, int index_cosine, int index_energy, int prob_type,
                        double* out);

/* BeamCudaPropagatorSingle::getProbability(ie, t) (beamcudapropagator.cu:146-160). */
int cp3_get_probability_beam(cp3_propagator* h, int index_energy, int prob_type, double* out);

/* getProbabilityArr(out, t) (atmoscudapropagator.cu:238-257): atmospheric order is
 * energy-major, cosine-minor (out[ie * n_cosines + ic]); beam out[ie]. */
int cp3_get_probability_arr(cp3_propagator* h, int prob_type, double* out);

/* No reference counterpart (zero-copy access): device pointer of the result in the layout
 * above; *is_float = 1 for MIXED handles.  Valid until the next compute or destroy. */
int cp3_device_result(cp3_propagator* h, const void** ptr, int* is_float, size_t* bytes);

/* No reference counterpart: asynchronous copy of the whole result, native element type and
 * device layout, into dst (bytes as reported by cp3_device_result) on `stream`
 * (NULL = the stream of the last compute; another stream waits for that compute on the
 * device). */
int cp3_copy_result_async(cp3_propagator* h, void* dst, void* stream);

/* ---- trajectory geometry (host only, no GPU) --------------------------------------------- */

/* No reference counterpart (inspection of what the atmospheric kernels walk; the geometry is
 * that of physics::calculate_atmos, getTraversedDistanceOfLayer, getDensityOfLayer[Poly],
 * physics.hpp:634-898).  Model as for cp3_set_layers (poly = 0: c1 = rho) or
 * cp3_set_layers_poly (poly = 1: c1, c2, c3 = a, b, c).  Call once with NULL outputs to get
 * *n_segments and *n_classes, then with arrays of those sizes: seg_offset[n_cosines + 1],
 * seg_len_km / seg_rho_e / seg_class[*n_segments] (segments l = 0..M of each cosine: air,
 * then shells inwards), class_rho_e[*n_classes] (class 0 = air; class 1 + i = shell i of the
 * constant model, so segment l of every row has class l; poly segments have class -1). */
int cp3_trajectory_table(const double* radii, const double* c1, const double* c2,
                         const double* c3, const double* ye, int n_radii, int poly,
                         const double* cosines, int n_cosines, double production_height_km,
                         int* n_segments, int* n_classes, int* seg_offset, double* seg_len_km,
                         double* seg_rho_e, int* seg_class, double* class_rho_e);

/* ---- profiling (the reference's TIMERSTART/TIMERSTOP macros, hpc_helpers.cuh:29-67) ------- */

/* enable != 0: record CUDA events around each kernel of every following compute. */
int cp3_set_profiling(cp3_propagator* h, int enable);

/* Device time of the last compute's kernels (waits for them): the eigen-table kernel and the
 * per-bin kernel, milliseconds.  eigen_ms is 0 where no table kernel runs (beam). */
int cp3_kernel_times(cp3_propagator* h, double* eigen_ms, double* bins_ms);

/* ---- batches: many problems, one run of a persistent kernel ------------------------------ */

/* No reference counterpart (the reference propagates one grid per call; a fit evaluates many
 * parameter sets with uneven grids, here in one run).  A batch holds atmospheric
 * problems (one Earth model and production height per batch, own cosine/energy grid each)
 * and beam problems (own energies, density and baselines), each with its own oscillation
 * parameters and neutrino type, computed in MIXED precision by one persistent kernel
 * replayed from a CUDA graph (one launch, or a table launch and a bin launch: see
 * cp3_batch_set_split_tables).  Results stay on the device:
 *   atmospheric problem  [9][n_cosines][n_energies] floats
 *   beam problem         [n_baselines][9][n_energies] floats */
typedef struct cp3_batch cp3_batch;

int cp3_batch_create(int device, cp3_batch** out);
int cp3_batch_destroy(cp3_batch* b);
const char* cp3_batch_last_error(const cp3_batch* b);

/* Earth model (as cp3_set_layers) and production height shared by the atmospheric problems. */
int cp3_batch_set_earth(cp3_batch* b, const double* radii, const double* rho, const double* ye,
                        int n, double production_height_km);
int cp3_batch_add_atmos(cp3_batch* b, const double* cosines, int n_cosines,
                        const double* energies, int n_energies, int* id);
/* rho in g/cm^3 (Ye = 0.5); all baselines of one problem share its eigen-decompositions. */
int cp3_batch_add_beam(cp3_batch* b, const double* energies, int n_energies, double rho,
                       const double* path_km, int n_baselines, int* id);
/* setMNSMatrix + setNeutrinoMasses + the neutrino type of one problem; may change between
 * runs after the commit (the next run uploads them). */
int cp3_batch_set_params(cp3_batch* b, int id, double theta12, double theta13, double theta23,
                         double dcp, int knutype, double dm12sq, double dm23sq,
                         int neutrino_type);
/* Freezes the problem list: trajectories, device arenas, the CUDA graph. */
int cp3_batch_commit(cp3_batch* b);
/* Tile shape of the persistent kernel (results do not depend on it): cosine rows per
 * atmospheric tile (1..16; a tile is 32 energies), resident blocks per SM (0 = as many as
 * fit), 32-energy groups per beam tile (1..64). */
int cp3_batch_set_shape(cp3_batch* b, int rows_per_tile, int blocks_per_sm, int beam_chunk);
int cp3_batch_get_shape(const cp3_batch* b, int* rows_per_tile, int* blocks_per_sm,
                        int* beam_chunk);
/* How a run with atmospheric problems is launched (results do not depend on it): on = 0,
 * one persistent launch in which each problem's bin tiles wait for its eigen-table tiles;
 * on != 0 (the default), a table launch followed by a bin launch, with no wait.  The
 * autotuner sets it. */
int cp3_batch_set_split_tables(cp3_batch* b, int on);
int cp3_batch_get_split_tables(const cp3_batch* b, int* on);
/* Testing aid for failure detection (no reference counterpart): with on != 0 the following
 * runs are single launches that hand out no eigen-table tile, so every atmospheric bin
 * tile's bounded wait (2 s) runs out; cp3_batch_synchronize then returns CP3_ERR_CUDA
 * ("wait limit") and the results of atmospheric problems are undefined.  on = 0 restores
 * normal runs.  Faults nothing. */
int cp3_batch_debug_withhold_tables(cp3_batch* b, int on);
/* Autotuner: times every candidate shape on this batch and keeps the fastest; use_cache != 0
 * reads and appends the choice to $CP3_TUNE_CACHE (default ~/.cache/cp3gb300_tune.txt),
 * keyed by GPU and batch size. */
int cp3_batch_tune(cp3_batch* b, int use_cache);
/* One run over every problem on `stream` (NULL = the batch's own stream). */
int cp3_batch_run(cp3_batch* b, void* stream);
/* One run with every result copied to dst, laid out as the arena (result_bytes bytes; each
 * problem at its cp3_batch_result_offset).  The bins run in n_pieces windows of whole
 * problems (0: one per 256 MB of results, at most 8); each window's range of the arena is
 * copied on the batch's copy stream while the next window computes, so with page-locked dst
 * the download overlaps the computation.  `stream` (NULL = the batch's own stream) waits for
 * the last copy.  The run always uses the split form (a table launch, then the bin launches)
 * and gives the same results as cp3_batch_run.  CP3_ERR_BAD_ARGUMENT for a null dst or more
 * than 8 pieces, CP3_ERR_UNSUPPORTED while cp3_batch_debug_withhold_tables is on.  (No
 * reference counterpart: the reference has no batches; its propagators download their
 * results in calculateProbabilities.) */
int cp3_batch_run_to_host(cp3_batch* b, void* dst, int n_pieces, void* stream);
/* Waits for the last run and for everything queued on the batch's own stream (result
 * copies with a NULL stream); *ms = the run's device time. */
int cp3_batch_synchronize(cp3_batch* b, double* ms);
/* Device pointer and float count of one problem's result. */
int cp3_batch_result(cp3_batch* b, int id, const float** ptr, size_t* count);
/* Asynchronous copy of one problem's result to dst (count floats) on `stream`, after the last
 * run on the device whatever its stream. */
int cp3_batch_copy_result(cp3_batch* b, int id, void* dst, void* stream);
/* The results of all problems sit in one arena of result_bytes / 4 floats (cp3_batch_info);
 * problem id's result starts at float *offset of it.  (No reference counterpart: the
 * reference has no batches.) */
int cp3_batch_result_offset(const cp3_batch* b, int id, size_t* offset);
/* Asynchronous copy of the arena's floats [first, first + count) to dst (host or device) on
 * `stream` (NULL: the batch's own stream), after the last run on the device whatever its
 * stream.  A caller that wants every result moves them in a few large copies instead of one
 * per problem; gaps between problems hold no results. */
int cp3_batch_copy_results(cp3_batch* b, size_t first, size_t count, void* dst, void* stream);
/* Bytes of one problem's parameter block (what a run uploads per problem after
 * cp3_batch_set_params). */
size_t cp3_batch_parameter_bytes(void);
int cp3_batch_info(const cp3_batch* b, int* n_problems, long long* total_bins,
                   size_t* result_bytes, long long* tiles);

/* ---- serving: continuous batching ------------------------------------------------------- */

/* No reference counterpart.  A request is one registered grid + one parameter set
 * + a neutrino type; submit returns at once.  A scheduler thread admits queued requests in
 * arrival order as device memory (a pool of pool_bytes for their tables and results) and one
 * of two launch slots free up, packs up to max_batch requests / max_bins_per_launch bins
 * into one run of the persistent kernel (a table launch and a bin launch where there are
 * atmospheric requests), and overlaps consecutive runs on two streams.  Grids stay
 * resident; a request's result stays on the device until cp3_server_release. */
typedef struct cp3_server cp3_server;

int cp3_server_create(int device, size_t pool_bytes, int max_batch,
                      long long max_bins_per_launch, cp3_server** out);
int cp3_server_destroy(cp3_server* s);
const char* cp3_server_last_error(const cp3_server* s);
int cp3_server_set_earth(cp3_server* s, const double* radii, const double* rho,
                         const double* ye, int n, double production_height_km);
int cp3_server_add_atmos_grid(cp3_server* s, const double* cosines, int n_cosines,
                              const double* energies, int n_energies, int* grid);
int cp3_server_add_beam_grid(cp3_server* s, const double* energies, int n_energies, double rho,
                             const double* path_km, int n_baselines, int* grid);
/* Uploads the grids, allocates the pool, captures the launch graphs, starts the loop. */
int cp3_server_start(cp3_server* s);
int cp3_server_submit(cp3_server* s, int grid, double theta12, double theta13, double theta23,
                      double dcp, int knutype, double dm12sq, double dm23sq, int neutrino_type,
                      unsigned long long* id);
/* Blocks up to timeout_s; *done = 1 when the request has finished.  A request whose launch
 * failed (a CUDA call of the launch, or the kernel's status word) finishes with *done = 1 and
 * CP3_ERR_CUDA, the reason in cp3_server_last_error; requests of other launches are not
 * affected. */
int cp3_server_wait(cp3_server* s, unsigned long long id, double timeout_s, int* done);
/* Device pointer / float count of a finished request's result (layout as for batches) and its
 * latency (submit to completion of its launch, ms).  Refused (CP3_ERR_CUDA) for a request
 * that finished with an error. */
int cp3_server_result(cp3_server* s, unsigned long long id, const float** ptr, size_t* count,
                      double* latency_ms);
/* Synchronous copy of a finished request's result to host memory (count floats). */
int cp3_server_copy_result(cp3_server* s, unsigned long long id, void* dst);
int cp3_server_release(cp3_server* s, unsigned long long id);
int cp3_server_stats(cp3_server* s, long long* launches, long long* completed,
                     long long* queued);
/* Completion queue for a client that multiplexes many requests from one thread (an MCMC
 * driver running many chains): writes to ids up to max_ids ids of requests that finished,
 * with or without error, since the previous poll, in completion order, and their number to
 * *n; blocks up to timeout_s while there is none.  Recording starts with the first call
 * (max_ids = 0 only starts it), so a client calls it once before its first submit. */
int cp3_server_poll(cp3_server* s, unsigned long long* ids, int max_ids, double timeout_s,
                    int* n);
/* Testing aid: the next `count` launches fail on the host before any of their GPU work, as a
 * launch whose CUDA calls fail does.  Their requests, and only theirs, finish with
 * CP3_ERR_CUDA. */
int cp3_server_debug_fail_launches(cp3_server* s, int count);

/* ---- atmospheric propagation without allocation ------------------------------------------ */

/* Size of the device scratch behind cp3_atmos_mixed_noalloc: one array per GPU the library
 * is used on, placed when the library's module is loaded on that GPU (at the latest by the
 * entry point's first call there), and held for the life of the process. */
#define CP3_NOALLOC_SCRATCH_BYTES (8u * 1024u * 1024u)

/* No counterpart in the reference: an addition for callers that cannot allocate device
 * memory when they propagate -- a fitter whose memory pool owns the whole GPU, code that
 * must not call cudaMalloc (it can synchronise the device, or is forbidden where the call
 * happens), or a host loop that must not touch any allocator.
 *
 * Computes what a CP3_MIXED atmospheric handle computes, for one oscillation-parameter set
 * and one neutrino type, without allocating anything: no cudaMalloc/cudaFree, no host heap.
 * Its working memory (the staged trajectory table and the per-(class, energy) eigen table)
 * is one fixed device array of CP3_NOALLOC_SCRATCH_BYTES; a grid that does not fit is
 * rejected with CP3_ERR_BAD_SIZE before anything runs.  The headline 59-shell 2000 x 2000
 * grid fits.
 *
 * Inputs and outputs stay the caller's:
 *   d_energies   device, n_energies doubles (GeV)
 *   seg_offset, seg_len_km, seg_class, class_rho_e   host arrays, exactly as filled by
 *                cp3_trajectory_table for the caller's cosines, model and production height
 *                (validated here: segment l of each row must have class l < n_classes; then
 *                copied in; pageable arrays may be reused as soon as the call returns,
 *                page-locked ones once the stream has passed this call)
 *   d_out        device, 9 * n_cosines * n_energies floats, layout [9][n_cosines][n_energies]
 *   stream       cudaStream_t (NULL = the legacy default stream); the call is asynchronous
 *                with respect to the device
 *   err          optional buffer for a message on failure (err_len bytes, NUL-terminated)
 *
 * Every call on a device shares the one scratch array, which keeps the last call's
 * contents; nothing in it has to start at zero (each call writes every element it reads).
 * Calls whose work overlaps on the GPU (other streams, or other host threads) race on that
 * array: order them on one stream or synchronise between them.
 *
 * The first call on each device is its set-up: with that device current it looks up the
 * array's device address (cudaGetSymbolAddress) and loads the kernels the call launches.
 * Under lazy module loading (the CUDA default) that is when the driver places the array and
 * the kernels in device memory, so the first call may allocate; make it where allocation is
 * still allowed, and before any stream capture on the device.  Later calls on that device
 * allocate nothing. */
int cp3_atmos_mixed_noalloc(int device, const double* d_energies, int n_energies,
                            const int* seg_offset, const double* seg_len_km,
                            const int* seg_class, int n_cosines, const double* class_rho_e,
                            int n_classes, double theta12, double theta13, double theta23,
                            double dcp, int knutype, double dm12sq, double dm23sq,
                            int neutrino_type, float* d_out, void* stream, char* err,
                            size_t err_len);

#ifdef __cplusplus
}
#endif
#endif
