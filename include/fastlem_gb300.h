/* fastlem_gb300.h -- C ABI of the GB300 landscape-evolution solve.
 *
 * The drop-in boundary for fastlem's `TerrainGenerator::generate()`.  A Rust crate
 * (or any FFI caller) keeps fastlem's public types and forwards to these calls;
 * no torch or CUDA types appear in any signature.  All arrays are host pointers.
 *
 * Status codes (int return values):
 *   FL_OK                          0
 *   FL_ERR_MODEL_NOT_SET           1  GenerationError::ModelNotSet            (lem/generator.rs:25)
 *   FL_ERR_PARAMETERS_NOT_SET      2  GenerationError::ParametersNotSet       (lem/generator.rs:23)
 *   FL_ERR_INVALID_NUM_PARAMETERS  3  GenerationError::InvalidNumberOfParameters (lem/generator.rs:21)
 *   FL_ERR_BUILDER_SITES_NOT_SET   4  ModelBuilderError::SitesNotSet          (models/surface/builder.rs:16)
 *   FL_ERR_BUILDER_BOUNDS_NOT_SET  5  ModelBuilderError::BoundsNotSet         (models/surface/builder.rs:18)
 *   FL_ERR_BUILDER_VORONOI         6  ModelBuilderError::VoronoiError         (models/surface/builder.rs:20)
 *   FL_ERR_INVALID_ARGUMENT       20  malformed graph (index out of range, NaN length, size limits)
 *   FL_ERR_CUDA                   21  a CUDA runtime call failed (message via fl_last_error)
 *   FL_ERR_OUT_OF_MEMORY          22  device allocation failed
 *   FL_ERR_DEVICE_LIMIT           23  a device-side loop hit its iteration cap (a graph whose
 *                                     receiver structure is not a forest; never expected)
 */
#ifndef FASTLEM_GB300_H
#define FASTLEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FL_OK 0
#define FL_ERR_MODEL_NOT_SET 1
#define FL_ERR_PARAMETERS_NOT_SET 2
#define FL_ERR_INVALID_NUM_PARAMETERS 3
#define FL_ERR_BUILDER_SITES_NOT_SET 4
#define FL_ERR_BUILDER_BOUNDS_NOT_SET 5
#define FL_ERR_BUILDER_VORONOI 6
#define FL_ERR_INVALID_ARGUMENT 20
#define FL_ERR_CUDA 21
#define FL_ERR_OUT_OF_MEMORY 22
#define FL_ERR_DEVICE_LIMIT 23

/* Opaque handle: one terrain model (graph, cell areas, default outlets) resident on
 * the current CUDA device, with the solver's device workspace. */
typedef struct fl_graph fl_graph;

/* Upload a model once.  Replaces `TerrainModel2D` as seen through the `Model`
 * trait (core/traits.rs:12-19, models/surface/model.rs:41-60):
 *   n                 = model.num()                     (graph.order())
 *   row_ptr[n+1], col[row_ptr[n]], len[row_ptr[n]]
 *                     = model.graph(): row i lists graph.neighbors_of(i) in
 *                       insertion order, col = neighbour, len = edge attribute
 *   area[n]           = model.areas()
 *   default_outlets   = model.default_outlets()
 * xs/ys (optional, may be NULL) are the site coordinates; they only steer the
 * device-side memory order and never change results.
 * Returns FL_OK and *out, or an error code. */
int fl_graph_create(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                    const double* area, const uint32_t* default_outlets, uint32_t n_default,
                    const double* xs, const double* ys, fl_graph** out);

/* Release a model and its device memory.  NULL is ignored. */
void fl_graph_destroy(fl_graph* g);

/* `TerrainGenerator::generate()` (lem/generator.rs:90-213) on model `g`.
 *   g == NULL                                  -> FL_ERR_MODEL_NOT_SET
 *   base/erodibility/uplift/is_outlet == NULL  -> FL_ERR_PARAMETERS_NOT_SET
 *   n_params != n                              -> FL_ERR_INVALID_NUM_PARAMETERS
 * The per-site parameter arrays are `TopographicalParameters` (core/parameters.rs:24-35)
 * as structure-of-arrays:
 *   base[i]        base_elevation
 *   erodibility[i] erodibility
 *   uplift[i]      uplift_rate
 *   is_outlet[i]   0 / 1
 *   max_slope[i]   radians; NaN means None.  max_slope == NULL means None everywhere.
 * max_iteration: negative means unset (`set_max_iteration` never called: the loop
 *                bound is u32::MAX); 0 .. u32::MAX as `set_max_iteration(m)` (0 runs no
 *                iteration and returns the initial elevations).
 * Outputs: out_elev[n] = Terrain2D::elevations() (models/surface/terrain.rs:31-33),
 *          *out_iterations = loop bodies executed (may be NULL). */
int fl_generate(fl_graph* g, uint32_t n_params, const double* base, const double* erodibility,
                const double* uplift, const uint8_t* is_outlet, const double* max_slope,
                int64_t max_iteration, double* out_elev, uint32_t* out_iterations);

/* Device-timed variant for benchmarks: same contract as fl_generate, and writes the
 * device time of the iteration loop (milliseconds, CUDA events on the solver's
 * stream) and of the whole call including host<->device copies. */
int fl_generate_timed(fl_graph* g, uint32_t n_params, const double* base,
                      const double* erodibility, const double* uplift, const uint8_t* is_outlet,
                      const double* max_slope, int64_t max_iteration, double* out_elev,
                      uint32_t* out_iterations, double* loop_ms, double* total_ms);

/* Page-locked host memory (no fastlem counterpart).  Parameter and output arrays in
 * such memory move between host and device by DMA at the link's rate and let the
 * parameter uploads overlap the host-side outlet scan; fl_generate accepts any host
 * memory.  *out is NULL after any failure; fl_host_alloc(0, ...) ->
 * FL_ERR_INVALID_ARGUMENT; fl_host_free(NULL) is ignored. */
int fl_host_alloc(uint64_t bytes, void** out);
void fl_host_free(void* p);

/* Number of vertices / adjacency slots of a model. */
uint32_t fl_graph_num_sites(const fl_graph* g);
uint64_t fl_graph_num_slots(const fl_graph* g);

/* ---- batched form (no fastlem counterpart: many generate() calls in one solve) ----
 *
 * `terrains` independent models packed into one graph with global site ids: terrain t
 * owns sites [site_off[t], site_off[t+1]) (its CSR rows, areas, coordinates) and
 * default outlets [def_off[t], def_off[t+1]) of `default_outlets`; no edge may cross
 * terrains.  xs / ys are each terrain's own coordinates (or NULL).  Each terrain is
 * solved exactly as fl_generate would solve it alone: its own outlet resolution
 * (generator.rs:120-132), its own StdRng noise stream (generator.rs:134-138) and its
 * own lake-heap order, so its elevations are bit-identical to a solo solve. */
int fl_batch_create(uint32_t terrains, const uint32_t* site_off, const uint32_t* row_ptr,
                    const uint32_t* col, const double* len, const double* area,
                    const uint32_t* def_off, const uint32_t* default_outlets, const double* xs,
                    const double* ys, fl_graph** out);

/* Number of packed terrains of a model (1 for fl_graph_create models). */
uint32_t fl_graph_num_terrains(const fl_graph* g);

/* Device memory a model holds (graph and workspace), in bytes. */
uint64_t fl_graph_device_bytes(const fl_graph* g);

/* An upper bound on fl_graph_device_bytes for a model of n sites and nnz adjacency
 * slots, before it is created (HBM planning; the served form's admission). */
uint64_t fl_model_device_bytes(uint32_t n, uint64_t nnz);

/* generate() for every packed terrain at once: per-site parameters over all sites, one
 * max_iteration for all.  out_terrain_iterations[t] = the loop bodies terrain t would
 * have run alone (its first iteration without an elevation change, or the limit);
 * out_iterations = loop bodies of the packed solve (the largest).  loop_ms / total_ms
 * as in fl_generate_timed; any of the last four pointers may be NULL. */
int fl_batch_generate(fl_graph* g, uint32_t n_params, const double* base,
                      const double* erodibility, const double* uplift, const uint8_t* is_outlet,
                      const double* max_slope, int64_t max_iteration, double* out_elev,
                      uint32_t* out_terrain_iterations, uint32_t* out_iterations,
                      double* loop_ms, double* total_ms);

/* The same pair with every terrain's arrays passed separately, in its own site
 * numbering (row_ptr[t] starts at 0, columns and default outlets are its own site
 * ids): no concatenated copy is made.  xs / ys may be null (caller order kept), else
 * every terrain has both.  max_slope may be null, and so may any of its entries (no
 * slope limit on that terrain). */
int fl_batch_create_parts(uint32_t terrains, const uint32_t* sites,
                          const uint32_t* const* row_ptr, const uint32_t* const* col,
                          const double* const* len, const double* const* area,
                          const uint32_t* n_default, const uint32_t* const* default_outlets,
                          const double* const* xs, const double* const* ys, fl_graph** out);
int fl_batch_generate_parts(fl_graph* g, const double* const* base,
                            const double* const* erodibility, const double* const* uplift,
                            const uint8_t* const* is_outlet, const double* const* max_slope,
                            int64_t max_iteration, double* const* out_elev,
                            uint32_t* out_terrain_iterations, uint32_t* out_iterations,
                            double* loop_ms, double* total_ms);

/* ---- served form (no fastlem counterpart: a request loop of generate() calls) ------
 *
 * Models are registered once (the server keeps a host copy); requests name a model
 * and carry their own parameters.  `slots` worker threads run up to that many requests
 * at once, each on its own CUDA stream, so their kernels overlap on the GPU.  A
 * request needs a device instance of its model (fl_graph_device_bytes of HBM); the
 * oldest waiting request starts once a slot is free and its model has an idle
 * instance or a new one fits `hbm_budget_bytes` after evicting idle instances (least
 * recently used first).  Instances stay resident for later requests on the same
 * model.  A request's elevations equal fl_generate's for the same model and
 * parameters.  Create and use the server on the device selected when it is created. */
typedef struct fl_server fl_server;

int fl_server_create(uint64_t hbm_budget_bytes, uint32_t slots, fl_server** out);

/* Registers a model (arguments as fl_graph_create; the arrays are copied).  The graph
 * itself is checked when a request first creates an instance of it. */
int fl_server_add_model(fl_server* s, uint32_t n, const uint32_t* row_ptr, const uint32_t* col,
                        const double* len, const double* area, const uint32_t* default_outlets,
                        uint32_t n_default, const double* xs, const double* ys,
                        uint32_t* model_id);

/* Queues generate() for a registered model; parameters as fl_generate (copied before
 * return).  out_elev (n entries) is written by the time fl_server_wait returns and
 * must stay valid until then.  FL_ERR_OUT_OF_MEMORY when the model can never fit the
 * budget. */
int fl_server_submit(fl_server* s, uint32_t model_id, const double* base,
                     const double* erodibility, const double* uplift, const uint8_t* is_outlet,
                     const double* max_slope, int64_t max_iteration, double* out_elev,
                     uint64_t* ticket);

/* Blocks until the request is done; returns its fl_generate status and, optionally,
 * its iterations, latency (submit to done), queueing and solve times in ms.  A ticket
 * can be waited for once. */
int fl_server_wait(fl_server* s, uint64_t ticket, uint32_t* out_iterations, double* latency_ms,
                   double* queue_ms, double* solve_ms);

/* Up to `cap` counters: requests completed, peak concurrent solves, peak and current
 * device bytes of instances, instances created, instances evicted, requests waiting,
 * packed solves run, requests solved in them. */
int fl_server_stats(fl_server* s, uint64_t* out, uint32_t cap);
/* Continuous batching on (1, the default) or off (0): requests on models of up to
 * 2,097,152 sites that find no resident instance are solved together with the other such
 * requests waiting at that moment (same iteration limit, up to 25,165,824 sites) as one
 * packed model; their results are those of their solo generate(). */
int fl_server_set_packing(fl_server* s, int enable);

/* Stops the workers after the requests they are running; waiting requests are
 * dropped (their out_elev is never written).  Frees every instance and the server:
 * no other fl_server_* call on `s` may run during or after it. */
void fl_server_destroy(fl_server* s);

/* Message for the last error on this thread ("" when none). */
const char* fl_last_error(void);

/* Make `device` current for this thread; fl_graph_create places the model on the
 * current device and every later call on that model runs there. */
int fl_select_device(int device);

/* ---- instrumentation -------------------------------------------------------------
 * Per kernel class: launches and algorithmic bytes are always counted; with timing
 * enabled each launch is also bracketed by CUDA events on the model's stream and its
 * device time accumulated.  Classes are numbered 0 .. fl_num_kernel_classes()-1. */
int fl_graph_set_timing(fl_graph* g, int enable);
void fl_graph_reset_stats(fl_graph* g);
/* Blocking host synchronisations the model's calls made since the last reset: one per
 * iteration of generate(), one more in an iteration that computes the lake order. */
uint64_t fl_graph_host_syncs(const fl_graph* g);

/* Launch shapes and switch points of the solve (no counterpart in the reference; the
 * results are the same bits whatever they are).  By default each model takes the
 * committed schedule's shapes for its size class (fastlem_gb300/schedule.json, listed by
 * fl_schedule_entry); fl_set_tuning overrides them process-wide, -1 restoring the
 * schedule:
 *   "low_ilp"        top-down Kahn rounds, sites in flight per thread: 1, 2 or 4
 *   "walk_per_sm"    chain walker blocks per SM, 1 .. 64 (at most what fits), 0: all that fit
 *   "kahn_min_width" Kahn rounds stop below this frontier width (where the chain walks
 *                    take over), 256 .. 2^24, or 0 for n / 512 clamped to [8192, 65536];
 *                    read when a model is created
 *   "sized_grids"    1: cooperative grids cut to the model's size (small models leave the
 *                    rest of the GPU to other streams' solves), 0: whole-GPU grids
 *   "gpu_rank"       1: the lake heap's order computed on the GPU where lengths decide it
 *                    (the host heap otherwise), 0: always the host heap
 * Change them only while no solve runs.  FL_LOW_ILP, FL_WALK_PER_SM, FL_KAHN_MIN_WIDTH,
 * FL_SIZED_GRIDS and FL_GPU_RANK in the environment set them at load. */
int fl_set_tuning(const char* name, int64_t value);
int64_t fl_get_tuning(const char* name);   /* -2 for an unknown name */
/* This model's cooperative grids: 1 cut to its size, 0 the whole GPU, -1 as the
 * schedule says.  A serving loop that runs several solves at once sets 1 on its
 * instances so that small solves leave room for the others. */
int fl_graph_set_sized_grids(fl_graph* g, int sized);
/* Schedule entry i (FL_ERR_INVALID_ARGUMENT past the end): models of up to max_sites
 * sites (packed batches when packed is 1) use these shapes; 0 width = the n / 512 rule. */
int fl_schedule_entry(uint32_t i, uint32_t* max_sites, int* packed, int* low_ilp,
                      uint32_t* walk_per_sm, uint32_t* kahn_min_width, int* sized_grids);

/* Where and how long the model's last lake-order computation ran: *on_gpu 1 (GPU), 0
 * (host heap) or -1 (none yet); *ms its host wall time. */
int fl_graph_rank_info(const fl_graph* g, double* ms, int* on_gpu);
uint32_t fl_num_kernel_classes(void);
int fl_graph_kernel_stats(const fl_graph* g, uint32_t cls, const char** name, uint64_t* launches,
                          double* device_ms, double* bytes);

/* Shape of the last basin pass (up to `cap` values): Kahn rounds run, leaves,
 * skeleton sites, skeleton chains, longest chain, skeleton sites needing the full
 * pull while walking, bottom-up and top-down hand-off wait iterations; then the
 * slowest bottom-up chain's walk time (ns), SM cycles spent in its full pulls and
 * their number; the slowest top-down chain's walk time (ns), SM cycles waiting for
 * its parent and its length.  Durations are kept to 64 ns, cycles to 128. */
int fl_graph_basin_stats(const fl_graph* g, uint64_t* out, uint32_t cap);

/* Round structure of the last basin pass (instrumentation; no fastlem counterpart).
 * *rounds = Kahn rounds run (r); for k <= min(cap - 1, r): offsets[k] = first order
 * slot of Kahn round k, up_ns[k] = device clock (ns) when bottom-up round k started
 * (up_ns[r] = end), down_ns[k] = when the k-th top-down round started (highest Kahn
 * round first; down_ns[r] = end).  Any output pointer may be NULL. */
int fl_graph_round_trace(fl_graph* g, uint32_t cap, uint32_t* rounds, uint32_t* offsets,
                         uint64_t* up_ns, uint64_t* down_ns);

/* ---- parity probes: one solver stage on host arrays (tests only) ---------------- */

/* Steepest-descent receivers (lem/stream_tree.rs:109-137); outlet_table[i] != 0 keeps
 * next[i] = i.  Returns FL_OK; *has_lake = 1 when a non-outlet site has no lower
 * neighbour (lem/stream_tree.rs:139-173). */
int fl_probe_receivers(fl_graph* g, const double* elev, const uint8_t* outlet_table,
                       uint32_t* next_out, int* has_lake);

/* Lake re-routing (lem/stream_tree.rs:175-243) of receivers `next_in` for the outlet
 * list `outlets` (order as generate() resolves it).  Writes the final receivers and
 * the basin label (root site) of every site before re-routing. */
int fl_probe_lakes(fl_graph* g, const uint32_t* outlets, uint32_t n_outlets,
                   const uint32_t* next_in, uint32_t* next_out, uint32_t* label_out);

/* One drainage-area / response-time / elevation pass (lem/generator.rs:144-203) on
 * final receivers `next`; elev is updated in place; returns *changed. */
int fl_probe_tree_pass(fl_graph* g, const uint32_t* outlets, uint32_t n_outlets,
                       const uint32_t* next, const double* erodibility, const double* uplift,
                       const double* max_slope, double* elev, double* drainage_out,
                       double* response_out, int* changed);

/* The order in which the reference's lake heap processes sites
 * (lem/stream_tree.rs:184-240), computed on the host: rank[v], UINT32_MAX if never. */
int fl_probe_prim_rank(fl_graph* g, const uint32_t* outlets, uint32_t n_outlets, uint32_t* rank);

/* The same order computed on the GPU (caller's site order): the outlets' tied prefix
 * replayed on the host, then the keyed part from the minimum spanning tree.  *used_gpu
 * is 0 when equal or non-positive lengths could let the heap's arrangement decide (rank
 * is then left untouched and fl_last_error says why).  Replaces the model's cached lake
 * order. */
int fl_probe_lake_rank_gpu(fl_graph* g, const uint32_t* outlets, uint32_t n_outlets,
                           uint32_t* rank, int* used_gpu);

/* x_k = (...((start + op_0) + op_1) ... + op_k) with every addition rounded, as the
 * reference's sequential accumulations do, evaluated by the solver's parallel exact
 * fold (the chain walks' arithmetic). */
int fl_probe_chain_fold(const double* operands, uint32_t n, double start, double* out);

/* `count` samples of StdRng::seed_from_u64(seed).gen::<f64>() drawn on the device,
 * starting at sample `first` (the initial-elevation noise of lem/generator.rs:134-138). */
int fl_probe_rng_f64(uint64_t seed, uint64_t first, uint64_t count, double* out);

/* ---- allocation-free variant ----------------------------------------------------- */

/* Basin labels (the root every site drains to, lem/stream_tree.rs:139-173) and
 * has_lake, for callers that must not allocate device memory -- e.g. a service whose
 * device memory comes from its own fixed pool, where a cudaMalloc would escape the
 * pool's accounting and synchronise the device.  No counterpart in the reference:
 * fastlem computes labels inside StreamTree::construct.
 *   next, outlet_table: device arrays of n entries (receivers; nonzero = outlet)
 *   labels:             device array of n entries, written
 *   has_lake:           host int (may be NULL)
 *   stream:             cudaStream_t (NULL = default stream)
 * Allocates nothing: the only scratch is a fixed 16 MiB device array inside the
 * library, held by every GPU that loads it, so n must not exceed 4,194,304
 * (FL_ERR_INVALID_ARGUMENT otherwise).  n == 0 returns FL_OK with has_lake 0 and
 * reads no array; otherwise the arrays must be non-null.  A receiver outside [0, n)
 * gives FL_ERR_INVALID_ARGUMENT, a receiver cycle (through no outlet)
 * FL_ERR_DEVICE_LIMIT.  The first call on a device looks up that array's address and
 * keeps it for the life of the process; make it before any stream capture, and do
 * not call this after a cudaDeviceReset of that device (the array may move).  Calls
 * share the scratch, so calls that overlap on one GPU race: serialise them. */
int fl_basin_labels_noalloc(uint32_t n, const uint32_t* next, const uint8_t* outlet_table,
                            uint32_t* labels, int* has_lake, void* stream);

/* ---- host model builder (models/surface/builder.rs) ------------------------------ */

/* `from_random_sites` sampler (builder.rs:38-52): x = gen_range(x0..x1), then
 * y = gen_range(y0..y1), per site.  zero_seed != 0 uses StdRng::from_seed([0; 32]) as
 * fastlem does; otherwise StdRng::seed_from_u64(seed). */
int fl_random_sites(uint64_t n, double x0, double y0, double x1, double y1, uint64_t seed,
                    int zero_seed, double* xs, double* ys);

/* `relaxate_sites(times)` (builder.rs:155-200): Lloyd relaxation in place. */
int fl_relax_sites(uint32_t n, double* xs, double* ys, double x0, double y0, double x1, double y1,
                   uint32_t times);

/* `build()` (builder.rs:202-281): Delaunay graph (a<b edge rule), clipped Voronoi
 * areas and hull outlets.  col/len hold `cap` slots (6n suffices); hull holds n. */
int fl_build_graph(uint32_t n, const double* xs, const double* ys, double x0, double y0,
                   double x1, double y1, uint32_t* row_ptr, uint32_t* col, double* len,
                   uint64_t cap, double* area, uint32_t* hull, uint64_t* out_nnz,
                   uint32_t* out_nhull);

/* The lake-heap processing order of remove_lakes_from_stream_tree
 * (lem/stream_tree.rs:175-243): rank[v] = the position at which the heap traversal
 * from `outlets` (pushed in order with key 0) processes site v, UINT32_MAX if never.
 * It depends only on the graph, the lengths and the outlet list (the solver computes
 * it once per model and outlet list).  Host computation.
 *   an out-of-range id or a NaN length met by the traversal -> FL_ERR_INVALID_ARGUMENT */
int fl_lake_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                 const uint32_t* outlets, uint32_t n_out, uint32_t* rank);

/* Raw triangulation (counter-clockwise triangles); returns the triangle count. */
int64_t fl_triangulate(uint32_t n, const double* xs, const double* ys, uint32_t* tri,
                       uint64_t cap);

/* ---- Terrain2D::get_elevation (models/surface/terrain.rs:35-38) ----
 *
 * `TerrainInterpolator2D::new(sites)` (models/surface/interpolator.rs:10-15) and its
 * `interpolate(elevations, site)` (interpolator.rs:17-29): Sibson natural-neighbour
 * interpolation, None outside the sites' convex hull.  fl_interpolate answers `count`
 * queries at once: out[i] = the interpolated value and found[i] = 1, or out[i] = NaN
 * and found[i] = 0 (the reference's None).  A query on a hull edge takes the linear
 * interpolant along it; a query equal to a site returns its value.  fl_interpolate
 * computes on host threads (large batches in grid-cell order).
 *   fewer than three sites / all collinear / a non-finite site -> FL_ERR_INVALID_ARGUMENT */
typedef struct fl_interpolator fl_interpolator;
int fl_interpolator_create(uint32_t n, const double* xs, const double* ys, fl_interpolator** out);
void fl_interpolator_destroy(fl_interpolator* it);
int fl_interpolate(const fl_interpolator* it, const double* values, uint64_t count,
                   const double* qx, const double* qy, double* out, uint8_t* found);

/* The same queries on the GPU, with the same results bit for bit: one thread per query
 * over the triangulation, which is uploaded to the current device on the first call
 * (later calls use that device).  fl_interpolate_gpu takes host arrays; in
 * fl_interpolate_device all five arrays are in that device's memory (for instance the
 * elevations of a solve and a rendering grid made on the device).  Both return when the
 * results are written.  A query whose natural-neighbour cavity exceeds 2048 triangles
 * (only with over two thousand sites on one circle) fails the call with
 * FL_ERR_INVALID_ARGUMENT; the host fl_interpolate has no such limit.
 *   null interpolator / a null array with count > 0 -> FL_ERR_INVALID_ARGUMENT (before any
 *   CUDA call); count == 0 -> FL_OK without device work */
int fl_interpolate_gpu(fl_interpolator* it, const double* values, uint64_t count, const double* qx,
                       const double* qy, double* out, uint8_t* found);
int fl_interpolate_device(fl_interpolator* it, const double* values, uint64_t count,
                          const double* qx, const double* qy, double* out, uint8_t* found);
/* Queries of the last GPU call whose first pass could not decide them (a predicate
 * filter inconclusive, a cavity over 32 triangles or a walk over 256 steps), answered by
 * the exact second pass. */
uint64_t fl_interpolator_last_deferred(const fl_interpolator* it);
/* Probe of the GPU queries' single-precision prefilters on count cases of 8 doubles
 * (a, b, c, q): out[4 i + 0, 1] the prefilter's orientation sign of (a, b, q) and
 * in-circle sign of (a, b, c, q), 0 where it leaves the case to double precision;
 * out[4 i + 2, 3] the exact signs. */
int fl_probe_prefilters(uint64_t count, const double* cases, int32_t* out);
/* Probe: the GPU natural-neighbour query code compiled for the host, one query at a time:
 * exact = 0 is the device's first pass (status 2: deferred to the second), exact = 1 the
 * second (status 3: cavity over 2048 triangles); status 0 outside, 1 found. */
int fl_probe_interp_query(const fl_interpolator* it, const double* values, uint64_t count,
                          const double* qx, const double* qy, int exact, double* out,
                          int32_t* status);

#ifdef __cplusplus
}
#endif

#endif /* FASTLEM_GB300_H */
