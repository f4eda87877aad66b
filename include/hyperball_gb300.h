/*
 * hyperball_gb300.h — C ABI of the GB300 (sm_103a) HyperBall library.
 *
 * This is the drop-in boundary for the HyperBall path of the Rust crate
 * webgraph-algo 0.1.0. Each entry point names the reference item it replaces
 * (paths are relative to that crate). A Rust wrapper binds these functions
 * with `extern "C"` and keeps the reference's builder/run/getter shape.
 *
 * Conventions
 *  - Every function returns an int status (HB_OK = 0) unless stated.
 *  - Graph inputs are host arrays; hb_create copies them to the device, so the
 *    caller keeps ownership. Outputs go into caller-provided host buffers.
 *  - One handle is driven by one host thread; distinct handles are independent.
 *  - On error, hb_last_error(handle) (or hb_global_last_error() for calls that
 *    have no handle) returns a message; the reference's anyhow errors map to
 *    HB_ERR_NOT_RUN / HB_ERR_NOT_REQUESTED / HB_ERR_INVALID below.
 *  - No torch or C++ types cross this boundary.
 */
#ifndef HYPERBALL_GB300_H
#define HYPERBALL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define HB_OK 0
#define HB_ERR_INVALID 1       /* bad argument (reference: builder asserts, HB:153-167, HB:211-238, HLL:379-403) */
#define HB_ERR_NOT_RUN 2       /* accessor before run (reference: ensure_iteration, HB:624-630) */
#define HB_ERR_NOT_REQUESTED 3 /* output not requested (reference: bail!, HB:645, HB:655, HB:669) */
#define HB_ERR_OOM 4           /* device allocation failed */
#define HB_ERR_CUDA 5          /* CUDA runtime error */
#define HB_ERR_TIMEOUT 6       /* a bounded device wait gave up */
#define HB_ERR_IO 7            /* file not readable */
#define HB_ERR_NO_DEVICE 8     /* no CUDA device: the library has no CPU fallback */

/* ---- hashers (reference: HyperLogLogBuilder::build_hasher, HLL:356-363) -- */
#define HB_HASH_SIP13 0   /* Rust std DefaultHasher (SipHash-1-3, zero keys), the default of HyperLogLogBuilder::new (HLL:244-251) */
#define HB_HASH_JENKINS 1 /* JenkinsHasher(seed) of tests/test_hyperball.rs:25-172 (Java dsiutils mix) */

/* ---- option flags --------------------------------------------------------- */
#define HB_SUM_OF_DISTANCES (1u << 0)         /* HyperBallBuilder::sum_of_distances(true), HB:262-265 */
#define HB_SUM_OF_INVERSE_DISTANCES (1u << 1) /* HyperBallBuilder::sum_of_inverse_distances(true), HB:268-271 */
#define HB_TRANSPOSE_ON_DEVICE (1u << 2)      /* build the transpose on the GPU (enables systolic iterations) */
#define HB_NO_I32_SHIFT_QUIRK (1u << 3)       /* count() with +2^-31 for register value 31 instead of Rust's i32 wrap (HLL:178) */
#define HB_TMA_GATHER (1u << 4)               /* far successors by TMA gathers instead of plain loads (tuning; same results) */
#define HB_NO_GRAPHS (1u << 5)                /* launch every iteration directly instead of replaying CUDA graphs of the iteration shapes an earlier run of the handle showed (same results) */

/* "choose automatically" value of the tuning fields of hb_options */
#define HB_AUTO 0xffffffffu

/* Which counter array hb_get_registers copies. */
#define HB_CURRENT_STATE 0
#define HB_NEXT_STATE 1

typedef struct hb_handle hb_handle;
typedef struct hb_graph hb_graph;

/* A CSR graph held by the caller (host memory): offsets[num_nodes + 1],
 * successors[num_arcs]; each successor list sorted ascending. This replaces
 * the reference's `G1: RandomAccessGraph` / `G2` transpose parameters and the
 * cumulative outdegree `D: Succ` (the offsets are that cumulative function). */
typedef struct hb_graph_view {
    uint64_t num_nodes;
    uint64_t num_arcs;
    const uint64_t* offsets;
    const uint32_t* successors;
} hb_graph_view;

/* Builder parameters (reference: HyperBallBuilder fields, HB:26-56, and
 * HyperLogLogBuilder, HLL:234-251). Initialise with hb_options_default. */
typedef struct hb_options {
    uint32_t struct_size;     /* sizeof(hb_options) */
    int32_t log2m;            /* log2 of registers per counter, >= 4 (HLL:379-383); default 4 */
    int32_t hash_kind;        /* HB_HASH_*; default HB_HASH_SIP13 */
    int32_t device;           /* CUDA device ordinal; default 0 */
    uint64_t hash_seed;       /* seed of HB_HASH_JENKINS */
    uint64_t num_elements;    /* HLL upper bound on elements; 0 = num_nodes (or sum of weights) (HLL:346-350) */
    uint32_t flags;           /* HB_* flags above */
    uint32_t far_rows;        /* with HB_TMA_GATHER: successors more than this many ids from their node are far; 0 = 8192 */
    uint64_t arc_granularity; /* accepted for parity with HB:280-283; 0 = 16 Ki. The device balances work by degree buckets. */
    const uint64_t* weights;  /* optional node weights, host array of num_nodes (HB:286-290); NULL = all 1 */
    uint64_t weight_seed;     /* seeds the values added for weights (the reference uses a non-reproducible RNG, HB:1167-1174) */
    void* stream;             /* cudaStream_t to launch on; NULL = legacy default stream */
    uint32_t small_max_degree;  /* tuning: nodes up to this out-degree run one lane-group each; HB_AUTO = 64 (see hb_tune_degree_buckets) */
    uint32_t medium_max_degree; /* tuning: nodes up to this out-degree run one 8-lane team each, above: one CTA; HB_AUTO = 4096 */
    uint32_t union_variant;     /* tuning: HB_AUTO = the autotuner picks the union-kernel variant per graph
                                   (see hb_union_variant_count); else the index of a fixed variant.
                                   Every variant gives bit-identical results. */
} hb_options;

/* Per-iteration statistics (reference: the progress-logger lines of
 * iterate(), HB:782-942). */
typedef struct hb_iter_stats {
    uint64_t iteration;          /* 1-based */
    uint64_t modified_counters;  /* HB:899-905 */
    uint64_t visited_arcs;       /* arcs (u,v), u != v, v modified in the previous iteration */
    uint64_t scanned_nodes;      /* nodes whose successors were enumerated */
    double neighborhood_function;/* value appended to the neighbourhood function */
    double relative_increment;   /* HB:929-941 */
    int32_t systolic, local, pre_local;
    int32_t union_variant;       /* variant of the union kernels this iteration ran */
    double union_ms;             /* device time of the union kernels of this iteration */
    double iteration_ms;         /* device time of the whole iteration */
    uint64_t scanned_arcs;       /* arcs of the scanned nodes (successor ids read) */
    uint64_t kernel_launches;    /* CUDA kernels this library launched for the iteration */
    int32_t from_graph;          /* 1: the iteration ran as a replay of a captured CUDA graph */
    int32_t reserved;
} hb_iter_stats;

/* Discount function: weight of distance d >= 1 (reference: the closures of
 * HyperBallBuilder::discount_function, HB:291-297). Called on the host once
 * per iteration with d = iteration + 1. */
typedef double (*hb_discount_fn)(uint64_t distance, void* ctx);

/* ---- lifecycle ------------------------------------------------------------ */

/* Fills defaults (log2m 4, SipHash-1-3, no optional outputs). */
void hb_options_default(hb_options* opts);

/* Builds a device-resident HyperBall instance.
 * Replaces HyperBallBuilder::with_hyper_log_log (HB:91-133), ::new (HB:152-181),
 * ::with_transpose (HB:204-256), the setters (HB:259-303) and ::build (HB:321-403).
 * `transpose` may be NULL; with HB_TRANSPOSE_ON_DEVICE the transpose is built on
 * the GPU instead. Without any transpose no systolic iteration runs (HB:795-796). */
int hb_create(const hb_graph_view* graph, const hb_graph_view* transpose, const hb_options* opts,
              hb_handle** out);

/* Adds a discount function (HB:291-297); call before the first run. */
int hb_add_discount_function(hb_handle* h, hb_discount_fn fn, void* ctx);

/* Frees every device and host resource of the handle. */
void hb_destroy(hb_handle* h);

/* ---- running (reference: HyperBall::run*, HB:534-621) --------------------- */

/* HyperBall::run(upper_bound, threshold) (HB:534-583): init, then iterate until
 * no counter changes, `upper_bound` (capped at num_nodes) iterations ran, or, when
 * `threshold` is not NaN, the relative increment after the fifth iteration is
 * below 1 + threshold. */
int hb_run(hb_handle* h, uint64_t upper_bound, double threshold);

/* HyperBall::run_until_stable(upper_bound) (HB:595-603). */
int hb_run_until_stable(hb_handle* h, uint64_t upper_bound);

/* HyperBall::run_until_done() (HB:614-621). */
int hb_run_until_done(hb_handle* h);

/* Autotuner of the degree buckets: which nodes run one lane group each
 * (out-degree up to small_max), one 8-lane team each (up to medium_max) or one
 * CTA each (above). Builds a handle per candidate pair (small_max in
 * {32, 64, 128, 256, 512, 1024}, medium_max in {4096, 16384, 65536}) from `opts`, times
 * the union kernels over `iterations` standard iterations (at least 2; the
 * first is not counted) and returns the fastest pair and its union time.
 * Pass the pair as hb_options.small_max_degree / medium_max_degree; every
 * pair gives identical results. No reference counterpart: the reference
 * splits work by arc granularity only (HB:280-283, HB:1012). */
int hb_tune_degree_buckets(const hb_graph_view* graph, const hb_options* opts, uint32_t iterations,
                           uint32_t* small_max, uint32_t* medium_max, double* union_ms);

/* Step-wise driving, as the reference's in-crate test does with init() and
 * iterate() (HB:1155-1213, HB:775-949). `out` may be NULL. */
int hb_init(hb_handle* h);
int hb_iterate(hb_handle* h, hb_iter_stats* out);

/* Number of completed iterations and the statistics of iteration i (0-based). */
uint64_t hb_num_iterations(const hb_handle* h);
int hb_get_iteration_stats(const hb_handle* h, uint64_t i, hb_iter_stats* out);

/* ---- results (reference: accessors, HB:633-757) ---------------------------- */

/* neighborhood_function() (HB:633-636): iterations + 1 values. Writes
 * min(capacity, len) values and stores len in *len. */
int hb_get_neighborhood_function(const hb_handle* h, double* dst, size_t capacity, size_t* len);
/* sum_of_distances() (HB:639-647); len must be num_nodes. */
int hb_get_sum_of_distances(const hb_handle* h, double* dst, size_t len);
/* harmonic_centralities() (HB:650-657). */
int hb_get_harmonic_centralities(const hb_handle* h, double* dst, size_t len);
/* discounted_centrality(index) (HB:663-671). */
int hb_get_discounted_centrality(const hb_handle* h, size_t index, double* dst, size_t len);
/* closeness_centrality() (HB:674-686): 1/d, 0 when d == 0. */
int hb_get_closeness_centrality(const hb_handle* h, double* dst, size_t len);
/* lin_centrality() (HB:691-712): count^2/d, 1 when d == 0. */
int hb_get_lin_centrality(const hb_handle* h, double* dst, size_t len);
/* nieminen_centrality() (HB:715-732): count^2 - d. */
int hb_get_nieminen_centrality(const hb_handle* h, double* dst, size_t len);
/* reachable_nodes() (HB:750-757). */
int hb_get_reachable_nodes(const hb_handle* h, double* dst, size_t len);
/* reachable_nodes_from(node) (HB:739-745). */
int hb_reachable_nodes_from(const hb_handle* h, uint64_t node, double* out);

/* Raw counter words of the current or next state, in the reference layout
 * (SliceCounterArray, src/utils/slice_counter_array.rs:166-169: counter i at
 * bytes [i*B, (i+1)*B), B = 2^log2m * 5 / 8, 5-bit registers packed LSB-first
 * in little-endian words). `bytes` must be num_nodes * B. */
int hb_get_registers(const hb_handle* h, int which, void* dst, size_t bytes);

/* Variants of the union kernels. They differ in how successor counters are
 * requested (plain loads, or software prefetch into L1 or L2 ahead of the
 * loads), in the registers per thread (2, 3 or 4 resident blocks per SM;
 * with 2, two counter loads in flight per lane), and in the kernel that runs
 * standard iterations (variants 5-8: the staged kernel, which copies each
 * work item's offsets, per-node sums and, in 5 and 6, successor ids into
 * shared memory one item ahead); they give bit-identical results. With union_variant = HB_AUTO the library
 * times them on the handle's own standard iterations (one iteration each,
 * per kind of iteration: merging every successor or only modified ones) and
 * keeps the fastest if it beats the first variant by 3%; systolic iterations
 * run the first variant. The choice is remembered for later handles of a
 * graph with the same nodes, arcs and log2m in the process. No reference
 * counterpart: the reference has one code path (HB:960-1152). */
int hb_union_variant_count(void);
/* The variant chosen for each kind of iteration (0: standard iterations
 * merging every successor, 1: standard iterations merging modified
 * successors, 2: systolic); -1 while still being timed. */
int hb_union_variant_chosen(const hb_handle* h, int32_t chosen[3]);

/* Counter size in bytes and register width (HLL:301-303). */
int hb_counter_layout(const hb_handle* h, uint64_t* counter_bytes, int* register_size);

/* Last error of a handle (never NULL). */
const char* hb_last_error(const hb_handle* h);
/* Last error of calls without a handle, per thread (never NULL). */
const char* hb_global_last_error(void);

/* ---- graphs: BVGraph input and synthetic workloads ------------------------- */

/* Decodes a BVGraph (basename.graph/.properties[/.offsets]) into host CSR.
 * Replaces webgraph's BvGraph::with_basename(..).load() as used at
 * src/main.rs:56-58 and tests/test_hyperball.rs:226-227. */
int hb_graph_load_bvgraph(const char* basename, hb_graph** out);
/* Directed out-regular Erdős–Rényi: d distinct uniform non-loop successors per node. */
int hb_graph_generate_er(uint64_t num_nodes, uint32_t d, uint64_t seed, hb_graph** out);
/* R-MAT with 2^scale nodes and edges_per_node * 2^scale drawn arcs, deduplicated, loop free. */
int hb_graph_generate_rmat(int scale, uint64_t edges_per_node, double a, double b, double c,
                           uint64_t seed, hb_graph** out);
/* Web-like: Zipf–Mandelbrot out-degrees (exponent 2.1, shift, capped), 4/5 of
 * successors within +-window of the source, 1/5 uniform. */
int hb_graph_generate_weblike(uint64_t num_nodes, uint64_t cap, double shift, uint64_t window,
                              uint64_t seed, hb_graph** out);
/* Host transpose (sorted rows). */
int hb_graph_transpose(const hb_graph* g, hb_graph** out);
/* Wraps caller arrays by copying them into a new graph. */
int hb_graph_from_csr(const hb_graph_view* view, hb_graph** out);
/* Borrowed view of a graph's arrays (valid until hb_graph_free). */
hb_graph_view hb_graph_get_view(const hb_graph* g);
void hb_graph_free(hb_graph* g);

/* ---- batches: many independent instances in one pass -------------------------- */

typedef struct hb_batch hb_batch;

/* Builds `count` independent HyperBall instances, graphs[i] (host CSR, copied)
 * with log2m[i] registers per counter; every other option (hash, flags,
 * device, stream, degree buckets) is shared; weights are not supported.
 * Instances with the same log2m run together as one disjoint union, so each
 * iteration is one pass of the union kernels over all of them. For every graph
 * the batch returns what HyperBallBuilder::build (HB:321-403) followed by
 * run_until_done (HB:614-621) returns for it alone: the same registers,
 * iteration count, neighbourhood function and per-node sums. The reference has
 * no batch API. */
int hb_batch_create(const hb_graph_view* graphs, uint32_t count, const int32_t* log2m,
                    const hb_options* opts, hb_batch** out);
/* Runs every instance until no counter of it changes. */
int hb_batch_run_until_done(hb_batch* b);
uint32_t hb_batch_num_graphs(const hb_batch* b);
/* Iterations graph `graph` ran (its own, as if alone). */
uint64_t hb_batch_num_iterations(const hb_batch* b, uint32_t graph);
/* Per-graph results, as the single-instance getters (HB:633-657). */
int hb_batch_get_neighborhood_function(const hb_batch* b, uint32_t graph, double* dst,
                                       size_t capacity, size_t* len);
int hb_batch_get_sum_of_distances(const hb_batch* b, uint32_t graph, double* dst, size_t len);
int hb_batch_get_harmonic_centralities(const hb_batch* b, uint32_t graph, double* dst, size_t len);
/* Counters of graph `graph` in the reference layout (see hb_get_registers). */
int hb_batch_get_registers(const hb_batch* b, uint32_t graph, void* dst, size_t bytes);
/* Totals over the batch: iterations of the longest group, visited arcs and
 * arc-register updates (visited arcs * 2^log2m) summed over every instance and
 * iteration, and the device time of the shared union launches of the run. */
int hb_batch_stats(const hb_batch* b, uint64_t* iterations, uint64_t* visited_arcs,
                   uint64_t* register_updates, double* device_ms);
/* Steps of the last run (one iteration of every running group each) that ran
 * as replays of a captured CUDA graph, and all steps (a step's launch
 * sequence is captured the second time its shape comes). No reference
 * counterpart. */
int hb_batch_graph_replays(const hb_batch* b, uint64_t* replayed, uint64_t* iterations);
void hb_batch_destroy(hb_batch* b);

/* ---- served jobs: continuous admission against a device-memory budget --------- */

/* Job states. */
#define HB_JOB_QUEUED 0
#define HB_JOB_RUNNING 1
#define HB_JOB_DONE 2
#define HB_JOB_FAILED 3

typedef struct hb_server hb_server;

typedef struct hb_server_options {
    uint32_t struct_size;      /* sizeof(hb_server_options) */
    int32_t device;            /* CUDA device ordinal */
    uint64_t hbm_budget_bytes; /* device bytes the running jobs may hold together; default 150e9 */
    uint32_t max_active;       /* jobs past admission at once, 1 to 48; default 16 */
    uint32_t keep_registers;   /* 1: keep each finished job's counters for hb_server_get_registers */
    uint32_t setup_threads;    /* threads that create jobs, and as many that fetch results; 0 = min(max_active, 2) */
    uint32_t union_sm_reserve; /* SMs the shared union launch leaves to the jobs' creation kernels; default 16 */
} hb_server_options;

typedef struct hb_job_info {
    int32_t state;             /* HB_JOB_* */
    int32_t error;             /* status of a failed job */
    uint64_t iterations;
    uint64_t visited_arcs;     /* summed over the iterations */
    uint64_t register_updates; /* visited arcs * 2^log2m */
    uint64_t footprint_bytes;  /* device bytes reserved for the job */
    double queue_ms;           /* submission to admission */
    double run_ms;             /* admission to results on the host */
    double latency_ms;         /* submission to results on the host */
} hb_job_info;

/* Fills defaults: device 0, 150 GB budget, 16 active jobs, no registers kept. */
void hb_server_options_default(hb_server_options* opts);
/* Starts a server. No reference counterpart. Jobs wait in arrival order. The
 * head job is admitted when a slot is free and its device footprint fits the
 * budget next to the running jobs. Each admitted job runs on its own stream,
 * so running jobs overlap on the device. A job's results equal those of
 * hb_create + hb_run_until_done on its graph alone. */
int hb_server_create(const hb_server_options* opts, hb_server** out);
/* Queues a job (the graph is copied; options as for hb_create, except that
 * weights, the stream and the device come from the server). HB_ERR_INVALID
 * when the job alone exceeds the budget. */
int hb_server_submit(hb_server* s, const hb_graph_view* graph, const hb_options* opts,
                     uint64_t* job);
/* The same without the copy: the graph's arrays must stay valid and unchanged
 * until hb_server_wait has returned for the job. Submitting then costs no
 * host time, so a stream of large jobs arrives on schedule. */
int hb_server_submit_borrowed(hb_server* s, const hb_graph_view* graph, const hb_options* opts,
                              uint64_t* job);
/* Waits until the job finished (timeout_s < 0: no limit); HB_ERR_TIMEOUT when
 * the limit passed first, the job's own status when it failed. */
int hb_server_wait(hb_server* s, uint64_t job, double timeout_s);
int hb_server_job_info(hb_server* s, uint64_t job, hb_job_info* info);
/* Results of a finished job, as the single-instance getters. */
int hb_server_get_neighborhood_function(hb_server* s, uint64_t job, double* dst, size_t capacity,
                                        size_t* len);
int hb_server_get_sum_of_distances(hb_server* s, uint64_t job, double* dst, size_t len);
int hb_server_get_harmonic_centralities(hb_server* s, uint64_t job, double* dst, size_t len);
int hb_server_get_registers(hb_server* s, uint64_t job, void* dst, size_t bytes);
/* Forgets a finished job and its host results. */
int hb_server_release(hb_server* s, uint64_t job);
/* Cancels queued jobs, waits for running ones, frees the server. */
void hb_server_destroy(hb_server* s);
/* Device bytes the server reserves for a job of this size. */
uint64_t hb_job_footprint(uint64_t num_nodes, uint64_t num_arcs, int log2m);
/* Last error of a server call on this thread (never NULL). */
const char* hb_server_last_error(void);
/* Stepping statistics of a server since its creation: steps run, their wall
 * time on the stepping thread (planning, launches, synchronisation and
 * bookkeeping of every running job), the device time of their shared union
 * launches, the jobs that took part summed over the steps, and the host time
 * the steps spent planning and launching. No reference counterpart: a
 * diagnostic of the continuous batching. */
int hb_server_stats(hb_server* s, uint64_t* steps, double* step_ms, double* union_ms,
                    uint64_t* job_steps, double* launch_ms);
/* Where the steps' time went, summed over the steps: device time from a
 * step's first launch to its union part (the jobs' pre-union kernels), of
 * the union part (the shared launch and the jobs' heavy-node kernels), and
 * from its end to the step's last launch (the post-union kernels and the
 * totals' copies); host time planning and launching, and waiting for the
 * steps to end. No reference counterpart: a diagnostic. */
int hb_server_step_times(hb_server* s, double* pre_ms, double* union_ms, double* post_ms,
                         double* host_ms, double* wait_ms);

/* ---- breadth-first visits ------------------------------------------------------ */
/* The fair parallel breadth-first visit of the reference (ParFair,
 * src/algo/visits/breadth_first/par_fair.rs:92-330) on the device. The
 * reference reports a visit through callbacks (EventPred::Unknown {node,
 * pred, distance}, Known, mod.rs:17-60), which cannot cross this boundary;
 * here a visit returns its Unknown events as arrays, level by level (within
 * a level in no particular order, as in the parallel reference), and counts
 * the Known ones. The visited set persists across visits until
 * hb_visit_reset (par_fair.rs:101, 322-324), so a second visit skips nodes
 * an earlier one reached, as the reference's does. */
typedef struct hb_visit hb_visit;

typedef struct hb_visit_stats {
    uint64_t visited;     /* Unknown events: nodes reached by this visit */
    uint64_t levels;      /* distinct distances of those nodes */
    uint64_t known_arcs;  /* Known events: arcs from the visit to already visited nodes */
    double device_ms;     /* device time of the visit's kernels (roots to the last level) */
} hb_visit_stats;

/* ParFair::new (par_fair.rs:117-124): copies the graph to `device` (checked
 * like hb_create); `stream` may be NULL (an own stream). The reference's
 * granularity has no equivalent: the device balances work by warps. */
int hb_visit_create(const hb_graph_view* graph, int device, void* stream, hb_visit** out);
void hb_visit_destroy(hb_visit* v);
/* Parallel::reset (par_fair.rs:322-324): forget every visited node. */
int hb_visit_reset(hb_visit* v);
/* One visit (par_visit_filtered_with, par_fair.rs:127-221) from `roots`
 * (roots already visited are skipped, par_fair.rs:142-156), with the filter
 * "distance <= max_distance" (UINT64_MAX: none; seq.rs:78-80 shows this
 * filter): nodes farther away are neither reported nor marked. Event k is
 * (nodes[k], preds[k], dists[k]); a root is its own predecessor at
 * distance 0. Any of the three arrays may be NULL. Fewer than the visit's
 * events fit in `capacity`: the first ones are written and HB_ERR_INVALID is
 * returned (the visit itself is complete). */
int hb_visit_run(hb_visit* v, const uint64_t* roots, size_t nroots, uint64_t max_distance,
                 uint32_t* nodes, uint32_t* preds, uint32_t* dists, size_t capacity,
                 hb_visit_stats* stats);
/* visit([root]) for each root in order, the pattern of the reference's tests
 * (tests/test_bfv.rs:89-101): dist[node] (and pred[node]) is set for every
 * node a visit reaches; other entries are left as they are. `len` must be
 * num_nodes; pred may be NULL. */
int hb_visit_each(hb_visit* v, const uint64_t* roots, size_t nroots, uint32_t* dist, uint32_t* pred,
                  size_t len);
const char* hb_visit_last_error(const hb_visit* v);

/* ---- ExactSumSweep ------------------------------------------------------------- */
/* The reference's ExactSumSweep (src/algo/exact_sum_sweep/: the OutputLevel
 * types All, AllForward, RadiusDiameter, Diameter, Radius of
 * output_level.rs, compute_directed and compute_undirected) on the device:
 * exact eccentricities, radius and diameter from a few breadth-first visits
 * with per-node bounds. */
enum {
    HB_SWEEP_ALL = 0,             /* forward and backward eccentricities, radius, diameter */
    HB_SWEEP_ALL_FORWARD = 1,     /* forward eccentricities, radius, diameter */
    HB_SWEEP_RADIUS_DIAMETER = 2,
    HB_SWEEP_DIAMETER = 3,
    HB_SWEEP_RADIUS = 4
};
/* a radius without radial vertices (usize::MAX in the reference) and an
 * iteration count the level did not compute */
#define HB_SWEEP_NONE UINT64_MAX
typedef struct hb_sweep_result {
    uint64_t diameter, radius;                 /* dir_outputs.rs / undir_outputs.rs */
    uint64_t diametral_vertex, radial_vertex;
    uint64_t radius_iterations, diameter_iterations;
    uint64_t forward_iterations, all_iterations;
    uint64_t sweeps;                           /* breadth-first visits run (no reference counterpart) */
    double device_ms;                          /* device time of the computation (no reference counterpart) */
} hb_sweep_result;
/* OutputLevel::compute_directed(graph, transpose, radial_vertices) when
 * `transpose` is given (output_level.rs:47-53), compute_undirected(graph)
 * for a symmetric graph when it is NULL (a symmetric graph's All is
 * AllForward, computer.rs:109-114). radial_vertices: num_nodes bytes
 * (nonzero: radial) or NULL, which takes the nodes that reach the largest
 * strongly connected component (computer.rs:487-542). Eccentricities (each
 * num_nodes words, or NULL) are written when the level computes them: All
 * gives forward and backward ones, AllForward the forward ones. Where the
 * reference's parallel visits leave the radial vertex open among several
 * nodes, the smallest is reported. An empty graph returns HB_ERR_INVALID with
 * the reference's assertion message. The component of the largest
 * out-degree node is found by device visits; the other components and the
 * arcs between components are computed on the host, sequentially, as in the
 * reference (sccs/tarjan.rs, sccs/symm_seq.rs, scc_graph.rs).
 * stream NULL: a stream of its own. Returns when the results are on the
 * host. */
int hb_exact_sum_sweep(const hb_graph_view* graph, const hb_graph_view* transpose, int level,
                       const uint8_t* radial_vertices, int device, void* stream,
                       uint64_t* forward_eccentricities, uint64_t* backward_eccentricities,
                       hb_sweep_result* out);
/* The message of the calling thread's last failed hb_exact_sum_sweep. */
const char* hb_sweep_last_error(void);

/* ---- device CSR utilities ----------------------------------------------------- */

/* Transpose of a device-resident CSR graph: d_offsets[num_nodes + 1] and
 * d_successors[num_arcs] (device pointers) into caller-allocated device arrays
 * d_t_offsets[num_nodes + 1] and d_t_successors[num_arcs], on `stream` (NULL =
 * legacy default stream); returns when the result is complete. Rows of the
 * transpose are in no particular order. Checks the input first (offsets[0] ==
 * 0, offsets[num_nodes] == num_arcs, non-decreasing offsets, successors <
 * num_nodes) and returns HB_ERR_INVALID otherwise. Allocates and frees about
 * 8 * (num_nodes + 1) bytes of temporary device memory on the stream.
 * The reference takes the transpose as an input of
 * HyperBallBuilder::with_transpose (HB:204-210), built on the host; this is
 * the same transpose built where the graph already is. */
int hb_device_transpose(const uint64_t* d_offsets, const uint32_t* d_successors, uint64_t num_nodes,
                        uint64_t num_arcs, uint64_t* d_t_offsets, uint32_t* d_t_successors,
                        void* stream);

/* hb_device_transpose without any device allocation, for callers that cannot
 * allocate: a serving loop whose device memory is reserved up front and must
 * not grow while it runs, a host program that hands all device memory to its
 * own allocator, or a process whose memory pool is exhausted. No reference
 * counterpart. Its scratch is one fixed array in the library's device memory
 * (a little over 8 MiB per device, held until the process exits), so
 * num_nodes is at most 1,048,576; larger graphs get HB_ERR_INVALID. That
 * array is shared by every call on a device: calls that overlap in time
 * (other streams or threads) race on it and must be serialized by the caller.
 * The first call on each device looks up the array's address
 * (cudaGetSymbolAddress) once; make that first call before any stream
 * capture. `stream` must belong to the current device (HB_ERR_INVALID
 * otherwise). The call checks the graph and waits for its stream like
 * hb_device_transpose. No claim is made about capturing the call in a CUDA
 * graph. Same arguments, checks and results as hb_device_transpose. */
int hb_device_transpose_noalloc(const uint64_t* d_offsets, const uint32_t* d_successors,
                                uint64_t num_nodes, uint64_t num_arcs, uint64_t* d_t_offsets,
                                uint32_t* d_t_successors, void* stream);

/* Test hook of the TMA far-gather variant (HB_TMA_GATHER): every bounded
 * mbarrier wait of the handle's union kernel gives up after `polls` polls
 * (0: the default limit), and `extra_tx_bytes` (at most 2^19) are added to
 * every expected transaction count, so that no wait can complete and the
 * timeout path runs: the kernel releases the extra bytes, waits (bounded)
 * for its copies in flight, issues no more TMA copies, and the iteration
 * returns HB_ERR_TIMEOUT. hb_init then starts a clean run. Pass (0, 0) to
 * restore the defaults. No reference counterpart. */
int hb_debug_far_wait(hb_handle* h, uint32_t polls, uint32_t extra_tx_bytes);
/* Test hook (process-wide): the device allocation of a handle (creation,
 * discount arrays) that is the (after + 1)-th from now fails once with
 * HB_ERR_OOM, as a cudaMalloc failure would; after < 0 turns it off. The
 * failing call releases what it had allocated. No reference counterpart. */
int hb_debug_fail_allocations(int64_t after);

/* ---- introspection ---------------------------------------------------------- */
/* Library build string, e.g. "hyperball_gb300 sm_103a". */
const char* hb_version(void);
/* CUDA kernels this library launched for the handle so far (creation, init and
 * every iteration). No reference counterpart: a diagnostic for benchmarks. */
uint64_t hb_kernel_launches(const hb_handle* h);

/* ---- device memory ------------------------------------------------------------ */
/* Handles, batches and served jobs take device memory from a pool the library
 * keeps per device; memory a destroyed handle gave back stays reserved there
 * for the next one, so creating and destroying handles in a loop maps no new
 * memory. This returns the reserved, unused memory of `device` to the device
 * (memory in use is untouched), and frees the small page-locked host blocks
 * that destroyed handles left for reuse. No reference counterpart. */
int hb_release_cached_memory(int device);

#ifdef __cplusplus
}
#endif

#endif /* HYPERBALL_GB300_H */
