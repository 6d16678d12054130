/*
 * grazelle_gb300.h -- native C ABI of the GB300 Grazelle engine (libgrazelle_gb300.so).
 *
 * One grz_graph holds one graph resident in the HBM of one GPU.  It holds the
 * vector-sparse edge lists, vertex indices, outdegrees and per-application
 * vertex state.  Every call that launches work enqueues it on the graph's CUDA
 * stream.  Calls that return data to host memory synchronise that stream.
 * Plain C types only; pointers may be host or device memory where noted.
 *
 * This is the context-handle form of the interface.  The reference's own entry
 * points (include/phases.h) are declared in grazelle_phases.h and act on the
 * graph bound with grz_phases_bind().
 *
 * Reference counterparts (paths in the Grazelle tree):
 *   grz_graph_load_pairs / _files   graph_data_read_from_file   source/graphdata.c:957-1049
 *   grz_graph_copy_list             graph_edges_{gather,scatter}_list_block_bufs_numa  include/graphdata.h:59-65
 *   grz_graph_copy_vertex_index     graph_vertex_{gather,scatter}_index_numa           include/graphdata.h:80-95
 *   grz_graph_copy_outdegrees       graph_vertex_outdegrees                            include/graphdata.h:38
 *   grz_pr_init                     execution_initialize_vertex_prop_pr                source/execution_pr.c:85-88
 *   grz_pr_iterate                  execution_impl_pr's loop                           source/execution_pr.c:92-168
 *   grz_cc_run                      execution_impl_cc                                  source/execution_cc.c:94-268
 *   grz_bfs_run                     execution_impl_bfs                                 source/execution_bfs.c:120-276
 *   grz_read_props                  graph_vertex_props                                 include/graphdata.h:32
 */
#ifndef GRAZELLE_GB300_H
#define GRAZELLE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GRZ_OK 0
#define GRZ_ERR_ARG -1        /* bad argument */
#define GRZ_ERR_CUDA -2       /* CUDA runtime error (no GPU, launch failure, ...) */
#define GRZ_ERR_NOMEM -3      /* device allocation failed */
#define GRZ_ERR_UNSORTED -4   /* an edge list is not grouped by its shared vertex in ascending order */
#define GRZ_ERR_RANGE -5      /* vertex ID >= V, or a size beyond the 32-bit device ID limit */
#define GRZ_ERR_STATE -6      /* call out of order (e.g. iterate before init) */
#define GRZ_ERR_IO -7         /* file missing, truncated or inconsistent with its header */
#define GRZ_ERR_TIMEOUT -8    /* a bounded device-side wait gave up */

/* application selectors (compile-time ALGORITHM in the reference, Makefile:179-223) */
#define GRZ_APP_PAGERANK 0
#define GRZ_APP_CONNECTED_COMPONENTS 1
#define GRZ_APP_BREADTH_FIRST_SEARCH 2

/* list selectors */
#define GRZ_LIST_PULL 0   /* in-edge (gather) list: shared vertex = destination */
#define GRZ_LIST_PUSH 1   /* out-edge (scatter) list: shared vertex = source */

typedef struct grz_graph grz_graph;

typedef struct grz_graph_info_t {
    uint64_t num_vertices;
    uint64_t num_edges;
    uint64_t pull_vectors;          /* graph_edges_gather_list_vector_count */
    uint64_t push_vectors;          /* graph_edges_scatter_list_vector_count */
    uint64_t pull_index_start, pull_index_end;   /* graph_vertex_gather_index_{start,end}_numa[0] */
    uint64_t push_index_start, push_index_end;
    const void* pull_list_device;   /* device address of the 256-bit pull vectors */
    const void* push_list_device;
    uint64_t device_bytes;          /* HBM held by this graph */
} grz_graph_info_t;

const char* grz_error_string(int code);
const char* grz_graph_last_error(const grz_graph* g);

/* stream: a cudaStream_t to run on, or NULL to create a private non-blocking stream */
int grz_graph_create(grz_graph** out, int device, void* stream);
int grz_graph_set_stream(grz_graph* g, void* stream);
void grz_graph_destroy(grz_graph* g);
int grz_sync(grz_graph* g);

/* Loads a graph from its two edge lists in Grazelle's file order: `pull_pairs` grouped by
 * destination, `push_pairs` grouped by source, each E interleaved (src, dst) uint64 pairs.
 * Host or device pointers.  push_pairs may be NULL (pull engine only).  Builds the
 * vector-sparse lists, vertex indices and outdegrees on the device. */
int grz_graph_load_pairs(grz_graph* g, uint64_t num_vertices, uint64_t num_edges,
                         const uint64_t* pull_pairs, const uint64_t* push_pairs);
/* The same with options (no counterpart in the reference).  GRZ_LOAD_DERIVE_PUSH, with
 * push_pairs NULL: build the -push list on the device from the -pull pairs (a stable sort by
 * source gives exactly the -push order), so only one list crosses the host link. */
#define GRZ_LOAD_DERIVE_PUSH 1
int grz_graph_load_pairs_ex(grz_graph* g, uint64_t num_vertices, uint64_t num_edges, const uint64_t* pull_pairs,
                            const uint64_t* push_pairs, int flags);
/* Reads `<base>-pull` and `<base>-push`, each a {V, E} header and E (src, dst) uint64 pairs
 * (source/graphdata.c:957-1049); push is optional.  The pairs are streamed to the device
 * through two pinned 64 MB staging buffers (parallel reads overlapping the copies). */
int grz_graph_load_files(grz_graph* g, const char* base);
/* The same with GRZ_LOAD_DERIVE_PUSH: only `<base>-pull` is read and the -push list is derived
 * on the device. */
int grz_graph_load_files_ex(grz_graph* g, const char* base, int flags);

/* The info's pull_list_device / push_list_device point at the reference-format 256-bit
 * vectors.  The engine runs on its own execution layout, so those vectors are derived from it
 * on the first request (this call, grz_graph_copy_list, or a phases.h binding) and then kept. */
int grz_graph_get_info(const grz_graph* g, grz_graph_info_t* out);
/* copies the reference-format 256-bit vectors (4 uint64 each) to host memory */
int grz_graph_copy_list(grz_graph* g, int list, uint64_t* host_vectors, uint64_t capacity_vectors);
/* copies the vertex index (V + 64 uint64) */
int grz_graph_copy_vertex_index(grz_graph* g, int list, uint64_t* host_index, uint64_t capacity);
int grz_graph_copy_outdegrees(grz_graph* g, double* host_outdeg, uint64_t capacity);

/* The reference's measurement experiments.  ITERATION_STATS (source/execution_cc.c:209-231):
 * while enabled, the CC/BFS edge phases count the vectors they process and those vectors'
 * valid lanes; grz_stats_take returns the counts since the last take and resets them (packing
 * efficiency = edges / (4 vectors)).  MODEL_LONG_VECTORS (source/graphdata.c:628-675): the
 * vectors a list would need with `lanes`-wide vectors. */
int grz_stats_enable(grz_graph* g, int on);
int grz_stats_take(grz_graph* g, uint64_t* vectors, uint64_t* edges);
int grz_graph_vector_model(grz_graph* g, int list, uint32_t lanes, uint64_t* vectors);

/* PageRank (FP64 props; exact fixed-point accumulation).  damping 0.875 reproduces the
 * reference's hard-coded constant (source/constants.asm:75-79). */
int grz_pr_init(grz_graph* g, double damping);
/* enqueues `iterations` fused edge-pull + vertex iterations (one kernel each) */
int grz_pr_iterate(grz_graph* g, uint32_t iterations);
/* PageRank props as the reference stores them (rank / outdegree'), V doubles to host */
int grz_read_props(grz_graph* g, double* host_props, uint64_t capacity);

/* timing helper: milliseconds of `iterations` fused PageRank iterations measured with CUDA
 * events on the graph's stream (state advances) */
int grz_pr_time_iterations(grz_graph* g, uint32_t iterations, float* ms_out);

/* -------- Connected Components and BFS -------- */

/* engine flags: the reference's compile-time EXPERIMENTS that change the CC/BFS driver
 * (Makefile:59-176); 0 = the default threshold heuristic (execution_bfs.c:146-168) */
#define GRZ_FLAG_FORCE_PULL 1       /* EXPERIMENT_EDGE_FORCE_PULL */
#define GRZ_FLAG_FORCE_PUSH 2       /* EXPERIMENT_EDGE_FORCE_PUSH */
#define GRZ_FLAG_WITHOUT_COUNT 4    /* EXPERIMENT_THRESHOLD_WITHOUT_COUNT */
#define GRZ_FLAG_WITHOUT_OUTDEG 8   /* EXPERIMENT_THRESHOLD_WITHOUT_OUTDEGREES */
#define GRZ_FLAG_HOST_LOOP 16       /* grz_cc_run / grz_bfs_run: one host round trip per iteration instead of one CUDA graph launch per run */

typedef struct grz_run_stats_t {
    uint32_t iterations;        /* total_iterations_executed */
    uint32_t pull_iterations;   /* total_iterations_used_gather */
    uint32_t push_iterations;   /* total_iterations_used_scatter */
    float ms;                   /* device time of the run (CUDA events) */
} grz_run_stats_t;

/* Connected Components to convergence (execution_impl_cc); labels via grz_read_props */
int grz_cc_run(grz_graph* g, int flags, grz_run_stats_t* stats);
/* BFS from `root` (the reference fixes root 0, source/execution_bfs.c:28); parents via
 * grz_read_props (-1 = unvisited or root), levels via grz_read_levels */
int grz_bfs_run(grz_graph* g, uint32_t root, int flags, grz_run_stats_t* stats);
int grz_read_levels(grz_graph* g, int64_t* host_levels, uint64_t capacity);
/* -------- kernel shapes (no counterpart in the reference) --------
 * Per-graph tuning knobs; the defaults are sound, the autotuner (grazelle/autotune.py) searches
 * them.  Results never depend on them. */
#define GRZ_TUNE_HUBS 0         /* hub sources encoded in the pull list at the next load (0..49152; 0 = none) */
#define GRZ_TUNE_CC_CACHE 1     /* hub labels the CC pull kernel keeps in shared memory (<= 49152) */
#define GRZ_TUNE_CC_THREADS 2   /* threads per block of the CC pull kernel: 256, 512 or 1024 */
#define GRZ_TUNE_CC_GRID 3      /* blocks of the persistent CC pull kernel (0 = SMs x resident blocks) */
#define GRZ_TUNE_PR_GRID 4      /* blocks of the persistent PageRank gather kernel (0 = SMs x resident blocks) */
#define GRZ_TUNE_BFS_PULL_SCAN 5 /* BFS pull over the whole list: 0 = only the wanted destinations' vectors (compacted), 1 = scan every vector */
#define GRZ_TUNE_PR_PROPS 6     /* props the PageRank gather reads, from the next grz_pr_init: 0 = by size (8-byte doubles when 16-byte fixed-point props exceed 6x L2), 1 = fixed point, 2 = doubles; results identical */
#define GRZ_TUNE_INGEST_CHUNKS 7 /* chunks of the pull-only ingest, from the next load (0 = one per 2^24 pairs, <= 64; the last is cut into up to four smaller pieces): each chunk is processed while the next crosses the host link */
#define GRZ_TUNE_PR_PERSISTENT 8 /* form of grz_pr_iterate: 0 = default (two kernels), 1 = two kernels per iteration (gather, apply), 2 or 3 = every iteration in one cooperative launch (6 or 8 blocks per SM) whose phases are separated by a grid barrier with bounded waits (the call then waits for the iterations) */
#define GRZ_TUNE_PULL_STAGING 13 /* CC pull's edge stream: 0 = streaming loads, 1 = bulk copies (cp.async.bulk) into shared memory, two tiles ahead; results identical */
#define GRZ_TUNE_CC_SEGMENTS 16 /* CC's first (full) pull over the source-segmented lists of GRZ_TUNE_PR_SEGMENT_BITS: 0 = when they are built (by grz_pr_init), 1 = never, 2 = built at the CC initialisation (with the default segment size when the graph is below the size threshold); results identical */
#define GRZ_TUNE_BFS_PULL_FIRST 17 /* BFS pull over the whole list: vectors each wanted destination reads, in order, in a first pass that stops at the first vector with a frontier source (1..64; 0 = no such pass, every vector of the wanted destinations is read); destinations left undecided are finished by the pass over their remaining vectors; results identical */
#define GRZ_TUNE_CC_PULL_FIRST 18 /* CC pull of an iteration without a usable previous minimum (the first of a run): each destination's first vector first, one destination per thread, then 1 = the whole list without the destinations at 0, 2 = only the remaining vectors of the destinations still above 0 (compacted; fewer bytes, but one iteration more on R-MAT), 3 = as 1, and the later pulls read only the destinations above the previous iteration's smallest written label (marked and compacted) instead of every vector's destination, 4 (default) = every pull over marked and compacted open destinations: in the first, every vector of the destinations still above 0 after their first vector; 0 = the whole list directly.  Results identical */
#define GRZ_TUNE_PR_SEGMENT_BITS 14 /* PageRank source segments, from the next grz_pr_init: 0 = by size (when the double props exceed 4x L2), 1 = none, 8..31 = 2^bits sources per segment.  The pull list is also kept cut by source segment, and each iteration gathers segment by segment so that a segment's props stay in L2; results identical (not with hub encoding) */
#define GRZ_TUNE_PR_WAIT_LIMIT_US 9 /* bound of one grid-barrier wait of the persistent PageRank kernel in microseconds (0 = 2 s); a wait that runs out makes grz_pr_iterate return GRZ_ERR_TIMEOUT and leaves PageRank uninitialised */
#define GRZ_TUNE_PR_WITHHOLD 10  /* fault injection for tests: block + 1 of the persistent PageRank kernel that never arrives at its first barrier (0 = none) */
#define GRZ_TUNE_RUN_MAX_ITERATIONS 11 /* CC/BFS iteration bound (0 = V + 2): a run that has not converged by then returns GRZ_ERR_TIMEOUT */
#define GRZ_TUNE_RUN_LIMIT_US 12  /* CC/BFS time bound of a run in microseconds (0 = 300 s), checked after each iteration: GRZ_ERR_TIMEOUT */
#define GRZ_TUNE_HUBS_LOADED 100 /* read-only: hubs encoded in the loaded pull list */
int grz_tune_set(grz_graph* g, int param, int64_t value);
int grz_tune_get(const grz_graph* g, int param, int64_t* value);

/* -------- batches: many PPR and BFS instances over many graphs (no counterpart in the reference) --------
 * Graphs of any size are added with their -pull pairs and merged into one block-diagonal union
 * on the device.  Each run processes up to GRZ_BATCH_K instances of every graph in one CUDA graph
 * launch.  Outputs are [union vertex][k]: graph g's local vertex v is row voff[g] + v, where voff
 * is the running sum of the vertex counts of the graphs added before g.
 * Personalized PageRank: the reference's PageRank vertex phase (source/phase_vertex_pr.asm:75-134)
 * with teleport and dangling mass sent to the seed: rank' = d*accum + [v == seed]*(d*(1-S) + 1-d),
 * starting from rank = one-hot(seed); edge sums exact (fixed point), rounded once to double.
 * Multi-source BFS: levels (-1 unreached), bit-parallel over the instances of a graph. */
#define GRZ_BATCH_K 8
typedef struct grz_batch grz_batch;
int grz_batch_create(grz_batch** out, int device, void* stream);
void grz_batch_destroy(grz_batch* b);
const char* grz_batch_last_error(const grz_batch* b);
/* pull_pairs: interleaved (src, dst) sorted by (dst, src); graphs need at least 32 vertices */
int grz_batch_add_graph(grz_batch* b, uint64_t num_vertices, uint64_t num_edges, const uint64_t* pull_pairs);
int grz_batch_build(grz_batch* b);
int grz_batch_info(const grz_batch* b, uint64_t* graphs, uint64_t* vertices, uint64_t* edges, uint64_t* vectors);
/* seeds / roots: [graphs][k] local vertex IDs, 0xffffffff = no instance; k <= GRZ_BATCH_K */
int grz_batch_ppr(grz_batch* b, const uint32_t* seeds, uint32_t k, uint32_t iterations, double damping,
                  double* ranks_out, grz_run_stats_t* stats);
int grz_batch_msbfs(grz_batch* b, const uint32_t* roots, uint32_t k, int32_t* levels_out, grz_run_stats_t* stats);
/* Both at once: PPR from `seeds` ([graphs][k]) and multi-source BFS from `roots` ([graphs][kb]) in one
 * CUDA graph launch whose two branches run the two loops side by side.  Results as the two calls
 * above (either output may be NULL); ppr_stats / bfs_stats time each branch inside the launch,
 * *total_ms the launch. */
int grz_batch_run(grz_batch* b, const uint32_t* seeds, uint32_t k, uint32_t iterations, double damping, const uint32_t* roots,
                  uint32_t kb, double* ranks_out, int32_t* levels_out, grz_run_stats_t* ppr_stats, grz_run_stats_t* bfs_stats,
                  float* total_ms);
/* kernel shapes of a batch (results never depend on them): resident blocks per SM of the
 * persistent PPR gather / apply and multi-source BFS pull kernels, 1..32 (default 8) */
#define GRZ_BATCH_TUNE_PPR_BLOCKS 0
#define GRZ_BATCH_TUNE_BFS_BLOCKS 1
#define GRZ_BATCH_TUNE_PPR_PROPS 2   /* props the PPR gather reads: 0 (default) or 1 = 16-byte fixed point, 2 = 8-byte doubles converted on the gather (measured slower: the gather is not DRAM-bound); results identical */
int grz_batch_tune_set(grz_batch* b, int param, int64_t value);
int grz_batch_tune_get(const grz_batch* b, int param, int64_t* value);
unsigned long long grz_batch_launch_count(const grz_batch* b);

/* Digest of the last CC/BFS result without reading it back (no counterpart in the reference):
 * out[0] = reached vertices (BFS) or components (CC: vertices whose label is their own ID),
 * out[1] = sum of the reached vertices' out-degrees (BFS; the TEPS numerator),
 * out[2] = order-independent checksum of the levels (BFS) or labels (CC). */
int grz_result_digest(grz_graph* g, uint64_t out[3]);

/* Step-wise driver for callers that choose the engine themselves (the learned switch):
 * begin, then call next until it returns 0 (converged); engine 1 = pull, 0 = push, -1 = the
 * threshold heuristic.  Returns 1 while running, 0 when the vote reached 0, < 0 on error. */
int grz_frontier_begin(grz_graph* g, int app, uint32_t root, int flags);
int grz_frontier_next(grz_graph* g, int engine, int* engine_used, uint64_t* vote);
/* the vote that decides the next iteration and the heuristic's engine for it */
int grz_frontier_current_vote(grz_graph* g, uint64_t* vote, int* threshold_engine);

/* -------- learned push/pull switch -------- */

/* The reference chooses the engine with a threshold on the vote (pull iff vote > E/5,
 * source/execution_bfs.c:146-168); that stays the default policy.  GRZ_POLICY_LEARNED asks a
 * small MLP (GRZ_MLP_FEATURES -> 32 -> 32 -> 1, FP32, hand-written CUDA kernels) before each
 * iteration whether pull will be faster.  Labels and levels do not depend on the choice. */
#define GRZ_MLP_FEATURES 12
#define GRZ_MLP_HIDDEN 32
#define GRZ_MLP_PARAMS 1505
#define GRZ_POLICY_THRESHOLD 0
#define GRZ_POLICY_LEARNED 1

typedef struct grz_mlp grz_mlp;
int grz_mlp_create(grz_mlp** out, int device, uint64_t seed);
void grz_mlp_destroy(grz_mlp* n);
int grz_mlp_get_params(grz_mlp* n, float* host_params, uint64_t capacity);
int grz_mlp_set_params(grz_mlp* n, const float* host_params, uint64_t count);
/* X: count x GRZ_MLP_FEATURES, Y: 1 if pull was faster, W: per-sample weight (e.g. |t_pull - t_push|);
 * loss = mean of W * BCE(logit, Y) */
int grz_mlp_gradients(grz_mlp* n, const float* X, const float* Y, const float* W, uint64_t count, float* host_grads,
                      float* loss);
int grz_mlp_train(grz_mlp* n, const float* X, const float* Y, const float* W, uint64_t count, uint32_t epochs, float lr,
                  float* final_loss);
int grz_mlp_predict(grz_mlp* n, const float* X, uint64_t count, float* host_logits);

int grz_frontier_set_policy(grz_graph* g, int policy, grz_mlp* mlp);
/* features of the state the next iteration starts from; *policy_choice = the current policy's engine */
int grz_frontier_features(grz_graph* g, float* host_features, uint64_t capacity, int* policy_choice);
int grz_frontier_last_features(grz_graph* g, float* host_features, uint64_t capacity);
/* time both engines from one state: snapshot, run one, restore, run the other */
int grz_frontier_snapshot(grz_graph* g);
int grz_frontier_restore(grz_graph* g);
int grz_frontier_next_timed(grz_graph* g, int engine, int* engine_used, uint64_t* vote, float* edge_ms);

/* Kernel profiling: when enabled, every launch is bracketed by a CUDA event pair on the graph's
 * stream (the GPU form of the reference's EXPERIMENT_ITERATION_PROFILE, source/main.c:43-55).
 * grz_profile_read synchronises, returns up to `capacity` (kind, milliseconds) records in launch
 * order, and clears the log. */
int grz_profile_enable(grz_graph* g, int on);
int grz_profile_read(grz_graph* g, int* kinds, float* ms, int capacity);
const char* grz_profile_kind_name(int kind);
/* while profiling: pull vectors the CC open-destination pulls (GRZ_TUNE_CC_PULL_FIRST 4) read, in
 * first pulls and in later pulls, since the last call (which resets them) */
int grz_profile_work(grz_graph* g, uint64_t* first_pull_vectors, uint64_t* later_pull_vectors);
/* number of kernels this graph has launched so far (monotonic) */
unsigned long long grz_launch_count(const grz_graph* g);

/* -------- allocation-free PageRank step -------- */

/* Largest graph (vertices) that grz_pr_step_noalloc accepts. */
#define GRZ_NOALLOC_MAX_VERTICES (1u << 18)

/* One PageRank iteration (edge-pull + vertex phase) on caller-owned device arrays, for callers
 * that cannot allocate device memory while they run: a framework whose own pool owns the
 * device memory, a latency-bound loop where cudaMalloc/cudaFree would synchronise the device,
 * or a sandbox that forbids allocation after start-up.  This function has no counterpart in
 * the reference.  It calls no cudaMalloc, cudaFree or other allocating routine.  Its scratch
 * (exact per-destination accumulators and per-block partial sums, about 4 MB) lives in a
 * fixed device array inside this library, held by every GPU that loads it until the process
 * exits.
 *   vectors      the reference's 256-bit pull vectors on the device (32-byte aligned), e.g.
 *                grz_graph_info_t.pull_list_device; num_vectors of them
 *   props_in     double[V] on the device: rank / outdegree', as the reference stores props
 *   outdeg       double[V] on the device: outdegree from the -pull list
 *   props_out    double[V] on the device: the props after one iteration; must not overlap
 *                props_in (GRZ_ERR_ARG)
 *   stream       cudaStream_t to run on (NULL = the legacy default stream)
 * Returns GRZ_ERR_RANGE if num_vertices is 0 or above GRZ_NOALLOC_MAX_VERTICES, GRZ_ERR_ARG
 * for a bad argument, GRZ_ERR_CUDA if a launch fails.
 * The first call on a device resolves the scratch array's device address (cudaGetSymbolAddress)
 * for that device, so make that first call before capturing a stream.  The address is kept until
 * the process exits: calling again after cudaDeviceReset is not supported.  Every call shares the
 * one array and clears the part it needs when it starts, so calls that overlap on the GPU (on
 * different streams, or from different host threads) race with each other: order them. */
int grz_pr_step_noalloc(const void* vectors, uint64_t num_vectors, uint64_t num_vertices, const double* props_in,
                        const double* outdeg, double damping, double* props_out, void* stream);
uint64_t grz_pr_step_noalloc_max_vertices(void);

/* Host-side diagnostics of the exact accumulation used by PageRank: values are converted
 * exactly to unsigned 4.124 fixed point, summed as 128-bit integers and rounded once to
 * double (round to nearest even).  Inputs and the total must stay in [0, 16); a total that
 * reaches 16 returns GRZ_ERR_RANGE. */
int grz_fixed_point_roundtrip(double x, double* out);
int grz_fixed_point_sum(const double* xs, uint64_t n, double* out);

#ifdef __cplusplus
}
#endif

#endif
