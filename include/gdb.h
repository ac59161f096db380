/* gdb.h -- C ABI of the GB300 occupancy-discovery / XF-barrier graph library.
 *
 * One process, one GPU.  A gdb_ctx owns a CUDA stream, the device-side
 * discovery context (protocol state plus XF barrier flags padded to 128-byte
 * lines) and a grow-only workspace; a gdb_graph owns (or borrows) a CSR in
 * HBM.  Plain pointers and sizes only -- no CUDA or C++ types cross this
 * boundary.  Every call is synchronous unless its name ends in _device, in
 * which case it is enqueued on the context's stream and all pointers are
 * device pointers.  Errors are negative gdb_status values; no exception
 * crosses the ABI.  A context is not thread-safe; distinct contexts are
 * independent.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   code/discovery_protocol/api/discovery.h          host discovery API
 *   code/discovery_protocol/api/discovery.cl         device protocol + XF barrier
 *   code/experiments/occupancy_tests/src (C files)   occupancy / protocol timing
 *   code/experiments/pannotia/graph_app/{sssp,mis,color,bc}/   mega-kernels
 *   code/experiments/lonestar_gpu_opencl/apps/{bfs,sssp,mst}/  port kernels
 */
#ifndef GDB_H
#define GDB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GDB_ABI_VERSION 10

/* Sentinels of the reference kernels. */
#define GDB_LONESTAR_INF 1000000000u /* lonestar/apps/bfs/kernel/bfs_common.cl:35 */
#define GDB_PANNOTIA_BIG 99999999    /* pannotia/graph_app/sssp/kernel/sssp_kernel.cl:68 */

typedef enum {
  GDB_OK = 0,
  GDB_ERR_INVALID = -1,        /* bad argument */
  GDB_ERR_CUDA = -2,           /* CUDA runtime error (see gdb_last_error) */
  GDB_ERR_OOM = -3,            /* device allocation failed */
  GDB_ERR_TIMEOUT = -4,        /* a device wait exceeded options.timeout_ns */
  GDB_ERR_CAPACITY = -5,       /* a device queue or table overflowed */
  GDB_ERR_NOT_CORESIDENT = -6, /* a fixed-occupancy launch above what fits */
  GDB_ERR_UNSUPPORTED = -7     /* option not available for this call */
} gdb_status;

/* Mutex of the discovery protocol (reference: locks.cl). */
typedef enum {
  GDB_LOCK_TICKET = 0, /* fair ticket lock, locks.cl:25-34 (reference default) */
  GDB_LOCK_SPIN = 1,   /* unfair exchange spin lock, locks.cl:11-20 */
  GDB_LOCK_FREE = 2    /* one atomic poll word: fetch_add to poll, fetch_or to close */
} gdb_lock_kind;

/* Inter-CTA barrier between supersteps. */
typedef enum {
  GDB_BARRIER_XF = 0,        /* discovery + XF master/slave flags (discovery.cl:129-190) */
  GDB_BARRIER_GRID_SYNC = 1, /* cooperative launch + cooperative_groups grid.sync() */
  GDB_BARRIER_RELAUNCH = 2,  /* one launch per superstep, host reads the stop flag */
  GDB_BARRIER_XF_FIXED = 3,  /* XF over all launched CTAs, no discovery (gbar_cl.h:15-74);
                                the grid is capped at the occupancy the API reports */
  GDB_BARRIER_RELAUNCH_GRAPH = 4 /* one launch per superstep from a CUDA graph: a WHILE
                                    node whose condition the last CTA of each superstep
                                    sets -- no host round trip (BFS, SSSP; in
                                    gdb_barrier_bench: captured relaunches replayed) */
} gdb_barrier_kind;

/* Schedule of the traversal options per superstep. */
typedef enum {
  GDB_SCHED_PLAIN = 0,    /* fixed: push, queue frontier, persistent */
  GDB_SCHED_ADAPTIVE = 1, /* per-superstep choice of push/pull (direction-optimising
                             thresholds); automatic near-far width for SSSP */
  GDB_SCHED_LEARNED = 2   /* the schedule selector's network (gdb_selector_set):
                             push/pull per BFS level, taken by the master CTA inside
                             each barrier; SSSP worklist / near-far width / graph
                             relaunch per run */
} gdb_schedule;

typedef struct {
  int device;          /* CUDA ordinal; -1 = current device */
  int block_size;      /* threads per CTA of the persistent kernels (0 = 512;
                          the graph kernels take at most 512) */
  int max_ctas;        /* cap on launched CTAs (0 = occupancy x SMs) */
  int oversubscribe;   /* >0: launch this many CTAs and let discovery pick
                          the co-resident ones (the reference launches 1000) */
  int lock;            /* gdb_lock_kind */
  int barrier;         /* gdb_barrier_kind */
  int schedule;        /* gdb_schedule */
  int xf_release;      /* XF form: 0 = master polls every slave's padded flag
                          and clears it (the reference's), 1 = same arrival,
                          one broadcast epoch word as release, 2 = combining:
                          slaves add to 16 padded arrival counters that one
                          master warp watches, one generation word as release,
                          3 = flat: every CTA adds to one counter and waits
                          for the barrier's count (the master arrives last
                          when a hook runs), 4 = flat up to 480 CTAs and
                          combining above (the default) */
  uint64_t timeout_ns; /* limit for every device spin (0 = 2e9) */
  /* direction-optimising BFS thresholds (GDB_SCHED_ADAPTIVE): switch to
     pull when frontier arcs > unvisited arcs / pull_alpha, back to push
     when the frontier has < V / push_beta vertices (0 = 14 / 24) */
  uint32_t pull_alpha;
  uint32_t push_beta;
  /* worklist SSSP bucket width: > 0 = near-far schedule with this width;
     0 = automatic width (32 x mean weight / mean degree) under
     GDB_SCHED_ADAPTIVE, the reference's label-correcting worklist under
     GDB_SCHED_PLAIN.  Distances are the same for every width. */
  uint32_t sssp_delta;
  /* light/heavy arc split of the near-far schedule (delta-stepping's edge
     classes): near supersteps relax only arcs lighter than the width, each
     bucket's heavy arcs are relaxed once when it runs dry.  0 = automatic
     (split when some weight >= the width), 1 = always, -1 = never. */
  int sssp_split;
  /* frontier bitmap of the direction-optimising BFS: a bottom-up (pull)
     level tests a neighbour's bit in its frontier's V-bit bitmap instead of
     loading the neighbour's level, and writes the next level's bitmap; the
     bitmap's first pull_bitmap_kb KB (the lowest vertex ids) are staged in
     every CTA's shared memory for the level.  1..64 = that stage everywhere,
     -1 = no bitmap (pull levels test the level array), 0 = automatic: 16 KB
     for a traversal that has the GPU to itself (gdb_bfs, gdb_bfs_multi,
     batches, traces), no bitmap for traversals that share it
     (gdb_bfs_sources, serving slots). */
  int pull_bitmap_kb;
} gdb_options;

typedef struct {
  uint32_t supersteps;       /* barrier intervals executed by the last run */
  uint32_t participating;    /* CTAs that took part (discovered or launched) */
  uint32_t launched;         /* CTAs launched */
  uint32_t launches;         /* kernel launches by the last run */
  uint64_t edges_processed;  /* arcs inspected (all passes) */
  uint64_t work_units;       /* edges/s work unit of the last run */
  double kernel_ms;          /* device time of the last run (CUDA events) */
  uint32_t phases;           /* SSSP near-far phase changes of the last run */
  uint32_t sssp_delta;       /* SSSP bucket width used (0 = plain worklist) */
  uint32_t sssp_light;       /* light-arc bound of the split (0 = no split) */
} gdb_run_stats;

typedef struct {
  uint64_t weight64;   /* exact forest weight */
  uint32_t weight32;   /* uint32 sum as the reference accumulates it (wraps) */
  uint32_t components; /* connected components (V - edges) */
  uint32_t edges;      /* forest edges */
  uint32_t rounds;     /* Boruvka rounds */
} gdb_mst_result;

typedef struct {
  int device;
  int sm_count;
  int cc_major, cc_minor;
  size_t total_mem;
  int occupancy_per_sm; /* resident CTAs per SM of the persistent kernels at
                           options.block_size */
  int flag_capacity;    /* barrier flags allocated (max participating CTAs) */
} gdb_device_info;

typedef struct gdb_ctx gdb_ctx;
typedef struct gdb_graph gdb_graph;

/* ------------------------------------------------------------ context */
void gdb_options_default(gdb_options* opt);
int gdb_ctx_create(const gdb_options* opt, gdb_ctx** out);
int gdb_ctx_destroy(gdb_ctx* ctx);
int gdb_ctx_set_options(gdb_ctx* ctx, const gdb_options* opt);
int gdb_ctx_get_options(gdb_ctx* ctx, gdb_options* opt);
int gdb_ctx_stream(gdb_ctx* ctx, void** cuda_stream); /* cudaStream_t */
int gdb_device_info_get(gdb_ctx* ctx, gdb_device_info* info);
const char* gdb_status_string(int status);
const char* gdb_last_error(gdb_ctx* ctx);
int gdb_last_run_stats(gdb_ctx* ctx, gdb_run_stats* stats);
int gdb_abi_version(void);

/* ------------------------------------------- discovery protocol / barrier */
/* Reset the device discovery context; replaces init_discovery_kernel_ctx
 * (code/discovery_protocol/api/discovery.h:10, kernel discovery.cl:194-202). */
int gdb_init_discovery_kernel_ctx(gdb_ctx* ctx);
/* Same with the skip flag (discovery.h:36): skip = 1 makes every launched CTA
 * participate without the protocol.  Only kernels capped at the occupancy
 * the CUDA API reports honour it; over-subscribed launches are refused. */
int gdb_init_discovery_kernel_ctx_skip(gdb_ctx* ctx, int skip);
/* Participating CTAs of the last discovery run (discovery.h:63); >= 0 count
 * or a negative status. */
int gdb_number_of_participating_groups(gdb_ctx* ctx);
/* Time one launch of the protocol-only kernel run_prot with upper_bound
 * CTAs of wgs threads (discovery.h:71, occupancy_tests/src/time_prot.c:20-85),
 * using options.lock.  *ns = device time of that launch. */
int gdb_time_protocol(gdb_ctx* ctx, int upper_bound, int wgs, double* ns);
/* run_test (occupancy_tests/src/kernels/occupancy_test.cl:8-12): protocol
 * then one XF barrier, with wgc CTAs of wgs threads and lms bytes of dynamic
 * shared memory each; *participating = CTAs discovered
 * (occupancy_tests/src/occupancy_test.c:21-89). */
int gdb_occupancy_test(gdb_ctx* ctx, int wgc, int wgs, int lms, int* participating);
/* Co-resident CTAs per the CUDA occupancy API for the run_test kernel
 * (replaces the reference's deadlock search, run_occupancy_tests.py:53-69). */
int gdb_api_occupancy(gdb_ctx* ctx, int wgs, int lms, int* ctas);
/* Barrier latency: `iters` empty supersteps with the given gdb_barrier_kind
 * on CTAs of wgs threads (0 = options.block_size) and options.max_ctas;
 * *ns_per_barrier = device time / iters, *groups = CTAs synchronised. */
int gdb_barrier_bench(gdb_ctx* ctx, int barrier_kind, int wgs, int iters,
                      double* ns_per_barrier, int* groups);
/* Fault-injection hook for tests: the XF master of the next run stops
 * releasing after `after_barriers` barriers, so every wait must end by the
 * timeout with GDB_ERR_TIMEOUT.  Negative = off. */
int gdb_debug_stall_master(gdb_ctx* ctx, int after_barriers);

/* ---------------------------------------------------------------- graphs */
/* Symmetric or directed CSR: row_ptr[V+1], col[E], optional w[E] (uint32).
 * Host arrays are copied to HBM.  Requires E < 2^32 and V < 2^31.  One
 * pass on the device checks the CSR (row_ptr[0] = 0, row_ptr[V] = E,
 * row_ptr non-decreasing, every column < V); GDB_ERR_INVALID otherwise. */
int gdb_graph_create(gdb_ctx* ctx, uint32_t V, uint64_t E, const uint32_t* row_ptr,
                     const uint32_t* col, const uint32_t* w, gdb_graph** out);
/* Same with device arrays, borrowed (not freed by gdb_graph_destroy). */
int gdb_graph_create_device(gdb_ctx* ctx, uint32_t V, uint64_t E, const uint32_t* d_row_ptr,
                            const uint32_t* d_col, const uint32_t* d_w, gdb_graph** out);
/* Replace the weight array (host array copied). */
int gdb_graph_set_weights(gdb_graph* g, const uint32_t* w);
/* Declare (1) that the graph is symmetric with symmetric weights: arc
   u -> v of weight w exists exactly when arc v -> u of weight w does (the
   undirected inputs of the reference's applications).  Pulls over in-arcs
   then read the out-arcs themselves instead of a transposed copy.  Results
   on a graph that does not satisfy the declaration are undefined.
   Default 0. */
int gdb_graph_set_symmetric(gdb_graph* g, int symmetric);
int gdb_graph_destroy(gdb_graph* g);
int gdb_graph_info(gdb_graph* g, uint32_t* V, uint64_t* E, uint32_t* heavy_vertices);

/* ---------------------------------------------------------- applications */
/* BFS levels from src; unreached = GDB_LONESTAR_INF.  Replaces LonestarGPU
 * drelax2 + host bfs() (lonestar/apps/bfs/kernel/bfs_port_kernel.cl:146-192,
 * lonestar/apps/bfs/bfs_port.cpp:62-194), which fixes src = 0. */
int gdb_bfs(gdb_ctx* ctx, gdb_graph* g, uint32_t src, uint32_t* dist);
int gdb_bfs_device(gdb_ctx* ctx, gdb_graph* g, uint32_t src, uint32_t* d_dist);

/* SSSP distances (uint32 weights); unreached = GDB_LONESTAR_INF.  Replaces
 * LonestarGPU worklist drelax2 (lonestar/apps/sssp/kernel/sssp_port_kernel.cl:152-197,
 * lonestar/apps/sssp/sssp_port.cpp). */
int gdb_sssp(gdb_ctx* ctx, gdb_graph* g, uint32_t src, uint32_t* dist);
int gdb_sssp_device(gdb_ctx* ctx, gdb_graph* g, uint32_t src, uint32_t* d_dist);

/* Pannotia Jacobi SSSP costs (int32); unreached = GDB_PANNOTIA_BIG.  The
 * graph is the CSR pulled over (the reference passes the transpose).
 * Replaces mega_kernel (pannotia/graph_app/sssp/kernel/sssp_kernel.cl:170-244,
 * host pannotia/graph_app/sssp/sssp_gb.cpp:92-343). */
int gdb_sssp_jacobi(gdb_ctx* ctx, gdb_graph* g, uint32_t src, int32_t* cost);
int gdb_sssp_jacobi_device(gdb_ctx* ctx, gdb_graph* g, uint32_t src, int32_t* d_cost);

/* Maximal independent set: s_array[v] = 2 in the set, 0 otherwise, for
 * float priorities node_value.  Where a round lets no vertex join the set
 * (adjacent vertices of equal priority; a NaN priority, or one of 99999999
 * and above, never wins), the reference never terminates; this call stops
 * at that round and returns GDB_ERR_INVALID.  Replaces mega_kernel
 * (pannotia/graph_app/mis/kernel/mis_kernel.cl:220-337). */
int gdb_mis(gdb_ctx* ctx, gdb_graph* g, const float* node_value, int32_t* s_array);
int gdb_mis_device(gdb_ctx* ctx, gdb_graph* g, const float* d_node_value, int32_t* d_s_array);

/* Greedy colouring: color[v] = round in which v beat every uncoloured
 * neighbour (1-based).  Replaces mega_kernel
 * (pannotia/graph_app/color/kernel/color_kernel.cl:159-252). */
int gdb_color(gdb_ctx* ctx, gdb_graph* g, const float* node_value, int32_t* color);
int gdb_color_device(gdb_ctx* ctx, gdb_graph* g, const float* d_node_value, int32_t* d_color);

/* Betweenness centrality (float32) summed over the given sources, no halving
 * for undirected graphs.  Replaces mega_bc_kernel
 * (pannotia/graph_app/bc/kernel/bc_kernel.cl:431-513) restricted to a source
 * list; bc is overwritten.  gdb_bc checks the sources; gdb_bc_device
 * ignores sources >= V (they add nothing). */
int gdb_bc(gdb_ctx* ctx, gdb_graph* g, const uint32_t* sources, uint32_t nsrc, float* bc);
int gdb_bc_device(gdb_ctx* ctx, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc,
                  float* d_bc);

/* Minimum spanning forest (Boruvka) over the graph's weights (one weight
 * per edge, the same on both arcs; arcs of weight 1e9 and above are never
 * chosen); arc_in_mst (nullable, E bytes) marks one arc of every forest
 * edge.  With unique weights the forest is the reference's; with equal
 * weights it is a minimum forest of the same weight, whose edges may
 * differ.  Replaces the LonestarGPU MST host loop and kernels
 * (lonestar/apps/mst/mst_port.cpp:202-312, mst_common.cl:41-194,
 * mst_port_kernel.cl:35-82). */
int gdb_mst(gdb_ctx* ctx, gdb_graph* g, gdb_mst_result* result, uint8_t* arc_in_mst);
int gdb_mst_device(gdb_ctx* ctx, gdb_graph* g, gdb_mst_result* d_result, uint8_t* d_arc_in_mst);

/* ---------------------------------------------------------- graph files */
/* Readers of the reference's graph formats into host CSR arrays that the
 * library allocates (free with gdb_csr_free); no GPU involved.
 *   GDB_FMT_GR      Lonestar .gr version 1 binary
 *                   (lonestar_gpu_opencl/include/graph.h:143-215);
 *   GDB_FMT_DIMACS  "p sp V E" / "a u v w" text, 1-based
 *                   (pannotia/graph_parser/parse.cpp:178-282); directed = 0
 *                   adds every arc reversed too, as the reference's
 *                   undirected mode does;
 *   GDB_FMT_METIS   METIS adjacency text, 1-based, edge weights when the
 *                   format field ends in 1 (parse.cpp:59-176).
 * GDB_FMT_AUTO picks by extension (.gr, .graph/.metis, .dimacs/.txt/.coo).
 * Arcs keep their file order within a source; every vertex has a row (the
 * reference drops the rows of vertices without arcs).  w is NULL when the
 * file carries no weights.  Errors: GDB_ERR_INVALID with the reason in
 * gdb_io_last_error(), GDB_ERR_OOM. */
#define GDB_FMT_AUTO 0
#define GDB_FMT_GR 1
#define GDB_FMT_DIMACS 2
#define GDB_FMT_METIS 3
typedef struct {
  uint32_t V;
  uint64_t E;
  uint32_t* row_ptr; /* V + 1 */
  uint32_t* col;     /* E */
  uint32_t* w;       /* E or NULL */
} gdb_csr;
int gdb_csr_read(const char* path, int format, int directed, gdb_csr* out);
void gdb_csr_free(gdb_csr* csr);
/* Write a CSR as a .gr version 1 file (weights as 4-byte edge data). */
int gdb_csr_write_gr(const char* path, const gdb_csr* csr);
const char* gdb_io_last_error(void);

/* ------------------------------------------------- schedule selector */
/* No reference counterpart.  A 12-32-32-6 ReLU MLP in FP32 (GDB_MLP_PARAMS
 * floats: feature shift[12], scale[12], W1[12][32], b1[32], W2[32][32],
 * b2[32], W3[32][6], b3[6]); its outputs are predicted log2 costs of the
 * options of a decision (0 push / 1 pull: a BFS level or an SSSP settle
 * superstep; 2 SSSP worklist, 3 SSSP near-far, 4 SSSP near-far 4x width,
 * 5 SSSP graph relaunch). */
#define GDB_MLP_FEATURES 12
#define GDB_MLP_OUTPUTS 6
#define GDB_MLP_PARAMS 1694

/* One BFS level as seen by the selector: its features, the mode it ran in
 * (0 push, 1 pull) and its duration (barrier to barrier, microseconds). */
typedef struct {
  float x[GDB_MLP_FEATURES];
  uint32_t mode;
  float us;
} gdb_level_trace;

/* Load (params != NULL) or clear the network used by GDB_SCHED_LEARNED. */
int gdb_selector_set(gdb_ctx* ctx, const float* params);
/* BFS with the mode of every level fixed (0 push, 1 pull) or chosen by
 * the loaded network (2), recording up to cap levels; *levels = levels
 * run.  Levels (dist) are the same for every mode. */
int gdb_bfs_trace(gdb_ctx* ctx, gdb_graph* g, uint32_t src, int mode, uint32_t* dist,
                  gdb_level_trace* trace, uint32_t cap, uint32_t* levels);
/* SSSP with the light/heavy split from src, the direction of every settle
 * superstep fixed (0 push, 1 pull) or chosen by the loaded network (2),
 * recording up to cap settle supersteps (features with decision kind 3, the
 * direction, the duration from the superstep's start to the next one's);
 * *settles = records written.  Distances are the same for every mode. */
int gdb_sssp_trace(gdb_ctx* ctx, gdb_graph* g, uint32_t src, int mode, uint32_t* dist,
                   gdb_level_trace* trace, uint32_t cap, uint32_t* settles);
/* Features of an SSSP run-level decision for g from nsrc sources. */
int gdb_sssp_features(gdb_ctx* ctx, gdb_graph* g, uint32_t nsrc, float* x);
/* Network outputs for n feature rows x[n][12] (host arrays). */
int gdb_mlp_forward(gdb_ctx* ctx, const float* params, const float* x, uint32_t n, float* y);
/* Masked squared loss L = sum(m * (y - t)^2) / sum(m) over rows x[n][12],
 * targets t[n][6], mask m[n][6], and its gradient over the whole blob
 * (the shift/scale entries get 0): CUDA forward/backward kernels with a
 * fixed reduction order (deterministic). */
int gdb_mlp_loss_grad(gdb_ctx* ctx, const float* params, const float* x, const float* t,
                      const float* m, uint32_t n, float* grad, double* loss);
/* Full-batch Adam on the GPU for `epochs` steps (lr, beta1 0.9, beta2
 * 0.999, eps 1e-8, weight decay wd on W1..W3); params updated in place,
 * *loss = loss before the last step (nullable). */
int gdb_mlp_train(gdb_ctx* ctx, float* params, const float* x, const float* t, const float* m,
                  uint32_t n, uint32_t epochs, float lr, float wd, double* loss);

/* ------------------------------------------------ multi-source forms */
/* No reference counterpart (they serve the batched form).  Every vertex
 * takes its level / distance from the nearest of the nsrc sources, as from
 * a super-source with zero-weight arcs to each of them; on a disjoint union
 * of graphs with one source per member graph this is every member's own
 * single-source answer.  Persistent barriers only (XF, XF_FIXED,
 * GRID_SYNC); other kinds return GDB_ERR_UNSUPPORTED.  The host forms check
 * the sources; the device forms ignore sources >= V. */
int gdb_bfs_multi(gdb_ctx* ctx, gdb_graph* g, const uint32_t* sources, uint32_t nsrc, uint32_t* dist);
int gdb_bfs_multi_device(gdb_ctx* ctx, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc,
                         uint32_t* d_dist);
int gdb_sssp_multi(gdb_ctx* ctx, gdb_graph* g, const uint32_t* sources, uint32_t nsrc, uint32_t* dist);
int gdb_sssp_multi_device(gdb_ctx* ctx, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc,
                          uint32_t* d_dist);

/* ------------------------------------------- independent many-source runs */
/* The single-source BFS / SSSP of each of n sources, source i's answer in
 * dist[i * V .. i * V + V): what n calls of gdb_bfs / gdb_sssp return (the
 * reference runs one source per call).  Under the XF barriers the runs are
 * spread over concurrent lanes -- streams with their own discovery
 * contexts, each launch with a share of the GPU's CTAs -- so that the
 * latency-bound supersteps of several sources overlap; other barrier kinds
 * run them one after another.  The host forms check the sources; the
 * device forms ignore sources >= V (their rows stay unreached). */
int gdb_bfs_sources(gdb_ctx* ctx, gdb_graph* g, const uint32_t* sources, uint32_t n, uint32_t* dist);
int gdb_bfs_sources_device(gdb_ctx* ctx, gdb_graph* g, const uint32_t* d_sources, uint32_t n,
                           uint32_t* d_dist);
int gdb_sssp_sources(gdb_ctx* ctx, gdb_graph* g, const uint32_t* sources, uint32_t n, uint32_t* dist);
int gdb_sssp_sources_device(gdb_ctx* ctx, gdb_graph* g, const uint32_t* d_sources, uint32_t n,
                            uint32_t* d_dist);

/* ---------------------------------------------------------- batched form */
/* No reference counterpart.  n host CSR graphs packed into one disjoint
 * union: member i's vertex v becomes vertex_offset[i] + v (vertex_offset:
 * n + 1 entries out, nullable).  w = NULL, or n weight arrays.  The union
 * must satisfy V < 2^31 and E < 2^32. */
int gdb_graph_create_batch(gdb_ctx* ctx, uint32_t n, const uint32_t* V, const uint64_t* E,
                           const uint32_t* const* row_ptr, const uint32_t* const* col,
                           const uint32_t* const* w, uint32_t* vertex_offset, gdb_graph** out);

#define GDB_BATCH_BFS 1u
#define GDB_BATCH_SSSP 2u
typedef struct gdb_batch gdb_batch;
/* Capture the persistent launches of `apps` (GDB_BATCH_* mask) over graph g
 * from the nsrc host sources (union vertex ids) into one CUDA graph, with a
 * workspace, result arrays, discovery context and barrier flags owned by
 * the batch.  Launch shape (block_size, max_ctas), lock, schedule and
 * timeout come from ctx's options at this call; the XF barrier uses the
 * combining XF form (valid on every replay).  g must outlive b. */
int gdb_batch_create(gdb_ctx* ctx, gdb_graph* g, uint32_t apps, const uint32_t* sources,
                     uint32_t nsrc, gdb_batch** out);
/* Replace the sources (same count) read by the next replay. */
int gdb_batch_set_sources(gdb_batch* b, const uint32_t* sources);
/* Replay on ctx's stream without waiting / wait for the replay, check the
 * device status and counters; *ms = device time of the replay (nullable). */
int gdb_batch_launch(gdb_batch* b);
int gdb_batch_wait(gdb_batch* b, double* ms);
int gdb_batch_run(gdb_batch* b, double* ms); /* launch + wait */
/* Copy the last replay's results to host arrays of V entries (NULL skips). */
int gdb_batch_results(gdb_batch* b, uint32_t* bfs_dist, uint32_t* sssp_dist);
/* Device array (V entries) of one app's results; NULL if not captured. */
const uint32_t* gdb_batch_device_result(gdb_batch* b, uint32_t app);
/* Arcs inspected and barrier intervals of one app in the last replay. */
int gdb_batch_app_stats(gdb_batch* b, uint32_t app, uint64_t* arcs, uint32_t* supersteps);
int gdb_batch_destroy(gdb_batch* b);

/* ------------------------------------------------------------- serving */
/* No reference counterpart.  A request loop over graphs resident in HBM
 * with continuous batching: a dispatcher thread admits queued requests, in
 * arrival order with bypass, into free slots as soon as a slot and the
 * request's device-memory footprint (result + workspace, first-fit in a
 * fixed pool) are free; each slot runs its request as a persistent launch
 * on its own stream with its own discovery context and barrier flags, so
 * requests admitted while others run overlap on the device.  Results are
 * those of gdb_bfs / gdb_sssp / gdb_bc from the same source. */
#define GDB_APP_BFS 1u
#define GDB_APP_SSSP 2u
#define GDB_APP_BC 3u
typedef struct gdb_server gdb_server;
typedef struct {
  uint64_t id;
  int32_t status;      /* GDB_OK or the request's error */
  uint32_t app, graph, src, slot;
  double queue_ms;     /* submit -> launch */
  double run_ms;       /* device time of the launch (CUDA events) */
  double total_ms;     /* submit -> result in the caller's buffer */
  uint64_t footprint;  /* device bytes held while running */
} gdb_request_info;
/* slots: concurrent requests (0 = 8); pool_bytes: device memory for
 * running requests (0 = 1 GiB); options (block size, CTA cap per launch,
 * lock, schedule, timeout) and the selector are taken from ctx. */
int gdb_server_create(gdb_ctx* ctx, uint32_t slots, uint64_t pool_bytes, gdb_server** out);
/* Register a resident graph created on ctx (weights needed for SSSP). */
int gdb_server_add_graph(gdb_server* s, gdb_graph* g, uint32_t* graph_id);
/* Queue a request; `out` (host, V entries: uint32 levels / distances, or
 * float BC scores) is written before the request completes.  Thread-safe.
 * GDB_ERR_CAPACITY if the footprint exceeds the whole pool. */
int gdb_server_submit(gdb_server* s, uint32_t graph_id, uint32_t app, uint32_t src, void* out,
                      uint64_t* request_id);
/* Completed requests since the last poll (up to max); *n = count. */
int gdb_server_poll(gdb_server* s, gdb_request_info* info, uint32_t max, uint32_t* n);
/* Block until every submitted request has completed (timeout_s <= 0: no
 * limit); GDB_ERR_TIMEOUT otherwise. */
int gdb_server_drain(gdb_server* s, double timeout_s);
int gdb_server_destroy(gdb_server* s);

/* ---------------------------------------------- Delaunay mesh refinement */
/* LonestarGPU DMR (lonestar_gpu_opencl/apps/dmr/dmr_port.cpp:160-316 host
 * loop over the refine kernel, dmr_port_kernel.cl:37-188, and
 * check_triangles, dmr_common.cl:144-187) as one persistent kernel over the
 * XF barrier.  Input: nnodes coordinates, nelements triples (triangles
 * counter-clockwise; a boundary segment's third node is GDB_DMR_SEGMENT).
 * Refines until no triangle has an angle below 30 degrees, with capacity
 * (maxfactor / 2) x nnodes nodes and maxfactor x nelements elements (the
 * reference's meshfiles.h:27,67).  A round's worklist is processed in chunks
 * of `chunk` items (1 .. GDB_DMR_MAX_CHUNK); the lowest item claiming an
 * element owns it and the winners take slots in item order, so the result
 * is deterministic and equals the same schedule run serially.  Outputs
 * (host, sized to the capacities): node coordinates, elements, neighbour
 * triples (GDB_DMR_SEGMENT = none), deleted flags; counts[5] = nodes,
 * elements, rounds, chunks, refinements.  GDB_ERR_CAPACITY when the mesh
 * outgrows the capacity or a cavity its slot. */
#define GDB_DMR_SEGMENT 1234567890u
#define GDB_DMR_MAX_CHUNK (1u << 16)
int gdb_dmr_refine(gdb_ctx* ctx, const double* x, const double* y, uint32_t nnodes,
                   const uint32_t* elements, uint32_t nelements, uint32_t maxfactor, uint32_t chunk,
                   double* x_out, double* y_out, uint32_t* elements_out, uint32_t* neighbours_out,
                   uint8_t* deleted_out, uint32_t* counts);

/* -------------------------------------------- allocation-free BFS variant */
/* No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory (a host whose own pool owns the GPU's
 * memory, a plug-in that must not trigger the device synchronisation of
 * cudaMalloc/cudaFree).  Same levels as gdb_bfs_device, from plain device
 * pointers, on the caller's stream (0 = default stream), without a
 * context, graph handle or workspace: queues, counters and the discovery
 * and barrier state live in one fixed device array inside the library
 * (about 8.6 MB, kept by every GPU that loads the library until the process
 * exits).  V above GDB_NOALLOC_MAX_VERTICES returns GDB_ERR_INVALID.
 * The first call on a device looks up that array's address and arms it.
 * All calls share the
 * array: calls that overlap on the GPU (other streams, other threads) race
 * and must be serialised by the caller.  Synchronous: every call waits
 * for its stream and reads the run's status back to host memory before it
 * returns. */
#define GDB_NOALLOC_MAX_VERTICES (1u << 20)
int gdb_bfs_noalloc(const uint32_t* d_row_ptr, const uint32_t* d_col, uint32_t V, uint64_t E,
                    uint32_t src, uint32_t* d_dist, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* GDB_H */
