/*
 * gx.h — C ABI of the GB300-native GraphMP hot path.
 *
 * The reference's operator interface is a C++ template engine,
 * GraphPS<T> (GraphMP/system/GraphPS.h:22-63), driven as
 *   init(path, V, P, maxIter)   (GraphPS.h:77)
 *   run()                       (GraphPS.h:171)
 * with a vertex program plugged in through the function pointer _comp
 * (GraphPS.h:25-34) and the virtual init_vertex() (GraphPS.h:60).  This ABI
 * replaces that engine: the shard files, vertex arrays, vertex programs and
 * termination rule are the reference's, the execution is CUDA on one GB300.
 * Every function returns gx_status; no C++ exception crosses this boundary;
 * gx_last_error() returns a thread-local message for the last failure.
 *
 * Plain pointers and sizes only.  Host pointers unless a parameter says
 * "device".  One gx_engine per host thread.
 */
#ifndef GX_H_
#define GX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gx_status {
  GX_OK = 0,
  GX_ERR_INVALID = 1,  /* bad argument */
  GX_ERR_IO = 2,       /* file missing / short read (reference: abort(), cnpy.h:131-134) */
  GX_ERR_FORMAT = 3,   /* shard header or .npy header mismatch */
  GX_ERR_OOM = 4,      /* device or pinned allocation failed */
  GX_ERR_CUDA = 5,     /* CUDA runtime error */
  GX_ERR_TIMEOUT = 6,  /* a bounded device-side wait gave up */
  GX_ERR_NODEVICE = 7, /* no CUDA device visible */
  GX_ERR_STATE = 8     /* call out of order (e.g. run before load) */
} gx_status;

/* Vertex programs.  GraphMP binds these through GraphPS<T>::_comp. */
typedef enum gx_app {
  /* comp_pagerank<float> (GraphMP/app/pagerank.cpp:20-84): FP32 pull sum of
   * Msg[u]/outdeg[u] (outdeg clamped to >=1), new = (double)acc*0.85 + 1.0/N
   * stored as float, init 1/N, dangling mass dropped. */
  GX_APP_PAGERANK_REF = 0,
  /* Standard PageRank: r' = (1-d)/N + d*(sum r[u]/outdeg[u] + D/N) with D the
   * rank held by vertices of out-degree 0.  No reference counterpart. */
  GX_APP_PAGERANK_STD = 1,
  /* comp_sssp<int32_t> (GraphMP/app/sssp.cpp:20-75): pull min-plus.  Unit
   * weights with INF = GPS_INF = 10000 (GraphMP/system/Global.h:50), or
   * uint32 weights with INF = 0xFFFFFFFF and saturating add. */
  GX_APP_SSSP = 2,
  /* comp_cc<int32_t> (GraphMP/app/cc.cpp:20-75): pull min-label, init l[v]=v. */
  GX_APP_CC = 3,
  /* comp_pagerank in GraphMP/app/cal.cpp:20-58: value = in-degree. */
  GX_APP_INDEGREE = 4
} gx_app;

typedef struct gx_engine gx_engine;

typedef struct gx_config {
  int32_t device;              /* CUDA device ordinal (default 0) */
  int64_t cache_budget_bytes;  /* HBM shard-cache budget for edge data; <0 = unlimited.
                                  Replaces EDGE_CACHE_SIZE (GraphMP/system/Global.h:52). */
  int32_t stream_slots;        /* device slots in the streaming ring (>=2, default 4) */
  int32_t copy_streams;        /* H2D copy streams the slots alternate over (default 1) */
  double selective_threshold;  /* BF_THRE (GraphMP/system/Global.h:57), default 0.001 */
  int32_t heavy_degree;        /* in-degree above which a vertex gets its own warp units, split
                                  into 2048-edge chunks (default 4096, minimum 32) */
  int32_t tile_edges;          /* edge cap of one warp tile (default 2048) */
  int32_t exact_order;         /* 1: fold every vertex's in-edges in edge order, as the reference's
                                  sequential loop does (PageRank bit-exact); 0: tree sums for
                                  vertices above heavy_degree (default 0) */
  int32_t push_sparse;         /* SSSP/CC: push over out-edges when selective (default 1) */
  int32_t use_graph;           /* replay the iteration loop as a CUDA graph (default 1) */
  uint32_t wait_limit;         /* polls (each of at least 64 ns) a device-side wait makes before it gives
                                  up and the call returns GX_ERR_TIMEOUT; bounds the CTA-team barrier
                                  of gx_batch_run and the grid barrier of gx_ppr (default 1<<24, over
                                  a second) */
  int32_t verbose;             /* per-iteration log lines on stderr (default 0) */
  int32_t profile;             /* time every pull launch with CUDA events (default 0) */
  int32_t compress_cache;      /* with a budget the plain shards exceed: keep every shard compressed
                                  (source ids as per-32-edge byte offsets from their minimum, weights as
                                  bytes when all fit), in HBM while the budget lasts and streamed
                                  otherwise; decoded in the pull kernel, same results as plain
                                  shards (default 1) */
  double push_edge_fraction;   /* SSSP/CC with push_sparse: also push when the frontier's out-edges are
                                  at most this fraction of E (default 0.5; 0 = push only when the
                                  step is selective, as the reference schedules it) */
  int32_t hot_vertices;        /* resident pull steps: sources [0, hot_vertices) are gathered from a
                                  table in shared memory, filled at the start of each pull launch
                                  (capped by the shared memory of one CTA; 0 = off, the default) */
  int32_t relabel;             /* 1: a load without a shard-cache budget renumbers the vertices of each
                                  shard by descending in-degree, ties by id (each in-list keeps its
                                  order), so the pull kernel's tiles hold lists of like length and the
                                  hot sources share cache lines.  The order is computed and the source
                                  ids renamed on the device, beside the upload.  Every call still speaks the caller's numbering (values, start
                                  values, sources, CC labels, weights, checkpoints, PPR rows);
                                  gx_batch_run and gx_get_device_graph refuse such an engine.  Ignored
                                  when E >= 2^32 or when bits(V) + bits(P) + 12 > 64.
                                  0 = off (the default) */
} gx_config;

typedef struct gx_run_params {
  gx_app app;
  int32_t max_iter;      /* reference: GraphPS::init's MaxIteration */
  double damping;        /* PageRank d, default 0.85 (pagerank.cpp:48) */
  int32_t source;        /* SSSP source vertex (reference hard-codes 1, sssp.cpp:72) */
  int32_t weighted;      /* SSSP: 1 = weights from gx_set_weights, 0 = unit weight */
  double tolerance;      /* PageRank: also stop once the L1 residual < tolerance (0 = off) */
  int32_t use_init;      /* 1 = start from gx_set_init values instead of the app's init_vertex */
  int32_t first_step;    /* resume: number the first superstep this (use_init must be set; the
                            step counter, the step-0 comparison against 0 and the stop rule
                            then continue as in the interrupted run; default 0) */
  int32_t async_mode;    /* SSSP/CC: 1 = Gauss-Seidel supersteps that update values in place, as
                            GraphH's USE_ASYNC; same final values, fewer supersteps, per-step
                            counts differ from the reference's Jacobi loop (default 0) */
  int32_t checkpoint_every;        /* write the values every this many supersteps (0 = off) */
  const char* checkpoint_prefix;   /* ... to {prefix}{step}.npy, step = supersteps completed */
} gx_run_params;

typedef struct gx_run_stats {
  int32_t iterations;       /* supersteps executed (reference: `step` at exit) */
  int32_t push_iterations;  /* of those, sparse push supersteps */
  int64_t changed_last;     /* _Changed_Vertex of the last step */
  double residual_l1_last;  /* PageRank: sum |new-old| of the last step */
  int64_t edges_scanned;    /* edges read over all steps */
  double ms_total;          /* wall time of gx_run's superstep loop (device events) */
  double ms_copy;           /* streamed-shard H2D time (copy stream busy time) */
  double ms_compute;        /* compute stream busy time */
  double overlap;           /* copy/compute overlap fraction (streamed runs) */
  int64_t h2d_bytes;        /* shard bytes streamed from pinned host memory */
  int32_t shards_resident;  /* shards held in the HBM shard cache */
  int32_t shards_streamed;  /* shard visits served by the streaming ring */
  int32_t kernel_launches;  /* device kernels launched by this run */
  int32_t pull_launches;    /* of those, pull kernels of executed steps */
  double ms_pull;           /* summed pull-kernel time (config.profile only) */
} gx_run_stats;

typedef struct gx_iter_stats {
  int64_t changed;        /* reference _Changed_Vertex: computed value != previous value */
  int64_t active;         /* |{v : MsgNew[v] != Msg[v]}| (next frontier) */
  int32_t shards_active;  /* shards swept this step */
  int32_t mode;           /* 0 dense pull, 1 selective pull, 2 push */
  double residual_l1;     /* PageRank: sum |new-old| */
  double dangling;        /* PageRank STD: dangling mass D used by the NEXT step */
  int64_t edges_scanned;
} gx_iter_stats;

/* ---- engine (replaces GraphPS<T>, GraphMP/system/GraphPS.h:22-387) ---- */

void gx_config_default(gx_config* cfg);
void gx_run_params_default(gx_run_params* p, gx_app app);
const char* gx_last_error(void);

gx_status gx_create(const gx_config* cfg, gx_engine** out);
gx_status gx_destroy(gx_engine* e);

/* Changes the engine's config.wait_limit (>= 1) for its later calls.  No
 * reference counterpart: the reference has no device-side waits. */
gx_status gx_set_wait_limit(gx_engine* e, uint32_t polls);

/* Engines draw device memory from a per-device pool that keeps blocks after
 * gx_destroy, so the next engine's load maps no new memory.  This returns
 * the cached blocks of `device` to the driver.  No reference counterpart. */
gx_status gx_release_cached_memory(int32_t device);

/* Loads the reference's shard directory: {p}.edge.npy for p in [0,P), each a
 * 1-D int32 .npy of [E_p, len(indices), len(indptr), start, end, indices...,
 * indptr...] (GraphMP/system/Comp.h:33-42, written by
 * GraphMP/tools/format_spark.py:148-154), and vertexout.npy (int32[V],
 * GraphPS.h:162-169).  `dir` ends with '/', as GraphPS::init expects.
 * Replaces GraphPS::init (GraphPS.h:77-151) + load_edge (Global.h:129-255). */
gx_status gx_load_shards(gx_engine* e, const char* dir, int32_t V, int32_t P);

/* Loads an in-memory graph in the same shard layout, as one global CSC:
 * bounds[P+1] destination ranges, off[V+1] in-edge offsets, col[off[V]]
 * source ids, outdeg[V] (NULL = computed from col). */
gx_status gx_load_csc(gx_engine* e, int32_t V, int32_t P, const int32_t* bounds,
                      const int64_t* off, const int32_t* col, const int32_t* outdeg);

/* SSSP edge weights aligned with col (uint32, >= 1). */
gx_status gx_set_weights(gx_engine* e, const uint32_t* w);

/* Initial vertex values (T[V]: float for PageRank, int32 for SSSP/CC);
 * the init_vertex() override (GraphPS.h:60). Used when params.use_init. */
gx_status gx_set_init(gx_engine* e, const void* host_vals);

/* Superstep loop of GraphPS<T>::run (GraphPS.h:256-386). */
gx_status gx_run(gx_engine* e, const gx_run_params* params, gx_run_stats* stats);

/* Copies the final _VertexMsg (T[V]) to host memory. */
gx_status gx_get_values(gx_engine* e, void* host_out);

/* Checkpoint/resume of vertex state.  gx_write_values_npy writes the current
 * values as a 1-D .npy ('<f4' PageRank, '<u4' weighted SSSP, '<i4' otherwise);
 * gx_read_values_npy reads such a file of exactly n elements into `out`, to be
 * passed to gx_set_init and resumed with params.use_init and params.first_step.
 * gx_run also writes them every params.checkpoint_every supersteps.  The
 * reference has no checkpoints (GraphPS.h keeps vertex state in memory only). */
gx_status gx_write_values_npy(gx_engine* e, const char* path);
gx_status gx_read_values_npy(const char* path, int64_t n, void* out);

/* The engine's resident graph as device pointers, for vertex programs that
 * run on it from the caller's own kernels (include/gx_program.cuh): the
 * plug-in point that GraphPS<T>'s _comp function pointer and init_vertex()
 * are in the reference (GraphMP/system/GraphPS.h:25-34,60).  Valid until the
 * next load or gx_destroy; GX_ERR_STATE when some shard is not resident. */
typedef struct gx_device_graph {
  int32_t V;
  int32_t P;
  int64_t E;
  const int64_t* off;      /* device: in-edge offsets, V+1 */
  const int32_t* col;      /* device: source ids, E (+ 8 readable entries past the end) */
  const uint32_t* w;       /* device: weights aligned with col, or NULL without gx_set_weights */
  const int32_t* outdeg;   /* device: out-degree, V */
  const int32_t* bounds;   /* device: shard bounds, P+1 */
  void* stream;            /* cudaStream_t the engine computes on */
} gx_device_graph;

gx_status gx_get_device_graph(gx_engine* e, gx_device_graph* out);

/* Per-step statistics of the last gx_run (the reference logs these per
 * iteration, GraphPS.h:375-382). */
gx_status gx_get_iter_stats(gx_engine* e, int32_t step, gx_iter_stats* out);

/* Triangles of the loaded graph taken as undirected (load the CSC of a
 * symmetrised, deduplicated edge list).  Orients u->v iff (deg u, u) <
 * (deg v, v) and intersects sorted out-lists.  No reference counterpart:
 * GraphH/list/system/GraphPS.h:15-95 ("tc") counts reciprocal edges, not
 * triangles.  *total receives the exact count. */
gx_status gx_triangle_count(gx_engine* e, uint64_t* total, gx_run_stats* stats);

/* Personalized PageRank for k <= 64 sources at once, as one sparse x dense
 * product per step over the loaded CSC: R <- restart*S + (1-restart)*A^T
 * D^-1 R, R0 = S (one-hot columns), dangling mass dropped, FP32.  Every step
 * runs in one persistent launch (a grid barrier between steps, bounded by
 * config.wait_limit: GX_ERR_TIMEOUT when it gives up), replayed as a CUDA
 * graph; rows are k rounded up to 8 columns.  No reference counterpart
 * (PageRank's pull, pagerank.cpp:44-48, on k vectors).  host_out (nullable)
 * receives R as float[V][k], row-major. */
gx_status gx_ppr(gx_engine* e, int32_t k, const int32_t* sources, int32_t iters, double restart,
                 float* host_out, gx_run_stats* stats);

/* Launch schedule of the batched kernel (chosen by gx_batch_autotune). */
typedef struct gx_batch_tuning {
  int32_t threads;      /* threads per CTA (multiple of 32, 64..1024) */
  int32_t lane_max;     /* in-lists up to this length are walked by one lane */
  int32_t ctas_per_sm;  /* resident CTAs per SM requested */
} gx_batch_tuning;

void gx_batch_tuning_default(gx_batch_tuning* t);

/* Many independent graphs packed into the loaded CSC (instance i owns
 * vertices [inst_vbegin[i], inst_vbegin[i+1]) and only edges among them),
 * run in ONE persistent launch replayed as a CUDA graph: for each instance
 * the reference's PageRank (pagerank.cpp, N = instance size) for up to
 * pr_iters supersteps, then its min-label CC (cc.cpp) until no label
 * changes (at most cc_max_iter), each with GraphPS::run's stop rule
 * (GraphPS.h:383) per instance.  pr_out float[V], cc_out int32[V]
 * (instance-local labels), pr_steps / cc_steps int32[n_inst]; all
 * nullable.  No reference counterpart for the batching itself. */
gx_status gx_batch_run(gx_engine* e, int32_t n_inst, const int32_t* inst_vbegin, int32_t pr_iters,
                       int32_t cc_max_iter, double damping, const gx_batch_tuning* tuning,
                       float* pr_out, int32_t* cc_out, int32_t* pr_steps, int32_t* cc_steps,
                       gx_run_stats* stats);

/* Times the batched launch under candidate schedules (threads per CTA,
 * lane_max, CTAs per SM) on the loaded batch, returns the fastest, and
 * appends a JSON line with every candidate's time to table_path
 * (nullable). */
gx_status gx_batch_autotune(gx_engine* e, int32_t n_inst, const int32_t* inst_vbegin, int32_t pr_iters,
                            int32_t cc_max_iter, const char* table_path, gx_batch_tuning* best,
                            double* best_ms);

/* ---- learned PageRank warm start (no reference counterpart) ----
 * MLP 6 -> 64 -> 64 -> 1 (GELU in tanh form, softplus output normalised to sum 1) over
 * per-vertex degree features: log1p(indeg), log1p(outdeg), mean and max of
 * in-neighbours' log1p(outdeg), log1p(2-hop in-degree sum), dangling flag.
 * BF16 weights, FP32 accumulation; inference on the tensor cores. */
typedef struct gx_mlp gx_mlp;

typedef struct gx_warm_stats {
  int32_t used_warm;            /* 0: fell back to the uniform start */
  int32_t iterations;           /* supersteps to the tolerance (incl. the first) */
  double resid_uniform_first;   /* L1 residual of one step from 1/N */
  double resid_warm_first;      /* L1 residual of one step from the prediction */
  double resid_last;
  double ms_features, ms_mlp, ms_pagerank, ms_total;
} gx_warm_stats;

int32_t gx_mlp_num_params(void);
gx_status gx_mlp_create(int32_t device, uint64_t seed, gx_mlp** out);
gx_status gx_mlp_destroy(gx_mlp* m);
/* params float[gx_mlp_num_params()] (FP32 master: W1[64][6], b1[64],
 * W2[64][64], b2[64], w3[64], b3), norm float[12] (feature mean, 1/std). */
gx_status gx_mlp_get_params(gx_mlp* m, float* params, float* norm);
gx_status gx_mlp_set_params(gx_mlp* m, const float* params, const float* norm);
/* Adds up to max_samples vertices of the engine's graph to the training
 * set, with targets log(N * r_v) of standard PageRank run to `tolerance`. */
gx_status gx_mlp_add_graph(gx_mlp* m, gx_engine* e, int32_t max_samples, int32_t max_iter,
                           double tolerance);
/* Adam on the squared error of log softplus(z) against the targets,
 * weighted by min(N * r_v, 100). */
gx_status gx_mlp_train(gx_mlp* m, int32_t epochs, int32_t batch, double lr, double* final_loss);
/* Gradient of the mean loss over n samples (raw features x[n][6], targets
 * t[n]) at the current weights, float[gx_mlp_num_params()]. */
gx_status gx_mlp_grad(gx_mlp* m, const float* x, const float* t, int32_t n, float* grad, double* loss);
/* Predicted start vector (sums to 1) for the engine's graph, left on the
 * device for gx_pagerank_warm; host_out (nullable) receives a copy. */
gx_status gx_mlp_predict(gx_mlp* m, gx_engine* e, double damping, float* host_out, double* ms_features,
                         double* ms_mlp);
/* Standard PageRank to `tolerance` (L1 residual) from the MLP's start, or
 * from the uniform start when the predicted start's first-step residual is
 * worse than the uniform start's. */
gx_status gx_pagerank_warm(gx_engine* e, gx_mlp* m, int32_t max_iter, double tolerance, double damping,
                           gx_warm_stats* out);

/* PageRank with the reference's semantics (GX_APP_PAGERANK_REF, default
 * tree-sum mode) over a CSC the caller already holds in device memory, for
 * callers that cannot allocate device memory themselves or let a library do
 * it: a plugin inside a host application whose allocator owns the GPU, a
 * serving path that must not allocate per request, or a process that has
 * reserved the device for its own pool.  No counterpart in the reference.
 *
 * Allocates nothing: its scratch is a fixed 12.7 MB array in the library's
 * device image, present on every GPU that loads the library until exit,
 * which bounds V to 1,048,576 and max_iter to 1024 (larger sizes are
 * rejected with GX_ERR_INVALID).  d_off int64[V+1], d_col int32 with room for
 * num_edges + 4 entries (col_capacity; the last four are read but unused),
 * d_outdeg int32[V]; d_rank float[V] receives the ranks.  All device
 * pointers; `stream` is a cudaStream_t (NULL = legacy default stream).
 * The CSC must satisfy off[0] == 0, off non-decreasing, off[V] == num_edges
 * and 0 <= d_col[k] < V; a kernel checks this on the device before any other
 * kernel indexes with it and, when it fails, no superstep runs.  Only a call
 * that passes iterations_out waits for the result and then returns
 * GX_ERR_INVALID for such a CSC (with *iterations_out = 0).
 * The first call on each device looks up the scratch's device address with
 * that device current and caches it for the life of the process; make that
 * first call before any stream capture, and do not call this entry point
 * after cudaDeviceReset on that device (the cached address is then stale).
 * Every call reuses the same scratch and resets it first, so calls that may
 * overlap on the GPU (other streams, other host threads) race with each
 * other and must be serialised by the caller.  iterations_out (nullable)
 * synchronises the stream and returns the supersteps run. */
gx_status gx_pagerank_noalloc(const int64_t* d_off, const int32_t* d_col, int64_t num_edges,
                              int64_t col_capacity, const int32_t* d_outdeg, int32_t V,
                              int32_t max_iter, double damping, float* d_rank, void* stream,
                              int32_t* iterations_out);

/* ---- graph construction and the reference's on-disk format (host) ---- */

enum { GX_BUILD_DROP_SELF = 1, GX_BUILD_DEDUP = 2, GX_BUILD_SYMMETRIZE = 4 };

/* Seeded R-MAT edge list: n edges over 2^scale vertices, quadrant
 * probabilities a, b, c (d = 1-a-b-c).  Edge i is a pure function of
 * (seed, i), so any range of edges can be generated independently. */
gx_status gx_rmat_edges(int32_t scale, int64_t n, double a, double b, double c,
                        uint64_t seed, int64_t first, int32_t* src, int32_t* dst);

/* Builds the CSC (in-edges grouped by destination, sources ascending) of an
 * edge list.  col must hold n entries (2n with GX_BUILD_SYMMETRIZE).
 * *n_out receives off[V]. */
gx_status gx_build_csc(int32_t V, int64_t n, const int32_t* src, const int32_t* dst,
                       int32_t flags, int64_t* off, int32_t* col, int64_t* n_out);

/* gx_build_csc computed on a GPU (`device`): same arguments, same output,
 * bit for bit.  Keys (dst, src) are radix-sorted on the device and runs of
 * equal keys collapse; replaces the offline Spark job and cal.cpp's degree
 * pass (GraphMP/tools/format_spark.py, GraphMP/app/cal.cpp). */
gx_status gx_build_csc_gpu(int32_t device, int32_t V, int64_t n, const int32_t* src, const int32_t* dst,
                           int32_t flags, int64_t* off, int32_t* col, int64_t* n_out);

/* The CSC of gx_rmat_edges(scale, n, a, b, c, seed, 0, ...) built by
 * gx_build_csc(2^scale, ..., flags), with the edges generated and the CSC
 * built on the GPU.  col must hold n entries (2n with GX_BUILD_SYMMETRIZE). */
gx_status gx_rmat_csc_gpu(int32_t device, int32_t scale, int64_t n, double a, double b, double c, uint64_t seed,
                          int32_t flags, int64_t* off, int32_t* col, int64_t* n_out);

/* Edge-balanced destination-range shard boundaries, the rule of
 * GraphMP/tools/format_spark.py:91-108: bounds[i] = first v with
 * off[v] >= ceil(E/P)*i, bounds[0] = 0, bounds[P] = V. */
gx_status gx_partition_bounds(int32_t V, const int64_t* off, int32_t P, int32_t* bounds);

/* outdeg[u] = number of CSC entries with source u. */
gx_status gx_out_degree(int32_t V, const int64_t* off, const int32_t* col, int32_t* outdeg);

/* Writes {p}.edge.npy, vertexout.npy and vertexin.npy in the reference layout. */
gx_status gx_write_shards(const char* dir, int32_t V, int32_t P, const int32_t* bounds,
                          const int64_t* off, const int32_t* col, const int32_t* outdeg);

/* Reads a shard directory into a global CSC (the host half of gx_load_shards).
 * Call first with off/col NULL to get *E_out; then with buffers. */
gx_status gx_read_shards(const char* dir, int32_t V, int32_t P, int32_t* bounds,
                         int64_t* off, int32_t* col, int32_t* outdeg, int64_t* E_out);

/* Edge-list text file ("src dst" per line, '#' or '%' comments) to the
 * reference's shard directory: replaces the offline Spark job
 * (GraphMP/tools/format_spark.py), with the same edge-balanced partition
 * rule.  flags as gx_build_csc; *n_edges_out receives the edges kept. */
gx_status gx_convert_edge_list(const char* path, int32_t V, int32_t P, int32_t flags, const char* out_dir,
                               int64_t* n_edges_out);

/* Seeded SSSP weights in [1,255], a pure function of (seed, u, v). */
gx_status gx_edge_weights(uint64_t seed, int32_t V, const int64_t* off, const int32_t* col,
                          uint32_t* w);

#ifdef __cplusplus
}
#endif
#endif /* GX_H_ */
