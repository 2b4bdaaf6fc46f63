/*
 * tc.h — C ABI of the GB300 exact triangle-counting engine.
 *
 * Every entry point takes plain pointers and sizes, returns a tc_status and
 * never exits the process.  Graphs use the GraphMiner CSR layout of the
 * reference project: int64 row pointers (eidType) of length n+1 and int32
 * column indices (vidType); counts are uint64 (AccType).
 *
 * Reference interfaces replaced (paths are inside the reference project):
 *   - TCSolver(Graph&, uint64_t&, int, int)    multigpu.cu:780,
 *       successful_push_pull/multigpu_nvshmem_pushpull.cu:29 (declared main.cc:5)
 *       -> tc_count_dag (count an oriented graph, the TCSolver contract) and
 *          tc_count (orientation + count on the device in one call).
 *   - Graph::orientation()                      successful_push_pull/graph.cc:252-298
 *       -> tc_orient (same kept-edge rule, same neighbour order, on the GPU).
 *   - Graph::Graph(prefix, ...) file loading    successful_push_pull/graph.cc:4-55
 *       -> tc_load_graphminer / tc_save_graphminer / tc_csr_free.
 *   - GraphGPU::init (H2D copy)                 successful_push_pull/graph_gpu.h:84-137
 *       -> folded into tc_count / tc_count_dag when tc_csr.on_device == 0.
 *   - warp_vertex kernel + intersect_num        bs_warp_vertex.cuh:2-35
 *       -> the strategy kernels behind tc_count / tc_count_dag.
 *
 * Threading: a tc_ctx owns one CUDA stream and a grow-only device arena; it
 * is not thread-safe (use one ctx per host thread).  Results are bit-exact
 * and independent of the strategy selected for each tile.
 */
#ifndef TC_H_
#define TC_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tc_status {
  TC_OK = 0,
  TC_ERR_INVALID_ARG = 1,    /* null pointer, bad size, bad option            */
  TC_ERR_INVALID_GRAPH = 2,  /* non-monotone rowptr, id out of range, unsorted */
  TC_ERR_CUDA = 3,           /* a CUDA runtime call failed                     */
  TC_ERR_OOM = 4,            /* device or host allocation failed               */
  TC_ERR_IO = 5,             /* file missing, truncated or malformed           */
  TC_ERR_TIMEOUT = 6,        /* a bounded device-side wait gave up             */
  TC_ERR_UNSUPPORTED = 7,    /* size beyond the engine's index limits          */
  TC_ERR_NO_DEVICE = 8       /* no CUDA device is visible                      */
} tc_status;

/* Compressed sparse rows.  For tc_count / tc_orient the graph is the
 * symmetric adjacency of a simple undirected graph (each row sorted strictly
 * ascending, no self loops), i.e. what Graph::Graph loads.  For tc_count_dag
 * it is an oriented graph with sorted rows (what Graph::orientation leaves). */
typedef struct tc_csr {
  int64_t n;               /* vertices                                        */
  int64_t nnz;             /* column entries (2m for a symmetric graph)       */
  const int64_t *rowptr;   /* [n+1], rowptr[0] == 0, rowptr[n] == nnz         */
  const int32_t *colidx;   /* [nnz]                                           */
  int32_t on_device;       /* 1: device pointers; 0: host pointers            */
} tc_csr;

/* Intersection strategies ("arms") a 4096-edge tile can be run with.  Every
 * arm is exact; they differ only in speed. */
typedef enum tc_arm {
  TC_ARM_BSEARCH_4 = 0,    /* 4 lanes per edge, binary search short->long     */
  TC_ARM_BSEARCH_32 = 1,   /* one warp per edge, binary search short->long    */
  TC_ARM_MERGE_8 = 2,      /* 8-lane windowed merge-path                      */
  TC_ARM_MERGE_32 = 3,     /* 32-lane windowed merge-path                     */
  TC_ARM_HASH = 4,         /* warp hash of the row's out-list, flattened probes */
  TC_ARM_BITMAP = 5,       /* block bitmap of the row's id window + probes    */
  TC_ARM_GALLOP_4 = 6,     /* 4 lanes per edge, each gallops a run of keys    */
  TC_ARM_MPATH_2 = 7,      /* 2 lanes per edge split the merge path evenly    */
  TC_ARM_FLAT = 8,         /* warp walks 32 edges' lookup lists as one run    */
  TC_ARM_PULL = 9,         /* edges grouped by target: hash N+(v) once, probe
                              every in-edge's row suffix against it           */
  TC_NUM_ARMS = 10
} tc_arm;

typedef enum tc_selector {
  TC_SELECT_FIXED = 0,     /* degree thresholds: default, fallback, baseline  */
  TC_SELECT_LEARNED = 1,   /* MLP cost model loaded into the ctx              */
  TC_SELECT_FORCE = 2      /* every tile uses opts.force_arm                  */
} tc_selector;

#define TC_DEFAULT_TILE_EDGES 4096

typedef struct tc_opts {
  int32_t selector;          /* tc_selector                                    */
  int32_t force_arm;         /* arm for TC_SELECT_FORCE                        */
  int32_t record_tile_costs; /* 1: record per-tile SM-cycle cost (training)    */
  int32_t validate;          /* 1 (default): check ids/rowptr/sortedness       */
} tc_opts;

/* Per-call timings (device milliseconds from CUDA events on the ctx stream)
 * and plan statistics. */
typedef struct tc_stats {
  float ms_h2d, ms_validate, ms_orient, ms_plan, ms_count, ms_scatter, ms_d2h, ms_total;
  int64_t m;                       /* oriented edges                          */
  int64_t tiles;                   /* 4096-edge tiles                         */
  int64_t tiles_per_arm[TC_NUM_ARMS];
  int64_t kernel_launches;         /* engine kernels launched by the call     */
  uint64_t h2d_bytes, d2h_bytes;
  float ms_arm[TC_NUM_ARMS];       /* device time of each arm's kernel        */
  /* Algorithmic bytes of each arm's tiles: sum over its edges u->v of
   * 4*(d+(u) + d+(v)) + 4 (both out-lists read once, as in a merge, plus the
   * edge itself); alg_bytes adds 8*(n+1) for the row pointers. */
  uint64_t alg_bytes_arm[TC_NUM_ARMS];
  uint64_t alg_bytes;
  /* The PULL arm's probing kernel alone (its grouping and bit-row kernels
   * excluded) and the number of edges it grouped (0 when no tile chose it). */
  float ms_pull_kernel;
  uint64_t pull_edges;
} tc_stats;

/* ---- context ---------------------------------------------------------- */
typedef struct tc_ctx tc_ctx;

tc_status tc_ctx_create(int device, tc_ctx **out);
void tc_ctx_destroy(tc_ctx *ctx);
/* Last error text of the ctx (or of the library when ctx is NULL). */
const char *tc_last_error(const tc_ctx *ctx);
const char *tc_status_str(tc_status s);
void tc_opts_default(tc_opts *o);
/* Device arena bytes currently reserved by the ctx. */
int64_t tc_ctx_arena_bytes(const tc_ctx *ctx);
/* Block until the ctx stream is idle. */
tc_status tc_ctx_sync(tc_ctx *ctx);
/* The ctx's CUDA stream (a cudaStream_t), for callers that time the engine
 * with their own events on the stream it launches on. */
void *tc_ctx_stream(tc_ctx *ctx);

/* ---- hot path --------------------------------------------------------- */

/* Orientation of a symmetric graph: keep u->v iff deg(v) > deg(u) or
 * (deg(v) == deg(u) and v > u), neighbours in input order (graph.cc:252-298).
 * dag_rowptr [n+1] and dag_colidx [capacity] receive the original-id DAG, in
 * the memory kind of g->on_device.  *m_out = number of oriented edges. */
tc_status tc_orient(tc_ctx *ctx, const tc_csr *g, int64_t *dag_rowptr, int32_t *dag_colidx,
                    int64_t dag_capacity, int64_t *m_out);

/* Orient on the device (rank by (degree, id), relabel, compact) and count
 * triangles.  *total is overwritten.  edge_counts (optional, capacity
 * edge_capacity) receives |N+(u) n N+(v)| for every oriented edge in the
 * order tc_orient produces; memory kind follows g->on_device. */
tc_status tc_count(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts, uint64_t *total,
                   uint32_t *edge_counts, int64_t edge_capacity, tc_stats *stats);

/* Count triangles of an already oriented graph (rows sorted ascending), the
 * contract of the reference TCSolver on a USE_DAG graph: the sum over every
 * edge u->v of |N+(u) n N+(v)|.  edge_counts follows the input edge order. */
tc_status tc_count_dag(tc_ctx *ctx, const tc_csr *dag, const tc_opts *opts, uint64_t *total,
                       uint32_t *edge_counts, int64_t edge_capacity, tc_stats *stats);

/* One shard of tc_count_dag: the edges of rows [row_begin, row_end) of an
 * oriented graph, each counted against the whole graph (every row's list is
 * read where it lies), so *total is the sum over u in the range, v in
 * N+(u), of |N+(u) n N+(v)|.  Contiguous row ranges that cover [0, n) give
 * partial counts that add up to tc_count_dag's total, with no exchange but
 * that one sum.  It replaces the reference's split of the rows over GPUs
 * (vertex u to device u % device_count, multigpu.cu:827-843) and its host
 * gather of the per-device counts (multigpu.cu:930-941).  edge_counts
 * (optional, edge_capacity >= rowptr[row_end] - rowptr[row_begin]) receives
 * the range's per-edge counts in input order.  Validation, when enabled,
 * checks the whole graph. */
tc_status tc_count_dag_range(tc_ctx *ctx, const tc_csr *dag, int64_t row_begin, int64_t row_end,
                             const tc_opts *opts, uint64_t *total, uint32_t *edge_counts, int64_t edge_capacity,
                             tc_stats *stats);

/* Triangles through every vertex of a symmetric graph: vertex_counts[u]
 * (n entries, input ids, memory kind of g->on_device) = number of triangles
 * that contain u, and *total = number of triangles.  The per-vertex counts
 * the reference's CPU intersection (Graph::intersect_num, graph.cc:376-406)
 * is the building block of, e.g. for clustering coefficients
 * 2*t(u) / (deg(u)*(deg(u)-1)).  Runs the PULL arm on every tile (the
 * selector in opts is ignored; validate is honoured). */
tc_status tc_count_vertices(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts, uint64_t *total,
                            uint64_t *vertex_counts, tc_stats *stats);

/* Labelled intersections on the oriented graph: for every oriented edge
 * u->v, the common out-neighbours w with vertex_labels[w] == label
 * (Graph::intersect_num(v, u, label), graph.cc:376-391 with the label test);
 * *total sums them over all edges (the triangles whose highest vertex
 * carries the label).  vertex_labels: n bytes, input ids, memory kind of
 * g->on_device; edge_counts as for tc_count.  Runs the PULL arm on every
 * tile (the selector in opts is ignored; validate is honoured). */
tc_status tc_count_labelled(tc_ctx *ctx, const tc_csr *g, const uint8_t *vertex_labels, int32_t label,
                            const tc_opts *opts, uint64_t *total, uint32_t *edge_counts, int64_t edge_capacity,
                            tc_stats *stats);

/* ---- tuning --------------------------------------------------------------- */

/* Work-chunk sizes of the PULL arm: a warp takes up to `item` grouped edges
 * at a time, shrinking to `item_min` as the launch runs out of work
 * (defaults 512 and 128; 32 <= item_min <= item <= 65536).  Results do not
 * depend on them; speed does, per graph. */
tc_status tc_set_pull_chunks(tc_ctx *ctx, int32_t item, int32_t item_min);
tc_status tc_get_pull_chunks(const tc_ctx *ctx, int32_t *item, int32_t *item_min);

/* Autotuner for the PULL work chunks: counts g (the tc_count contract) with
 * each of the ncand candidate chunk sizes (item_min = max(32, item / 4)),
 * `reps` times each after one warm-up call, and keeps the candidate with the
 * lowest device time (CUDA events on the ctx stream, best of reps) in the
 * ctx.  ms[i] (optional, ncand entries) receives candidate i's time, *best
 * (optional) the chosen size.  Every candidate's total must agree, else
 * TC_ERR_INVALID_GRAPH is returned and the ctx keeps its previous sizes. */
tc_status tc_autotune_pull(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts, const int32_t *candidates,
                           int32_t ncand, int32_t reps, float *ms, int32_t *best);

/* Run-time tuning of one ctx.  Results never depend on it; speed does, per
 * graph.
 *   pull_item, pull_item_min  PULL work chunks (tc_set_pull_chunks)
 *   pull_block_tiles          4096-edge tiles per PULL source block: the hub
 *                             targets' in-edges are grouped per block of rows
 *                             so that the rows they probe stay in L2
 *                             (default 2560 = 42 MB of adjacency)
 *   pull_dense_num / _den     a hub-hub edge is counted by ANDing bit rows
 *                             when its row suffix holds more than num/den
 *                             entries per 32-bit word of the target's bitmap
 *                             (default 1/1)
 *   orient_blocks_per_sm      entry-chunk geometry of the orientation passes:
 *                             chunks per SM of the kept-count and placement
 *                             passes (default 6, the blocks resident per SM)
 * This replaces the reference's fixed launch shape (multigpu.cu:203-206,
 * grid from BLOCK_SIZE and the vertex count). */
typedef struct tc_tuning {
  int32_t pull_item, pull_item_min;
  int32_t pull_block_tiles;
  int32_t pull_dense_num, pull_dense_den;
  int32_t orient_blocks_per_sm;
} tc_tuning;

tc_status tc_get_tuning(const tc_ctx *ctx, tc_tuning *out);
/* Checks ranges: 32 <= item_min <= item <= 65536, 64 <= block_tiles <=
 * 1<<20, 1 <= dense_num, dense_den <= 64, 1 <= orient_blocks_per_sm <= 64. */
tc_status tc_set_tuning(tc_ctx *ctx, const tc_tuning *t);

/* Autotuner for the ctx's tuning: coordinate descent over the PULL chunk
 * size (256, 512, 1024), the source-block size (1280, 2560, 5120 tiles),
 * the dense ratio (1/2, 1/1, 2/1) and the orientation geometry (3, 6, 12
 * chunks per SM), one dimension at a time with the others at their best so
 * far.  Every trial counts g (the tc_count contract) once to warm up and
 * `reps` times, keeping the best device time (CUDA events on the ctx
 * stream); every trial must count the same triangles, else
 * TC_ERR_INVALID_GRAPH is returned and the ctx keeps its previous tuning.
 * best (optional) receives the chosen tuning, *best_ms its time and
 * *trials (optional) the number of settings timed. */
tc_status tc_autotune(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts, int32_t reps, tc_tuning *best,
                      float *best_ms, int32_t *trials);

/* ---- measurement ---------------------------------------------------------- */

/* L2 read ceiling of the ctx's GPU: one kernel reads a device buffer of
 * `bytes` (small enough to stay in L2, e.g. 32 MB) `passes` times with
 * 16-byte loads that bypass L1; *gbs = bytes * passes / kernel time (CUDA
 * events on the ctx stream, best of 5 launches after a warm-up).  The
 * roofline of the PULL arm, whose row suffixes and tables come mostly from
 * L2, is reported against it beside the HBM copy bandwidth. */
tc_status tc_l2_bandwidth(tc_ctx *ctx, int64_t bytes, int32_t passes, double *gbs);

/* ---- allocation-free variant ------------------------------------------- */

/* Size of the fixed device scratch array behind tc_count_dag_noalloc.  Every
 * GPU that loads the library holds it until the process exits. */
#define TC_NOALLOC_SCRATCH_BYTES (4u << 20)

/* No counterpart in the reference: an extra entry point for callers that
 * must not allocate device memory while counting — applications whose
 * runtime owns the whole GPU through its own memory pool (and forbids
 * cudaMalloc outside it), plugins loaded into such applications, and
 * latency-bound loops that cannot afford cudaMalloc's implicit device
 * synchronisation.  It counts the triangles of an oriented graph (the
 * tc_count_dag contract, sorted rows, ids in [0, n)) with no ctx and no
 * allocation of any kind: its scratch is a fixed static device array of
 * TC_NOALLOC_SCRATCH_BYTES, which caps m at about 536 million edges; larger
 * inputs are rejected with TC_ERR_UNSUPPORTED.
 *   rowptr [n+1], colidx [m], total [1] and the optional edge_counts [m] are
 *   DEVICE pointers on `device`; stream is a cudaStream_t (NULL: the legacy
 *   default stream).  The call is asynchronous: *total is valid once the
 *   stream has been synchronised.  Inputs are not validated on the device.
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress), and so does the first call after the device's
 * context has been replaced (cudaDeviceReset); make such a call before any
 * stream capture.
 * All calls share the one array and every call overwrites it: calls whose
 * work overlaps on the GPU (other streams or threads without ordering) race
 * and return wrong counts.  Errors are reported by tc_last_error(NULL). */
tc_status tc_count_dag_noalloc(int device, const int64_t *rowptr, const int32_t *colidx, int64_t n, int64_t m,
                               uint64_t *total, uint32_t *edge_counts, void *stream);

/* ---- batched path ------------------------------------------------------ */

/* A batch of graphs, each a symmetric CSR with local ids, concatenated:
 * graph g owns vertices [vtx_off[g], vtx_off[g+1]) and entries
 * [rowptr[vtx_off[g]], rowptr[vtx_off[g+1]]) of one global rowptr whose
 * values are global entry offsets; colidx values are LOCAL ids. */
typedef struct tc_batch {
  int64_t num_graphs;
  const int64_t *vtx_off;   /* [num_graphs+1]                                  */
  const int64_t *rowptr;    /* [vtx_off[num_graphs]+1]                         */
  const int32_t *colidx;    /* [rowptr[last]]                                  */
  int32_t on_device;
} tc_batch;

/* Count every graph of the batch in one pass of the engine over the batch's
 * disjoint union (one persistent launch per arm over (graph, tile) items).
 * totals [num_graphs] receives each graph's exact count (host memory). */
tc_status tc_batch_count(tc_ctx *ctx, const tc_batch *b, const tc_opts *opts, uint64_t *totals,
                         tc_stats *stats);

/* ---- learned selector -------------------------------------------------- */

#define TC_MLP_FEATURES 16
#define TC_MLP_HIDDEN 64

/* Per-tile features and per-arm costs of a graph, for training.  features is
 * [tiles][TC_MLP_FEATURES] float, costs is [tiles][TC_NUM_ARMS] float
 * (SM-cycles); both host memory with room for `capacity` tiles. */
tc_status tc_tile_profile(tc_ctx *ctx, const tc_csr *g, float *features, float *costs,
                          int64_t capacity, int64_t *tiles_out);

/* The arm the selector of `opts` picks for every tile of a graph (host
 * int32 array with room for `capacity` tiles). */
tc_status tc_plan_arms(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts, int32_t *arms, int64_t capacity,
                       int64_t *tiles_out);

/* Train the MLP cost model on the device (forward/backward/Adam kernels of
 * this library) from host arrays of features and costs; the trained weights
 * stay loaded in the ctx.  weight_decay is decoupled (AdamW: every step also
 * scales the weights by 1 - lr * weight_decay).  loss_out (optional)
 * receives the final loss. */
tc_status tc_selector_train(tc_ctx *ctx, const float *features, const float *costs,
                            int64_t tiles, int32_t epochs, float lr, float weight_decay,
                            uint64_t seed, float *loss_out);
/* Weights as a flat float blob (TC_MLP_PARAM_COUNT floats). */
#define TC_MLP_PARAM_COUNT (TC_MLP_FEATURES * TC_MLP_HIDDEN + TC_MLP_HIDDEN + \
                            TC_MLP_HIDDEN * TC_MLP_HIDDEN + TC_MLP_HIDDEN +   \
                            TC_MLP_HIDDEN * TC_NUM_ARMS + TC_NUM_ARMS)
tc_status tc_selector_set_weights(tc_ctx *ctx, const float *params, int64_t count);
/* The learned selector keeps the fixed rule's arm for a tile unless the cost
 * model predicts another arm at least `margin` cheaper in log2 cost (0: any
 * predicted gain switches; default 0).  The PULL decision always stays with
 * the fixed rule: a PULL tile's cost depends on how many of its targets'
 * in-edges other PULL tiles share, which per-tile profiles cannot show. */
tc_status tc_selector_set_margin(tc_ctx *ctx, float margin);
tc_status tc_selector_get_weights(tc_ctx *ctx, float *params, int64_t count);
/* Predicted per-arm costs for host feature rows (inference kernel). */
tc_status tc_selector_predict(tc_ctx *ctx, const float *features, int64_t rows, float *pred);
/* One forward+backward pass on a host mini-batch: loss and parameter
 * gradients (for checking against a CPU restatement). */
tc_status tc_selector_grad(tc_ctx *ctx, const float *params, const float *features,
                           const float *costs, int64_t rows, float *loss, float *grad);

/* ---- graph construction, generators and files --------------------------- */

/* Symmetrise + drop self loops + dedup an edge list into a sorted symmetric
 * CSR on the device.  src/dst host or device per on_device; rowptr [n+1] and
 * colidx [capacity] are outputs in the same memory kind. */
tc_status tc_csr_from_edges(tc_ctx *ctx, int64_t n, int64_t num_edges, const int32_t *src,
                            const int32_t *dst, int32_t on_device, int64_t *rowptr,
                            int32_t *colidx, int64_t capacity, int64_t *nnz_out);

/* Count the triangles of an undirected edge list (COO; duplicates, both
 * directions and self loops allowed), the reference's edge-list input form
 * (Graph::init_edgelist, successful_push_pull/graph.cc:316-345): the list is
 * symmetrised and deduplicated on the device (tc_csr_from_edges), then
 * oriented and counted as tc_count does.  src/dst host or device per
 * on_device; *total is overwritten. */
tc_status tc_count_edges(tc_ctx *ctx, int64_t n, int64_t num_edges, const int32_t *src, const int32_t *dst,
                         int32_t on_device, const tc_opts *opts, uint64_t *total, tc_stats *stats);

/* Seeded generators (counter-based RNG, identical on host and device). */
typedef enum tc_gen_kind { TC_GEN_ER = 0, TC_GEN_RMAT = 1, TC_GEN_RGG = 2, TC_GEN_CHUNG_LU = 3 } tc_gen_kind;
typedef struct tc_gen_params {
  int32_t kind;            /* tc_gen_kind                                     */
  int64_t n;               /* vertices (RMAT: ignored, n = 2^scale)           */
  int32_t scale;           /* RMAT scale                                      */
  double avg_degree;       /* ER / RGG / Chung-Lu target average degree       */
  double edge_factor;      /* RMAT edges per vertex                           */
  double a, b, c;          /* RMAT quadrant probabilities (d = 1-a-b-c)       */
  double gamma;            /* Chung-Lu degree exponent                        */
  uint64_t seed;
} tc_gen_params;

/* Number of edge samples the generator draws (RGG: an upper bound). */
int64_t tc_gen_num_samples(const tc_gen_params *p);
/* Vertex count of the generated graph. */
int64_t tc_gen_num_vertices(const tc_gen_params *p);
/* Draw edge samples on the host (OpenMP).  *count_out = samples written. */
tc_status tc_gen_edges_host(const tc_gen_params *p, int32_t *src, int32_t *dst, int64_t capacity,
                            int64_t *count_out);
/* Same samples drawn by a device kernel into device buffers (ER, RMAT, CL). */
tc_status tc_gen_edges_device(tc_ctx *ctx, const tc_gen_params *p, int32_t *src, int32_t *dst,
                              int64_t capacity, int64_t *count_out);
/* A seeded batch of small graphs of mixed families for tc_batch_count:
 * graph g draws n log-uniform in [n_min, n_max] and an average degree
 * uniform in [deg_min, deg_max]; families cycle Erdos-Renyi, R-MAT
 * (a, b, c; n rounded to the nearest power of two) and random geometric.
 * Built in parallel over graphs (OpenMP).  vtx_off [num_graphs+1] is caller
 * memory; rowptr/colidx are malloc'd (tc_csr_free). */
typedef struct tc_batch_spec {
  int64_t num_graphs;
  int64_t n_min, n_max;
  double deg_min, deg_max;
  double a, b, c;
  uint64_t seed;
} tc_batch_spec;
tc_status tc_gen_batch_host(const tc_batch_spec *spec, int64_t *vtx_off, int64_t **rowptr_out,
                            int32_t **colidx_out, int64_t *nnz_out);
/* Host symmetric CSR builder (sort + unique), the host twin of
 * tc_csr_from_edges, for callers without a device. */
tc_status tc_csr_from_edges_host(int64_t n, int64_t num_edges, const int32_t *src,
                                 const int32_t *dst, int64_t **rowptr_out, int32_t **colidx_out,
                                 int64_t *nnz_out);

/* GraphMiner on-disk format (graph.cc:31-55): prefix.meta.txt with
 * "n nnz vid_size eid_size vlabel_size elabel_size max_degree feat_len
 * num_vertex_classes num_edge_classes", prefix.vertex.bin int64[n+1],
 * prefix.edge.bin int32[nnz].  Loaded arrays are malloc'd host memory
 * released with tc_csr_free. */
tc_status tc_load_graphminer(const char *prefix, int64_t *n, int64_t *nnz, int64_t **rowptr,
                             int32_t **colidx, int64_t *max_degree);
tc_status tc_save_graphminer(const char *prefix, int64_t n, int64_t nnz, const int64_t *rowptr,
                             const int32_t *colidx);
void tc_csr_free(int64_t *rowptr, int32_t *colidx);
/* Vertex labels of a GraphMiner graph: prefix.vlabel.bin, one byte per
 * vertex (graph.cc, "read vertex labels"); saving also records the label
 * size and class count in prefix.meta.txt, which must exist. */
tc_status tc_load_vlabels(const char *prefix, int64_t n, uint8_t *labels);
tc_status tc_save_vlabels(const char *prefix, int64_t n, const uint8_t *labels);

/* One partition of a METIS-partitioned GraphMiner graph, the files the
 * reference's partitioner writes (PartitionedGraph::metis_write_into_file,
 * successful_push_pull/graph_partition.cc:501-594) and its partitioned
 * loader reads (successful_push_pull/graph.cc:16-58 under USE_METIS):
 *   prefix.meta.txt         n n_real nnz max_subg_nv max_subg_ne max_degree
 *   prefix.vertex.bin       int64[n+1]: rows of all n vertices, only the
 *                           partition's own vertices have entries
 *   prefix.edge.bin         int32[nnz]: neighbours, global ids
 *   prefix.vertex_list.bin  int32[n_real]: the partition's own vertices
 *   prefix.part.bin         int64[n]: the partition of every vertex
 * prefix names one file set, e.g. "<graph dir>/metis/pgraph0".  The
 * partitioner runs on the oriented graph (metis_partition.cc:11), so the
 * rows are out-lists of the degree-ordered DAG.  Read-only here: building
 * partitions needs libmetis, which this engine does not use. */
typedef struct tc_metis_part {
  int64_t n, n_real, nnz, max_subg_nv, max_subg_ne, max_degree;
  int64_t *rowptr;       /* [n+1]    malloc'd                                 */
  int32_t *colidx;       /* [nnz]    malloc'd                                 */
  int32_t *vertex_list;  /* [n_real] malloc'd                                 */
  int64_t *part;         /* [n]      malloc'd                                 */
} tc_metis_part;

/* Read one partition; checks the sizes against the meta file and that the
 * rows are monotone with ids in [0, n).  Release with tc_metis_part_free. */
tc_status tc_load_metis_part(const char *prefix, tc_metis_part *out);
void tc_metis_part_free(tc_metis_part *p);

/* The whole oriented graph from its num_parts partition file sets
 * prefix0 .. prefix{num_parts-1} (prefix e.g. "<graph dir>/metis/pgraph"):
 * row v comes from the partition that owns v.  Checks that every file set
 * has the same n and part table, that part values lie in [0, num_parts),
 * that each vertex_list is exactly the partition's vertices in ascending
 * order and that only owned rows hold entries.  The sets are read one at a
 * time, twice (checks and row lengths, then the rows): memory is the result
 * plus one set.  rowptr/colidx are released with tc_csr_free, part
 * (optional, int64[n]) with tc_host_free. */
tc_status tc_assemble_metis(const char *prefix, int32_t num_parts, int64_t *n, int64_t *nnz, int64_t **rowptr,
                            int32_t **colidx, int64_t **part);
void tc_host_free(void *p);

/* Which partition an edge u->v's intersection is credited to. */
typedef enum tc_part_rule {
  /* part[u]: the owner of the row (the local loop of the reference's
   * partitioned solver, successful_push_pull/bs_warp_vertex_nvshmem.cuh:25-40,
   * and its pull path, :133-136) */
  TC_PART_BY_SOURCE = 0,
  /* the reference's push/pull split: an edge whose ends lie in different
   * partitions with d+(u) < d+(v) is pushed to and counted by part[v]
   * (bs_warp_vertex_nvshmem.cuh:127-132 and the receiver, :224-232); every
   * other edge by part[u] */
  TC_PART_PUSH_PULL = 1
} tc_part_rule;

/* Per-partition partial counts on an oriented graph (the tc_count_dag
 * contract) whose vertices are split by part[v] in [0, num_parts):
 * part_totals[p] = sum of |N+(u) n N+(v)| over the edges u->v that `rule`
 * credits to p, i.e. what PE p of the reference's partitioned solver adds to
 * its total; *total = their sum.  part: int64[n] (the part.bin type), memory
 * kind of dag->on_device; part_totals: uint64[num_parts], host memory.  A
 * part value outside [0, num_parts) is rejected with TC_ERR_INVALID_ARG. */
tc_status tc_count_dag_parts(tc_ctx *ctx, const tc_csr *dag, const int64_t *part, int32_t num_parts,
                             int32_t rule, const tc_opts *opts, uint64_t *total, uint64_t *part_totals,
                             tc_stats *stats);

/* Host CSR checks: rowptr monotone, ids in range, rows strictly ascending,
 * no self loops (the contract of tc_count). */
tc_status tc_check_csr_host(int64_t n, int64_t nnz, const int64_t *rowptr, const int32_t *colidx,
                            int32_t require_sorted_simple);

#ifdef __cplusplus
}
#endif
#endif /* TC_H_ */
