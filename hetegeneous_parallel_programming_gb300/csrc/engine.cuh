// Engine-internal interfaces between orient.cu, count.cu, mlp.cu and capi.cu.
#pragma once
#include "dev_common.cuh"

namespace tc {

constexpr int TILE_EDGES = TC_DEFAULT_TILE_EDGES;   // selector granularity
constexpr int ENTRY_TILE = 2048;                    // orientation tile (entries)

// Validation flag bits (ctx->d_flags[0]).
enum : unsigned {
  VF_ROWPTR_ENDS = 1u,     // rowptr[0] != 0 or rowptr[n] != nnz
  VF_ROWPTR_ORDER = 2u,    // rowptr not monotone
  VF_ID_RANGE = 4u,        // column id outside [0, n)
  VF_SELF_LOOP = 8u,
  VF_UNSORTED = 16u,       // row not strictly ascending (or duplicate)
  VF_TIMEOUT = 32u,        // a bounded device wait gave up
  VF_PART_RANGE = 64u      // a partition id outside [0, num_parts)
};

// A CSR resident on the device.
struct DevCSR {
  int64_t n = 0, nnz = 0;
  const int64_t *rowptr = nullptr;
  const int32_t *col = nullptr;
};

// An oriented graph ready for counting.  For the relabelled DAG of tc_count
// (restrict_after = 1) every edge r->s has s > r and rows are sorted, so only
// the part of N+(r) after s can meet N+(s).
struct DevDag {
  int64_t n = 0, m = 0;
  const int64_t *rowptr = nullptr;   // [n+1]
  const int32_t *col = nullptr;      // [m]
  const int32_t *src = nullptr;      // [m] row of each edge
  const uint32_t *perm = nullptr;    // [m] output slot of each edge (null: identity)
  const int32_t *indeg = nullptr;    // [n] in-degree of each vertex in the DAG (caller-oriented DAGs)
  const int2 *dv = nullptr;          // [n] (out-degree, in-degree) of each vertex (relabelled DAGs)
  uint32_t *top = nullptr;           // [m] per-vertex mode: triangles in which edge e joins the
                                     // lowest and the highest vertex (PULL arm only)
  const uint8_t *vlabel = nullptr;   // [n] labelled mode: vertex labels (relabelled ids; PULL arm only)
  int label = 0;                     // labelled mode: count common neighbours with this label
  int restrict_after = 0;
  unsigned *flags = nullptr;         // VF_* error bits (ctx->d_flags): a bounded device wait that gave up
  // PULL dense edges: bit rows of the DAG rows of the top hub ids, one row of
  // hub_wpr4 16-byte words per hub (null: dense path off)
  const uint4 *hub_bits = nullptr;
  int hub_wpr4 = 0;
};

// Validation: sets VF_* bits in ctx->d_flags[0].
tc_status launch_validate(tc_ctx *ctx, const DevCSR &g, bool require_sorted_simple);
tc_status launch_validate_rowptr(tc_ctx *ctx, const DevCSR &g);
// in-degree of every vertex of a caller-oriented DAG (histogram of col)
tc_status launch_indeg(tc_ctx *ctx, const int32_t *col, int64_t n, int64_t m, int32_t *indeg);

// Orientation.  Phase A (before the host learns m): degree keys, rank sort,
// kept counts per row and per block.  Phase B: compaction + relabel sort.
struct OrientBufs {
  // phase A
  uint64_t *vkeys0, *vkeys1;   // [n]
  int32_t *rank;               // [n]
  int64_t *kept;               // [n+1] kept out-degree per original row
  int64_t *bcount;             // [G+1] kept per block chunk
  int64_t *d_m;                // [1]
  void *sort_scratch;          // radix + scan scratch
  int64_t *orowptr;            // [n+1] original-order DAG row pointers
  int64_t *nrowptr;            // [n+1] relabelled row pointers
  int64_t *dnew;               // [n+1] relabelled row lengths
  int2 *dv;                    // [n] (out-degree, in-degree) per relabelled vertex
  int32_t *mid_list, *big_list, *huge_list;  // [n] rows for the warp / block / global sorts
  unsigned *seg_counts;        // [4]: mid, big, huge rows; big rows left to the block sort
  int32_t *rv = nullptr;       // [nnz] rank of every entry's target, written by the kept-count pass
  // phase B
  int32_t *ncol, *nsrc;        // [m]
  uint32_t *perm;              // [m] original slot of each relabelled edge (optional)
  int32_t *dag_col;            // optional original-id DAG output [m]
  int G;                       // blocks of the entry-chunk kernels
  int64_t chunk;
  // optional vertex groups (batched graphs): ranks sort by (group, degree,
  // id), so every group owns the contiguous rank range of its vertices.
  const int32_t *vgroup = nullptr;
  int group_bits = 0;
  // batched graphs whose column ids are local: the kept-count pass adds
  // vtx_off[vgroup[u]] to every id of row u (and range-checks it); only the
  // kept-count pass reads the column array then (the placement streams the
  // target ranks it wrote)
  const int64_t *vtx_off = nullptr;
  // check ids, sortedness and self loops inside the kept-count pass
  bool validate = false;
  // column array arriving in `pieces` uploads (ctx->piece_ev): piece k is
  // blocks [k * ceil(G / pieces), ...) of the entry-chunk geometry, and the
  // kept-count pass runs piece by piece as they land
  int pieces = 1;
};
// Entry-chunk geometry: about 6 resident blocks per SM, times `pieces` when
// the column array arrives in pieces (each piece then fills the GPU).
void orient_geometry(const tc_ctx *ctx, int64_t nnz, int pieces, int *G, int64_t *chunk);
tc_status orient_phase_a(tc_ctx *ctx, const DevCSR &g, OrientBufs &b);
// out == nullptr: only the original-id DAG columns (b.dag_col) are written.
tc_status orient_phase_b(tc_ctx *ctx, const DevCSR &g, OrientBufs &b, int64_t m, bool want_perm,
                         bool want_dag_cols, DevDag *out);

// Row of every entry of a CSR (for counting a caller-oriented DAG).
tc_status launch_expand_src(tc_ctx *ctx, const int64_t *rowptr, int64_t n, int64_t m, int32_t *src);
tc_status launch_shift_rowptr(tc_ctx *ctx, const int64_t *rowptr, int64_t n, int64_t shift, int64_t *out);

// Counting.
struct CountBufs {
  float *features;        // [T][TC_MLP_FEATURES]
  uint64_t *qkeys0, *qkeys1;  // [T]
  uint32_t *qvals0, *qvals1;  // [T]
  int32_t *arm;           // [T]
  int64_t *qoff;          // [TC_NUM_ARMS+1]
  unsigned long long *tile_cycles;  // [T] (optional)
  unsigned long long *tile_bytes;   // [T] algorithmic bytes per tile
  unsigned long long *arm_bytes;    // [TC_NUM_ARMS]
  uint32_t *pull_pos;     // [keys+1] PULL grouping: key counts, then group offsets
  uint2 *pull_er;         // [m] PULL grouping: (edge id, row) grouped by key (source block, target)
  uint4 *hub_bits;        // [hub rows][hub words / 4] PULL dense edges: bit rows of the hubs' out-lists
  void *sort_scratch;
};
size_t count_scratch_bytes(const tc_ctx *ctx, int64_t n, int64_t m);
// out[rank[u]] = in[u] for n one-byte values (vertex labels into relabelled ids)
tc_status launch_relabel_u8(tc_ctx *ctx, const uint8_t *in, const int32_t *rank, int64_t n, uint8_t *out);
// per-vertex triangle counts from the per-edge and top counts of a relabelled
// DAG, written per input id (rank[u] is u's relabelled id); t is [n] scratch
tc_status launch_vertex_sums(tc_ctx *ctx, const DevDag &g, const uint32_t *c, const uint32_t *top,
                             unsigned long long *t, const int32_t *rank, unsigned long long *out);
// Per-partition sums of the per-edge counts c: out[p] += c[e] for the edges
// that `rule` (tc_part_rule) credits to partition p; part ids are checked
// (VF_PART_RANGE).  out: num_parts device counters, zeroed here.
tc_status launch_part_sums(tc_ctx *ctx, const DevDag &g, const uint32_t *c, const int64_t *part, int num_parts,
                           int rule, unsigned long long *out);
tc_status count_carve(const tc_ctx *ctx, int64_t n, int64_t m, Bump &bump, CountBufs &cb, bool want_cycles);
// Enqueues plan, queue build and every arm kernel on the ctx stream (no host
// sync, so it can be captured into a CUDA graph); adds the count into
// ctx->d_total (which the caller zeroes) and writes per-edge counts to
// out[perm[e]] when out is set.  The queue offsets land in pinned host
// memory; count_stats reads them (and the timing events) after a sync.
tc_status run_count(tc_ctx *ctx, const DevDag &dag, const tc_opts &opts, CountBufs &cb, uint32_t *out, bool timing);
void count_stats(tc_ctx *ctx, tc_stats *st, bool timing);

// Shared by the entry points (capi.cu, batch.cu).
// pieces > 1 (host input only): rowptr is copied on the ctx stream, the
// column array in `pieces` uploads on ctx->copy_stream, each recording
// ctx->piece_ev[k]; the orientation's kept-count pass waits for them.
tc_status stage_csr(tc_ctx *ctx, const tc_csr *g, Bump &bump, DevCSR &d, uint64_t *h2d, int pieces = 1);
void orient_sizes(const tc_ctx *ctx, int64_t n, int64_t nnz, bool perm, bool dagcol, Sizer &sz, int pieces = 1);
void orient_carve(const tc_ctx *ctx, int64_t n, int64_t nnz, bool perm, bool dagcol, Bump &bump, OrientBufs &b,
                  int pieces = 1);
tc_status orient_front(tc_ctx *ctx, const DevCSR &d, const tc_opts &o, OrientBufs &ob, int64_t *m, float *ms_validate,
                       float *ms_a);
// orient_front in two halves: the launches (graph-capturable: kernels, event
// records and the queued copies of m and the flags) and the wait for them.
tc_status orient_front_launch(tc_ctx *ctx, const DevCSR &d, const tc_opts &o, OrientBufs &ob);
tc_status orient_front_finish(tc_ctx *ctx, int64_t *m, float *ms_validate, float *ms_a);
float elapsed(cudaEvent_t a, cudaEvent_t b);
const char *flag_text(unsigned f);
tc_status init_arm_occupancy(tc_ctx *ctx);

// Learned selector inference parameters live in ctx->d_mlp (fp32 master
// copy); the plan kernel rounds them to bf16 when it stages them.
}  // namespace tc
