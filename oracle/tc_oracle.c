/*
 * tc_oracle.c — CPU oracle for exact triangle counting.  TEST INFRASTRUCTURE
 * ONLY: the tests, the smoke check and the CPU-baseline leg of the bench load
 * it as the checker; the engine never links, calls or ships it.
 *
 * It restates the reference project's CPU path (file:line inside the
 * reference project):
 *   - orientation:  successful_push_pull/graph.cc:252-298 (Graph::orientation):
 *       deg(v) = row length; keep src->dst iff deg(dst) > deg(src) or
 *       (deg(dst) == deg(src) and dst > src) (graph.cc:265-266); kept
 *       neighbours stay in input order (graph.cc:279-290); rowptr is the
 *       exclusive prefix sum of kept degrees (graph.cc:276).
 *   - counting:     bs_warp_vertex.cuh:13-21: total = sum over u, over
 *       v in N+(u), of |N+(u) n N+(v)|, each intersection by the two-pointer
 *       merge of Graph::intersect_num (graph.cc:376-391) without the vertex
 *       label predicate.
 *   - neighbour sort: graph.cc:156-164 (std::sort per row).
 *   - symmetrise / dedup / self-loop removal: the clean input the reference
 *     assumes (main.cc:17, graph.cc:329); restated as sort + unique per row.
 *
 * Parity status: pinned to the reference's own code.  oracle/build_ref.sh
 * compiles the reference's successful_push_pull/graph.cc unchanged into
 * oracle/_ref; tests/test_ref_pin.py checks that this file gives the same
 * oriented arrays, per-edge, total and labelled counts on the golden and
 * seeded graphs, and tests/golden/reference_outputs.json keeps what the
 * reference produced.  It is also pinned to networkx 3.6.1 triangle counts,
 * analytic answers (K_n, K_{a,b}, wheels, grids) and exhaustive enumeration
 * (tests/golden/triangles.json).
 *
 * Build: oracle/build_oracle.sh -> oracle/_build/libtc_oracle.so (gcc -O2 -fopenmp).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

/* graph.cc:252-298.  out_rowptr [n+1]; out_colidx must hold nnz entries
 * (an upper bound).  Returns the number of oriented edges. */
int64_t oracle_orient(int64_t n, const int64_t *rowptr, const int32_t *colidx, int64_t *out_rowptr,
                      int32_t *out_colidx) {
  int64_t *newdeg = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  if (!newdeg) return -1;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t src = 0; src < n; ++src) {
    const int64_t dsrc = rowptr[src + 1] - rowptr[src];
    int64_t k = 0;
    for (int64_t e = rowptr[src]; e < rowptr[src + 1]; ++e) {
      const int32_t dst = colidx[e];
      const int64_t ddst = rowptr[dst + 1] - rowptr[dst];
      if (ddst > dsrc || (ddst == dsrc && dst > src)) ++k;
    }
    newdeg[src] = k;
  }
  out_rowptr[0] = 0;
  for (int64_t v = 0; v < n; ++v) out_rowptr[v + 1] = out_rowptr[v] + newdeg[v];
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t src = 0; src < n; ++src) {
    const int64_t dsrc = rowptr[src + 1] - rowptr[src];
    int64_t w = out_rowptr[src];
    for (int64_t e = rowptr[src]; e < rowptr[src + 1]; ++e) {
      const int32_t dst = colidx[e];
      const int64_t ddst = rowptr[dst + 1] - rowptr[dst];
      if (ddst > dsrc || (ddst == dsrc && dst > src)) out_colidx[w++] = dst;
    }
  }
  free(newdeg);
  return out_rowptr[n];
}

/* graph.cc:376-391 without the label test. */
static inline uint32_t merge_count(const int32_t *a, int64_t na, const int32_t *b, int64_t nb) {
  int64_t i = 0, j = 0;
  uint32_t num = 0;
  while (i < na && j < nb) {
    const int32_t x = a[i], y = b[j];
    if (x <= y) ++i;
    if (y <= x) ++j;
    if (x == y) ++num;
  }
  return num;
}

/* bs_warp_vertex.cuh:13-21 over rows [row_begin, row_end) of an oriented
 * graph with sorted rows.  per_edge (optional, indexed like colidx) receives
 * each edge's intersection size. */
uint64_t oracle_count_rows(int64_t n, const int64_t *rowptr, const int32_t *colidx, int64_t row_begin,
                           int64_t row_end, int64_t row_step, uint32_t *per_edge) {
  uint64_t total = 0;
  if (row_step < 1) row_step = 1;
  if (row_end > n) row_end = n;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (int64_t u = row_begin; u < row_end; u += row_step) {
    const int32_t *nu = colidx + rowptr[u];
    const int64_t du = rowptr[u + 1] - rowptr[u];
    for (int64_t k = 0; k < du; ++k) {
      const int32_t v = nu[k];
      const uint32_t c = merge_count(nu, du, colidx + rowptr[v], rowptr[v + 1] - rowptr[v]);
      if (per_edge) per_edge[rowptr[u] + k] = c;
      total += c;
    }
  }
  return total;
}

uint64_t oracle_count(int64_t n, const int64_t *rowptr, const int32_t *colidx, uint32_t *per_edge) {
  return oracle_count_rows(n, rowptr, colidx, 0, n, 1, per_edge);
}

/* graph.cc:376-391 with the label test: over every edge u->v of an oriented
 * graph with sorted rows, the common out-neighbours w with labels[w] ==
 * label.  per_edge (optional, indexed like colidx) receives each edge's
 * count. */
uint64_t oracle_count_labelled(int64_t n, const int64_t *rowptr, const int32_t *colidx, const uint8_t *labels,
                               int label, uint32_t *per_edge) {
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (int64_t u = 0; u < n; ++u) {
    const int32_t *nu = colidx + rowptr[u];
    const int64_t du = rowptr[u + 1] - rowptr[u];
    for (int64_t k = 0; k < du; ++k) {
      const int32_t v = nu[k];
      const int32_t *nv = colidx + rowptr[v];
      const int64_t dv = rowptr[v + 1] - rowptr[v];
      int64_t i = 0, j = 0;
      uint32_t num = 0;
      while (i < du && j < dv) {
        const int32_t a = nu[i], b = nv[j];
        if (a <= b) ++i;
        if (b <= a) ++j;
        if (a == b && labels[a] == label) ++num;
      }
      if (per_edge) per_edge[rowptr[u] + k] = num;
      total += num;
    }
  }
  return total;
}

/* Triangles through every vertex of an oriented graph with sorted rows: the
 * merge of graph.cc:376-391 enumerates, for every edge u->v, each common
 * out-neighbour w; triangle {u, v, w} adds one to t[u], t[v] and t[w]
 * (t has n entries, zeroed here).  Returns the number of triangles. */
uint64_t oracle_count_vertices(int64_t n, const int64_t *rowptr, const int32_t *colidx, uint64_t *t) {
  for (int64_t i = 0; i < n; ++i) t[i] = 0;
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (int64_t u = 0; u < n; ++u) {
    const int32_t *nu = colidx + rowptr[u];
    const int64_t du = rowptr[u + 1] - rowptr[u];
    for (int64_t k = 0; k < du; ++k) {
      const int32_t v = nu[k];
      const int32_t *nv = colidx + rowptr[v];
      const int64_t dv = rowptr[v + 1] - rowptr[v];
      int64_t i = 0, j = 0;
      uint64_t c = 0;
      while (i < du && j < dv) {
        if (nu[i] < nv[j]) ++i;
        else if (nv[j] < nu[i]) ++j;
        else {
#pragma omp atomic
          t[nu[i]] += 1;
          ++c;
          ++i;
          ++j;
        }
      }
      if (c) {
#pragma omp atomic
        t[u] += c;
#pragma omp atomic
        t[v] += c;
      }
      total += c;
    }
  }
  return total;
}

/* Orientation restricted to a sample of rows (every row_step-th row), for
 * the bounded CPU baseline: same work per sampled row as oracle_orient.
 * Returns the number of kept edges of the sampled rows. */
int64_t oracle_orient_rows_cost(int64_t n, const int64_t *rowptr, const int32_t *colidx, int64_t row_step) {
  int64_t kept = 0;
  if (row_step < 1) row_step = 1;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : kept)
  for (int64_t src = 0; src < n; src += row_step) {
    const int64_t dsrc = rowptr[src + 1] - rowptr[src];
    for (int64_t e = rowptr[src]; e < rowptr[src + 1]; ++e) {
      const int32_t dst = colidx[e];
      const int64_t ddst = rowptr[dst + 1] - rowptr[dst];
      if (ddst > dsrc || (ddst == dsrc && dst > src)) ++kept;
    }
  }
  return kept;
}

static int cmp_i32(const void *x, const void *y) {
  const int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
  return (a > b) - (a < b);
}

/* graph.cc:156-164: sort every row ascending (in place). */
void oracle_sort_neighbors(int64_t n, const int64_t *rowptr, int32_t *colidx) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < n; ++v)
    qsort(colidx + rowptr[v], (size_t)(rowptr[v + 1] - rowptr[v]), sizeof(int32_t), cmp_i32);
}

/* Symmetrise, drop self loops and duplicates: rowptr [n+1], colidx holds up
 * to 2*num_edges entries.  Returns nnz or -1 on a bad id. */
int64_t oracle_csr_from_edges(int64_t n, int64_t num_edges, const int32_t *src, const int32_t *dst,
                              int64_t *rowptr, int32_t *colidx) {
  int64_t *deg = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  if (!deg) return -1;
  for (int64_t i = 0; i < num_edges; ++i) {
    if (src[i] < 0 || src[i] >= n || dst[i] < 0 || dst[i] >= n) { free(deg); return -1; }
    if (src[i] == dst[i]) continue;
    deg[src[i] + 1]++;
    deg[dst[i] + 1]++;
  }
  for (int64_t v = 0; v < n; ++v) deg[v + 1] += deg[v];
  int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(deg[n] + 1));
  if (!cur || !tmp) { free(deg); free(cur); free(tmp); return -1; }
  memcpy(cur, deg, sizeof(int64_t) * (size_t)(n + 1));
  for (int64_t i = 0; i < num_edges; ++i) {
    if (src[i] == dst[i]) continue;
    tmp[cur[src[i]]++] = dst[i];
    tmp[cur[dst[i]]++] = src[i];
  }
  oracle_sort_neighbors(n, deg, tmp);
  rowptr[0] = 0;
  for (int64_t v = 0; v < n; ++v) {
    int64_t w = rowptr[v];
    for (int64_t e = deg[v]; e < deg[v + 1]; ++e)
      if (e == deg[v] || tmp[e] != tmp[e - 1]) colidx[w++] = tmp[e];
    rowptr[v + 1] = w;
  }
  free(deg); free(cur); free(tmp);
  return rowptr[n];
}

/* Per-graph counts of a concatenated batch (local ids, global rowptr),
 * parallel over graphs (the per-graph calls run serially inside). */
void oracle_batch_count(int64_t num_graphs, const int64_t *vtx_off, const int64_t *rowptr,
                        const int32_t *colidx, uint64_t *totals) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t g = 0; g < num_graphs; ++g) {
    const int64_t v0 = vtx_off[g], n = vtx_off[g + 1] - v0;
    const int64_t base = rowptr[v0];
    int64_t *lrow = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    int64_t *orow = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    const int64_t nnz = rowptr[v0 + n] - base;
    int32_t *ocol = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nnz + 1));
    for (int64_t v = 0; v <= n; ++v) lrow[v] = rowptr[v0 + v] - base;
    oracle_orient(n, lrow, colidx + base, orow, ocol);
    totals[g] = oracle_count(n, orow, ocol, NULL);
    free(lrow); free(orow); free(ocol);
  }
}

int oracle_max_threads(void) { return omp_get_max_threads(); }
void oracle_set_threads(int t) { if (t > 0) omp_set_num_threads(t); }

/* ---- seeded generators, for CPU-only callers --------------------------------
 * The same samples as the engine's tc_gen_edges_host (kinds 0 ER, 1 R-MAT,
 * 3 Chung-Lu), from the shared counter-based sampling functions of
 * tc_gen_common.h, with the per-workload parameters (sample count, R-MAT
 * quadrant thresholds, Chung-Lu cumulative weights) derived here, so a
 * process that only times the CPU path need not load the engine library.
 * tests/test_ref_pin.py checks that both produce identical samples. */
#include <math.h>
#include "tc_gen_common.h"

int64_t oracle_gen_num_samples(int32_t kind, int64_t n, int32_t scale, double avg_degree, double edge_factor) {
  if (kind == 1) return (int64_t)floor(edge_factor * (double)((int64_t)1 << scale));
  if (kind == 0 || kind == 3) return (int64_t)floor((double)n * avg_degree / 2.0);
  return -1;
}

/* Writes the samples into src/dst (capacity entries); returns their number,
 * or -1 for an unknown kind or too small a buffer. */
int64_t oracle_gen_edges(int32_t kind, int64_t n, int32_t scale, double avg_degree, double edge_factor, double a,
                         double b, double c, double gamma, uint64_t seed, int32_t *src, int32_t *dst,
                         int64_t capacity) {
  const int64_t M = oracle_gen_num_samples(kind, n, scale, avg_degree, edge_factor);
  if (M < 0 || M > capacity) return -1;
  if (kind == 0) {
    const uint64_t key = tc_stream_key(seed, TC_SID_ER);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) tc_er_sample(key, (uint64_t)n, (uint64_t)i, &src[i], &dst[i]);
  } else if (kind == 1) {
    const double s = 4294967296.0;  /* cumulative quadrant probabilities in 2^-32 units */
    const uint64_t t1 = (uint64_t)floor(a * s), t2 = (uint64_t)floor((a + b) * s),
                   t3 = (uint64_t)floor((a + b + c) * s);
    const uint64_t key = tc_stream_key(seed, TC_SID_RMAT);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) tc_rmat_sample(key, scale, t1, t2, t3, (uint64_t)i, &src[i], &dst[i]);
  } else {
    /* expected degree of vertex i proportional to (i+1)^(-1/(gamma-1)),
     * scaled to mean avg_degree, capped at sqrt(n * avg_degree), in 20-bit
     * fixed point (at least 1), accumulated */
    uint64_t *cum = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    double *w = (double *)malloc(sizeof(double) * (size_t)n);
    if (!cum || !w) { free(cum); free(w); return -1; }
    const double alpha = 1.0 / (gamma - 1.0);
    double sum = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      w[i] = pow((double)(i + 1), -alpha);
      sum += w[i];
    }
    const double scl = avg_degree * (double)n / sum, cap = sqrt((double)n * avg_degree);
    uint64_t acc = 0;
    for (int64_t i = 0; i < n; ++i) {
      const double d = fmin(w[i] * scl, cap);
      uint64_t fx = (uint64_t)llround(d * 1048576.0);
      acc += fx ? fx : 1;
      cum[i] = acc;
    }
    free(w);
    const uint64_t key = tc_stream_key(seed, TC_SID_CL);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) tc_cl_sample(key, cum, n, (uint64_t)i, &src[i], &dst[i]);
    free(cum);
  }
  return M;
}
