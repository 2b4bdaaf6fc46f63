/*
 * ref_driver.cc — C entry points over the reference's own Graph class.
 * TEST INFRASTRUCTURE ONLY: oracle/build_ref.sh compiles this file together
 * with the reference's successful_push_pull/graph.cc, unchanged and read
 * where it lies, into oracle/_ref/libtc_ref.so.  The tests use it to pin the
 * C restatement (oracle/tc_oracle.c) and the golden fixtures to the
 * reference's code; the engine never links or calls it.
 *
 * What runs is the reference's code:
 *   - Graph::Graph(prefix, use_dag, ...)   graph.cc:4-142 (GraphMiner files,
 *                                          meta :31-49, binaries :51-55)
 *   - Graph::orientation()                 graph.cc:252-298 (use_dag)
 *   - Graph::sort_neighbors()              graph.cc:156-164 (main.cc:30-31)
 *   - Graph::intersect_num(v, u, label)    graph.cc:376-391
 * and this file adds only the counting loop of the reference kernel
 * (bs_warp_vertex.cuh:13-21: for every vertex u and every v in N(u), add
 * |N(u) n N(v)|), run over vertices in parallel with OpenMP and recording
 * each edge's count at its CSR slot.  The label test of intersect_num is
 * kept: an unlabelled count loads an all-zero label file (one class) and
 * asks for label 0, so every common neighbour matches.
 */
#include "graph.h"

#include <sstream>

namespace {

// Graph's constructor and orientation print progress to std::cout; the
// tests want a quiet library.
struct QuietCout {
  std::ostringstream sink;
  std::streambuf *old;
  QuietCout() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~QuietCout() { std::cout.rdbuf(old); }
};

}  // namespace

extern "C" {

void *ref_graph_open(const char *prefix, int use_dag, int use_vlabel, int sort_neighbors) {
  QuietCout q;
  Graph *g = new Graph(std::string(prefix), use_dag != 0, false, use_vlabel != 0);
  if (sort_neighbors) g->sort_neighbors();
  return g;
}

void ref_graph_close(void *h) { delete static_cast<Graph *>(h); }

int64_t ref_graph_num_vertices(void *h) { return static_cast<Graph *>(h)->V(); }
int64_t ref_graph_num_edges(void *h) { return static_cast<Graph *>(h)->E(); }
int64_t ref_graph_max_degree(void *h) { return static_cast<Graph *>(h)->get_max_degree(); }

/* Copies the graph's CSR (after orientation when opened with use_dag). */
void ref_graph_arrays(void *h, int64_t *rowptr, int32_t *colidx) {
  Graph *g = static_cast<Graph *>(h);
  const eidType *rp = g->out_rowptr();
  for (int64_t v = 0; v <= g->V(); ++v) rowptr[v] = rp[v];
  for (int64_t e = 0; e < g->E(); ++e) colidx[e] = g->getEdgeDst(e);
}

/* bs_warp_vertex.cuh:13-21 over vertices [row_begin, row_end) with step
 * `row_step`, each intersection by Graph::intersect_num(u, v, label).
 * per_edge (optional, E() entries) receives the count of every edge u->v of
 * the visited rows at its CSR slot. */
uint64_t ref_graph_count(void *h, int32_t label, int64_t row_begin, int64_t row_end, int64_t row_step,
                         uint32_t *per_edge) {
  Graph *g = static_cast<Graph *>(h);
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : total)
  for (int64_t u = row_begin; u < row_end; u += row_step) {
    for (eidType e = g->edge_begin((vidType)u); e < g->edge_end((vidType)u); ++e) {
      const vidType v = g->getEdgeDst(e);
      const vidType c = g->intersect_num((vidType)u, v, (vlabel_t)label);
      if (per_edge) per_edge[e] = (uint32_t)c;
      total += (uint64_t)c;
    }
  }
  return total;
}

}  // extern "C"
