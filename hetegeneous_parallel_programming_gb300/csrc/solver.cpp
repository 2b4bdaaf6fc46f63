// C++ Graph / TCSolver mirror of the reference host interface, over the C ABI.
#include <algorithm>
#include <cstdio>
#include <iostream>
#include <mutex>
#include <stdexcept>

#include "../../include/tc_graph.hpp"

namespace {

std::mutex g_mu;
tc_ctx *g_ctx = nullptr;

tc_ctx *shared_ctx() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ctx) {
    tc_status s = tc_ctx_create(0, &g_ctx);
    if (s != TC_OK) throw std::runtime_error(std::string("tc_ctx_create: ") + tc_last_error(nullptr));
  }
  return g_ctx;
}

void check(tc_status s, tc_ctx *ctx, const char *what) {
  if (s != TC_OK) throw std::runtime_error(std::string(what) + ": " + tc_status_str(s) + ": " + tc_last_error(ctx));
}

}  // namespace

Graph::Graph(std::string prefix, bool use_dag, bool directed, bool, bool, bool, bool, int) : directed_(directed) {
  size_t i = prefix.rfind('/');
  if (i != std::string::npos) inputfile_path_ = prefix.substr(0, i);
  i = inputfile_path_.rfind('/');
  name_ = (i != std::string::npos) ? inputfile_path_.substr(i + 1) : inputfile_path_;
  int64_t n = 0, nnz = 0, maxd = 0;
  int64_t *rp = nullptr;
  int32_t *cl = nullptr;
  check(tc_load_graphminer(prefix.c_str(), &n, &nnz, &rp, &cl, &maxd), nullptr, "tc_load_graphminer");
  n_vertices_ = (vidType)n;
  vertices_.assign(rp, rp + n + 1);
  edges_.assign(cl, cl + nnz);
  tc_csr_free(rp, cl);
  max_degree_ = compute_max_degree();
  if (use_dag) {
    if (directed) throw std::runtime_error("orientation needs an undirected graph");
    orientation();
  }
}

Graph::Graph(vidType nv, eidType ne) { allocateFrom(nv, ne); }

Graph::Graph(vidType nv, eidType ne, const eidType *rowptr, const vidType *colidx, bool oriented)
    : oriented_(oriented), n_vertices_(nv) {
  vertices_.assign(rowptr, rowptr + nv + 1);
  edges_.assign(colidx, colidx + ne);
  max_degree_ = compute_max_degree();
}

void Graph::allocateFrom(vidType nv, eidType ne) {
  n_vertices_ = nv;
  vertices_.assign((size_t)nv + 1, 0);
  edges_.assign((size_t)ne, 0);
}

vidType Graph::compute_max_degree() const {
  vidType m = 0;
  for (vidType v = 0; v < n_vertices_; ++v) m = std::max<vidType>(m, (vidType)(vertices_[v + 1] - vertices_[v]));
  return m;
}

void Graph::orientation() {
  if (oriented_) return;
  tc_ctx *ctx = shared_ctx();
  tc_csr g{n_vertices_, (int64_t)edges_.size(), vertices_.data(), edges_.data(), 0};
  std::vector<eidType> dag_row((size_t)n_vertices_ + 1);
  std::vector<vidType> dag_col(edges_.size());
  int64_t m = 0;
  check(tc_orient(ctx, &g, dag_row.data(), dag_col.data(), (int64_t)dag_col.size(), &m), ctx, "tc_orient");
  dag_col.resize((size_t)m);
  sym_vertices_.swap(vertices_);
  sym_edges_.swap(edges_);
  vertices_.swap(dag_row);
  edges_.swap(dag_col);
  oriented_ = true;
  max_degree_ = compute_max_degree();
}

void Graph::sort_neighbors() {
#pragma omp parallel for schedule(dynamic, 1024)
  for (vidType v = 0; v < n_vertices_; ++v) std::sort(edges_.begin() + vertices_[v], edges_.begin() + vertices_[v + 1]);
}

void Graph::print_meta_data() const {
  std::cout << "|V|: " << n_vertices_ << ", |E|: " << edges_.size() << ", Max Degree: " << max_degree_
            << (oriented_ ? " (oriented)" : "") << "\n";
}

void TCSolver(Graph &g, uint64_t &total, int n_gpu, int chunk_size) {
  (void)chunk_size;  // unused by the reference as well
  (void)n_gpu;       // one GB300 holds every supported graph: device 0 counts it
  tc_ctx *ctx = shared_ctx();
  uint64_t t = 0;
  tc_stats st;
  if (!g.symmetric_rowptr().empty()) {
    // Oriented from a symmetric graph held alongside: orient + count on the device.
    tc_csr s{g.V(), (int64_t)g.symmetric_colidx().size(), g.symmetric_rowptr().data(), g.symmetric_colidx().data(), 0};
    check(tc_count(ctx, &s, nullptr, &t, nullptr, 0, &st), ctx, "tc_count");
  } else if (g.is_oriented()) {
    tc_csr d{g.V(), g.E(), g.out_rowptr(), g.out_colidx(), 0};
    check(tc_count_dag(ctx, &d, nullptr, &t, nullptr, 0, &st), ctx, "tc_count_dag");
  } else {
    tc_csr s{g.V(), g.E(), g.out_rowptr(), g.out_colidx(), 0};
    check(tc_count(ctx, &s, nullptr, &t, nullptr, 0, &st), ctx, "tc_count");
  }
  std::cout << "runtime [gpu0] = " << st.ms_total << " ms\n";
  total += t;
}
