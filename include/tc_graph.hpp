// tc_graph.hpp — C++ host interface mirroring the reference project's Graph
// class and TCSolver entry point, implemented over the C ABI in tc.h.
//
// Reference interfaces (paths inside the reference project):
//   Graph(prefix, use_dag, ...)         successful_push_pull/graph.h:58-60, graph.cc:4-142
//   V() E() get_degree edge_begin ...   successful_push_pull/graph.h:68-96
//   orientation()                       successful_push_pull/graph.cc:252-298
//   sort_neighbors()                    successful_push_pull/graph.cc:156-164
//   TCSolver(Graph&, uint64_t&, int, int)  multigpu.cu:780, main.cc:5
//
// Differences a reference user sees: orientation() runs on the GPU (same
// kept edges, same neighbour order); TCSolver counts on one GPU (n_gpu > 1
// still uses device 0 — one GB300 holds every supported graph) and keeps the
// reference's "total +=" contract; errors throw std::runtime_error with the
// engine's message instead of printing and calling exit(-1).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "tc.h"

typedef int32_t vidType;
typedef int64_t eidType;
typedef uint64_t AccType;

class Graph {
 public:
  // Loads prefix.meta.txt / .vertex.bin / .edge.bin; orients when use_dag.
  explicit Graph(std::string prefix, bool use_dag = false, bool directed = false, bool use_vlabel = false,
                 bool use_elabel = false, bool need_reverse = false, bool bipartite = false, int my_id = 0);
  // Empty graph with room for nv vertices and ne column entries.
  Graph(vidType nv, eidType ne);
  // Takes a copy of a CSR.
  Graph(vidType nv, eidType ne, const eidType *rowptr, const vidType *colidx, bool oriented = false);
  Graph(const Graph &) = delete;
  Graph &operator=(const Graph &) = delete;
  ~Graph() = default;

  vidType V() const { return n_vertices_; }
  eidType E() const { return (eidType)edges_.size(); }
  vidType size() const { return n_vertices_; }
  eidType sizeEdges() const { return E(); }
  vidType num_vertices() const { return n_vertices_; }
  eidType num_edges() const { return E(); }
  vidType get_max_degree() const { return max_degree_; }
  std::string get_name() const { return name_; }
  bool is_directed() const { return directed_; }
  bool is_oriented() const { return oriented_; }

  vidType get_degree(vidType v) const { return (vidType)(vertices_[v + 1] - vertices_[v]); }
  vidType out_degree(vidType v) const { return get_degree(v); }
  eidType edge_begin(vidType v) const { return vertices_[v]; }
  eidType edge_end(vidType v) const { return vertices_[v + 1]; }
  vidType N(vidType v, vidType i) const { return edges_[vertices_[v] + i]; }
  vidType *adj_ptr(vidType v) { return &edges_[vertices_[v]]; }
  vidType getEdgeDst(eidType e) const { return edges_[e]; }
  eidType *out_rowptr() { return vertices_.data(); }
  vidType *out_colidx() { return edges_.data(); }
  const eidType *out_rowptr() const { return vertices_.data(); }
  const vidType *out_colidx() const { return edges_.data(); }

  void allocateFrom(vidType nv, eidType ne);
  void constructEdge(eidType eid, vidType dst) { edges_[eid] = dst; }
  void fixEndEdge(vidType vid, eidType row_end) { vertices_[vid + 1] = row_end; }

  // Degree-ordered DAG (keeps the symmetric graph for TCSolver's fast path).
  void orientation();
  void sort_neighbors();
  void print_meta_data() const;

  // The symmetric graph this one was oriented from (empty if none).
  const std::vector<eidType> &symmetric_rowptr() const { return sym_vertices_; }
  const std::vector<vidType> &symmetric_colidx() const { return sym_edges_; }

 private:
  vidType compute_max_degree() const;
  std::string name_, inputfile_path_;
  bool directed_ = false, oriented_ = false;
  vidType n_vertices_ = 0, max_degree_ = 0;
  std::vector<eidType> vertices_;
  std::vector<vidType> edges_;
  std::vector<eidType> sym_vertices_;
  std::vector<vidType> sym_edges_;
};

// total += number of triangles of g (oriented or symmetric).
void TCSolver(Graph &g, uint64_t &total, int n_gpu, int chunk_size);
