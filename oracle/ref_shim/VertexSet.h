/*
 * VertexSet.h — stand-in for the GraphMiner header that the reference's
 * successful_push_pull/graph.h includes (graph.h:2) and that the reference
 * does not vendor (GraphMiner/ is an empty, unpinned submodule).  TEST
 * INFRASTRUCTURE ONLY: it exists so that the reference's graph.cc compiles
 * unchanged into oracle/_ref (oracle/build_ref.sh), which pins the oracle.
 *
 * It supplies what graph.cc and graph.h use and nothing else:
 *   - the GraphMiner typedefs.  vidType is int32 (the reference reads colidx
 *     with nvshmem int32 gets, successful_push_pull/bs_warp_vertex_nvshmem.cuh:134),
 *     eidType int64 (int64 gets on rowptr, same file :114), vlabel_t one byte
 *     (graph.cc:44 checks sizeof(vlabel_t) against the meta file's
 *     vlabel_size, which GraphMiner files set to 1);
 *   - VertexSet: a read-only view of a neighbour list (pointer, size, owner)
 *     with size(), operator[], add() and range iteration, plus the static
 *     MAX_DEGREE and release_buffers() that Graph::Graph touches;
 *   - read_file / map_file / custom_alloc_global / custom_free and Timer.
 */
#pragma once
#include <algorithm>
#include <cassert>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <set>
#include <string>
#include <vector>
#include <omp.h>
#include <sys/mman.h>

typedef int32_t vidType;
typedef int64_t eidType;
typedef uint8_t vlabel_t;
typedef int32_t elabel_t;
typedef float feat_t;
typedef uint64_t AccType;
typedef std::vector<vidType> VertexList;
typedef std::map<vlabel_t, int> nlf_map;

class VertexSet {
 public:
  static inline vidType MAX_DEGREE = 1;
  static void release_buffers() {}

  VertexSet() = default;
  VertexSet(vidType *p, eidType n, vidType owner) : ptr_(p), size_(n), vid_(owner) {}

  vidType size() const { return (vidType)size_; }
  vidType get_vid() const { return vid_; }
  vidType operator[](size_t i) const { return ptr_ ? ptr_[i] : owned_[i]; }
  void add(vidType v) { owned_.push_back(v); ++size_; }
  const vidType *begin() const { return ptr_ ? ptr_ : owned_.data(); }
  const vidType *end() const { return begin() + size_; }

 private:
  vidType *ptr_ = nullptr;
  eidType size_ = 0;
  vidType vid_ = 0;
  std::vector<vidType> owned_;
};

template <typename T>
T *custom_alloc_global(size_t n) {
  return static_cast<T *>(std::malloc(std::max<size_t>(n, 1) * sizeof(T)));
}

template <typename T>
void custom_free(T *p, size_t) {
  std::free(p);
}

/* Allocates `ptr` and fills it with `n` elements of the binary file. */
template <typename T>
void read_file(const std::string &fname, T *&ptr, size_t n) {
  ptr = custom_alloc_global<T>(n);
  FILE *f = std::fopen(fname.c_str(), "rb");
  if (!f || std::fread(ptr, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "read_file: cannot read %zu elements from %s\n", n, fname.c_str());
    std::abort();
  }
  std::fclose(f);
}

/* The reference only maps files when its map_* constants are true; they are
 * false (graph.h:7-11), so this is never called. */
template <typename T>
void map_file(const std::string &fname, T *&ptr, size_t n) {
  read_file(fname, ptr, n);
}

class Timer {
 public:
  void Start() { t0_ = std::chrono::steady_clock::now(); }
  void Stop() { t1_ = std::chrono::steady_clock::now(); }
  double Seconds() const { return std::chrono::duration<double>(t1_ - t0_).count(); }
  double Millisecs() const { return Seconds() * 1e3; }

 private:
  std::chrono::steady_clock::time_point t0_{}, t1_{};
};
