/*
 * scan.h — stand-in for the GraphMiner scan header that the reference's
 * successful_push_pull/graph.cc includes (graph.cc:2), un-vendored there.
 * TEST INFRASTRUCTURE ONLY (see VertexSet.h).
 *
 * parallel_prefix_sum<In, Out>(in, out) writes the exclusive prefix sum of
 * `in` into out[0 .. in.size()]: out[0] = 0, out[i+1] = out[i] + in[i].
 * Graph::orientation (graph.cc:276) uses it to turn the kept out-degrees
 * into the DAG's row pointers and reads out[n] as the edge count.  A scan's
 * result does not depend on how it is parallelised, so a sequential loop
 * states it exactly.
 */
#pragma once
#include <vector>

template <typename In, typename Out>
void parallel_prefix_sum(const std::vector<In> &in, Out *out) {
  Out acc = 0;
  out[0] = 0;
  for (size_t i = 0; i < in.size(); ++i) {
    acc += (Out)in[i];
    out[i + 1] = acc;
  }
}
