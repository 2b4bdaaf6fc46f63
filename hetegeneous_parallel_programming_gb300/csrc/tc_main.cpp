// Command line with the reference's usage (main.cc:11-36):
//   tc_main <graph-prefix> [num_gpu(1)] [chunk_size(1024)] [adj_sorted(1)]
#include <cstdlib>
#include <iostream>
#include <stdexcept>

#include "../../include/tc_graph.hpp"

int main(int argc, char *argv[]) {
  if (argc < 2) {
    std::cout << "Usage: " << argv[0] << " <graph> [num_gpu(1)] [chunk_size(1024)] [adj_sorted(1)]\n";
    std::cout << "Example: " << argv[0] << " /graph_inputs/mico/graph\n";
    return 1;
  }
  try {
    int n_devices = 1, chunk_size = 1024, adj_sorted = 1;
    if (argc > 2) n_devices = atoi(argv[2]);
    if (argc > 3) chunk_size = atoi(argv[3]);
    if (argc > 4) adj_sorted = atoi(argv[4]);
    Graph g(argv[1], false);
    if (!adj_sorted) g.sort_neighbors();
    g.orientation();
    g.print_meta_data();
    uint64_t total = 0;
    TCSolver(g, total, n_devices, chunk_size);
    std::cout << "total_num_triangles = " << total << "\n";
  } catch (const std::exception &e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
