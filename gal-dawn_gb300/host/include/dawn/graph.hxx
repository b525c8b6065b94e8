// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Graph container and loader entry point, API of include/dawn/graph.hxx in
// the reference project.
#pragma once
#include <dawn/include.hxx>
#include <dawn/matrix.hxx>

namespace DAWN {
namespace Graph {

class Graph_t {
 public:
  int rows = 0;
  int cols = 0;
  uint64_t nnz = 0;
  DAWN::Matrix::Csr_t csr;
  DAWN::Matrix::Coo_t coo;
  int thread = 1;
  int interval = 100;
  int stream = 1;      // accepted for compatibility; the GB300 path picks its own
  int block_size = 1024;  // accepted for compatibility; ignored
  int source = 0;
  bool print = false;
  bool weighted = false;
  // true unless every edge is stored in both directions; createGraph sets it
  // from the file header.  The default is the safe one for a hand-filled CSR.
  bool directed = true;
  std::vector<int> msource;  // source list for multi-source algorithms
};

// Reads a MatrixMarket coordinate file into graph (rows, cols, nnz, csr,
// directed); graph.weighted selects the weighted reader.
void createGraph(std::string& input_path, DAWN::Graph::Graph_t& graph);

}  // namespace Graph
}  // namespace DAWN
