// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// MatrixMarket header handling and reader dispatch (API and messages of
// src/graph.cpp:9-77 in the reference project).
#include <dawn/graph.hxx>
#include <dawn/io.hxx>

namespace DAWN {
namespace Graph {

void createGraph(std::string& input_path, Graph_t& graph) {
  std::ifstream file(input_path);
  if (!file.is_open()) {
    std::cerr << "Error opening file " << input_path << std::endl;
    return;
  }
  std::string line;
  std::getline(file, line);
  std::stringstream ss(line);
  std::string format, object, matrixtype, datatype, direct;
  ss >> format >> object >> matrixtype >> datatype >> direct;
  if (format == "%%MatrixMarket" && matrixtype == "coordinate") {
    const bool file_weighted = datatype != "pattern";
    if (!file_weighted && graph.weighted)
      std::cout << "This is an unweighted graph, but it has been instructed "
                   "to use weighted functions for computation."
                << std::endl;
    if (file_weighted && !graph.weighted)
      std::cout << "This is a weighted graph, and it has been instructed "
                   "to use unweighted functions for computation. "
                << std::endl;
    graph.directed = direct != "symmetric";
  } else {
    std::cout << "invalid file" << std::endl;
    return;
  }
  int rows = 0, cols = 0, nnz = 0;
  while (std::getline(file, line)) {
    if (!line.empty() && line[0] == '%') continue;
    std::stringstream sz(line);
    sz >> rows >> cols >> nnz;
    break;
  }
  file.close();
  graph.rows = rows;
  graph.cols = cols;
  graph.nnz = (uint64_t)nnz;
  if (rows > 0) graph.source = graph.source % rows;
  std::cout << "Read Input Graph" << std::endl;
  if (graph.directed) {
    if (graph.weighted)
      DAWN::IO::readGraph_Directed_Weighted(input_path, graph);
    else
      DAWN::IO::readGraph_Directed(input_path, graph);
  } else {
    if (graph.weighted)
      DAWN::IO::readGraph_Weighted(input_path, graph);
    else
      DAWN::IO::readGraph(input_path, graph);
  }
}

}  // namespace Graph
}  // namespace DAWN
