// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Betweenness centrality on the GPU, API of include/dawn/algorithm/gpu/bc.cuh
// in the reference project (declared there, with no implementation).
#pragma once
#include <dawn/algorithm/gpu/bfs.cuh>

namespace DAWN {
namespace BC_GPU {

// BCDAWN betweenness of every vertex, every vertex a source: the quantity
// BC_CPU::Betweenness_Centrality computes (src/algorithm/cpu/bc.cpp:9-39),
// written with IO::outfile(rows, values, output_path) as the CPU tool does;
// returns seconds.  The values agree with the CPU path to float rounding.
float Betweenness_Centrality(Graph::Graph_t& graph, std::string& output_path);

// Declared by the reference without a definition; not provided here either.
float Betweenness_Centrality_Weighted(Graph::Graph_t& graph, std::string& output_path);

}  // namespace BC_GPU
}  // namespace DAWN
