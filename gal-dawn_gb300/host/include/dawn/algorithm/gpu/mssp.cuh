// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Multi-source BFS / shortest paths on the GPU, API of
// include/dawn/algorithm/gpu/mssp.cuh in the reference project.
#pragma once
#include <dawn/algorithm/gpu/bfs.cuh>
#include <dawn/algorithm/gpu/sssp.cuh>

namespace DAWN {
namespace MSSP_GPU {

float run(Graph::Graph_t& graph, std::string& output_path);
float run_Weighted(Graph::Graph_t& graph, std::string& output_path);

}  // namespace MSSP_GPU
}  // namespace DAWN
