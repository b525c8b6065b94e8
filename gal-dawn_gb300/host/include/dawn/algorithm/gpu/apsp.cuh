// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// All-pairs BFS / shortest paths on the GPU, API of
// include/dawn/algorithm/gpu/apsp.cuh in the reference project.
#pragma once
#include <dawn/algorithm/gpu/bfs.cuh>
#include <dawn/algorithm/gpu/sssp.cuh>

namespace DAWN {
namespace APSP_GPU {

float run(Graph::Graph_t& graph, std::string& output_path);
float run_Weighted(Graph::Graph_t& graph, std::string& output_path);

}  // namespace APSP_GPU
}  // namespace DAWN
