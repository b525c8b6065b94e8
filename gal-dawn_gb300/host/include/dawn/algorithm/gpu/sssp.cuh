// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Single-source weighted shortest paths on the GPU, API of
// include/dawn/algorithm/gpu/sssp.cuh in the reference project.
#pragma once
#include <dawn/dawn.cuh>

namespace DAWN {
namespace SSSP_GPU {

float run(Graph::Graph_t& graph, std::string& output_path);

}  // namespace SSSP_GPU
}  // namespace DAWN
