// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Single-source BFS on the GPU, API of include/dawn/algorithm/gpu/bfs.cuh
// in the reference project (the reference's thrust-based kernel() helper is
// internal and not part of this API).
#pragma once
#include <dawn/dawn.cuh>

namespace DAWN {
namespace BFS_GPU {

// Hop distances from graph.source; writes output_path when graph.print.
// Returns the traversal time in seconds.  An isolated source prints
// "Source [s] is isolated node" and exits(0), as the reference does.
float run(Graph::Graph_t& graph, std::string& output_path);

}  // namespace BFS_GPU
}  // namespace DAWN
