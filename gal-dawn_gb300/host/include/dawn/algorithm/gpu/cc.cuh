// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Closeness centrality on the GPU, API of include/dawn/algorithm/gpu/cc.cuh
// in the reference project.
#pragma once
#include <dawn/algorithm/gpu/bfs.cuh>
#include <dawn/algorithm/gpu/sssp.cuh>

namespace DAWN {
namespace CC_GPU {

// The reference's value: (rows - 1) / sum of distances, the unweighted form
// dividing int by int (src/algorithm/gpu/cc.cu:305-307) and the weighted form
// summing FLT_MAX for unreachable vertices (src/algorithm/gpu/cc.cu:405-407).
float run(Graph::Graph_t& graph, int source);
float run_Weighted(Graph::Graph_t& graph, int source);

// Exact closeness: (rows - 1) / sum over the reached v != source of d(s, v),
// summed exactly and divided in float64 (dawn_closeness).
double closeness(Graph::Graph_t& graph, int source, bool weighted);

}  // namespace CC_GPU
}  // namespace DAWN
