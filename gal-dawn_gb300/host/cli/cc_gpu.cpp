// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// cc_gpu: the reference's command-line tool (algorithm/gpu/cc_gpu/cc_gpu.cu)
// over the GB300 path.  The closeness line keeps the reference's value; set
// DAWN_EXACT_CC=1 to print the exact float64 closeness instead.
#include <dawn/algorithm/gpu/cc.cuh>

int main(int argc, char* argv[]) {
  DAWN::IO::parameters_t params = DAWN::IO::parameters(argc, argv);
  DAWN::Graph::Graph_t graph;
  graph.source = params.source;
  graph.print = params.print;
  graph.weighted = params.weighted;
  graph.thread = 1;
  graph.stream = 1;
  graph.block_size = 1024;
  DAWN::Graph::createGraph(params.input_path, graph);
  const char* exact = std::getenv("DAWN_EXACT_CC");
  double cc;
  if (exact && std::string(exact) == "1")
    cc = DAWN::CC_GPU::closeness(graph, graph.source, graph.weighted);
  else
    cc = graph.weighted ? DAWN::CC_GPU::run_Weighted(graph, graph.source) : DAWN::CC_GPU::run(graph, graph.source);
  printf("%-21s%3.5d\n", "Source:", graph.source);
  printf("%-21s%3.5lf\n", "Closeness Centrality:", cc);
  return 0;
}
