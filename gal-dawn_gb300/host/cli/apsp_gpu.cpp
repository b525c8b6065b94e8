// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// apsp_gpu: the reference's command-line tool (algorithm/gpu/apsp_gpu/apsp_gpu.cu)
// over the GB300 path: same flags, console lines and output file.
#include <dawn/algorithm/gpu/apsp.cuh>

int main(int argc, char* argv[]) {
  DAWN::IO::parameters_t params = DAWN::IO::parameters(argc, argv);
  DAWN::Graph::Graph_t graph;
  graph.source = params.source;
  graph.print = params.print;
  graph.weighted = params.weighted;
  graph.thread = 1;
  graph.stream = 4;
  graph.block_size = 1024;
  graph.interval = 100;
  DAWN::Graph::createGraph(params.input_path, graph);

  float elapsed_time = graph.weighted ? DAWN::APSP_GPU::run_Weighted(graph, params.output_path)
                                      : DAWN::APSP_GPU::run(graph, params.output_path);
  printf("%-21s%3.5d\n", "Nodes:", graph.rows);
  printf("%-21s%3.5ld\n", "Edges:", (long)graph.nnz);
  printf("%-21s%3.5lf\n", "Time:", (double)elapsed_time);
  return 0;
}
