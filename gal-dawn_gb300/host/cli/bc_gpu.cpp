// bc_gpu: betweenness centrality of every vertex on the GB300 path, with the
// interface of the reference's CPU tool (algorithm/cpu/bc_cpu/bc_cpu.cpp):
// the same flags, the Nodes / Edges / Time lines and the output file of
// IO::outfile(rows, values, path).
#include <dawn/algorithm/gpu/bc.cuh>

int main(int argc, char* argv[]) {
  DAWN::IO::parameters_t params = DAWN::IO::parameters(argc, argv);
  DAWN::Graph::Graph_t graph;
  graph.print = true;
  graph.interval = 100;
  graph.weighted = false;
  DAWN::Graph::createGraph(params.input_path, graph);
  printf("%-21s%3.5d\n", "Nodes:", graph.rows);
  printf("%-21s%3.5ld\n", "Edges:", graph.nnz);
  float elapsed_time = DAWN::BC_GPU::Betweenness_Centrality(graph, params.output_path);
  printf("%-21s%3.5lf\n", "Time:", elapsed_time);
  return 0;
}
