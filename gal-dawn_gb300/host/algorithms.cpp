// GAL-DAWN's GPU algorithm entry points over the C ABI of libdawn_gb300.so.
//
// Each run() keeps the reference's contract (src/algorithm/gpu/*.cu):
// the same arguments, return value (seconds of traversal), console messages,
// isolated-source handling and output file; the traversal itself is one
// dawn_* call on the GB300 kernels.  The graph is uploaded once per run()
// (the reference copies it once per source, see bfs.cuh:14-19).
#include <dawn/algorithm/gpu/apsp.cuh>
#include <dawn/algorithm/gpu/bc.cuh>
#include <dawn/algorithm/gpu/cc.cuh>
#include <dawn/algorithm/gpu/mssp.cuh>

#include "dawn_gb300.h"

namespace DAWN {
namespace {

[[noreturn]] void die(dawn_status s, const char* what) {
  std::fprintf(stderr, "dawn: %s failed (status %d): %s\n", what, (int)s, dawn_last_error());
  std::exit(EXIT_FAILURE);
}

struct Device {
  dawn_graph* g = nullptr;
  Device(Graph::Graph_t& graph, bool weighted) {
    const uint32_t flags = graph.directed ? 0u : DAWN_GRAPH_SYMMETRIC;
    dawn_status s = dawn_graph_create(graph.csr.row_ptr, graph.csr.col, weighted ? graph.csr.val : nullptr,
                                      weighted ? DAWN_W_F32 : DAWN_W_NONE, graph.rows, (int64_t)graph.nnz, flags,
                                      nullptr, &g);
    if (s != DAWN_OK) die(s, "dawn_graph_create");
  }
  ~Device() {
    if (g) dawn_graph_destroy(g);
  }
};

bool isolated(const Graph::Graph_t& graph, int s) { return graph.csr.row_ptr[s] == graph.csr.row_ptr[s + 1]; }

// C-ABI hop distances -> the reference's encoding (0 = unvisited or source).
void to_reference(std::vector<int32_t>& d, int source) {
  for (auto& x : d)
    if (x < 0) x = 0;
  d[source] = 0;
}

std::vector<int32_t> hops(Device& dev, const Graph::Graph_t& graph, int source, dawn_stats* st) {
  std::vector<int32_t> d(graph.rows);
  dawn_status s = dawn_bfs(dev.g, &source, 1, d.data(), DAWN_VARIANT_DO, st);
  if (s != DAWN_OK) die(s, "dawn_bfs");
  return d;
}

std::vector<float> weighted(Device& dev, const Graph::Graph_t& graph, int source, dawn_stats* st) {
  std::vector<float> d(graph.rows);
  dawn_status s = dawn_sssp(dev.g, &source, 1, d.data(), DAWN_VARIANT_AUTO, st);
  if (s != DAWN_OK) die(s, "dawn_sssp");
  return d;
}

// Sources of a multi-source call: msource modulo rows, isolated ones
// reported and skipped (src/algorithm/gpu/mssp.cu:26-34).
std::vector<int32_t> usable_sources(const Graph::Graph_t& graph, bool report) {
  std::vector<int32_t> out;
  out.reserve(graph.msource.size());
  for (int s0 : graph.msource) {
    const int s = s0 % graph.rows;
    if (isolated(graph, s)) {
      if (report) std::printf("Source [%d] is isolated node\n", s);
      continue;
    }
    out.push_back(s);
  }
  return out;
}

// Multi-source traversal in chunks; distances stay on the device.
float batched(Device& dev, const std::vector<int32_t>& srcs, bool is_weighted, int total, int interval, int thread,
              bool progress) {
  float ms = 0.0f;
  const int chunk = 4096;
  int done = 0;
  for (size_t i = 0; i < srcs.size(); i += chunk) {
    const int c = (int)std::min<size_t>(chunk, srcs.size() - i);
    dawn_stats st;
    dawn_status s = is_weighted ? dawn_sssp(dev.g, srcs.data() + i, c, nullptr, DAWN_VARIANT_AUTO, &st)
                                : dawn_bfs(dev.g, srcs.data() + i, c, nullptr, DAWN_VARIANT_AUTO, &st);
    if (s != DAWN_OK) die(s, is_weighted ? "dawn_sssp" : "dawn_bfs");
    ms += st.device_ms;
    if (progress)
      for (int k = 0; k < c; k++) Tool::infoprint(++done, total, interval, thread, ms);
  }
  return ms;
}

void print_source(Device& dev, Graph::Graph_t& graph, bool is_weighted, std::string& output_path) {
  std::printf("Start print\n");
  if (is_weighted) {
    std::vector<float> d = weighted(dev, graph, graph.source, nullptr);
    IO::outfile(graph.rows, d.data(), graph.source, output_path);
  } else {
    std::vector<int32_t> d = hops(dev, graph, graph.source, nullptr);
    to_reference(d, graph.source);
    IO::outfile(graph.rows, d.data(), graph.source, output_path);
  }
}

}  // namespace

float BFS_GPU::run(Graph::Graph_t& graph, std::string& output_path) {
  const int source = graph.source;
  if (isolated(graph, source)) {
    std::printf("Source [%d] is isolated node\n", source);
    std::exit(0);
  }
  Device dev(graph, false);
  dawn_stats st;
  std::vector<int32_t> d = hops(dev, graph, source, &st);
  if (graph.print) {
    std::printf("Start print\n");
    to_reference(d, source);
    IO::outfile(graph.rows, d.data(), source, output_path);
  }
  return st.device_ms / 1000.0f;
}

float SSSP_GPU::run(Graph::Graph_t& graph, std::string& output_path) {
  const int source = graph.source;
  if (isolated(graph, source)) {
    std::printf("Source [%d] is isolated node\n", source);
    std::exit(0);
  }
  Device dev(graph, true);
  dawn_stats st;
  std::vector<float> d = weighted(dev, graph, source, &st);
  if (graph.print) {
    std::printf("Start print\n");
    IO::outfile(graph.rows, d.data(), source, output_path);
  }
  return st.device_ms / 1000.0f;
}

static float mssp(Graph::Graph_t& graph, std::string& output_path, bool is_weighted) {
  if (is_weighted) std::cout << "Initialize Input Matrices" << std::endl;
  Device dev(graph, is_weighted);
  const std::vector<int32_t> srcs = usable_sources(graph, true);
  const float ms = batched(dev, srcs, is_weighted, (int)srcs.size(), graph.interval, graph.thread, false);
  // The reference writes the output file only for the source equal to
  // graph.source (src/algorithm/gpu/bfs.cu:97).
  if (graph.print && std::find(srcs.begin(), srcs.end(), graph.source) != srcs.end())
    print_source(dev, graph, is_weighted, output_path);
  return ms / (graph.thread * 1000.0f);
}

float MSSP_GPU::run(Graph::Graph_t& graph, std::string& output_path) { return mssp(graph, output_path, false); }
float MSSP_GPU::run_Weighted(Graph::Graph_t& graph, std::string& output_path) {
  return mssp(graph, output_path, true);
}

static float apsp(Graph::Graph_t& graph, std::string& output_path, bool is_weighted) {
  Device dev(graph, is_weighted);
  std::cout << ">>>>>>>>>>>>>>>>>>>>>>>>>>> APSP start <<<<<<<<<<<<<<<<<<<<<<<<<<<" << std::endl;
  std::vector<int32_t> srcs;
  int skipped = 0;
  for (int s = 0; s < graph.rows; s++) {
    if (isolated(graph, s)) {
      skipped++;
      continue;
    }
    srcs.push_back(s);
  }
  float ms = batched(dev, srcs, is_weighted, graph.rows, graph.interval, graph.thread, true);
  for (int k = 0; k < skipped; k++)
    Tool::infoprint((int)srcs.size() + k + 1, graph.rows, graph.interval, graph.thread, ms);
  std::cout << ">>>>>>>>>>>>>>>>>>>>>>>>>>> APSP end <<<<<<<<<<<<<<<<<<<<<<<<<<<" << std::endl;
  if (graph.print && !isolated(graph, graph.source)) print_source(dev, graph, is_weighted, output_path);
  return ms / (graph.thread * 1000.0f);
}

float APSP_GPU::run(Graph::Graph_t& graph, std::string& output_path) { return apsp(graph, output_path, false); }
float APSP_GPU::run_Weighted(Graph::Graph_t& graph, std::string& output_path) {
  return apsp(graph, output_path, true);
}

static void cc_report(const Graph::Graph_t& graph, float seconds) {
  std::printf("%-21s%3.5d\n", "Node:", graph.rows);
  std::printf("%-21s%3.5ld\n", "Edges:", (long)graph.nnz);
  std::printf("%-21s%3.5lf\n", "Time:", (double)seconds / graph.thread);
}

float CC_GPU::run(Graph::Graph_t& graph, int source) {
  if (isolated(graph, source)) {
    std::printf("Source [%d] is isolated node\n", source);
    std::exit(0);
  }
  Device dev(graph, false);
  dawn_stats st;
  std::vector<int32_t> d = hops(dev, graph, source, &st);
  to_reference(d, source);
  // int accumulate and int division, as src/algorithm/gpu/cc.cu:305-307
  uint32_t acc = 0;
  for (int32_t x : d) acc += (uint32_t)x;
  const int32_t sum = (int32_t)acc;
  const float cc = sum ? (float)((graph.rows - 1) / sum) : 0.0f;
  cc_report(graph, st.device_ms / 1000.0f);
  return cc;
}

float CC_GPU::run_Weighted(Graph::Graph_t& graph, int source) {
  if (isolated(graph, source)) {
    std::printf("Source [%d] is isolated node\n", source);
    std::exit(0);
  }
  Device dev(graph, true);
  dawn_stats st;
  std::vector<float> d = weighted(dev, graph, source, &st);
  d[source] = 0.0f;
  // float accumulate over every entry, unreachable FLT_MAX included, as
  // src/algorithm/cpu/cc.cpp:133-134 (the GPU form's reduction order is
  // unspecified)
  const float sum = std::accumulate(d.begin(), d.end(), 0.0f);
  const float cc = (float)((1.0 * graph.rows - 1.0f) / sum);
  cc_report(graph, st.device_ms / 1000.0f);
  return cc;
}

double CC_GPU::closeness(Graph::Graph_t& graph, int source, bool is_weighted) {
  Device dev(graph, is_weighted);
  double cc = 0.0;
  dawn_status s = dawn_closeness(dev.g, &source, 1, is_weighted ? 1 : 0, &cc, nullptr, nullptr, nullptr);
  if (s != DAWN_OK) die(s, "dawn_closeness");
  return cc;
}

float BC_GPU::Betweenness_Centrality(Graph::Graph_t& graph, std::string& output_path) {
  Device dev(graph, false);
  std::vector<int32_t> sources(graph.rows);
  for (int i = 0; i < graph.rows; i++) sources[i] = i;
  std::vector<double> bc(graph.rows);
  dawn_stats st;
  const dawn_status s = dawn_betweenness(dev.g, sources.data(), graph.rows, bc.data(), &st);
  if (s != DAWN_OK) die(s, "dawn_betweenness");
  std::vector<float> out(bc.begin(), bc.end());
  IO::outfile(graph.rows, out.data(), output_path);
  return st.device_ms / 1000.0f;
}

}  // namespace DAWN
