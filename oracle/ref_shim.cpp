// ORACLE — test infrastructure only.
//
// C entry points around the reference's own, unmodified CPU algorithm files
// (src/algorithm/cpu/{bfs,sssp,cc,mssp,bc}.cpp, src/matrix.cpp, src/tool.cpp),
// compiled from where they lie by oracle/Makefile into oracle/_ref/.  The
// reference reports results only through DAWN::IO::outfile
// (src/io.cpp:215-281); this file defines those four overloads to capture
// the distance array instead of writing text, so the reference's results
// can be compared in-process.

#include <dawn/algorithm/cpu/bc.hxx>
#include <dawn/algorithm/cpu/bfs.hxx>
#include <dawn/algorithm/cpu/cc.hxx>
#include <dawn/algorithm/cpu/mssp.hxx>
#include <dawn/algorithm/cpu/sssp.hxx>

#include <cstring>
#include <mutex>

namespace {
thread_local int32_t* g_cap_i = nullptr;
thread_local float* g_cap_f = nullptr;
// Multi-source capture: source vertex -> destination row (first index wins).
std::mutex g_mu;
int32_t** g_rows_i = nullptr;
float** g_rows_f = nullptr;
}  // namespace

namespace DAWN {
namespace IO {
void outfile(int n, int* result, int source, std::string&) {
  if (g_cap_i) {
    std::memcpy(g_cap_i, result, sizeof(int) * (size_t)n);
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_rows_i && g_rows_i[source])
    std::memcpy(g_rows_i[source], result, sizeof(int) * (size_t)n);
}
void outfile(int n, float* result, int source, std::string&) {
  if (g_cap_f) {
    std::memcpy(g_cap_f, result, sizeof(float) * (size_t)n);
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_rows_f && g_rows_f[source])
    std::memcpy(g_rows_f[source], result, sizeof(float) * (size_t)n);
}
void outfile(int, int*, std::string&) {}
void outfile(int n, float* result, std::string&) {
  if (g_cap_f) std::memcpy(g_cap_f, result, sizeof(float) * (size_t)n);
}
}  // namespace IO
}  // namespace DAWN

extern "C" {

// BFS_CPU::BFS_kernel (queue form, bfs.cpp:79-132).
void ref_bfs_kernel(const int32_t* row_ptr, const int32_t* col, int32_t n,
                    int32_t source, int32_t* dist) {
  std::string path;
  g_cap_i = dist;
  DAWN::BFS_CPU::BFS_kernel(const_cast<int*>(row_ptr), const_cast<int*>(col), n,
                            source, true, path);
  g_cap_i = nullptr;
}

// BFS_CPU::BFS (bitmap form, bfs.cpp:23-77).
void ref_bfs_bitmap(const int32_t* row_ptr, const int32_t* col, int32_t n,
                    int32_t source, int32_t* dist) {
  std::string path;
  g_cap_i = dist;
  DAWN::BFS_CPU::BFS(const_cast<int*>(row_ptr), const_cast<int*>(col), n,
                     source, true, path);
  g_cap_i = nullptr;
}

// SSSP_CPU::SSSP (bitmap min-plus, sssp.cpp:23-80).  Runs on one OpenMP
// thread: with more, the unsynchronised min at sssp.cpp:186-189 loses
// updates and returns wrong distances.
void ref_sssp(const int32_t* row_ptr, const int32_t* col, const float* val,
              int32_t n, int32_t source, float* dist) {
  std::string path;
  const int saved = omp_get_max_threads();
  omp_set_num_threads(1);
  g_cap_f = dist;
  DAWN::SSSP_CPU::SSSP(const_cast<int*>(row_ptr), const_cast<int*>(col),
                       const_cast<float*>(val), n, source, true, path);
  g_cap_f = nullptr;
  omp_set_num_threads(saved);
}

// Same call on the reference's default OpenMP team (racy; for the record).
void ref_sssp_threaded(const int32_t* row_ptr, const int32_t* col,
                       const float* val, int32_t n, int32_t source,
                       float* dist) {
  std::string path;
  g_cap_f = dist;
  DAWN::SSSP_CPU::SSSP(const_cast<int*>(row_ptr), const_cast<int*>(col),
                       const_cast<float*>(val), n, source, true, path);
  g_cap_f = nullptr;
}

// CC_CPU::kernel / kernel_Weighted (cc.cpp:37-142); returns the reference's value.
float ref_cc(const int32_t* row_ptr, const int32_t* col, const float* val,
             int32_t n, int32_t source) {
  float t = 0.0f;
  if (val) {
    const int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    float cc = DAWN::CC_CPU::kernel_Weighted(const_cast<int*>(row_ptr),
                                             const_cast<int*>(col),
                                             const_cast<float*>(val), n, source, t);
    omp_set_num_threads(saved);
    return cc;
  }
  return DAWN::CC_CPU::kernel(const_cast<int*>(row_ptr), const_cast<int*>(col),
                              n, source, t);
}

// BC_CPU::Betweenness_Centrality (bc.cpp:9-39): BCDAWN summed over every
// vertex as a source, float32, as the reference's bc_cpu computes it.
void ref_bc(const int32_t* row_ptr, const int32_t* col, int32_t n, float* bc) {
  DAWN::Graph::Graph_t graph;
  graph.rows = n;
  graph.cols = n;
  graph.nnz = (uint64_t)row_ptr[n];
  graph.csr.row_ptr = const_cast<int*>(row_ptr);
  graph.csr.col = const_cast<int*>(col);
  std::string path;
  g_cap_f = bc;
  DAWN::BC_CPU::Betweenness_Centrality(graph, path);
  g_cap_f = nullptr;
  graph.csr.row_ptr = nullptr;
  graph.csr.col = nullptr;
}

// MSSP_CPU::run (mssp.cpp:9-32) over a caller CSR.  With dist == NULL the
// reference runs with print = false (the timed configuration); otherwise
// each distinct source's row is captured into dist (nsrc x n).
float ref_mssp_run(const int32_t* row_ptr, const int32_t* col,
                   const float* val, int32_t n, int64_t nnz,
                   const int32_t* sources, int32_t nsrc, int32_t weighted,
                   int32_t* dist, float* dist_f) {
  DAWN::Graph::Graph_t g;
  g.rows = n;
  g.cols = n;
  g.nnz = (uint64_t)nnz;
  g.csr.row_ptr = const_cast<int*>(row_ptr);
  g.csr.col = const_cast<int*>(col);
  g.csr.val = const_cast<float*>(val);
  g.thread = 1;
  g.interval = 100;
  g.stream = 1;
  g.block_size = 1024;
  g.source = 0;
  g.weighted = weighted != 0;
  g.directed = true;
  g.print = dist != nullptr || dist_f != nullptr;
  g.msource.assign(sources, sources + nsrc);
  std::vector<int32_t*> rows_i;
  std::vector<float*> rows_f;
  if (dist) {
    std::memset(dist, 0, sizeof(int32_t) * (size_t)nsrc * n);
    rows_i.assign((size_t)n, nullptr);
    for (int32_t i = nsrc - 1; i >= 0; i--)
      rows_i[sources[i] % n] = dist + (size_t)i * n;
    g_rows_i = rows_i.data();
  }
  if (dist_f) {
    for (size_t i = 0; i < (size_t)nsrc * n; i++) dist_f[i] = 0.0f;
    rows_f.assign((size_t)n, nullptr);
    for (int32_t i = nsrc - 1; i >= 0; i--)
      rows_f[sources[i] % n] = dist_f + (size_t)i * n;
    g_rows_f = rows_f.data();
  }
  std::string path;
  float t = DAWN::MSSP_CPU::run(g, path);
  g_rows_i = nullptr;
  g_rows_f = nullptr;
  if (dist) {  // duplicate sources: copy the captured row to every slot
    for (int32_t i = 0; i < nsrc; i++) {
      int32_t* first = rows_i[sources[i] % n];
      if (first != dist + (size_t)i * n)
        std::memcpy(dist + (size_t)i * n, first, sizeof(int32_t) * (size_t)n);
    }
  }
  g.csr.row_ptr = nullptr;
  return t;
}

}  // extern "C"
