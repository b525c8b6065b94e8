// ORACLE — test infrastructure only.
//
// C entry points around the reference's own, unmodified single-source GPU
// path: SOVM and the BFS_GPU::kernel level loop
// (src/algorithm/gpu/bfs.cu:9-105), GOVM and the SSSP_GPU::kernel level loop
// (src/algorithm/gpu/sssp.cu:30-129).  oracle/Makefile (target ref-gpu)
// compiles those files from where they lie, for sm_103a, into
// oracle/_ref/libdawn_ref_gpu.so.  They serve one purpose: timing the
// reference's GPU kernels on this GPU next to this library's, after checking
// what they compute.  The reference hands its distances only to
// DAWN::IO::outfile (src/io.cpp:215-281); this file defines the two
// per-source overloads to copy the array out instead of writing text.
//
// BFS_GPU::run / SSSP_GPU::run (bfs.cu:107-129, sssp.cu:131-157) upload the
// CSR and then call kernel(); here the upload happens once per handle and
// kernel() is called per source with the same arguments run() passes
// (the CSR device vectors by value, as the reference's signature takes
// them).  run()'s isolated-source check ends the process with exit(0), so
// the caller must pass sources with at least one out-edge; ref_gpu_bfs and
// ref_gpu_sssp refuse others with -2.  A CUDA error (thrust throws them)
// comes back as a negative status, never as an exception across the C ABI.

#include <dawn/algorithm/gpu/bfs.cuh>
#include <dawn/algorithm/gpu/sssp.cuh>

#include <cstring>

namespace {
thread_local int32_t* g_cap_i = nullptr;
thread_local float* g_cap_f = nullptr;
}  // namespace

namespace DAWN {
namespace IO {
void outfile(int n, int* result, int, std::string&) {
  if (g_cap_i) std::memcpy(g_cap_i, result, sizeof(int) * (size_t)n);
}
void outfile(int n, float* result, int, std::string&) {
  if (g_cap_f) std::memcpy(g_cap_f, result, sizeof(float) * (size_t)n);
}
}  // namespace IO
}  // namespace DAWN

namespace {
struct RefGpu {
  std::vector<int> row_ptr, col;
  std::vector<float> val;
  thrust::device_vector<int> d_row_ptr, d_col;
  thrust::device_vector<float> d_val;
  DAWN::Graph::Graph_t graph;
  cudaStream_t stream = nullptr;
};

int cuda_status() {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? 0 : -(int)e - 1000;
}
}  // namespace

extern "C" {

// Host copies of the CSR (the level loops read the source's row on the
// host) and one device upload, as BFS_GPU::run / SSSP_GPU::run make it.
// val may be null (hop distances only).  block_size: the reference's
// graph.block_size (1024 in its GPU drivers, algorithm/gpu/*/*.cu).
void* ref_gpu_open(const int32_t* row_ptr, const int32_t* col, const float* val, int32_t n, int64_t nnz,
                   int32_t block_size) try {
  auto* h = new RefGpu();
  h->row_ptr.assign(row_ptr, row_ptr + (size_t)n + 1);
  h->col.assign(col, col + (size_t)nnz);
  if (val) h->val.assign(val, val + (size_t)nnz);
  h->d_row_ptr = h->row_ptr;
  h->d_col = h->col;
  if (val) h->d_val = h->val;
  DAWN::Graph::Graph_t& g = h->graph;
  g.rows = n;
  g.cols = n;
  g.nnz = (uint64_t)nnz;
  g.csr.row_ptr = h->row_ptr.data();
  g.csr.col = h->col.data();
  g.csr.val = val ? h->val.data() : nullptr;
  g.thread = 1;
  g.interval = 100;
  g.stream = 1;
  g.block_size = block_size;
  g.source = 0;
  g.print = true;
  g.weighted = val != nullptr;
  g.directed = true;
  cudaStreamCreate(&h->stream);
  if (cuda_status() != 0) {
    delete h;
    return nullptr;
  }
  return h;
} catch (...) {  // thrust reports CUDA errors by exception
  return nullptr;
}

void ref_gpu_close(void* p) {
  auto* h = static_cast<RefGpu*>(p);
  if (!h) return;
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

// BFS_GPU::kernel from one source: dist receives the array it prints
// (0 = unreached, as in the reference); *ms its own elapsed time (host
// clock around the level loop, bfs.cu:75-101).  0 on success.
int ref_gpu_bfs(void* p, int32_t source, int32_t* dist, float* ms) try {
  auto* h = static_cast<RefGpu*>(p);
  DAWN::Graph::Graph_t& g = h->graph;
  if (source < 0 || source >= g.rows || g.csr.row_ptr[source] == g.csr.row_ptr[source + 1]) return -2;
  g.source = source;
  std::string path;
  g_cap_i = dist;
  *ms = DAWN::BFS_GPU::kernel(g, source, h->stream, h->d_row_ptr, h->d_col, path);
  g_cap_i = nullptr;
  return cuda_status();
} catch (...) {
  g_cap_i = nullptr;
  return -4;
}

// SSSP_GPU::kernel from one source (float weights): dist receives the
// printed array (FLT_MAX = unreached); *ms as above (sssp.cu:91-120).
int ref_gpu_sssp(void* p, int32_t source, float* dist, float* ms) try {
  auto* h = static_cast<RefGpu*>(p);
  DAWN::Graph::Graph_t& g = h->graph;
  if (!g.weighted) return -3;
  if (source < 0 || source >= g.rows || g.csr.row_ptr[source] == g.csr.row_ptr[source + 1]) return -2;
  g.source = source;
  std::string path;
  g_cap_f = dist;
  *ms = DAWN::SSSP_GPU::kernel(g, source, h->stream, h->d_row_ptr, h->d_col, h->d_val, path);
  g_cap_f = nullptr;
  return cuda_status();
} catch (...) {
  g_cap_f = nullptr;
  return -4;
}

}  // extern "C"
