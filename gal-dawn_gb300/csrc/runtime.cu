// Host runtime of libdawn_gb300.so: error state, device buffers, the driver
// that runs a single-source traversal as one conditional CUDA graph per
// source, CSR validation, in-edge (transpose) construction and the exact
// closeness reductions.
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "dawn_device.cuh"

namespace dawn {

namespace {
thread_local char g_err[1024] = "";
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
void clear_error() { g_err[0] = 0; }
const char* last_error() { return g_err; }

namespace {
std::once_flag g_pool_once[64];
}

dawn_status pool_alloc(void** p, size_t bytes, cudaStream_t s) {
  int dev = 0;
  DAWN_CUDA(cudaGetDevice(&dev));
  std::call_once(g_pool_once[dev & 63], [dev]() {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  });
  DAWN_CUDA(cudaMallocAsync(p, bytes ? bytes : 16, s));
  return DAWN_OK;
}

void pool_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

namespace {
std::mutex g_pin_mu;
std::vector<void*> g_pin_free;
constexpr int kPinnedChunkSlots = 64;
}  // namespace

dawn_status pinned_slot(void** p) {
  std::lock_guard<std::mutex> lock(g_pin_mu);
  if (g_pin_free.empty()) {
    char* chunk = nullptr;
    DAWN_CUDA(cudaMallocHost((void**)&chunk, kPinnedSlot * kPinnedChunkSlots));
    for (int i = kPinnedChunkSlots - 1; i >= 0; i--) g_pin_free.push_back(chunk + (size_t)i * kPinnedSlot);
  }
  *p = g_pin_free.back();
  g_pin_free.pop_back();
  return DAWN_OK;
}

void pinned_slot_release(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lock(g_pin_mu);
  g_pin_free.push_back(p);
}

dawn_status ensure(DevBuf& b, size_t bytes, cudaStream_t s) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return DAWN_OK;
  if (b.p) pool_free(b.p, b.stream);
  b.p = nullptr;
  b.bytes = 0;
  DAWN_CHECK(pool_alloc(&b.p, bytes, s));
  b.bytes = bytes;
  b.stream = s;
  return DAWN_OK;
}

void release(DevBuf& b) {
  if (b.p) pool_free(b.p, b.stream);
  b.p = nullptr;
  b.bytes = 0;
}

bool cluster_fits(const void* fn, int ctas, int threads) {
  static std::mutex mu;
  static std::vector<std::pair<const void*, bool>> known;
  std::lock_guard<std::mutex> lock(mu);
  for (const auto& k : known)
    if (k.first == fn) return k.second;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(threads);
  int clusters = 0;
  const bool fits = cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) == cudaSuccess && clusters > 0;
  cudaGetLastError();
  known.emplace_back(fn, fits);
  return fits;
}

int persistent_blocks(const void* fn, int block, size_t smem, int cap) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  if (cap > 0 && cap < per_sm) per_sm = cap;
  return sms * per_sm;
}

dawn_status upload_ctl(dawn_graph* g, const SsCtl& c) {
  // Pageable source: the runtime stages it before returning, so the stack
  // copy may go out of scope while the transfer is still queued.
  DAWN_CUDA(cudaMemcpyAsync(g->ss_ctl.p, &c, sizeof(SsCtl), cudaMemcpyHostToDevice, g->stream));
  return DAWN_OK;
}

dawn_status download_ctl(dawn_graph* g, SsCtl* out) {
  DAWN_CUDA(cudaMemcpyAsync(&g->h_ctl[1], g->ss_ctl.p, sizeof(SsCtl), cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  *out = g->h_ctl[1];
  return DAWN_OK;
}

namespace {

// The persisting-L2 carve-out of each device, set once to the device's
// maximum (a limit of this process's context; it ends with the process).
struct L2Persist {
  std::once_flag once;
  size_t carve = 0, max_window = 0;
};
L2Persist g_l2[64];

// Access-policy window of a family's body kernels: its hot arrays (the
// frontier words every level gathers from) marked persisting, so the edge
// arrays that stream through L2 at every level do not evict them.
bool family_window(const SsFamily& fam, cudaAccessPolicyWindow* w) {
  if (!fam.l2_base || fam.l2_bytes == 0) return false;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  L2Persist& p = g_l2[dev];
  std::call_once(p.once, [&p, dev] {
    int carve = 0, win = 0;
    if (cudaDeviceGetAttribute(&carve, cudaDevAttrMaxPersistingL2CacheSize, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&win, cudaDevAttrMaxAccessPolicyWindowSize, dev) != cudaSuccess || carve <= 0 ||
        win <= 0 || cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)carve) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    p.carve = (size_t)carve;
    p.max_window = (size_t)win;
  });
  if (p.carve == 0) return false;
  w->base_ptr = const_cast<void*>(fam.l2_base);
  w->num_bytes = fam.l2_bytes < p.max_window ? fam.l2_bytes : p.max_window;
  w->hitRatio = (float)((double)p.carve / (double)w->num_bytes);
  if (w->hitRatio > 1.0f) w->hitRatio = 1.0f;
  w->hitProp = cudaAccessPropertyPersisting;
  w->missProp = cudaAccessPropertyStreaming;
  return true;
}

dawn_status add_kernel(cudaGraph_t graph, cudaGraphNode_t* node, const cudaGraphNode_t* dep, const Launch& l,
                       const cudaAccessPolicyWindow* w = nullptr) {
  cudaKernelNodeParams p = {};
  p.func = const_cast<void*>(l.fn);
  p.gridDim = l.grid;
  p.blockDim = l.block;
  p.sharedMemBytes = (unsigned)l.smem;
  p.kernelParams = l.args;
  p.extra = nullptr;
  DAWN_CUDA(cudaGraphAddKernelNode(node, graph, dep, dep ? 1 : 0, &p));
  if (w) {
    cudaKernelNodeAttrValue v = {};
    v.accessPolicyWindow = *w;
    DAWN_CUDA(cudaGraphKernelNodeSetAttribute(*node, cudaKernelNodeAttributeAccessPolicyWindow, &v));
  }
  return DAWN_OK;
}

dawn_status build_graph(SsFamily& fam, cudaGraphExec_t* exec) {
  cudaGraph_t graph = nullptr;
  DAWN_CUDA(cudaGraphCreate(&graph, 0));
  dawn_status st = DAWN_OK;
  do {
    cudaGraphNode_t prev = nullptr, node = nullptr, loop = nullptr;
    for (int i = 0; i < fam.npre && st == DAWN_OK; i++) {
      st = add_kernel(graph, &node, prev ? &prev : nullptr, fam.pre[i]);
      prev = node;
    }
    if (st != DAWN_OK) break;
    cudaGraphConditionalHandle h = 0;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) {
      set_error("cudaGraphConditionalHandleCreate: %s", cudaGetErrorString(e));
      st = DAWN_ERR_CUDA;
      break;
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    e = cudaGraphAddNode(&loop, graph, prev ? &prev : nullptr, nullptr, prev ? 1 : 0, &cp);
    if (e != cudaSuccess) {
      set_error("cudaGraphAddNode(while): %s", cudaGetErrorString(e));
      st = DAWN_ERR_CUDA;
      break;
    }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    *fam.handle = h;
    *fam.in_graph = 1;
    cudaAccessPolicyWindow win;
    const bool has_win = family_window(fam, &win);
    cudaGraphNode_t bprev = nullptr;
    for (int i = 0; i < fam.nbody && st == DAWN_OK; i++) {
      st = add_kernel(body, &node, bprev ? &bprev : nullptr, fam.body[i], has_win ? &win : nullptr);
      bprev = node;
    }
    if (st != DAWN_OK) break;
    cudaGraphNode_t pprev = loop;
    for (int i = 0; i < fam.npost && st == DAWN_OK; i++) {
      st = add_kernel(graph, &node, &pprev, fam.post[i]);
      pprev = node;
    }
    if (st != DAWN_OK) break;
    e = cudaGraphInstantiate(exec, graph, 0);
    if (e != cudaSuccess) {
      set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
      *exec = nullptr;
      st = DAWN_ERR_CUDA;
      break;
    }
  } while (0);
  cudaGraphDestroy(graph);
  *fam.in_graph = 0;
  *fam.handle = 0;
  return st;
}

dawn_status launch(const Launch& l, cudaStream_t s, const cudaAccessPolicyWindow* w = nullptr) {
  if (!w) {
    DAWN_CUDA(cudaLaunchKernel(l.fn, l.grid, l.block, l.args, l.smem, s));
    return DAWN_OK;
  }
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeAccessPolicyWindow;
  attr.val.accessPolicyWindow = *w;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = l.grid;
  cfg.blockDim = l.block;
  cfg.dynamicSmemBytes = l.smem;
  cfg.stream = s;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  DAWN_CUDA(cudaLaunchKernelExC(&cfg, l.fn, l.args));
  return DAWN_OK;
}

constexpr int kPollLevels = 4;  // host-loop form: levels launched between polls

}  // namespace

// Traced form: level by level from the host, CUDA events around each kernel
// that does work at that level, one trace record per kernel.
dawn_status ss_run_traced(dawn_graph* g, SsFamily& fam, int32_t nruns) {
  *fam.in_graph = 0;
  cudaAccessPolicyWindow win;
  const bool has_win = family_window(fam, &win);
  for (int i = 0; i < 10; i++)
    if (!g->trace_ev[i]) DAWN_CUDA(cudaEventCreate(&g->trace_ev[i]));
  std::vector<unsigned char> host(fam.ctl_bytes);
  struct Pending {
    int body;
    LevelProbe p;
  };
  // Times the launches of one stage (pre or post kernels) as level 0 / -1 records.
  auto timed_stage = [&](const Launch* ls, int cnt, int run, int level) -> dawn_status {
    for (int j = 0; j < cnt; j++) {
      DAWN_CUDA(cudaEventRecord(g->trace_ev[0], g->stream));
      DAWN_CHECK(launch(ls[j], g->stream));
      DAWN_CUDA(cudaEventRecord(g->trace_ev[1], g->stream));
      DAWN_CUDA(cudaEventSynchronize(g->trace_ev[1]));
      dawn_trace_rec r = {};
      std::snprintf(r.kernel, sizeof(r.kernel), "%s", ls[j].name);
      r.run = run;
      r.level = level;
      r.mode = -1;
      DAWN_CUDA(cudaEventElapsedTime(&r.ms, g->trace_ev[0], g->trace_ev[1]));
      g->trace_log.push_back(r);
    }
    return DAWN_OK;
  };
  for (int32_t run = 0; run < nruns; run++) {
    DAWN_CHECK(timed_stage(fam.pre, fam.npre, run, 0));
    for (;;) {
      DAWN_CUDA(cudaMemcpyAsync(host.data(), fam.ctl, fam.ctl_bytes, cudaMemcpyDeviceToHost, g->stream));
      DAWN_CUDA(cudaStreamSynchronize(g->stream));
      LevelProbe p;
      fam.probe(host.data(), &p);
      if (p.done) break;
      Pending pend[5];
      int np = 0;
      const int nwork = fam.decide_in_body ? fam.nbody : fam.nbody - 1;
      for (int b = 0; b < nwork; b++) {
        const int bm = fam.body[b].mode;
        const bool match = bm < 0 || bm == p.mode || (bm == kModeStep && (p.mode == kModePush || p.mode == kModePull));
        if (!match) continue;
        DAWN_CUDA(cudaEventRecord(g->trace_ev[2 * np], g->stream));
        DAWN_CHECK(launch(fam.body[b], g->stream, has_win ? &win : nullptr));
        DAWN_CUDA(cudaEventRecord(g->trace_ev[2 * np + 1], g->stream));
        pend[np++] = {b, p};
        if (fam.decide_in_body) break;  // the kernel ran the level and its bookkeeping
      }
      if (!fam.decide_in_body) DAWN_CHECK(launch(fam.body[fam.nbody - 1], g->stream, has_win ? &win : nullptr));
      DAWN_CUDA(cudaStreamSynchronize(g->stream));
      for (int i = 0; i < np; i++) {
        dawn_trace_rec r = {};
        std::snprintf(r.kernel, sizeof(r.kernel), "%s", fam.body[pend[i].body].name);
        r.run = run;
        r.level = pend[i].p.level;
        r.mode = pend[i].p.mode;
        r.frontier = pend[i].p.frontier;
        r.frontier_edges = pend[i].p.frontier_edges;
        r.unvisited_edges = pend[i].p.unvisited_edges;
        DAWN_CUDA(cudaEventElapsedTime(&r.ms, g->trace_ev[2 * i], g->trace_ev[2 * i + 1]));
        g->trace_log.push_back(r);
      }
    }
    DAWN_CHECK(timed_stage(fam.post, fam.npost, run, -1));
  }
  return DAWN_OK;
}

dawn_status ss_run(dawn_graph* g, SsFamily& fam, int32_t nruns, cudaGraphExec_t* exec) {
  if (g->trace && fam.probe) return ss_run_traced(g, fam, nruns);
  if (g->graphs_ok && !*exec) {
    if (build_graph(fam, exec) != DAWN_OK) {
      g->graphs_ok = false;  // report once, then run the host level loop
      std::fprintf(stderr, "dawn: conditional graphs unavailable (%s); using the host level loop\n",
                   last_error());
      cudaGetLastError();
      clear_error();
    }
  }
  if (g->graphs_ok && *exec) {
    for (int32_t i = 0; i < nruns; i++) DAWN_CUDA(cudaGraphLaunch(*exec, g->stream));
    return DAWN_OK;
  }
  *fam.in_graph = 0;
  cudaAccessPolicyWindow win;
  const bool has_win = family_window(fam, &win);
  int32_t* h_done = &g->h_ctl[1].done;
  for (int32_t i = 0; i < nruns; i++) {
    for (int j = 0; j < fam.npre; j++) DAWN_CHECK(launch(fam.pre[j], g->stream));
    for (;;) {
      for (int j = 0; j < kPollLevels; j++)
        for (int b = 0; b < fam.nbody; b++) DAWN_CHECK(launch(fam.body[b], g->stream, has_win ? &win : nullptr));
      DAWN_CUDA(cudaMemcpyAsync(h_done, fam.done_flag, sizeof(int32_t), cudaMemcpyDeviceToHost, g->stream));
      DAWN_CUDA(cudaStreamSynchronize(g->stream));
      if (*h_done) break;
    }
    for (int j = 0; j < fam.npost; j++) DAWN_CHECK(launch(fam.post[j], g->stream));
  }
  return DAWN_OK;
}

// --- CSR validation -----------------------------------------------------------

namespace {

__device__ __forceinline__ int check_entry(int32_t c, int32_t n, const void* val, int wtype, size_t k) {
  int f = (c < 0 || c >= n) ? 8 : 0;
  if (wtype == DAWN_W_I32 && static_cast<const int32_t*>(val)[k] < 0) f |= 16;
  if (wtype == DAWN_W_F32) {
    const float w = static_cast<const float*>(val)[k];
    if (!(w >= 0.0f) || isinf(w)) f |= 16;
  }
  return f;
}

// One pass over row_ptr and col (128-bit loads) checking the CSR invariants
// the kernels rely on: monotone row_ptr from 0 to m, columns in [0, n),
// weights finite and non-negative.
__global__ void validate_csr_kernel(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                    const void* __restrict__ val, int wtype, int32_t n, long long m,
                                    int* __restrict__ flags) {
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  int f = 0;
  if (tid == 0) {
    if (rp[0] != 0) f |= 1;
    if ((long long)rp[n] != m) f |= 2;
  }
  for (size_t i = tid; i < (size_t)n; i += stride)
    if (rp[i] > rp[i + 1]) f |= 4;
  const size_t m4 = (size_t)m / 4;
  const int4* c4 = reinterpret_cast<const int4*>(col);
  for (size_t q = tid; q < m4; q += stride) {
    const int4 c = c4[q];
    const int32_t cc[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int j = 0; j < 4; j++) f |= check_entry(cc[j], n, val, wtype, 4 * q + j);
  }
  for (size_t k = 4 * m4 + tid; k < (size_t)m; k += stride) f |= check_entry(col[k], n, val, wtype, k);
  if (f) atomicOr(flags, f);
}

}  // namespace

dawn_status validate_csr(dawn_graph* g) {
  int* d_flags = nullptr;
  DAWN_CUDA(cudaMallocAsync(&d_flags, sizeof(int), g->stream));
  DAWN_CUDA(cudaMemsetAsync(d_flags, 0, sizeof(int), g->stream));
  validate_csr_kernel<<<g->geo.sms * 8, kBlock, 0, g->stream>>>(g->row_ptr, g->col, g->val, g->wtype, g->n, g->m,
                                                                 d_flags);
  DAWN_CUDA(cudaGetLastError());
  int flags = 0;
  DAWN_CUDA(cudaMemcpyAsync(&flags, d_flags, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaFreeAsync(d_flags, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  if (flags) {
    set_error("invalid CSR:%s%s%s%s%s", (flags & 1) ? " row_ptr[0] != 0;" : "",
              (flags & 2) ? " row_ptr[n] != m;" : "", (flags & 4) ? " row_ptr decreases;" : "",
              (flags & 8) ? " col index outside [0, n);" : "",
              (flags & 16) ? " negative or non-finite weight;" : "");
    return DAWN_ERR_INVALID_ARG;
  }
  return DAWN_OK;
}

// --- exclusive scan (int64), used for the in-edge CSR ---------------------------

namespace {

constexpr int kScanBlock = 1024;

__global__ void __launch_bounds__(kScanBlock) scan_block(const int64_t* __restrict__ in, int64_t* __restrict__ out,
                                                         long long n, int64_t* __restrict__ sums) {
  __shared__ long long warp_tot[kScanBlock / 32];
  const long long i = blockIdx.x * (long long)kScanBlock + threadIdx.x;
  const long long x = i < n ? in[i] : 0;
  long long v = x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    long long y = __shfl_up_sync(kFull, v, d);
    if (lane >= d) v += y;
  }
  if (lane == 31) warp_tot[w] = v;
  __syncthreads();
  if (w == 0) {
    long long t = warp_tot[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      long long y = __shfl_up_sync(kFull, t, d);
      if (lane >= d) t += y;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  const long long incl = v + (w ? warp_tot[w - 1] : 0);
  if (i < n) out[i] = incl - x;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = incl;
}

__global__ void add_block_offsets(int64_t* __restrict__ out, long long n, const int64_t* __restrict__ offs) {
  const long long i = blockIdx.x * (long long)kScanBlock + threadIdx.x;
  if (i < n) out[i] += offs[blockIdx.x];
}

}  // namespace

dawn_status exclusive_scan_i64(const int64_t* d_in, int64_t* d_out, int64_t n, cudaStream_t s) {
  if (n <= 0) return DAWN_OK;
  const long long nb = (n + kScanBlock - 1) / kScanBlock;
  int64_t* sums = nullptr;
  DAWN_CUDA(cudaMallocAsync(&sums, sizeof(int64_t) * 2 * nb, s));
  scan_block<<<(unsigned)nb, kScanBlock, 0, s>>>(d_in, d_out, n, sums);
  DAWN_CUDA(cudaGetLastError());
  if (nb > 1) {
    DAWN_CHECK(exclusive_scan_i64(sums, sums + nb, nb, s));
    add_block_offsets<<<(unsigned)nb, kScanBlock, 0, s>>>(d_out, n, sums + nb);
    DAWN_CUDA(cudaGetLastError());
  }
  DAWN_CUDA(cudaFreeAsync(sums, s));
  return DAWN_OK;
}

// --- in-edge CSR -------------------------------------------------------------------

namespace {

__global__ void count_in_degree(const int32_t* __restrict__ col, long long m,
                                unsigned long long* __restrict__ deg) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < (size_t)m; k += stride)
    atomicAdd(deg + col[k], 1ull);
}

__global__ void offsets_to_rowptr(const int64_t* __restrict__ off, int32_t* __restrict__ rp,
                                  unsigned long long* __restrict__ cursor, int32_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i <= (size_t)n; i += stride) {
    rp[i] = (int32_t)off[i];
    cursor[i] = (unsigned long long)off[i];
  }
}

__global__ void scatter_in_edges(const int32_t* __restrict__ rp, const int32_t* __restrict__ col, int32_t n,
                                 unsigned long long* __restrict__ cursor, int32_t* __restrict__ t_col) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
    const int e = rp[u + 1];
    for (int k = rp[u] + lane; k < e; k += 32) {
      const int32_t v = col[k];
      t_col[atomicAdd(cursor + v, 1ull)] = u;
    }
  }
}

__global__ void init_cursor(const int32_t* __restrict__ t_row_ptr, unsigned long long* __restrict__ cursor,
                            int32_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride)
    cursor[i] = (unsigned long long)t_row_ptr[i];
}

__global__ void scatter_weighted_in_edges(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                          const int32_t* __restrict__ val, int32_t n,
                                          unsigned long long* __restrict__ cursor, int32_t* __restrict__ t_col,
                                          int32_t* __restrict__ t_val) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
    const int e = rp[u + 1];
    for (int k = rp[u] + lane; k < e; k += 32) {
      const unsigned long long slot = atomicAdd(cursor + col[k], 1ull);
      t_col[slot] = u;
      t_val[slot] = val[k];
    }
  }
}

}  // namespace

dawn_status build_weighted_in_edges(dawn_graph* g) {
  if (g->wt_col.p) return DAWN_OK;
  const int32_t n = g->n;
  const cudaStream_t s = g->stream;
  unsigned long long* cursor = nullptr;
  DAWN_CHECK(pool_alloc((void**)&cursor, sizeof(unsigned long long) * ((size_t)n + 1), s));
  DAWN_CHECK(ensure(g->wt_col, sizeof(int32_t) * (size_t)(g->m > 0 ? g->m : 1) + 16, s));
  DAWN_CHECK(ensure(g->wt_val, sizeof(int32_t) * (size_t)(g->m > 0 ? g->m : 1) + 16, s));
  const int grid = g->geo.sms * 8;
  init_cursor<<<grid, kBlock, 0, s>>>(g->t_row_ptr, cursor, n);
  DAWN_CUDA(cudaGetLastError());
  // 32-bit weights (int32 or float32 bit patterns) move as words
  scatter_weighted_in_edges<<<grid, kBlock, 0, s>>>(g->row_ptr, g->col, static_cast<const int32_t*>(g->val), n,
                                                    cursor, g->wt_col.as<int32_t>(), g->wt_val.as<int32_t>());
  DAWN_CUDA(cudaGetLastError());
  pool_free(cursor, s);
  return DAWN_OK;
}

dawn_status build_transpose(dawn_graph* g) {
  const int32_t n = g->n;
  const cudaStream_t s = g->stream;
  unsigned long long* deg = nullptr;
  int64_t* off = nullptr;
  DAWN_CUDA(cudaMallocAsync(&deg, sizeof(unsigned long long) * ((size_t)n + 1), s));
  DAWN_CUDA(cudaMallocAsync(&off, sizeof(int64_t) * ((size_t)n + 1), s));
  DAWN_CUDA(cudaMemsetAsync(deg, 0, sizeof(unsigned long long) * ((size_t)n + 1), s));
  const int grid = g->geo.sms * 8;
  count_in_degree<<<grid, kBlock, 0, s>>>(g->col, g->m, deg);
  DAWN_CUDA(cudaGetLastError());
  DAWN_CHECK(exclusive_scan_i64(reinterpret_cast<const int64_t*>(deg), off, (int64_t)n + 1, s));
  DAWN_CHECK(pool_alloc((void**)&g->t_row_ptr, sizeof(int32_t) * ((size_t)n + 1), s));
  DAWN_CHECK(pool_alloc((void**)&g->t_col, sizeof(int32_t) * (size_t)(g->m > 0 ? g->m : 1) + 32, s));
  offsets_to_rowptr<<<grid, kBlock, 0, s>>>(off, g->t_row_ptr, deg, n);
  DAWN_CUDA(cudaGetLastError());
  scatter_in_edges<<<grid, kBlock, 0, s>>>(g->row_ptr, g->col, n, deg, g->t_col);
  DAWN_CUDA(cudaGetLastError());
  DAWN_CUDA(cudaFreeAsync(deg, s));
  DAWN_CUDA(cudaFreeAsync(off, s));
  return DAWN_OK;
}

// --- closeness: exact per-row reductions ----------------------------------------------

namespace {

// kind 0: hop rows (-1 unreachable); 1: int32 weights (INT32_MAX); 2: float (FLT_MAX).
template <bool kDegree>
__global__ void __launch_bounds__(kBlock) row_sums(const void* __restrict__ dist, int32_t n,
                                                   const int32_t* __restrict__ row_ptr,
                                                   const int32_t* __restrict__ sources, int kind, int row0,
                                                   long long* __restrict__ isum, double* __restrict__ fsum,
                                                   unsigned long long* __restrict__ cnt) {
  const int row = row0 + blockIdx.y;
  const int32_t s = sources[row];
  long long is = 0;
  double fs = 0.0;
  unsigned long long c = 0;
  const size_t base = (size_t)row * n;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    bool reached;
    double fd = 0.0;
    long long id = 0;
    if (kind == 2) {
      const float d = static_cast<const float*>(dist)[base + v];
      reached = d != 3.402823466e+38f;
      fd = (double)d;
    } else {
      const int32_t d = static_cast<const int32_t*>(dist)[base + v];
      reached = kind == 0 ? d >= 0 : d != 0x7fffffff;
      id = d;
    }
    if (kDegree) {
      if (reached) is += row_ptr[v + 1] - row_ptr[v];
    } else if (reached && v != s) {
      if (kind == 2) fs += fd; else is += id;
      c++;
    }
  }
  __shared__ long long s_i[kBlock / 32];
  __shared__ double s_f[kBlock / 32];
  __shared__ unsigned long long s_c[kBlock / 32];
  for (int d = 16; d; d >>= 1) {
    is += __shfl_xor_sync(kFull, is, d);
    fs += __shfl_xor_sync(kFull, fs, d);
    c += __shfl_xor_sync(kFull, c, d);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    s_i[w] = is;
    s_f[w] = fs;
    s_c[w] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long ti = 0;
    double tf = 0;
    unsigned long long tc = 0;
    for (int i = 0; i < kBlock / 32; i++) {
      ti += s_i[i];
      tf += s_f[i];
      tc += s_c[i];
    }
    if (ti) atomicAdd(reinterpret_cast<unsigned long long*>(isum + row), (unsigned long long)ti);
    if (tf != 0.0) atomicAdd(fsum + row, tf);
    if (tc) atomicAdd(cnt + row, tc);
  }
}

}  // namespace

dawn_status row_reduce(dawn_graph* g, const void* d_dist, int32_t nsrc, const int32_t* d_sources, int kind,
                       int degree, double* d_sum, long long* d_cnt) {
  // Integer sums are exact; a float64 sum is exact while the distances are
  // integer-valued (the benchmark weights), otherwise order-dependent in the
  // last bits.  d_sum holds int64 bits for kinds 0/1 and for degree sums.
  DAWN_CUDA(cudaMemsetAsync(d_sum, 0, sizeof(double) * nsrc, g->stream));
  DAWN_CUDA(cudaMemsetAsync(d_cnt, 0, sizeof(long long) * nsrc, g->stream));
  int bx = (g->n + kBlock * 8 - 1) / (kBlock * 8);
  if (bx > 4 * g->geo.sms) bx = 4 * g->geo.sms;
  if (bx < 1) bx = 1;
  for (int32_t r0 = 0; r0 < nsrc; r0 += 65535) {
    const int rows = nsrc - r0 < 65535 ? nsrc - r0 : 65535;
    dim3 grid(bx, rows);
    if (degree)
      row_sums<true><<<grid, kBlock, 0, g->stream>>>(d_dist, g->n, g->row_ptr, d_sources, kind, r0,
                                                     reinterpret_cast<long long*>(d_sum), d_sum,
                                                     reinterpret_cast<unsigned long long*>(d_cnt));
    else
      row_sums<false><<<grid, kBlock, 0, g->stream>>>(d_dist, g->n, g->row_ptr, d_sources, kind, r0,
                                                      reinterpret_cast<long long*>(d_sum), d_sum,
                                                      reinterpret_cast<unsigned long long*>(d_cnt));
    DAWN_CUDA(cudaGetLastError());
  }
  return DAWN_OK;
}

}  // namespace dawn
