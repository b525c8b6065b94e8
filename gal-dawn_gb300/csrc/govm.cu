// Single-source min-plus relax (GOVM) on sm_103a.
//
// Replaces the reference's GOVM kernel, its CAS-loop float atomicMin and the
// host loop around them (src/algorithm/gpu/sssp.cu:18-129).  The reference
// sweeps all n rows every level, clears the consumed frontier with an extra
// thrust::fill_n launch and retries a CAS loop per relaxation.  Here:
//   * distances live as 32-bit words compared as signed integers: int32
//     weights natively, float32 weights through their bit pattern, which
//     orders exactly like the value for the non-negative floats the graph
//     validation admits, so one hardware atomicMin replaces the CAS loop;
//   * the frontier is a compacted queue expanded warp-cooperatively (the same
//     edge dealing as the boolean expand), with a per-level "queued" bitmap
//     so a vertex improved by several edges is queued once;
//   * the source row is resolved as the reference CPU path does
//     (src/algorithm/cpu/sssp.cpp:41-46): each distinct neighbour takes the
//     weight of its last CSR entry, all of them form the first frontier, the
//     source is set to 0 and is never relaxed afterwards.
// Any relaxation order reaches the same fixed point, so the distances equal
// the reference's for integer-valued weights.
#include "dawn_device.cuh"

namespace dawn {
namespace {

__device__ __forceinline__ int32_t relax_sum(int32_t dv, int k, const int32_t* __restrict__ wi,
                                             const float* __restrict__ wf, bool is_float) {
  if (is_float) return __float_as_int(__fadd_rn(__int_as_float(dv), __ldg(wf + k)));
  return dv + __ldg(wi + k);
}

__global__ void __launch_bounds__(kBlock) sssp_clear(SsCtl* __restrict__ ctl, uint32_t* __restrict__ inq,
                                                     int32_t n, int32_t nwords, int32_t inf) {
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride) dist[i] = inf;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)2 * nwords; i += stride) inq[i] = 0;
}

// One CTA: resolve the source row (last CSR entry of a repeated neighbour
// wins), seed the first frontier, then set the source to 0.
__global__ void __launch_bounds__(kBlock) sssp_init(SsCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                                                    const int32_t* __restrict__ col, const int32_t* __restrict__ wi,
                                                    const float* __restrict__ wf, int is_float,
                                                    unsigned long long* __restrict__ last, int32_t* __restrict__ q,
                                                    Seg* __restrict__ segs, int32_t n) {
  const int32_t s = ctl->sources[ctl->src_idx];
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  const int rs = row_ptr[s], re = row_ptr[s + 1];
  if (threadIdx.x == 0) {
    ctl->source = s;
    ctl->qsize[0] = 0;
    ctl->qsize[1] = 0;
    ctl->lpack[0] = 0;
    ctl->lpack[1] = 0;
    ctl->level = 1;
    ctl->n_push = 0;
    ctl->n_pull = 0;
    ctl->reached = 0;
  }
  for (int k = rs + threadIdx.x; k < re; k += blockDim.x) last[col[k]] = 0;
  __syncthreads();
  for (int k = rs + threadIdx.x; k < re; k += blockDim.x) atomicMax(last + col[k], (unsigned long long)(k + 1));
  __syncthreads();
  for (int k = rs + threadIdx.x; k < re; k += blockDim.x) {
    const int32_t u = col[k];
    if (last[u] == (unsigned long long)(k + 1)) {
      dist[u] = is_float ? __float_as_int(__ldg(wf + k)) : __ldg(wi + k);
      // winners are unique: no dedup bit needed
      const int urs = row_ptr[u], udeg = row_ptr[u + 1] - urs;
      if (udeg >= kLongRow) {
        const int nseg = (udeg + kSeg - 1) / kSeg;
        const unsigned long long old = atomicAdd(&ctl->lpack[0], (1ull << 32) | (unsigned)nseg);
        for (int j = 0; j < nseg; j++) segs[(uint32_t)old + j] = Seg{u, urs + j * kSeg};
      } else {
        q[atomicAdd(&ctl->qsize[0], 1)] = u;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    dist[s] = 0;
    ctl->done = ctl->qsize[0] == 0 && ctl->lpack[0] == 0;
  }
}

__global__ void __launch_bounds__(kBlock) sssp_relax(const int32_t* __restrict__ row_ptr,
                                                     const int32_t* __restrict__ col, const int32_t* __restrict__ wi,
                                                     const float* __restrict__ wf, int is_float,
                                                     SsCtl* __restrict__ ctl, int32_t* __restrict__ q,
                                                     Seg* __restrict__ segs, size_t segcap,
                                                     uint32_t* __restrict__ inq, int32_t n, int32_t nwords) {
  __shared__ int s_excl[kBlock / 32][32];
  __shared__ int s_rs[kBlock / 32][32];
  __shared__ int s_v[kBlock / 32][32];
  __shared__ int32_t s_q[kBlock / 32][kWarpQueue];
  if (ctl->done) return;
  const int L = ctl->level;
  const int pin = (L - 1) & 1, pout = L & 1;
  const int32_t* qin = q + (size_t)pin * n;
  const Seg* sin = segs + (size_t)pin * segcap;
  int32_t* qout = q + (size_t)pout * n;
  Seg* sout = segs + (size_t)pout * segcap;
  unsigned long long* lpack = &ctl->lpack[pout];
  const int ln = seg_count(ctl->lpack[pin]);
  uint32_t* inq_in = inq + (size_t)pin * nwords;
  uint32_t* inq_out = inq + (size_t)pout * nwords;
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  int32_t* qcount = &ctl->qsize[pout];
  const int32_t source = ctl->source;
  const int qn = ctl->qsize[pin];
  const int wib = threadIdx.x >> 5;

  // The input queue's dedup bits are free again once the level has started:
  // this level claims in inq_out only.
  const size_t gstride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)(qn + ln); i += gstride) {
    const int32_t v = i < (size_t)qn ? qin[i] : sin[i - qn].v;
    atomicAnd(inq_in + (v >> 5), ~(1u << (v & 31)));
  }

  WarpQueue wq(s_q[wib], qout, qcount);
  auto op = [&](int32_t v, int k, bool valid) {
    bool found = false;
    int32_t u = -1;
    if (valid) {
      u = __ldg(col + k);
      if (u != source) {
        const int32_t nd = relax_sum(__ldcg(dist + v), k, wi, wf, is_float != 0);
        if (nd < __ldcg(dist + u)) {
          const int32_t old = atomicMin(dist + u, nd);
          if (nd < old) found = claim_bit(inq_out, u);
        }
      }
    }
    int deg = 0, rs = 0;
    if (found) {
      rs = row_ptr[u];
      deg = row_ptr[u + 1] - rs;
    }
    emit_routed(found, u, deg, rs, wq, sout, lpack);
  };
  seg_expand(row_ptr, sin, ln, op);
  warp_expand(row_ptr, qin, qn, s_excl[wib], s_rs[wib], s_v[wib], op);
  wq.flush();
}

__global__ void sssp_decide(SsCtl* __restrict__ ctl, int32_t n, cudaGraphConditionalHandle loop, int in_graph) {
  if (threadIdx.x != 0) return;
  if (ctl->done) {
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  const int L = ctl->level, pout = L & 1;
  ctl->n_push++;
  // The reference stops after n levels at most (src/algorithm/cpu/sssp.cpp:34);
  // with non-negative weights the queue empties long before.
  if ((ctl->qsize[pout] == 0 && ctl->lpack[pout] == 0) || L >= n) {
    ctl->done = 1;
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  ctl->qsize[pout ^ 1] = 0;
  ctl->lpack[pout ^ 1] = 0;
  ctl->level = L + 1;
}

__global__ void sssp_next(SsCtl* __restrict__ ctl) {
  if (threadIdx.x != 0) return;
  ctl->total_levels += ctl->level;
  ctl->total_push += ctl->n_push;
  ctl->src_idx += 1;
}

void probe_sssp(const void* p, LevelProbe* out) {
  const SsCtl* c = static_cast<const SsCtl*>(p);
  out->level = c->level;
  out->mode = kModePush;
  out->done = c->done;
  out->frontier = c->qsize[(c->level - 1) & 1] + (int64_t)(c->lpack[(c->level - 1) & 1] >> 32);
  out->frontier_edges = 0;
  out->unvisited_edges = 0;
}

}  // namespace

dawn_status sssp_single(dawn_graph* g, const int32_t* sources, int32_t nsrc, void* d_dist) {
  const int32_t n = g->n;
  const int32_t nwords = (n + 31) / 32;
  DAWN_CHECK(ensure(g->ss_queues, sizeof(int32_t) * 2 * (size_t)n, g->stream));
  size_t segcap = seg_capacity(n, g->m);
  DAWN_CHECK(ensure(g->ss_segs, sizeof(Seg) * 2 * segcap, g->stream));
  DAWN_CHECK(ensure(g->ss_bitmaps, sizeof(uint32_t) * 4 * (size_t)nwords, g->stream));
  DAWN_CHECK(ensure(g->ss_scratch, sizeof(unsigned long long) * (size_t)n, g->stream));
  DAWN_CHECK(ensure(g->ss_ctl, sizeof(SsCtl), g->stream));
  DAWN_CHECK(ensure(g->ss_sources, sizeof(int32_t) * (size_t)nsrc, g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->ss_sources.p, sources, sizeof(int32_t) * nsrc, cudaMemcpyHostToDevice,
                            g->stream));
  const int is_float = g->wtype == DAWN_W_F32;
  SsCtl c = {};
  c.policy = DAWN_VARIANT_PUSH;
  c.weighted = is_float;
  c.nsrc = nsrc;
  c.dist_base = static_cast<int32_t*>(d_dist);
  c.sources = g->ss_sources.as<int32_t>();
  DAWN_CHECK(upload_ctl(g, c));

  struct {
    SsCtl* ctl;
    const int32_t *row_ptr, *col, *wi;
    const float* wf;
    int is_float;
    unsigned long long* last;
    int32_t* q;
    Seg* segs;
    size_t segcap;
    uint32_t* inq;
    int32_t n, nwords, inf;
    cudaGraphConditionalHandle handle;
    int in_graph;
  } a;
  a.ctl = g->ss_ctl.as<SsCtl>();
  a.row_ptr = g->row_ptr;
  a.col = g->col;
  a.wi = is_float ? nullptr : static_cast<const int32_t*>(g->val);
  a.wf = is_float ? static_cast<const float*>(g->val) : nullptr;
  a.is_float = is_float;
  a.last = g->ss_scratch.as<unsigned long long>();
  a.q = g->ss_queues.as<int32_t>();
  a.segs = g->ss_segs.as<Seg>();
  a.segcap = segcap;
  a.inq = g->ss_bitmaps.as<uint32_t>();
  a.n = n;
  a.nwords = nwords;
  a.inf = is_float ? 0x7f7fffff : 0x7fffffff;  // FLT_MAX bits / INT32_MAX
  a.handle = 0;
  a.in_graph = 0;
  void* clear_args[] = {&a.ctl, &a.inq, &a.n, &a.nwords, &a.inf};
  void* init_args[] = {&a.ctl, &a.row_ptr, &a.col, &a.wi, &a.wf, &a.is_float, &a.last, &a.q, &a.segs, &a.n};
  void* relax_args[] = {&a.row_ptr, &a.col, &a.wi, &a.wf, &a.is_float, &a.ctl, &a.q, &a.segs, &a.segcap,
                        &a.inq, &a.n, &a.nwords};
  void* decide_args[] = {&a.ctl, &a.n, &a.handle, &a.in_graph};
  void* next_args[] = {&a.ctl};

  const int sms = g->geo.sms;
  SsFamily fam;
  fam.npre = 2;
  fam.pre[0] = {(const void*)sssp_clear, clear_args, dim3(sms * 4), dim3(kBlock)};
  fam.pre[1] = {(const void*)sssp_init, init_args, dim3(1), dim3(kBlock)};
  fam.nbody = 2;
  fam.body[0] = {(const void*)sssp_relax, relax_args,
                 dim3(persistent_blocks((const void*)sssp_relax, kBlock, 0, g->blocks_per_sm)), dim3(kBlock), "sssp_relax"};
  fam.body[1] = {(const void*)sssp_decide, decide_args, dim3(1), dim3(32), "sssp_decide"};
  fam.npost = 1;
  fam.post[0] = {(const void*)sssp_next, next_args, dim3(1), dim3(32), "sssp_next"};
  fam.ctl = a.ctl;
  fam.ctl_bytes = sizeof(SsCtl);
  fam.probe = probe_sssp;
  fam.handle = &a.handle;
  fam.in_graph = &a.in_graph;
  fam.done_flag = &a.ctl->done;
  if (g->sssp_exec && g->sssp_exec_weighted != is_float) {
    cudaGraphExecDestroy(g->sssp_exec);
    g->sssp_exec = nullptr;
  }
  g->sssp_exec_weighted = is_float;
  return ss_run(g, fam, nsrc, &g->sssp_exec);
}

}  // namespace dawn
