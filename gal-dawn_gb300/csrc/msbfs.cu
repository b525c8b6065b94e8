// Batched boolean expand over 64-source bitset frontiers on sm_103a.
//
// The reference runs multi-source and all-pairs BFS as a serial loop of
// single-source traversals (src/algorithm/gpu/mssp.cu:26-43,
// src/algorithm/gpu/apsp.cu:183-200), re-reading the whole CSR once per
// source.  Here up to 64 sources share one traversal: every vertex carries
// one uint64 word per state (visited, frontier, next), bit b standing for
// source b of the batch, so one pass over an adjacency row serves all 64
// sources.  Hop distances come out identical to 64 separate traversals:
// bit b of a vertex is set at level L exactly when source b first reaches it
// at L.
//
// A level runs in one of two directions, chosen on the device:
//   pull: each unfinished vertex (some source has not reached it) ORs the
//         frontier words of its in-neighbours, stopping early once every
//         missing bit is found; the vertex owns its words, so no atomics;
//   push: the active vertices' rows are dealt to warps; new bits are
//         atomicOr-ed into `next`, the first toucher queues the target, and
//         an update pass folds `next` into visited / frontier.
// Both write each new (source, vertex) distance exactly once.
#include "dawn_device.cuh"

namespace dawn {
namespace {

struct BsCtl {
  int32_t aq_size[2];          // active (frontier) queue sizes by level parity
  int32_t tq_size;             // push: vertices touched this level
  int32_t aq_prev;             // stale entries of the output frontier to clear
  int32_t level, mode, done, policy;
  unsigned long long mf[2];    // out-degree sums of the active queues
  long long mu;                // degree sum of vertices not yet finished
  long long mu_dec;            // degree of vertices finished this level
  unsigned long long reached;  // TEPS numerator of the batch
  unsigned long long full;     // this batch's source bits
  int32_t batch, nsrc, n_push, n_pull;
  int32_t* dist_base;
  const int32_t* sources;
  unsigned long long total_reached;
  int32_t total_levels, total_push, total_pull, pad;
};

constexpr long long kPushRatio = 3;  // push while 3 * frontier edges < unfinished edges

__device__ __forceinline__ void write_new_bits(int32_t* __restrict__ dist_base, int32_t n, int batch, int32_t u,
                                               unsigned long long nw, int32_t level) {
  const size_t base = (size_t)batch * 64;
  while (nw) {
    const int b = __ffsll((long long)nw) - 1;
    nw &= nw - 1;
    dist_base[(base + b) * (size_t)n + u] = level;
  }
}

__global__ void __launch_bounds__(kBlock) bs_clear(unsigned long long* __restrict__ words, size_t count) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  ulonglong2* w2 = reinterpret_cast<ulonglong2*>(words);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count / 2; i += stride)
    w2[i] = make_ulonglong2(0ull, 0ull);
  if (blockIdx.x == 0 && threadIdx.x == 0 && (count & 1)) words[count - 1] = 0;
}

__global__ void bs_init(BsCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                        unsigned long long* __restrict__ visit, unsigned long long* __restrict__ fr0,
                        int32_t* __restrict__ aq0, int32_t n, long long m) {
  __shared__ unsigned long long s_mf, s_reached, s_dec;
  const int b = threadIdx.x;
  const int batch = ctl->batch;
  const int nb = min(64, ctl->nsrc - batch * 64);
  if (b == 0) {
    s_mf = 0;
    s_reached = 0;
    s_dec = 0;
    ctl->aq_size[0] = 0;
    ctl->aq_size[1] = 0;
    ctl->tq_size = 0;
    ctl->aq_prev = 0;
    ctl->full = nb == 64 ? ~0ull : ((1ull << nb) - 1ull);
  }
  __syncthreads();
  int32_t s = -1;
  bool first = false;
  if (b < nb) {
    s = ctl->sources[batch * 64 + b];
    const unsigned long long bit = 1ull << b;
    atomicOr(visit + s, bit);
    first = atomicOr(fr0 + s, bit) == 0ull;
    ctl->dist_base[((size_t)batch * 64 + b) * (size_t)n + s] = 0;
    atomicAdd(&s_reached, (unsigned long long)(row_ptr[s + 1] - row_ptr[s]));
  }
  __syncthreads();
  if (first) {
    const unsigned long long deg = (unsigned long long)(row_ptr[s + 1] - row_ptr[s]);
    aq0[atomicAdd(&ctl->aq_size[0], 1)] = s;
    atomicAdd(&s_mf, deg);
    if (visit[s] == ctl->full) atomicAdd(&s_dec, deg);
  }
  __syncthreads();
  if (b == 0) {
    ctl->mf[0] = s_mf;
    ctl->mf[1] = 0;
    ctl->reached = s_reached;
    ctl->mu = m - (long long)s_dec;
    ctl->mu_dec = 0;
    ctl->level = 1;
    ctl->mode = kModePush;
    ctl->done = 0;
    ctl->n_push = 0;
    ctl->n_pull = 0;
  }
}

// Per-thread accumulators of a level, flushed once per warp.
struct LevelAcc {
  unsigned long long mf = 0, reached = 0;
  long long dec = 0;
  __device__ __forceinline__ void flush(BsCtl* ctl, int pout) {
    mf = warp_sum(mf);
    reached = warp_sum(reached);
    dec = (long long)warp_sum((unsigned long long)dec);
    if (lane_id() == 0) {
      if (mf) atomicAdd(&ctl->mf[pout], mf);
      if (reached) atomicAdd(&ctl->reached, reached);
      if (dec) atomicAdd(reinterpret_cast<unsigned long long*>(&ctl->mu_dec), (unsigned long long)dec);
    }
  }
};

__global__ void __launch_bounds__(kBlock) bs_pull(const int32_t* __restrict__ row_ptr,
                                                  const int32_t* __restrict__ t_row_ptr,
                                                  const int32_t* __restrict__ t_col, BsCtl* __restrict__ ctl,
                                                  unsigned long long* __restrict__ visit,
                                                  unsigned long long* __restrict__ fr,
                                                  int32_t* __restrict__ aq, int32_t n) {
  if (ctl->done || ctl->mode != kModePull) return;
  const int L = ctl->level;
  const int pin = (L - 1) & 1, pout = L & 1;
  const unsigned long long* __restrict__ fin = fr + (size_t)pin * n;
  unsigned long long* __restrict__ fout = fr + (size_t)pout * n;
  int32_t* aq_out = aq + (size_t)pout * n;
  const unsigned long long full = ctl->full;
  const int batch = ctl->batch;
  int32_t* dist_base = ctl->dist_base;
  LevelAcc acc;
  // Grid-stride over all vertices; the trip count is uniform per warp so the
  // warp-aggregated append below sees all 32 lanes.
  const int total = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += total) {
    const int32_t u = base + threadIdx.x;
    unsigned long long nw = 0;
    if (u < n) {
      const unsigned long long vis = visit[u];
      if (vis != full) {
        unsigned long long got = 0;
        const int e = t_row_ptr[u + 1];
        for (int k = t_row_ptr[u]; k < e; k++) {
          got |= __ldg(fin + __ldg(t_col + k));
          if ((got | vis) == full) break;
        }
        nw = got & ~vis;
        if (nw) {
          visit[u] = vis | nw;
          const unsigned long long deg = (unsigned long long)(row_ptr[u + 1] - row_ptr[u]);
          acc.mf += deg;
          acc.reached += deg * (unsigned long long)__popcll(nw);
          if ((vis | nw) == full) acc.dec += (long long)deg;
          write_new_bits(dist_base, n, batch, u, nw, L);
        }
      }
      fout[u] = nw;
    }
    const int pos = warp_append(nw != 0, &ctl->aq_size[pout]);
    if (nw) aq_out[pos] = u;
  }
  acc.flush(ctl, pout);
}

__global__ void __launch_bounds__(kBlock) bs_push_scatter(const int32_t* __restrict__ row_ptr,
                                                          const int32_t* __restrict__ col, BsCtl* __restrict__ ctl,
                                                          const unsigned long long* __restrict__ visit,
                                                          unsigned long long* __restrict__ fr,
                                                          unsigned long long* __restrict__ nxt,
                                                          int32_t* __restrict__ aq, int32_t* __restrict__ tq,
                                                          int32_t n) {
  __shared__ int s_excl[kBlock / 32][32];
  __shared__ int s_rs[kBlock / 32][32];
  __shared__ int s_v[kBlock / 32][32];
  if (ctl->done || ctl->mode != kModePush) return;
  const int L = ctl->level;
  const int pin = (L - 1) & 1, pout = L & 1;
  const unsigned long long* __restrict__ fin = fr + (size_t)pin * n;
  unsigned long long* __restrict__ fout = fr + (size_t)pout * n;
  const int32_t* aq_in = aq + (size_t)pin * n;
  const int32_t* aq_old = aq + (size_t)pout * n;
  const int qn = ctl->aq_size[pin];
  // The output frontier still holds the words of two levels ago.
  const int stale = ctl->aq_prev;
  const size_t gstride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)stale; i += gstride)
    fout[aq_old[i]] = 0ull;
  const int wib = threadIdx.x >> 5;
  warp_expand(row_ptr, aq_in, qn, s_excl[wib], s_rs[wib], s_v[wib], [&](int32_t v, int k, bool valid) {
    bool first = false;
    int32_t u = -1;
    if (valid) {
      u = __ldg(col + k);
      const unsigned long long bits = __ldg(fin + v) & ~__ldcg(visit + u);
      if (bits) first = atomicOr(nxt + u, bits) == 0ull;
    }
    const int pos = warp_append(first, &ctl->tq_size);
    if (first) tq[pos] = u;
  });
}

__global__ void __launch_bounds__(kBlock) bs_push_update(const int32_t* __restrict__ row_ptr,
                                                         BsCtl* __restrict__ ctl,
                                                         unsigned long long* __restrict__ visit,
                                                         unsigned long long* __restrict__ fr,
                                                         unsigned long long* __restrict__ nxt,
                                                         int32_t* __restrict__ aq, const int32_t* __restrict__ tq,
                                                         int32_t n) {
  if (ctl->done || ctl->mode != kModePush) return;
  const int L = ctl->level;
  const int pout = L & 1;
  unsigned long long* __restrict__ fout = fr + (size_t)pout * n;
  int32_t* aq_out = aq + (size_t)pout * n;
  const unsigned long long full = ctl->full;
  const int batch = ctl->batch;
  int32_t* dist_base = ctl->dist_base;
  const int tn = ctl->tq_size;
  LevelAcc acc;
  const int total = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < tn; base += total) {
    const int i = base + threadIdx.x;
    unsigned long long nw = 0;
    int32_t u = -1;
    if (i < tn) {
      u = tq[i];
      const unsigned long long x = nxt[u];
      nxt[u] = 0ull;
      const unsigned long long vis = visit[u];
      nw = x & ~vis;
      fout[u] = nw;
      if (nw) {
        visit[u] = vis | nw;
        const unsigned long long deg = (unsigned long long)(row_ptr[u + 1] - row_ptr[u]);
        acc.mf += deg;
        acc.reached += deg * (unsigned long long)__popcll(nw);
        if ((vis | nw) == full) acc.dec += (long long)deg;
        write_new_bits(dist_base, n, batch, u, nw, L);
      }
    }
    const int pos = warp_append(nw != 0, &ctl->aq_size[pout]);
    if (nw) aq_out[pos] = u;
  }
  acc.flush(ctl, pout);
}

__global__ void bs_decide(BsCtl* __restrict__ ctl, int32_t n, cudaGraphConditionalHandle loop, int in_graph) {
  if (threadIdx.x != 0) return;
  if (ctl->done) {
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  const int L = ctl->level, pin = (L - 1) & 1, pout = L & 1;
  if (ctl->mode == kModePush) ctl->n_push++; else ctl->n_pull++;
  ctl->mu -= ctl->mu_dec;
  ctl->mu_dec = 0;
  const int nf = ctl->aq_size[pout];
  if (nf == 0 || L >= n) {
    ctl->done = 1;
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  // Next level writes the frontier buffer this level read.
  ctl->aq_prev = ctl->aq_size[pin];
  ctl->aq_size[pin] = 0;
  ctl->mf[pin] = 0;
  ctl->tq_size = 0;
  int mode;
  if (ctl->policy == DAWN_VARIANT_PUSH) {
    mode = kModePush;
  } else {
    mode = (long long)ctl->mf[pout] * kPushRatio < ctl->mu ? kModePush : kModePull;
  }
  ctl->mode = mode;
  ctl->level = L + 1;
}

__global__ void bs_next(BsCtl* __restrict__ ctl) {
  if (threadIdx.x != 0) return;
  ctl->total_reached += ctl->reached;
  ctl->total_levels += ctl->level;
  ctl->total_push += ctl->n_push;
  ctl->total_pull += ctl->n_pull;
  ctl->batch += 1;
}

void probe_bs(const void* p, LevelProbe* out) {
  const BsCtl* c = static_cast<const BsCtl*>(p);
  const int pin = (c->level - 1) & 1;
  out->level = c->level;
  out->mode = c->mode;
  out->done = c->done;
  out->frontier = c->aq_size[pin];
  out->frontier_edges = (int64_t)c->mf[pin];
  out->unvisited_edges = c->mu;
}

}  // namespace

dawn_status bfs_bitset(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_dist) {
  const int32_t n = g->n;
  const size_t nn = (size_t)n;
  // words: visit | fr0 | fr1 | nxt
  DAWN_CHECK(ensure(g->bs_words, sizeof(unsigned long long) * 4 * nn));
  DAWN_CHECK(ensure(g->bs_queues, sizeof(int32_t) * 3 * nn));
  DAWN_CHECK(ensure(g->bs_ctl, sizeof(BsCtl)));
  DAWN_CHECK(ensure(g->bs_sources, sizeof(int32_t) * (size_t)nsrc));
  DAWN_CUDA(cudaMemcpyAsync(g->bs_sources.p, sources, sizeof(int32_t) * nsrc, cudaMemcpyHostToDevice,
                            g->stream));
  DAWN_CUDA(cudaMemsetAsync(d_dist, 0xff, sizeof(int32_t) * (size_t)nsrc * nn, g->stream));
  BsCtl c = {};
  c.nsrc = nsrc;
  c.policy = DAWN_VARIANT_BITSET;
  c.dist_base = d_dist;
  c.sources = g->bs_sources.as<int32_t>();
  DAWN_CUDA(cudaMemcpyAsync(g->bs_ctl.p, &c, sizeof(BsCtl), cudaMemcpyHostToDevice, g->stream));

  struct {
    BsCtl* ctl;
    const int32_t *row_ptr, *col, *t_row_ptr, *t_col;
    unsigned long long *words, *visit, *fr, *fr0, *nxt;
    int32_t *aq, *aq0, *tq;
    size_t nwords;
    int32_t n;
    long long m;
    cudaGraphConditionalHandle handle;
    int in_graph;
  } a;
  a.ctl = g->bs_ctl.as<BsCtl>();
  a.row_ptr = g->row_ptr;
  a.col = g->col;
  a.t_row_ptr = g->t_row_ptr;
  a.t_col = g->t_col;
  a.words = g->bs_words.as<unsigned long long>();
  a.visit = a.words;
  a.fr = a.words + nn;
  a.fr0 = a.fr;
  a.nxt = a.words + 3 * nn;
  a.aq = g->bs_queues.as<int32_t>();
  a.aq0 = a.aq;
  a.tq = a.aq + 2 * nn;
  a.nwords = 4 * nn;
  a.n = n;
  a.m = g->m;
  a.handle = 0;
  a.in_graph = 0;
  void* clear_args[] = {&a.words, &a.nwords};
  void* init_args[] = {&a.ctl, &a.row_ptr, &a.visit, &a.fr0, &a.aq0, &a.n, &a.m};
  void* pull_args[] = {&a.row_ptr, &a.t_row_ptr, &a.t_col, &a.ctl, &a.visit, &a.fr, &a.aq, &a.n};
  void* scatter_args[] = {&a.row_ptr, &a.col, &a.ctl, &a.visit, &a.fr, &a.nxt, &a.aq, &a.tq, &a.n};
  void* update_args[] = {&a.row_ptr, &a.ctl, &a.visit, &a.fr, &a.nxt, &a.aq, &a.tq, &a.n};
  void* decide_args[] = {&a.ctl, &a.n, &a.handle, &a.in_graph};
  void* next_args[] = {&a.ctl};

  const int sms = g->geo.sms;
  SsFamily fam;
  fam.npre = 2;
  fam.pre[0] = {(const void*)bs_clear, clear_args, dim3(sms * 8), dim3(kBlock)};
  fam.pre[1] = {(const void*)bs_init, init_args, dim3(1), dim3(64)};
  fam.nbody = 4;
  fam.body[0] = {(const void*)bs_pull, pull_args, dim3(persistent_blocks((const void*)bs_pull, kBlock, 0)),
                 dim3(kBlock), "bs_pull", kModePull};
  fam.body[1] = {(const void*)bs_push_scatter, scatter_args,
                 dim3(persistent_blocks((const void*)bs_push_scatter, kBlock, 0)), dim3(kBlock),
                 "bs_push_scatter", kModePush};
  fam.body[2] = {(const void*)bs_push_update, update_args,
                 dim3(persistent_blocks((const void*)bs_push_update, kBlock, 0)), dim3(kBlock),
                 "bs_push_update", kModePush};
  fam.body[3] = {(const void*)bs_decide, decide_args, dim3(1), dim3(32), "bs_decide"};
  fam.post = {(const void*)bs_next, next_args, dim3(1), dim3(32), "bs_next"};
  fam.ctl = a.ctl;
  fam.ctl_bytes = sizeof(BsCtl);
  fam.probe = probe_bs;
  fam.handle = &a.handle;
  fam.in_graph = &a.in_graph;
  fam.done_flag = &a.ctl->done;
  const int nbatches = (nsrc + 63) / 64;
  return ss_run(g, fam, nbatches, &g->bs_exec);
}

dawn_status bfs_bitset_stats(dawn_graph* g, dawn_stats* st, int32_t nsrc) {
  BsCtl h;
  DAWN_CUDA(cudaMemcpyAsync(&h, g->bs_ctl.p, sizeof(BsCtl), cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  st->edges_traversed = (int64_t)h.total_reached;
  st->levels = h.total_levels;
  st->push_levels = h.total_push;
  st->pull_levels = h.total_pull;
  st->batches = (nsrc + 63) / 64;
  return DAWN_OK;
}

}  // namespace dawn
