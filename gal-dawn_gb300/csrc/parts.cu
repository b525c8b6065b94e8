// Many independent graphs in one persistent launch, on sm_103a.
//
// The reference traverses one graph per process call: MSSP_GPU::run
// (src/algorithm/gpu/mssp.cu:9-51) copies a CSR, loops over its sources and
// frees it.  A workload of hundreds of small graphs then pays a CSR upload,
// per-level launches and host syncs for every (graph, source).  Here the
// graphs are the parts of one disjoint-union CSR (part p owns the vertex
// range [off[p], off[p+1]) and no edge leaves its part), and one persistent
// kernel runs every (part, batch of up to 64 sources) task:
//
//   * a thread-block cluster (kPartCluster CTAs on as many SMs) takes the
//     next task from a device counter (tasks sorted by estimated cost,
//     longest first, so the long ones start early) and runs the whole
//     multi-source bitset traversal of that part, its CTAs splitting every
//     vertex and row sweep, with cluster barriers between phases and the
//     level counters summed through distributed shared memory: no launch
//     per level, no host sync, and no wait on another cluster;
//   * its working words live in a per-cluster slot of global memory
//     (visited, two frontier words, a push accumulator and bit-sliced
//     levels, one uint64 per vertex each); the part's words stay in L2
//     while the cluster works on them;
//   * each level is a push (frontier rows scattered with atomicOr into the
//     accumulator, then a sweep folding it in) or a pull (each unfinished
//     vertex ORs its in-neighbours' frontier words, stopping once no
//     missing bit is left), chosen by the same frontier-edge rule as the
//     single-graph bitset traversal;
//   * the distances of a task are emitted once, at its end, from the level
//     slices, with coalesced stores, and the emit pass zeroes every word the
//     task used, so the slot is clean for the next task without a separate
//     clearing pass.
//
// Hop distances are those of a separate BFS of each part from each source:
// bit b of a vertex's word appears at level L exactly when source b first
// reaches it at L, whatever the direction of each level.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "dawn_device.cuh"

namespace dawn {
namespace {

using u64 = unsigned long long;
constexpr int kPartBlock = 1024;
constexpr int kPartSlices = 8;  // level slices kept in registers by the emit pass
constexpr int kPartLaneMax = 64;  // rows below this many entries are walked by one lane
constexpr int kPartCluster = 8;   // CTAs (SMs) per task: a thread-block cluster (1 where 8 do not fit)

struct PartsCtl {
  int32_t next_task;    // task counter of the persistent grid
  int32_t ntasks;
  int32_t push_ratio;   // push while ratio * frontier edges < unfinished in-edges
  int32_t pad0;
  const PartTask* tasks;
  const int32_t* sources;  // part-local source ids, in task order
  int32_t* dist;           // output base
  unsigned long long reached;  // TEPS numerator, all tasks
  unsigned long long levels, push_levels, pull_levels;
  unsigned long long* task_log;  // tracing: 4 words per task, else NULL
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned sm_id() {
  unsigned r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}

__device__ __forceinline__ u64 block_reduce_add(u64 x, u64* s_slot) {
  x = warp_sum(x);
  if (lane_id() == 0 && x) atomicAdd(s_slot, x);
  return x;
}

// Distances of one vertex for the task's nb sources from its visited word
// and level slices; NB slices are read into registers, the rest (levels of
// 256 and above) from memory.
template <int NB>
__device__ __forceinline__ void emit_part_vertex(int32_t* __restrict__ dist, int32_t np, int nb, int u, u64 vis,
                                                 u64* __restrict__ slices, int32_t maxn, int nbits) {
  u64 w[NB > 0 ? NB : 1];
#pragma unroll
  for (int k = 0; k < NB; k++) {
    w[k] = slices[(size_t)k * maxn + u];
    slices[(size_t)k * maxn + u] = 0ull;
  }
  for (int b = 0; b < nb; b++) {
    int32_t v = -1;
    if ((vis >> b) & 1ull) {
      v = 0;
#pragma unroll
      for (int k = 0; k < NB; k++) v |= (int32_t)((w[k] >> b) & 1ull) << k;
      for (int k = NB; k < nbits; k++) v |= (int32_t)((slices[(size_t)k * maxn + u] >> b) & 1ull) << k;
    }
    dist[(size_t)b * np + u] = v;
  }
  for (int k = NB; k < nbits; k++) slices[(size_t)k * maxn + u] = 0ull;
}

template <int C>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(kPartBlock, 1)
    parts_traverse(PartsCtl* __restrict__ ctl,
                                                           const int32_t* __restrict__ row_ptr,
                                                           const int32_t* __restrict__ col,
                                                           const int32_t* __restrict__ t_row_ptr,
                                                           const int32_t* __restrict__ t_col,
                                                           const int32_t* __restrict__ voff,
                                                           u64* __restrict__ scratch, size_t slot_words,
                                                           int32_t maxn) {
  // Per level (by parity): frontier out-edges, in-edges of the vertices
  // finished, vertices reached.  Each CTA counts its own; the cluster's
  // totals are read through distributed shared memory after the level's
  // barrier, and a CTA resets its counters of the other parity then (every
  // reader of those passed the barrier).
  __shared__ int s_task;
  __shared__ u64 s_cnt[2][3];
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const int ctid = crank * kPartBlock + tid;  // thread index within the cluster
  constexpr int kThreads = C * kPartBlock;
  const int lane = lane_id(), wib = tid >> 5;
  const int cwarp = crank * (kPartBlock / 32) + wib;
  u64* const visit = scratch + (size_t)(blockIdx.x / C) * slot_words;
  u64* const fa = visit + maxn;
  u64* const fb = fa + maxn;
  u64* const acc = fb + maxn;
  u64* const slices = acc + maxn;
  const int ratio = ctl->push_ratio;
  u64 my_reached = 0;
  u64 t_levels = 0, t_push = 0, t_pull = 0;

  auto totals = [&](int par, u64& mf_t, u64& dec_t, u64& nf_t) {
    mf_t = dec_t = nf_t = 0;
#pragma unroll
    for (int r = 0; r < C; r++) {
      const u64* c = cluster.map_shared_rank(&s_cnt[par][0], r);
      mf_t += c[0];
      dec_t += c[1];
      nf_t += c[2];
    }
  };
  for (;;) {
    if (crank == 0 && tid == 0) s_task = atomicAdd(&ctl->next_task, 1);
    if (tid < 6) (&s_cnt[0][0])[tid] = 0;
    cluster.sync();
    const int t = *cluster.map_shared_rank(&s_task, 0);
    if (t >= ctl->ntasks) break;
    const PartTask task = ctl->tasks[t];
    const int32_t v0 = voff[task.part];
    const int32_t np = voff[task.part + 1] - v0;
    const int nb = task.nsrc;
    const u64 full = nb == 64 ? ~0ull : ((1ull << nb) - 1ull);
    const int32_t* src = ctl->sources + task.src0;
    const long long mp = (long long)row_ptr[v0 + np] - row_ptr[v0];
    unsigned long long t_start = 0, push0 = t_push;
    if (ctid == 0 && ctl->task_log) t_start = global_ns();
    // Seed: source b sets bit b at its vertex (the cluster's first CTA;
    // its level-0 counters take the seeds' rows).
    if (ctid < nb) {
      const int32_t s = src[ctid];
      atomicOr(visit + s, 1ull << ctid);
      atomicOr(fa + s, 1ull << ctid);
    }
    __syncthreads();
    if (ctid < nb) {
      const int32_t s = src[ctid];
      const int32_t gs = v0 + s;
      const u64 deg = (u64)(row_ptr[gs + 1] - row_ptr[gs]);
      my_reached += deg;
      // the thread of the lowest bit at a vertex counts the vertex once
      if ((fa[s] & ((1ull << ctid) - 1ull)) == 0ull) {
        atomicAdd(&s_cnt[0][0], deg);
        if (visit[s] == full) atomicAdd(&s_cnt[0][1], (u64)(t_row_ptr[gs + 1] - t_row_ptr[gs]));
      }
    }
    cluster.sync();
    long long mf, mu;
    {
      u64 a0, a1, a2;
      totals(0, a0, a1, a2);
      mf = (long long)a0;
      mu = mp - (long long)a1;
    }
    u64* cur = fa;
    u64* nxt = fb;
    int L = 1;
    for (;;) {
      const bool push = mf * ratio < mu;
      const int par = L & 1;  // this level's counters; level 0 used the other parity
      if (push) {
        // scatter: the frontier rows of 32 consecutive vertices per warp
        // task; rows of >= kPartLaneMax entries swept by the whole warp,
        // shorter ones walked by one lane each (no shared-memory search per
        // edge: these loops are bound by their L1/TEX traffic)
        for (int base = cwarp * 32; base < np; base += kThreads) {
          const int v = base + lane;
          const u64 f = v < np ? cur[v] : 0ull;
          int rs = 0, re = 0;
          if (f) {
            rs = row_ptr[v0 + v];
            re = row_ptr[v0 + v + 1];
          }
          const int deg = re - rs;
          if (__ballot_sync(kFull, deg > 0) == 0u) continue;
          uint32_t big = __ballot_sync(kFull, deg >= kPartLaneMax);
          while (big) {
            const int leader = __ffs(big) - 1;
            big &= big - 1;
            const u64 lf = __shfl_sync(kFull, f, leader);
            const int ks = __shfl_sync(kFull, rs, leader), ke = __shfl_sync(kFull, re, leader);
            for (int k = ks + lane; k < ke; k += 32) {
              const int u = __ldg(col + k) - v0;
              const u64 bits = lf & ~visit[u];
              if (bits) atomicOr(acc + u, bits);
            }
          }
          // short rows: one lane each, four targets in flight
          if (deg > 0 && deg < kPartLaneMax) {
            for (int k = rs; k < re; k += 4) {
              int u[4];
#pragma unroll
              for (int j = 0; j < 4; j++) u[j] = k + j < re ? __ldg(col + k + j) - v0 : -1;
              u64 bits[4];
#pragma unroll
              for (int j = 0; j < 4; j++) bits[j] = u[j] >= 0 ? f & ~visit[u[j]] : 0ull;
#pragma unroll
              for (int j = 0; j < 4; j++)
                if (bits[j]) atomicOr(acc + u[j], bits[j]);
            }
          }
        }
      }
      if (push) cluster.sync();  // the scatter's ORs are in before the sweep reads them
      u64 lmf = 0, ldec = 0, lnf = 0;
      for (int base = cwarp * 32; base < np; base += kThreads) {
        const int u = base + lane;
        const bool in = u < np;
        const int gu = v0 + u;
        // every load of the vertex's own words and row bounds is issued at
        // once, ahead of the gathers that need them
        u64 vis = full, x = 0ull;
        int rp0 = 0, rp1 = 0, tr0 = 0, tr1 = 0;
        if (in) {
          vis = visit[u];
          rp0 = row_ptr[gu];
          rp1 = row_ptr[gu + 1];
          tr0 = t_row_ptr[gu];
          tr1 = t_row_ptr[gu + 1];
          if (push) x = acc[u];
        }
        u64 nw = 0ull;
        if (push) {
          if (x) {
            acc[u] = 0ull;
            nw = x & ~vis;
          }
        } else {
          // pull: unfinished vertices OR their in-neighbours' frontier
          // words; long rows by the whole warp, short rows by one lane
          // each, both stopping once no missing bit is left
          const bool active = vis != full;
          const int rs = active ? tr0 : 0, re = active ? tr1 : 0;
          const int deg = re - rs;
          u64 got = 0ull;
          uint32_t big = __ballot_sync(kFull, deg >= kPartLaneMax);
          while (big) {
            const int leader = __ffs(big) - 1;
            big &= big - 1;
            const u64 lvis = __shfl_sync(kFull, vis, leader);
            const int ks = __shfl_sync(kFull, rs, leader), ke = __shfl_sync(kFull, re, leader);
            u64 w = 0ull;
            for (int k0 = ks; k0 < ke; k0 += 128) {
              const int k = k0 + lane;
              const int32_t c0 = k < ke ? __ldg(t_col + k) : -1;
              const int32_t c1 = k + 32 < ke ? __ldg(t_col + k + 32) : -1;
              const int32_t c2 = k + 64 < ke ? __ldg(t_col + k + 64) : -1;
              const int32_t c3 = k + 96 < ke ? __ldg(t_col + k + 96) : -1;
              if (c0 >= 0) w |= cur[c0 - v0];
              if (c1 >= 0) w |= cur[c1 - v0];
              if (c2 >= 0) w |= cur[c2 - v0];
              if (c3 >= 0) w |= cur[c3 - v0];
              if ((warp_or(w) | lvis) == full) break;
            }
            w = warp_or(w);
            if (lane == leader) got = w;
          }
          // short rows: one lane each, four in-neighbours in flight,
          // stopping once the missing bits are all found
          if (active && deg < kPartLaneMax) {
            u64 w = 0ull;
            for (int k = rs; k < re; k += 4) {
              int32_t c[4];
#pragma unroll
              for (int j = 0; j < 4; j++) c[j] = k + j < re ? __ldg(t_col + k + j) : -1;
#pragma unroll
              for (int j = 0; j < 4; j++)
                if (c[j] >= 0) w |= cur[c[j] - v0];
              if ((w | vis) == full) break;
            }
            got = w;
          }
          nw = got & ~vis;
        }
        if (!in) continue;
        nxt[u] = nw;
        if (nw) {
          visit[u] = vis | nw;
          // the bits are new to every slice, so an OR without a return
          // (no load on the thread's path) records them
          for (unsigned l = (unsigned)L; l; l &= l - 1) atomicOr(slices + (size_t)(__ffs(l) - 1) * maxn + u, nw);
          const u64 od = (u64)(rp1 - rp0);
          lmf += od;
          my_reached += od * (u64)__popcll(nw);
          lnf++;
          if ((vis | nw) == full) ldec += (u64)(tr1 - tr0);
        }
      }
      block_reduce_add(lmf, &s_cnt[par][0]);
      block_reduce_add(ldec, &s_cnt[par][1]);
      block_reduce_add(lnf, &s_cnt[par][2]);
      if (push) t_push++; else t_pull++;
      cluster.sync();
      u64 mf_t, dec_t, nf_t;
      totals(par, mf_t, dec_t, nf_t);
      // every reader of the other parity's counters is past the barrier,
      // and this CTA's next-level sums wait for the reset
      if (tid < 3) s_cnt[par ^ 1][tid] = 0;
      __syncthreads();
      if (nf_t == 0 || L >= np) break;
      mf = (long long)mf_t;
      mu -= (long long)dec_t;
      u64* tmp = cur;
      cur = nxt;
      nxt = tmp;
      L++;
    }
    t_levels += (u64)L;
    // Emit: the last level found nothing, so the deepest level is L - 1.
    const int deepest = L - 1;
    const int nbits = deepest > 0 ? 32 - __clz(deepest) : 0;
    int32_t* dist = ctl->dist + task.out0;
    for (int u = ctid; u < np; u += kThreads) {
      const u64 vis = visit[u];
      visit[u] = 0ull;
      fa[u] = 0ull;
      fb[u] = 0ull;
      switch (nbits < kPartSlices ? nbits : kPartSlices) {
        case 0: emit_part_vertex<0>(dist, np, nb, u, vis, slices, maxn, nbits); break;
        case 1: emit_part_vertex<1>(dist, np, nb, u, vis, slices, maxn, nbits); break;
        case 2: emit_part_vertex<2>(dist, np, nb, u, vis, slices, maxn, nbits); break;
        case 3: emit_part_vertex<3>(dist, np, nb, u, vis, slices, maxn, nbits); break;
        case 4: emit_part_vertex<4>(dist, np, nb, u, vis, slices, maxn, nbits); break;
        case 5: emit_part_vertex<5>(dist, np, nb, u, vis, slices, maxn, nbits); break;
        case 6: emit_part_vertex<6>(dist, np, nb, u, vis, slices, maxn, nbits); break;
        case 7: emit_part_vertex<7>(dist, np, nb, u, vis, slices, maxn, nbits); break;
        default: emit_part_vertex<kPartSlices>(dist, np, nb, u, vis, slices, maxn, nbits); break;
      }
    }
    cluster.sync();  // the slot is clean before the next task seeds it
    if (ctid == 0 && ctl->task_log) {
      unsigned long long* r = ctl->task_log + 4 * (size_t)t;
      r[0] = t_start;
      r[1] = global_ns();
      r[2] = ((unsigned long long)L << 32) | (unsigned)(t_push - push0);
      r[3] = sm_id();
    }
  }
  cluster.sync();  // no CTA exits while another may still read its task slot
  my_reached = warp_sum(my_reached);
  if (lane_id() == 0 && my_reached) atomicAdd(&ctl->reached, my_reached);
  if (ctid == 0 && t_levels) {
    atomicAdd(&ctl->levels, t_levels);
    atomicAdd(&ctl->push_levels, t_push);
    atomicAdd(&ctl->pull_levels, t_pull);
  }
}

// Block-diagonal check: every column of a part's rows lies in that part.
__global__ void __launch_bounds__(kBlock) parts_check(const int32_t* __restrict__ row_ptr,
                                                      const int32_t* __restrict__ col,
                                                      const int32_t* __restrict__ voff, int32_t nparts,
                                                      int* __restrict__ flag) {
  const int32_t p = blockIdx.y * gridDim.x + blockIdx.x;
  if (p >= nparts) return;
  const int32_t lo = voff[p], hi = voff[p + 1];
  const int k0 = row_ptr[lo], k1 = row_ptr[hi];
  int bad = 0;
  for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const int32_t c = col[k];
    bad |= c < lo || c >= hi;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

// Row-pointer values at the part boundaries (edge positions of each part).
__global__ void parts_bounds(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ voff, int32_t count,
                             long long* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = row_ptr[voff[i]];
}

// Per (part, source) row: sum of the hop distances of the reached vertices
// other than the source, and their count.  One CTA per row.
__global__ void __launch_bounds__(kBlock) parts_row_sums(const int32_t* __restrict__ dist,
                                                         const PartRow* __restrict__ rows, int32_t nrows,
                                                         long long* __restrict__ sum,
                                                         long long* __restrict__ cnt) {
  __shared__ long long s_sum, s_cnt;
  for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
    if (threadIdx.x == 0) {
      s_sum = 0;
      s_cnt = 0;
    }
    __syncthreads();
    const PartRow row = rows[r];
    const int32_t* d = dist + row.off;
    long long ls = 0, lc = 0;
    for (int v = threadIdx.x; v < row.len; v += blockDim.x) {
      const int32_t x = d[v];
      if (x > 0) {
        ls += x;
        lc++;
      }
    }
    ls = (long long)warp_sum((u64)ls);
    lc = (long long)warp_sum((u64)lc);
    if (lane_id() == 0 && lc) {
      atomicAdd(reinterpret_cast<u64*>(&s_sum), (u64)ls);
      atomicAdd(reinterpret_cast<u64*>(&s_cnt), (u64)lc);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      sum[r] = s_sum;
      cnt[r] = s_cnt;
    }
    __syncthreads();
  }
}

}  // namespace

dawn_status parts_set(dawn_graph* g, int32_t nparts, const int32_t* offsets) {
  if (nparts < 1 || !offsets) {
    set_error("parts: need nparts >= 1 and an offsets array of nparts + 1 entries");
    return DAWN_ERR_INVALID_ARG;
  }
  if (offsets[0] != 0 || offsets[nparts] != g->n) {
    set_error("parts: offsets must start at 0 and end at n = %d", g->n);
    return DAWN_ERR_INVALID_ARG;
  }
  int32_t maxn = 0;
  for (int32_t p = 0; p < nparts; p++) {
    const int32_t np = offsets[p + 1] - offsets[p];
    if (np < 1) {
      set_error("parts: part %d is empty or the offsets decrease", p);
      return DAWN_ERR_INVALID_ARG;
    }
    maxn = std::max(maxn, np);
  }
  if (maxn > kPartMaxVertices) {
    set_error("parts: a part of %d vertices exceeds the per-part limit of %d; traverse it as its own graph",
              maxn, kPartMaxVertices);
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CHECK(ensure(g->pt_voff, sizeof(int32_t) * ((size_t)nparts + 1), g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->pt_voff.p, offsets, sizeof(int32_t) * ((size_t)nparts + 1), cudaMemcpyHostToDevice,
                            g->stream));
  {
    long long* d_pos = nullptr;
    DAWN_CHECK(pool_alloc((void**)&d_pos, sizeof(long long) * ((size_t)nparts + 1), g->stream));
    parts_bounds<<<(nparts + 1 + kBlock - 1) / kBlock, kBlock, 0, g->stream>>>(g->row_ptr, g->pt_voff.as<int32_t>(),
                                                                              nparts + 1, d_pos);
    g->pt_pos.resize((size_t)nparts + 1);
    const cudaError_t le = cudaGetLastError();
    const cudaError_t ce = cudaMemcpyAsync(g->pt_pos.data(), d_pos, sizeof(long long) * ((size_t)nparts + 1),
                                           cudaMemcpyDeviceToHost, g->stream);
    pool_free(d_pos, g->stream);
    DAWN_CUDA(le);
    DAWN_CUDA(ce);
  }
  if (!(g->flags & DAWN_GRAPH_NO_VALIDATE)) {
    int* d_flag = nullptr;
    DAWN_CHECK(pool_alloc((void**)&d_flag, sizeof(int), g->stream));
    DAWN_CUDA(cudaMemsetAsync(d_flag, 0, sizeof(int), g->stream));
    const int gx = std::min(nparts, 65535);
    const int gy = (nparts + gx - 1) / gx;
    parts_check<<<dim3(gx, gy), kBlock, 0, g->stream>>>(g->row_ptr, g->col, g->pt_voff.as<int32_t>(), nparts,
                                                         d_flag);
    DAWN_CUDA(cudaGetLastError());
    int flag = 0;
    DAWN_CUDA(cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    pool_free(d_flag, g->stream);
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    if (flag) {
      set_error("parts: an edge leaves its part (the graph is not the disjoint union the offsets describe)");
      return DAWN_ERR_INVALID_ARG;
    }
  }
  // Per-cluster slots: visited, two frontiers, accumulator and one slice
  // per level bit (levels never exceed the part's vertex count).  The grid
  // is as many clusters as the device holds at once.
  const int nbits = 32 - __builtin_clz((unsigned)maxn);
  const size_t slot_words = (size_t)(4 + nbits) * (size_t)maxn;
  int cluster = kPartCluster, clusters = 0;
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kPartCluster);
    cfg.blockDim = dim3(kPartBlock);
    if (cudaOccupancyMaxActiveClusters(&clusters, (const void*)parts_traverse<kPartCluster>, &cfg) != cudaSuccess ||
        clusters < 1) {
      // no room for clusters of kPartCluster CTAs (a small partition of the
      // device): one CTA per task, one per SM
      cudaGetLastError();
      cluster = 1;
      clusters = g->geo.sms;
    }
  }
  const int slots = clusters * cluster;  // CTAs of the grid
  const size_t bytes = sizeof(u64) * slot_words * (size_t)clusters;
  if (g->pt_scratch.bytes < bytes) {
    DAWN_CHECK(ensure(g->pt_scratch, bytes, g->stream));
    if (g->pt_exec) {
      cudaGraphExecDestroy(g->pt_exec);
      g->pt_exec = nullptr;
    }
  }
  // Slots are clean between calls: each task zeroes what it used.
  DAWN_CUDA(cudaMemsetAsync(g->pt_scratch.p, 0, bytes, g->stream));
  if (g->pt_exec && (g->pt_slots != slots || g->pt_slot_words != slot_words || g->pt_maxn != maxn ||
                     g->pt_cluster != cluster)) {
    cudaGraphExecDestroy(g->pt_exec);
    g->pt_exec = nullptr;
  }
  g->pt_off.assign(offsets, offsets + nparts + 1);
  g->pt_slots = slots;
  g->pt_cluster = cluster;
  g->pt_slot_words = slot_words;
  g->pt_maxn = maxn;
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  return DAWN_OK;
}

dawn_status parts_bfs(dawn_graph* g, const int32_t* source_offset, const int32_t* sources, int32_t* d_dist,
                      std::vector<PartRow>* rows_out, dawn_stats* st) {
  const int32_t nparts = (int32_t)g->pt_off.size() - 1;
  if (nparts < 1) {
    set_error("parts: the graph has no parts (dawn_graph_set_parts)");
    return DAWN_ERR_INVALID_ARG;
  }
  if (!source_offset || source_offset[0] != 0) {
    set_error("parts: source_offset must have nparts + 1 entries starting at 0");
    return DAWN_ERR_INVALID_ARG;
  }
  const std::vector<int32_t>& off = g->pt_off;
  std::vector<PartTask> tasks;
  long long out = 0;
  for (int32_t p = 0; p < nparts; p++) {
    const int32_t s0 = source_offset[p], s1 = source_offset[p + 1];
    const int32_t np = off[p + 1] - off[p];
    if (s1 < s0) {
      set_error("parts: source_offset decreases at part %d", p);
      return DAWN_ERR_INVALID_ARG;
    }
    for (int32_t i = s0; i < s1; i++)
      if (sources[i] < 0 || sources[i] >= np) {
        set_error("parts: source %d of part %d is outside [0, %d)", sources[i], p, np);
        return DAWN_ERR_INVALID_ARG;
      }
    for (int32_t i = s0; i < s1; i += 64) {
      PartTask t;
      t.part = p;
      t.src0 = i;
      t.nsrc = std::min(64, s1 - i);
      t.pad = 0;
      t.out0 = out + (long long)(i - s0) * np;
      tasks.push_back(t);
    }
    if (rows_out)
      for (int32_t i = s0; i < s1; i++) rows_out->push_back(PartRow{out + (long long)(i - s0) * np, np, p});
    out += (long long)(s1 - s0) * np;
  }
  if (st) std::memset(st, 0, sizeof(*st));
  if (tasks.empty()) return DAWN_OK;
  // Longest tasks first, so they start while the grid is full.  Measured
  // on 512 random parts (the per-task trace), a task takes about
  // levels x (n + m / 60) time units: the per-level sweep of the part's
  // vertices costs far more than its edges.  A random part of n vertices
  // and average degree d is about ln n / ln d + 3 ln n / d levels deep
  // (correlation 0.98 with the traced depths).
  const std::vector<long long>& pos = g->pt_pos;
  std::vector<double> cost(nparts);
  for (int32_t p = 0; p < nparts; p++) {
    const double np = (double)(off[p + 1] - off[p]), mp = (double)(pos[p + 1] - pos[p]);
    const double d = np > 0 ? std::max(2.0, mp / np) : 2.0;
    const double ln = std::log(std::max(np, 2.0));
    cost[p] = (np + mp / 60.0) * std::max(1.0, ln / std::log(d) + 3.0 * ln / d);
  }
  std::stable_sort(tasks.begin(), tasks.end(),
                   [&](const PartTask& a, const PartTask& b) { return cost[a.part] > cost[b.part]; });
  const int32_t nsrc = source_offset[nparts];
  DAWN_CHECK(ensure(g->pt_tasks, sizeof(PartTask) * tasks.size(), g->stream));
  DAWN_CHECK(ensure(g->pt_sources, sizeof(int32_t) * (size_t)std::max(nsrc, 1), g->stream));
  DAWN_CHECK(ensure(g->pt_ctl, sizeof(PartsCtl), g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->pt_tasks.p, tasks.data(), sizeof(PartTask) * tasks.size(), cudaMemcpyHostToDevice,
                            g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->pt_sources.p, sources, sizeof(int32_t) * (size_t)nsrc, cudaMemcpyHostToDevice,
                            g->stream));
  PartsCtl c = {};
  c.ntasks = (int32_t)tasks.size();
  c.push_ratio = g->bs_push_ratio;
  c.tasks = g->pt_tasks.as<PartTask>();
  c.sources = g->pt_sources.as<int32_t>();
  c.dist = d_dist;
  unsigned long long* d_log = nullptr;
  if (g->trace) {
    DAWN_CHECK(pool_alloc((void**)&d_log, sizeof(unsigned long long) * 4 * tasks.size(), g->stream));
    c.task_log = d_log;
  }
  DAWN_CUDA(cudaMemcpyAsync(g->pt_ctl.p, &c, sizeof(PartsCtl), cudaMemcpyHostToDevice, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));  // c lives on this stack frame

  PartsCtl* ctl = g->pt_ctl.as<PartsCtl>();
  const int32_t* voff = g->pt_voff.as<int32_t>();
  u64* scratch = g->pt_scratch.as<u64>();
  size_t slot_words = g->pt_slot_words;
  int32_t maxn = g->pt_maxn;
  const bool capturable = g->stream != nullptr && g->stream != cudaStreamLegacy && g->stream != cudaStreamPerThread;
  if (!g->pt_exec && g->graphs_ok && capturable) {
    // One persistent launch, captured once per handle and replayed: every
    // per-call value travels in the control block.
    cudaGraph_t graph = nullptr;
    cudaStream_t cs = g->stream;
    DAWN_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    (g->pt_cluster == kPartCluster ? parts_traverse<kPartCluster> : parts_traverse<1>)<<<g->pt_slots, kPartBlock, 0, cs>>>(ctl, g->row_ptr, g->col, g->t_row_ptr, g->t_col, voff, scratch,
                                                  slot_words, maxn);
    const cudaError_t le = cudaGetLastError();
    const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      set_error("parts: capture failed: %s", cudaGetErrorString(le != cudaSuccess ? le : ce));
      return DAWN_ERR_CUDA;
    }
    const cudaError_t ie = cudaGraphInstantiate(&g->pt_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      g->pt_exec = nullptr;
      set_error("parts: graph instantiation failed: %s", cudaGetErrorString(ie));
      return DAWN_ERR_CUDA;
    }
  }
  if (g->pt_exec) {
    DAWN_CUDA(cudaGraphLaunch(g->pt_exec, g->stream));
  } else {
    (g->pt_cluster == kPartCluster ? parts_traverse<kPartCluster> : parts_traverse<1>)<<<g->pt_slots, kPartBlock, 0, g->stream>>>(ctl, g->row_ptr, g->col, g->t_row_ptr, g->t_col, voff,
                                                         scratch, slot_words, maxn);
    DAWN_CUDA(cudaGetLastError());
  }
  if (d_log) {
    // one trace record per task: device-clock start and duration
    std::vector<unsigned long long> h(4 * tasks.size());
    DAWN_CUDA(cudaMemcpyAsync(h.data(), d_log, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost,
                              g->stream));
    pool_free(d_log, g->stream);
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    unsigned long long t0 = ~0ull;
    for (size_t i = 0; i < tasks.size(); i++) t0 = std::min(t0, h[4 * i]);
    for (size_t i = 0; i < tasks.size(); i++) {
      dawn_trace_rec r = {};
      std::snprintf(r.kernel, sizeof(r.kernel), "parts_task");
      const int p = tasks[i].part;
      r.run = p;
      r.level = (int32_t)(h[4 * i + 2] >> 32);
      r.mode = (int32_t)(h[4 * i + 2] & 0xffffffffu);
      r.pad = (int32_t)h[4 * i + 3];
      r.frontier = tasks[i].nsrc;
      r.frontier_edges = g->pt_pos[p + 1] - g->pt_pos[p];
      r.unvisited_edges = (int64_t)(h[4 * i] - t0);
      r.ms = (float)((double)(h[4 * i + 1] - h[4 * i]) * 1e-6);
      g->trace_log.push_back(r);
    }
  }
  if (st) {
    PartsCtl h;
    DAWN_CUDA(cudaMemcpyAsync(&h, ctl, sizeof(PartsCtl), cudaMemcpyDeviceToHost, g->stream));
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    st->edges_traversed = (int64_t)h.reached;
    st->levels = (int32_t)h.levels;
    st->push_levels = (int32_t)h.push_levels;
    st->pull_levels = (int32_t)h.pull_levels;
    st->batches = (int32_t)tasks.size();
  }
  return DAWN_OK;
}

dawn_status parts_row_reduce(dawn_graph* g, const int32_t* d_dist, const std::vector<PartRow>& rows,
                             long long* h_sum, long long* h_cnt) {
  if (rows.empty()) return DAWN_OK;
  const size_t nr = rows.size();
  DAWN_CHECK(ensure(g->pt_rows, sizeof(PartRow) * nr, g->stream));
  DAWN_CHECK(ensure(g->cc_out, 2 * sizeof(long long) * nr, g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->pt_rows.p, rows.data(), sizeof(PartRow) * nr, cudaMemcpyHostToDevice, g->stream));
  long long* d_sum = g->cc_out.as<long long>();
  long long* d_cnt = d_sum + nr;
  const int grid = (int)std::min<size_t>(nr, (size_t)g->geo.sms * 8);
  parts_row_sums<<<grid, kBlock, 0, g->stream>>>(d_dist, g->pt_rows.as<PartRow>(), (int32_t)nr, d_sum, d_cnt);
  DAWN_CUDA(cudaGetLastError());
  DAWN_CUDA(cudaMemcpyAsync(h_sum, d_sum, sizeof(long long) * nr, cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaMemcpyAsync(h_cnt, d_cnt, sizeof(long long) * nr, cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  return DAWN_OK;
}

}  // namespace dawn
