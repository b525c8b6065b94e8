// Single-source boolean expand (BOVM) on sm_103a.
//
// Replaces the reference's SOVM kernel and its host level loop
// (src/algorithm/gpu/bfs.cu:9-105).  The reference launches one thread per
// vertex over all n rows every level, walks each row serially and polls a
// racy flag from the host every third level.  Here a level is one of
//   push: the compacted frontier queue is expanded warp-cooperatively; rows
//         of >= 32 entries are swept by the whole warp with coalesced col
//         loads, shorter rows are packed across lanes through a warp scan;
//         a visited bitmap (L2-resident, n/8 bytes) is claimed with atomicOr;
//   pull: every still-unvisited vertex scans its in-edges and stops at the
//         first neighbour in the frontier bitmap (one warp owns 32 vertices,
//         so bitmap words are written without atomics);
// and a one-thread decide kernel picks the next level's direction (Beamer's
// alpha/beta rule) on the device.  Both kernels emit the next frontier as a
// queue and as a bitmap, so either direction can follow.  Distances are
// written once, when a vertex is claimed.
#include <cooperative_groups.h>
#include <climits>
#include <mutex>

#include "cluster_levels.cuh"
#include "dawn_device.cuh"
#include "selector.cuh"

namespace dawn {
namespace {

constexpr long long kAlpha = 14, kBeta = 24;


__device__ __forceinline__ uint32_t* rot(uint32_t* fbm, int i, int nwords) {
  return fbm + (size_t)(i % 3) * nwords;
}

// Fill the current source's distance row with -1 and clear the bitmaps.
__global__ void __launch_bounds__(kBlock) bfs_clear(SsCtl* __restrict__ ctl, uint32_t* __restrict__ bitmaps,
                                                    int32_t n, int32_t nwords) {
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride) dist[i] = -1;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)4 * nwords; i += stride)
    bitmaps[i] = 0;
}

// The first level of the current source (one thread): distance 0, the
// source in the visited bitmap and the level-0 frontier, its row as the
// level-1 work, the level counters.
__device__ __forceinline__ void init_source(SsCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                                            int32_t* __restrict__ q, Seg* __restrict__ segs,
                                            uint32_t* __restrict__ vbm, int32_t n, long long m) {
  const int32_t s = ctl->sources[ctl->src_idx];
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  const int32_t deg = row_ptr[s + 1] - row_ptr[s];
  ctl->source = s;
  dist[s] = 0;
  vbm[s >> 5] |= 1u << (s & 31);
  // level-0 frontier bitmap (the first of the three rotating ones, right
  // after the visited words): read when the first level is a pull
  vbm[(n + 31) / 32 + (s >> 5)] |= 1u << (s & 31);
  if (deg >= kLongRow) {
    const int nseg = (deg + kSeg - 1) / kSeg;
    for (int j = 0; j < nseg; j++) segs[j] = Seg{s, row_ptr[s] + j * kSeg};
    ctl->qsize[0] = 0;
    ctl->lpack[0] = (1ull << 32) | (unsigned)nseg;
  } else {
    q[0] = s;
    ctl->qsize[0] = 1;
    ctl->lpack[0] = 0;
  }
  ctl->qsize[1] = 0;
  ctl->lpack[1] = 0;
  ctl->mf[0] = (unsigned long long)deg;
  ctl->mf[1] = 0;
  ctl->mu = m - deg;
  ctl->reached = (unsigned long long)deg;
  ctl->level = 1;
  ctl->mode = ctl->force - 1 == kVarPull ? kModePull : kModePush;
  ctl->done = deg == 0;
  ctl->prev_nf = 1;
  ctl->n_push = 0;
  ctl->n_pull = 0;
}

__global__ void bfs_init(SsCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                         int32_t* __restrict__ q, Seg* __restrict__ segs, uint32_t* __restrict__ vbm, int32_t n,
                         long long m) {
  if (threadIdx.x != 0) return;
  init_source(ctl, row_ptr, q, segs, vbm, n, m);
}

// bfs_clear and bfs_init in one launch: the distance row filled with -1
// (16-byte stores over its aligned middle) and the bitmaps cleared, then
// the last CTA to finish (arrival count in the control block, which it
// resets) seeds the source.
__global__ void __launch_bounds__(kBlock) bfs_start(SsCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                                                    int32_t* __restrict__ q, Seg* __restrict__ segs,
                                                    uint32_t* __restrict__ bitmaps, int32_t n, int32_t nwords,
                                                    long long m) {
  __shared__ int s_last;
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
  const size_t head = ((16 - (reinterpret_cast<uintptr_t>(dist) & 15)) & 15) / 4;
  const size_t h = head < (size_t)n ? head : (size_t)n;
  const size_t nvec = ((size_t)n - h) / 4;
  if (tid < h) dist[tid] = -1;
  int4* d4 = reinterpret_cast<int4*>(dist + h);
  for (size_t i = tid; i < nvec; i += stride) d4[i] = make_int4(-1, -1, -1, -1);
  for (size_t i = h + 4 * nvec + tid; i < (size_t)n; i += stride) dist[i] = -1;
  for (size_t i = tid; i < (size_t)4 * nwords; i += stride) bitmaps[i] = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&ctl->arrive, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    ctl->arrive = 0;
    init_source(ctl, row_ptr, q, segs, bitmaps, n, m);
  }
}

// Shared memory of one level kernel: the push's row dealing and the
// queue staging both directions use.
struct LevelSmem {
  int excl[kBlock / 32][32];
  int rs[kBlock / 32][32];
  int v[kBlock / 32][32];
  int32_t q[kBlock / 32][kWarpQueueBig];
};

// Top-down level: the frontier's rows are dealt to warps; unvisited
// targets are claimed in the visited bitmap and queued for the next level.
__device__ __forceinline__ void push_level(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                           SsCtl* __restrict__ ctl, int32_t* __restrict__ q,
                                           Seg* __restrict__ segs, size_t segcap, uint32_t* __restrict__ vbm,
                                           uint32_t* __restrict__ fbm, int32_t n, int32_t nwords, LevelSmem& sm) {
  const int L = ctl->level;
  const int pin = (L - 1) & 1, pout = L & 1;
  const int32_t* qin = q + (size_t)pin * n;
  const Seg* sin = segs + (size_t)pin * segcap;
  int32_t* qout = q + (size_t)pout * n;
  Seg* sout = segs + (size_t)pout * segcap;
  uint32_t* fout = rot(fbm, L, nwords);
  uint32_t* fclr = rot(fbm, L + 1, nwords);
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  int32_t* qcount = &ctl->qsize[pout];
  unsigned long long* lpack = &ctl->lpack[pout];
  const int qn = ctl->qsize[pin], ln = seg_count(ctl->lpack[pin]);
  const int lane = lane_id(), wib = threadIdx.x >> 5;

  const size_t gstride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)nwords; i += gstride) fclr[i] = 0;

  unsigned long long my_mf = 0;
  WarpQueueBig wq(sm.q[wib], qout, qcount);
  auto op = [&](int32_t, int k, bool valid) {
    const int32_t u = valid ? __ldg(col + k) : -1;
    const bool found = valid && claim_bit(vbm, u);
    int deg = 0, rs = 0;
    if (found) {
      rs = row_ptr[u];
      deg = row_ptr[u + 1] - rs;
      dist[u] = L;
      atomicOr(fout + (u >> 5), 1u << (u & 31));
      my_mf += (unsigned long long)deg;
    }
    emit_routed(found, u, deg, rs, wq, sout, lpack);
  };
  seg_expand(row_ptr, sin, ln, op);
  warp_expand(row_ptr, qin, qn, sm.excl[wib], sm.rs[wib], sm.v[wib], op);
  wq.flush();
  my_mf = warp_sum(my_mf);
  if (lane == 0 && my_mf) atomicAdd(&ctl->mf[pout], my_mf);
}

__global__ void __launch_bounds__(kBlock) bfs_push(const int32_t* __restrict__ row_ptr,
                                                   const int32_t* __restrict__ col, SsCtl* __restrict__ ctl,
                                                   int32_t* __restrict__ q, Seg* __restrict__ segs, size_t segcap,
                                                   uint32_t* __restrict__ vbm, uint32_t* __restrict__ fbm,
                                                   int32_t n, int32_t nwords) {
  __shared__ LevelSmem sm;
  if (ctl->done || ctl->mode != kModePush) return;
  push_level(row_ptr, col, ctl, q, segs, segcap, vbm, fbm, n, nwords, sm);
}

// Small frontiers: a single cluster of kSmallCtas CTAs runs push levels one
// after another in one launch.
//   * Each CTA appends the vertices its warps discover to its own shared-
//     memory slice (by level parity); the next level deals the rows of all
//     the cluster's slices to the cluster's warps, reading them through
//     distributed shared memory, so the frontier never goes through HBM.
//   * One cluster barrier per level (release/acquire at cluster scope)
//     orders the slices and the visited-bitmap claims; a kept vertex's
//     distance is written when the next level reads it from its slice;
//     after it every warp reads the eight slices' counters and takes the same
//     continue/stop decision.  A CTA resets its slice of the other parity
//     after the barrier: every reader of that slice (the level before) has
//     arrived at it.
//   * The loop stops after a level whose frontier is empty, holds a row of
//     >= kLongRow entries, outgrows kSmallFrontier vertices, kSmallEdges
//     out-edges or one slice (the entries past it went to the global queue
//     at once), at level n - 1, or after kSmallMaxLevels levels.  That last
//     level is handed to the per-level kernels in their format: slices ->
//     global queue and segment lists, a fresh frontier bitmap of the level
//     (the three rotating bitmaps are cleared first, since these levels did
//     not maintain them), and the counters the decide kernel reads, which
//     then does that level's bookkeeping as after a push.
// The first level reads the global queue and segments the kernels before
// wrote; its input counters are zeroed (behind one extra barrier) before a
// later level of that parity can spill into them.
__device__ __forceinline__ void decide_level(SsCtl* __restrict__ ctl, int32_t n, const float* __restrict__ sel_w,
                                             cudaGraphConditionalHandle loop, int in_graph);

__global__ void __cluster_dims__(kSmallCtas, 1, 1) __launch_bounds__(kSmallBlock)
    bfs_small(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col, SsCtl* ctl, int32_t* q,
              Seg* segs, size_t segcap, uint32_t* __restrict__ vbm, uint32_t* __restrict__ fbm, int32_t n,
              int32_t nwords, const float* __restrict__ sel_w, cudaGraphConditionalHandle loop, int in_graph) {
  __shared__ SmallSlice s_sl[2];
  // per parity: vertices appended (past kSmallCap they spilled), whether
  // one has a row of >= kLongRow entries, and their out-degree sum (the
  // degrees of distinct vertices sum to at most m < 2^31)
  __shared__ int32_t s_cnt[2], s_nlong[2];
  __shared__ uint32_t s_mf[2];
  if (ctl->done || ctl->mode != kModeSmall) return;
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  constexpr int kWarps = kSmallBlock / 32;
  const int cwarp = rank * kWarps + wib;  // warp index within the cluster
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  if (threadIdx.x < 2) {
    s_cnt[threadIdx.x] = 0;
    s_nlong[threadIdx.x] = 0;
    s_mf[threadIdx.x] = 0;
  }
  __syncthreads();

  int L = ctl->level;
  int pre = INT_MAX, tot = 0;       // dealing of the previous level's slices (lane r < kSmallCtas: slice r)
  unsigned long long sum_mf = 0;    // out-edges of the levels finished here
  int nlev = 0, last_nf = 0, nf = 0;
  unsigned long long mf = 0;
  for (int iter = 0;; iter++) {
    const int p = L & 1;
    uint32_t my_mf = 0;
    bool my_long = false;
    auto op = [&](int k, bool valid, int32_t) {
      const int32_t u = valid ? __ldg(col + k) : -1;
      bool found = false;
      int rs = 0, deg = 0;
      if (valid) {
        // the row bounds are loaded alongside the claim (most claims
        // succeed on small frontiers), so they add no round trip
        const uint32_t bit = 1u << (u & 31);
        rs = __ldg(row_ptr + u);
        const int re = __ldg(row_ptr + u + 1);
        found = !(atomicOr(vbm + (u >> 5), bit) & bit);
        deg = re - rs;
      }
      if (found) {
        my_mf += (uint32_t)deg;
        my_long |= deg >= kLongRow;
      }
      const uint32_t m = __ballot_sync(kFull, found);
      if (m == 0) return;
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(&s_cnt[p], __popc(m));
      const int slot = __shfl_sync(kFull, base, leader) + __popc(m & lanemask_lt());
      if (found && slot < kSmallCap) {
        s_sl[p].u[slot] = u;
        s_sl[p].rs[slot] = rs;
        s_sl[p].deg[slot] = deg;
      }
      const bool spill = found && slot >= kSmallCap;
      if (spill) dist[u] = L;  // kept vertices get theirs when the next level reads them
      if (__any_sync(kFull, spill))
        emit_routed(spill, u, deg, rs, q + (size_t)p * n, &ctl->qsize[p], segs + (size_t)p * segcap, &ctl->lpack[p]);
    };
    if (iter == 0) {
      // the previous level in the global format
      const int pin = p ^ 1;
      const int32_t* qin = q + (size_t)pin * n;
      const int qn = ctl->qsize[pin], ln = seg_count(ctl->lpack[pin]);
      seg_expand(row_ptr, segs + (size_t)pin * segcap, ln, [&](int32_t, int k, bool valid) { op(k, valid, 0); });
      const int bs = batch_rows(qn);
      for (int b = cwarp * bs; b < qn; b += kSmallCtas * kWarps * bs) {
        const int i = b + lane;
        const bool ok = lane < bs && i < qn;
        int rs = 0, deg = 0;
        if (ok) {
          const int32_t v = qin[i];
          rs = row_ptr[v];
          deg = row_ptr[v + 1] - rs;
        }
        expand_rows(ok, rs, deg, 0, op);
      }
    } else {
      // the previous level's slices, across the cluster
      const int bs = batch_rows(tot);
      for (int b = cwarp * bs; b < tot; b += kSmallCtas * kWarps * bs) {
        const int e = lane < bs ? b + lane : INT_MAX;
        int r = 0;  // last slice whose first index is <= e
#pragma unroll
        for (int step = kSmallCtas / 2; step; step >>= 1) {
          const int ex = __shfl_sync(kFull, pre, r + step);
          if (ex <= e) r += step;
        }
        const int off = e - __shfl_sync(kFull, pre, r);
        int rs = 0, deg = 0;
        if (e < tot) {
          const SmallSlice* src = cluster.map_shared_rank(&s_sl[p ^ 1], r);
          rs = src->rs[off];
          deg = src->deg[off];
          dist[src->u[off]] = L - 1;
        }
        expand_rows(e < tot, rs, deg, 0, op);
      }
    }
    my_mf = __reduce_add_sync(kFull, my_mf);
    my_long = __any_sync(kFull, my_long);
    if (lane == 0) {
      if (my_mf) atomicAdd(&s_mf[p], my_mf);
      if (my_long) s_nlong[p] = 1;
    }
    cluster.sync();
    // this level's counters, slice by slice (lane r reads slice r)
    int cnt = 0, nl = 0;
    uint32_t mr = 0;
    if (lane < kSmallCtas) {
      cnt = *cluster.map_shared_rank(&s_cnt[p], lane);
      nl = *cluster.map_shared_rank(&s_nlong[p], lane);
      mr = *cluster.map_shared_rank(&s_mf[p], lane);
    }
    const int kept = cnt < kSmallCap ? cnt : kSmallCap;
    int incl = kept;  // inclusive scan over the kSmallCtas slice lanes
#pragma unroll
    for (int d = 1; d < kSmallCtas; d <<= 1) {
      const int t = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl += t;
    }
    nf = (int)__reduce_add_sync(kFull, (uint32_t)cnt);
    mf = __reduce_add_sync(kFull, mr);
    const bool longs = __any_sync(kFull, nl != 0);
    const bool over = __any_sync(kFull, cnt > kSmallCap);
    const bool stop = nf == 0 || longs || over || nf > kSmallFrontier || (long long)mf > kSmallEdges ||
                      L + 1 >= n || iter + 1 == kSmallMaxLevels;
    if (stop) break;
    pre = lane < kSmallCtas ? incl - kept : INT_MAX;
    tot = __shfl_sync(kFull, incl, kSmallCtas - 1);
    sum_mf += mf;
    nlev++;
    last_nf = nf;
    if (threadIdx.x == 0) {
      s_cnt[p ^ 1] = 0;
      s_nlong[p ^ 1] = 0;
      s_mf[p ^ 1] = 0;
      if (iter == 0 && rank == 0) {
        ctl->qsize[p ^ 1] = 0;
        ctl->lpack[p ^ 1] = 0;
        ctl->mf[p ^ 1] = 0;
      }
    }
    if (iter == 0) cluster.sync(); else __syncthreads();
    L++;
  }

  // hand-off of level L (slice parity p) to the per-level kernels
  const int p = L & 1;
  const int mine = s_cnt[p] < kSmallCap ? s_cnt[p] : kSmallCap;
  for (int b = wib * 32; b < mine; b += kWarps * 32) {
    const int i = b + lane;
    const bool ok = i < mine;
    const int32_t u = ok ? s_sl[p].u[i] : 0;
    if (ok) dist[u] = L;
    emit_routed(ok, u, ok ? s_sl[p].deg[i] : 0, ok ? s_sl[p].rs[i] : 0, q + (size_t)p * n, &ctl->qsize[p],
                segs + (size_t)p * segcap, &ctl->lpack[p]);
  }
  const size_t tid = (size_t)rank * kSmallBlock + threadIdx.x;
  const size_t stride = (size_t)kSmallCtas * kSmallBlock;
  for (size_t i = tid; i < (size_t)3 * nwords; i += stride) fbm[i] = 0;
  if (rank == 0 && threadIdx.x == 0) {
    ctl->mf[p] = mf;
    ctl->reached += sum_mf;
    ctl->mu -= (long long)sum_mf;
    ctl->n_push += nlev;
    if (nlev) ctl->prev_nf = last_nf;
    ctl->level = L;
  }
  cluster.sync();  // also keeps every CTA resident until no one reads its shared memory
  uint32_t* fcur = rot(fbm, L, nwords);
  const int qn = __ldcg(&ctl->qsize[p]), ln = seg_count(__ldcg(&ctl->lpack[p]));
  for (size_t i = tid; i < (size_t)qn; i += stride) {
    const int32_t v = __ldcg(q + (size_t)p * n + i);
    atomicOr(fcur + (v >> 5), 1u << (v & 31));
  }
  // a long row's segments are contiguous: its first one sets the bit
  const Seg* sl = segs + (size_t)p * segcap;
  for (size_t i = tid; i < (size_t)ln; i += stride) {
    const int32_t v = __ldcg(&sl[i].v);
    if (i == 0 || __ldcg(&sl[i - 1].v) != v) atomicOr(fcur + (v >> 5), 1u << (v & 31));
  }
  // The handed-off level's bookkeeping, as after a push level.  Every
  // counter it reads was written before the cluster barrier above; it
  // writes the other parity's counters and the level fields, which no CTA
  // reads after that barrier.
  if (rank == 0 && threadIdx.x < 32) {
    __threadfence();
    decide_level(ctl, n, sel_w, loop, in_graph);
  }
}

// Bottom-up level: a warp owns 32 vertices (one bitmap word); each
// unvisited one scans its in-edges until a frontier bit.
__device__ __forceinline__ void pull_level(const int32_t* __restrict__ row_ptr,
                                           const int32_t* __restrict__ t_row_ptr,
                                           const int32_t* __restrict__ t_col, SsCtl* __restrict__ ctl,
                                           int32_t* __restrict__ q, Seg* __restrict__ segs, size_t segcap,
                                           uint32_t* __restrict__ vbm, uint32_t* __restrict__ fbm, int32_t n,
                                           int32_t nwords, LevelSmem& sm) {
  const int L = ctl->level;
  const int pout = L & 1;
  int32_t* qout = q + (size_t)pout * n;
  Seg* sout = segs + (size_t)pout * segcap;
  unsigned long long* lpack = &ctl->lpack[pout];
  const uint32_t* fin = rot(fbm, L - 1, nwords);
  uint32_t* fout = rot(fbm, L, nwords);
  uint32_t* fclr = rot(fbm, L + 1, nwords);
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  int32_t* qcount = &ctl->qsize[pout];
  const int lane = lane_id();

  const size_t gstride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)nwords; i += gstride) fclr[i] = 0;

  unsigned long long my_mf = 0;
  WarpQueueBig wq(sm.q[threadIdx.x >> 5], qout, qcount);
  for (int w = global_warp(); w < nwords; w += num_warps()) {
    const uint32_t vis = vbm[w];
    uint32_t unv = ~vis;
    if (w == nwords - 1 && (n & 31)) unv &= (1u << (n & 31)) - 1u;
    if (unv == 0) continue;
    const int32_t u = w * 32 + lane;
    bool found = false;
    if ((unv >> lane) & 1u) {
      const int e = t_row_ptr[u + 1];
      for (int k = t_row_ptr[u]; k < e; k++) {
        if (test_bit(fin, __ldg(t_col + k))) {
          found = true;
          break;
        }
      }
    }
    const uint32_t fm = __ballot_sync(kFull, found);
    if (fm) {
      if (lane == 0) {
        vbm[w] = vis | fm;
        fout[w] = fm;
      }
      int deg = 0, rs = 0;
      if (found) {
        rs = row_ptr[u];
        deg = row_ptr[u + 1] - rs;
        dist[u] = L;
        my_mf += (unsigned long long)deg;
      }
      emit_routed(found, u, deg, rs, wq, sout, lpack);
    }
  }
  wq.flush();
  my_mf = warp_sum(my_mf);
  if (lane == 0 && my_mf) atomicAdd(&ctl->mf[pout], my_mf);
}

__global__ void __launch_bounds__(kBlock) bfs_pull(const int32_t* __restrict__ row_ptr,
                                                   const int32_t* __restrict__ t_row_ptr,
                                                   const int32_t* __restrict__ t_col, SsCtl* __restrict__ ctl,
                                                   int32_t* __restrict__ q, Seg* __restrict__ segs, size_t segcap,
                                                   uint32_t* __restrict__ vbm, uint32_t* __restrict__ fbm,
                                                   int32_t n, int32_t nwords) {
  __shared__ LevelSmem sm;
  if (ctl->done || ctl->mode != kModePull) return;
  pull_level(row_ptr, t_row_ptr, t_col, ctl, q, segs, segcap, vbm, fbm, n, nwords, sm);
}

// One warp (all 32 lanes).  Ends the loop when the frontier is empty,
// otherwise picks the next level's direction: the forced variant if one is
// set, else the learned selector if weights are loaded (direction-
// optimising calls only), else Beamer's alpha/beta rule.  The control block
// is read through volatile loads: when this runs at the end of the level
// kernel itself, counters other CTAs just raised may sit stale in this
// SM's L1.
__device__ __forceinline__ void decide_level(SsCtl* __restrict__ ctl, int32_t n, const float* __restrict__ sel_w,
                                             cudaGraphConditionalHandle loop, int in_graph) {
  const int lane = lane_id();
  if (sel_w) sel_prefetch(sel_w);
  const volatile SsCtl* vc = ctl;
  // every lane reads the control block before lane 0 changes it
  const int done = vc->done;
  const int L = vc->level, pout = L & 1;
  const int nf = vc->qsize[pout] + long_vertices(vc->lpack[pout]);
  const unsigned long long mf = vc->mf[pout];
  const long long mu = vc->mu - (long long)mf;
  const int cur_mode = vc->mode, prev_nf = vc->prev_nf, policy = vc->policy, force = vc->force;
  const bool sel = vc->use_sel && sel_w;
  const long long m = vc->m;
  const int small = vc->small;
  const unsigned long long nlong = long_vertices(vc->lpack[pout]);
  const float margin = vc->sel_margin;
  __syncwarp();
  if (done) {
    if (lane == 0 && in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  if (lane == 0) {
    ctl->reached += mf;
    ctl->mu = mu;
    if (cur_mode == kModePull) ctl->n_pull++; else ctl->n_push++;
  }
  if (nf == 0 || L >= n) {
    if (lane == 0) {
      ctl->done = 1;
      if (in_graph) cudaGraphSetConditional(loop, 0);
    }
    return;
  }
  int mode = cur_mode == kModePull ? kModePull : kModePush;  // cluster levels are push levels
  if (policy == DAWN_VARIANT_DO) {
    if (mode == kModePush) {
      if ((long long)mf * kAlpha > mu && nf > prev_nf) mode = kModePull;
    } else {
      if ((long long)nf * kBeta < (long long)n && nf < prev_nf) mode = kModePush;
    }
  }
  if (force) {
    mode = force - 1 == kVarPull ? kModePull : kModePush;
  } else if (policy == DAWN_VARIANT_DO && sel) {
    float x[kSelIn];
    sel_features(x, (float)n, (float)m, (float)nf, (float)mf, (float)mu, (float)(L + 1), (float)prev_nf, 1.0f);
    const int h = mode == kModePull ? kVarPull : kVarPush;
    mode = sel_pick(sel_w, x, (1u << kVarPush) | (1u << kVarPull), h, margin) == kVarPull ? kModePull
                                                                                         : kModePush;
  }
  // small levels start from frontiers without long rows: a long row's
  // neighbourhood tends to hold more, which end the cluster levels at once
  if (mode == kModePush && small && !force && policy == DAWN_VARIANT_DO && nf <= kSmallFrontier &&
      (long long)mf <= kSmallEdges && nlong == 0)
    mode = kModeSmall;
  if (lane == 0) {
    ctl->qsize[pout ^ 1] = 0;
    ctl->lpack[pout ^ 1] = 0;
    ctl->mf[pout ^ 1] = 0;
    ctl->prev_nf = nf;
    ctl->mode = mode;
    ctl->level = L + 1;
  }
}

__global__ void bfs_decide(SsCtl* __restrict__ ctl, int32_t n, const float* __restrict__ sel_w,
                           cudaGraphConditionalHandle loop, int in_graph) {
  decide_level(ctl, n, sel_w, loop, in_graph);
}

// One launch per push or pull level: the level's work, then its end-of-
// level bookkeeping by the last CTA to finish (an arrival count in the
// control block, reset by that CTA), so a level costs one kernel instead of
// a work kernel and a decide kernel.  Returns at once at cluster levels.
__global__ void __launch_bounds__(kBlock, 5) bfs_step(const int32_t* __restrict__ row_ptr,
                                                   const int32_t* __restrict__ col,
                                                   const int32_t* __restrict__ t_row_ptr,
                                                   const int32_t* __restrict__ t_col, SsCtl* __restrict__ ctl,
                                                   int32_t* __restrict__ q, Seg* __restrict__ segs, size_t segcap,
                                                   uint32_t* __restrict__ vbm, uint32_t* __restrict__ fbm,
                                                   int32_t n, int32_t nwords, const float* __restrict__ sel_w,
                                                   cudaGraphConditionalHandle loop, int in_graph) {
  __shared__ LevelSmem sm;
  __shared__ int s_last;
  if (ctl->done) {
    // a traversal that ended before its first level (an isolated source)
    // or at a cluster level: the loop still has to be told
    if (in_graph && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(loop, 0);
    return;
  }
  const int mode = ctl->mode;
  if (mode == kModePush)
    push_level(row_ptr, col, ctl, q, segs, segcap, vbm, fbm, n, nwords, sm);
  else if (mode == kModePull)
    pull_level(row_ptr, t_row_ptr, t_col, ctl, q, segs, segcap, vbm, fbm, n, nwords, sm);
  else
    return;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&ctl->arrive, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x < 32) {
    __threadfence();
    if (threadIdx.x == 0) ctl->arrive = 0;
    decide_level(ctl, n, sel_w, loop, in_graph);
  }
}

__global__ void ss_next(SsCtl* __restrict__ ctl) {
  if (threadIdx.x != 0) return;
  ctl->total_reached += ctl->reached;
  ctl->total_levels += ctl->level;
  ctl->total_push += ctl->n_push;
  ctl->total_pull += ctl->n_pull;
  ctl->src_idx += 1;
}

void probe_ss(const void* p, LevelProbe* out) {
  const SsCtl* c = static_cast<const SsCtl*>(p);
  const int pin = (c->level - 1) & 1;
  out->level = c->level;
  out->mode = c->mode;
  out->done = c->done;
  out->frontier = c->qsize[pin] + (int64_t)(c->lpack[pin] >> 32);
  out->frontier_edges = (int64_t)c->mf[pin];
  out->unvisited_edges = c->mu;
}

}  // namespace

dawn_status bfs_single(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_dist,
                       int32_t policy) {
  const int32_t n = g->n;
  int32_t nwords = (n + 31) / 32;
  long long m = g->m;
  DAWN_CHECK(ensure(g->ss_queues, sizeof(int32_t) * 2 * (size_t)n, g->stream));
  size_t segcap = seg_capacity(n, m);
  DAWN_CHECK(ensure(g->ss_segs, sizeof(Seg) * 2 * segcap, g->stream));
  DAWN_CHECK(ensure(g->ss_bitmaps, sizeof(uint32_t) * 4 * (size_t)nwords, g->stream));
  DAWN_CHECK(ensure(g->ss_ctl, sizeof(SsCtl), g->stream));
  DAWN_CHECK(ensure(g->ss_sources, sizeof(int32_t) * (size_t)nsrc, g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->ss_sources.p, sources, sizeof(int32_t) * nsrc, cudaMemcpyHostToDevice,
                            g->stream));
  SsCtl c = {};
  c.policy = policy;
  c.nsrc = nsrc;
  c.dist_base = d_dist;
  c.sources = g->ss_sources.as<int32_t>();
  c.use_sel = g->sel_call;
  c.sel_margin = g->sel_margin;
  c.force = g->force_variant == 3 ? 1 + kVarPush : g->force_variant;
  c.small = g->small_levels && cluster_fits((const void*)bfs_small, kSmallCtas, kSmallBlock) ? 1 : 0;
  c.m = m;
  DAWN_CHECK(upload_ctl(g, c));

  struct {
    SsCtl* ctl;
    const int32_t *row_ptr, *col, *t_row_ptr, *t_col;
    int32_t* q;
    Seg* segs;
    size_t segcap;
    uint32_t *bitmaps, *vbm, *fbm;
    int32_t n, nwords;
    long long m;
    cudaGraphConditionalHandle handle;
    int in_graph;
    const float* sel_w;
  } a;
  a.sel_w = g->sel_slot.as<float>();
  a.ctl = g->ss_ctl.as<SsCtl>();
  a.row_ptr = g->row_ptr;
  a.col = g->col;
  a.t_row_ptr = g->t_row_ptr;
  a.t_col = g->t_col;
  a.q = g->ss_queues.as<int32_t>();
  a.segs = g->ss_segs.as<Seg>();
  a.segcap = segcap;
  a.bitmaps = g->ss_bitmaps.as<uint32_t>();
  a.vbm = a.bitmaps;
  a.fbm = a.bitmaps + nwords;
  a.n = n;
  a.nwords = nwords;
  a.m = m;
  a.handle = 0;
  a.in_graph = 0;
  void* start_args[] = {&a.ctl, &a.row_ptr, &a.q, &a.segs, &a.bitmaps, &a.n, &a.nwords, &a.m};
  void* step_args[] = {&a.row_ptr, &a.col, &a.t_row_ptr, &a.t_col, &a.ctl, &a.q, &a.segs, &a.segcap, &a.vbm,
                       &a.fbm, &a.n, &a.nwords, &a.sel_w, &a.handle, &a.in_graph};
  void* small_args[] = {&a.row_ptr, &a.col, &a.ctl, &a.q, &a.segs, &a.segcap, &a.vbm, &a.fbm, &a.n, &a.nwords,
                        &a.sel_w, &a.handle, &a.in_graph};
  void* next_args[] = {&a.ctl};

  const int sms = g->geo.sms;
  SsFamily fam;
  fam.npre = 1;
  fam.pre[0] = {(const void*)bfs_start, start_args, dim3(sms * 8), dim3(kBlock), "bfs_start"};
  // Two kernels per loop iteration, each ending its level with the
  // bookkeeping (no separate decide launch): the push/pull level kernel and
  // the cluster levels; the one whose mode does not match returns at once.
  fam.nbody = 2;
  fam.decide_in_body = true;
  fam.body[0] = {(const void*)bfs_step, step_args,
                 dim3(persistent_blocks((const void*)bfs_step, kBlock, 0, g->blocks_per_sm)), dim3(kBlock),
                 "bfs_step", kModeStep};
  fam.body[1] = {(const void*)bfs_small, small_args, dim3(kSmallCtas), dim3(kSmallBlock), "bfs_small", kModeSmall};
  fam.npost = 1;
  fam.post[0] = {(const void*)ss_next, next_args, dim3(1), dim3(32), "ss_next"};
  fam.ctl = a.ctl;
  fam.ctl_bytes = sizeof(SsCtl);
  fam.probe = probe_ss;
  fam.handle = &a.handle;
  fam.in_graph = &a.in_graph;
  fam.done_flag = &a.ctl->done;
  return ss_run(g, fam, nsrc, &g->bfs_exec);
}

// --- single-source BFS with static scratch (dawn_bfs_static) ---------------
//
// Some callers may not allocate device memory at the moment they traverse:
// a serving loop whose device memory is entirely reserved by another
// allocator, or one that must never wait on the allocator (an allocation
// can synchronise the device, or fail under fragmentation, at a point where
// neither is acceptable).  For them the push traversal above runs over a
// fixed block of device memory that the library declares at file scope, so
// the call allocates nothing: the caller owns the CSR and the distance row,
// and every other word the traversal touches lives in `g_static_scratch`.
//
// The block holds a graph of at most kStaticMaxVertices vertices and
// kStaticMaxEdges edges (about 12.5 MiB).  It exists on a GPU once the
// library's kernels are loaded there (with lazy module loading, at the
// first launch of one of them on that device) and stays until the process
// exits.  There is one block per device,
// so calls that overlap on one device (from two host threads, or on two
// streams) race on it: the caller serialises them.

constexpr int32_t kStaticMaxVertices = DAWN_STATIC_MAX_VERTICES;
constexpr long long kStaticMaxEdges = DAWN_STATIC_MAX_EDGES;
constexpr size_t kStaticSegCap = 2 * (size_t)(kStaticMaxEdges / kSeg) + 64;  // seg_capacity at the maxima
constexpr size_t kStaticWords = (size_t)(kStaticMaxVertices + 31) / 32;
// layout (byte offsets, each 256-aligned): control block | source | flags |
// 4 bitmaps | 2 vertex queues | 2 segment lists
constexpr size_t kStaticCtlOff = 0;
constexpr size_t kStaticSrcOff = 512;
constexpr size_t kStaticFlagOff = 768;
constexpr size_t kStaticBitmapOff = 1024;
constexpr size_t kStaticQueueOff = kStaticBitmapOff + 4 * kStaticWords * sizeof(uint32_t);
constexpr size_t kStaticSegOff = kStaticQueueOff + 2 * (size_t)kStaticMaxVertices * sizeof(int32_t);
constexpr size_t kStaticBytes = kStaticSegOff + 2 * kStaticSegCap * sizeof(Seg);
static_assert(sizeof(SsCtl) <= kStaticSrcOff, "control block overlaps the source slot");
static_assert(kStaticQueueOff % 256 == 0 && kStaticSegOff % 256 == 0, "scratch regions must stay 256-aligned");

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

namespace {

constexpr int kStaticPollLevels = 8;  // levels launched between two reads of the done flag
constexpr int kStaticMaxDevices = 64;

struct StaticDevice {
  std::once_flag once;
  cudaError_t err = cudaSuccess;
  unsigned char* scratch = nullptr;
  int clear_blocks = 0, push_blocks = 0, check_blocks = 0;
};
StaticDevice g_static_dev[kStaticMaxDevices];

// Set-up of one device, run once with that device current: the address of
// its copy of the scratch block and the launch shapes.
void static_setup(StaticDevice& d) {
  d.err = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.scratch), g_static_scratch);
  if (d.err != cudaSuccess) return;
  int dev = 0, sms = 0, per_sm = 0;
  if ((d.err = cudaGetDevice(&dev)) != cudaSuccess) return;
  if ((d.err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return;
  if ((d.err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bfs_push, kBlock, 0)) != cudaSuccess) return;
  d.push_blocks = sms * (per_sm > 0 ? per_sm : 1);
  d.clear_blocks = sms * 4;
  d.check_blocks = sms * 8;
}

// CSR checks of the static path: same invariants as the upload-time
// validation, with scalar loads (the caller's arrays carry no alignment
// promise beyond 4 bytes).  Flags: 1 row_ptr[0] != 0, 2 row_ptr[n] != m,
// 4 row_ptr decreases, 8 column outside [0, n).
__global__ void __launch_bounds__(kBlock) static_check_csr(const int32_t* __restrict__ rp,
                                                           const int32_t* __restrict__ col, int32_t n, long long m,
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
  for (size_t k = tid; k < (size_t)m; k += stride) {
    const int32_t c = __ldg(col + k);
    if (c < 0 || c >= n) f |= 8;
  }
  if (f) atomicOr(flags, f);
}

// Writes the control block of a one-source push traversal into the
// scratch (every field, so nothing is left from an earlier call) and clears
// the flag word.
__global__ void static_begin(SsCtl* __restrict__ ctl, int32_t* __restrict__ src_slot, int* __restrict__ flags,
                             int32_t source, int32_t* dist) {
  if (threadIdx.x != 0) return;
  SsCtl c = {};
  c.policy = DAWN_VARIANT_PUSH;
  c.nsrc = 1;
  c.dist_base = dist;
  c.sources = src_slot;
  *ctl = c;
  *src_slot = source;
  *flags = 0;
}

}  // namespace

dawn_status bfs_static(const int32_t* row_ptr, const int32_t* col, int32_t n, int64_t m, int32_t source,
                       int32_t* dist, uint32_t flags, cudaStream_t stream) {
  if (!row_ptr || !dist || (m > 0 && !col)) {
    set_error("dawn_bfs_static: row_ptr, col and dist must be device pointers (col may be NULL only when m = 0)");
    return DAWN_ERR_INVALID_ARG;
  }
  if (n < 1 || n > kStaticMaxVertices) {
    set_error("dawn_bfs_static: n = %d outside [1, %d], the vertex limit of the static scratch block", n,
              kStaticMaxVertices);
    return DAWN_ERR_INVALID_ARG;
  }
  if (m < 0 || m > kStaticMaxEdges) {
    set_error("dawn_bfs_static: m = %lld outside [0, %lld], the edge limit of the static scratch block",
              (long long)m, kStaticMaxEdges);
    return DAWN_ERR_INVALID_ARG;
  }
  if (source < 0 || source >= n) {
    set_error("dawn_bfs_static: source %d outside [0, %d)", source, n);
    return DAWN_ERR_INVALID_ARG;
  }
  int dev = 0;
  DAWN_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kStaticMaxDevices) {
    set_error("dawn_bfs_static: device %d beyond the %d devices the library tracks", dev, kStaticMaxDevices);
    return DAWN_ERR_UNSUPPORTED;
  }
  const void* ptrs[3] = {row_ptr, col, dist};
  for (const void* p : ptrs) {
    if (!p) continue;
    cudaPointerAttributes at;
    DAWN_CUDA(cudaPointerGetAttributes(&at, p));
    if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) || at.device != dev) {
      set_error("dawn_bfs_static: row_ptr, col and dist must be memory of the current device (%d)", dev);
      return DAWN_ERR_INVALID_ARG;
    }
  }
  StaticDevice& d = g_static_dev[dev];
  std::call_once(d.once, static_setup, std::ref(d));
  DAWN_CUDA(d.err);

  SsCtl* ctl = reinterpret_cast<SsCtl*>(d.scratch + kStaticCtlOff);
  int32_t* src_slot = reinterpret_cast<int32_t*>(d.scratch + kStaticSrcOff);
  int* d_flags = reinterpret_cast<int*>(d.scratch + kStaticFlagOff);
  uint32_t* bitmaps = reinterpret_cast<uint32_t*>(d.scratch + kStaticBitmapOff);
  int32_t* q = reinterpret_cast<int32_t*>(d.scratch + kStaticQueueOff);
  Seg* segs = reinterpret_cast<Seg*>(d.scratch + kStaticSegOff);
  const int32_t nwords = (n + 31) / 32;
  uint32_t* vbm = bitmaps;
  uint32_t* fbm = bitmaps + nwords;

  static_begin<<<1, 32, 0, stream>>>(ctl, src_slot, d_flags, source, dist);
  DAWN_CUDA(cudaGetLastError());
  if (!(flags & DAWN_GRAPH_NO_VALIDATE)) {
    static_check_csr<<<d.check_blocks, kBlock, 0, stream>>>(row_ptr, col, n, (long long)m, d_flags);
    DAWN_CUDA(cudaGetLastError());
    int f = 0;
    DAWN_CUDA(cudaMemcpyAsync(&f, d_flags, sizeof(int), cudaMemcpyDeviceToHost, stream));
    DAWN_CUDA(cudaStreamSynchronize(stream));
    if (f) {
      set_error("dawn_bfs_static: invalid CSR:%s%s%s%s", (f & 1) ? " row_ptr[0] != 0;" : "",
                (f & 2) ? " row_ptr[n] != m;" : "", (f & 4) ? " row_ptr decreases;" : "",
                (f & 8) ? " col index outside [0, n);" : "");
      return DAWN_ERR_INVALID_ARG;
    }
  }
  // bfs_clear fills the distance row with -1 and zeroes the visited and
  // frontier bitmaps; bfs_init seeds the source.  Queues and segment lists
  // are read only up to the sizes the control block records.
  bfs_clear<<<d.clear_blocks, kBlock, 0, stream>>>(ctl, bitmaps, n, nwords);
  DAWN_CUDA(cudaGetLastError());
  bfs_init<<<1, 32, 0, stream>>>(ctl, row_ptr, q, segs, vbm, n, (long long)m);
  DAWN_CUDA(cudaGetLastError());
  // Levels after the last one return at once (done is set), so the host
  // reads the flag only every kStaticPollLevels levels.  Each level sets
  // done once its frontier is empty or the level count reaches n.
  for (;;) {
    for (int j = 0; j < kStaticPollLevels; j++) {
      bfs_push<<<d.push_blocks, kBlock, 0, stream>>>(row_ptr, col, ctl, q, segs, kStaticSegCap, vbm, fbm, n,
                                                      nwords);
      bfs_decide<<<1, 32, 0, stream>>>(ctl, n, nullptr, 0, 0);
    }
    DAWN_CUDA(cudaGetLastError());
    int32_t done = 0;
    DAWN_CUDA(cudaMemcpyAsync(&done, &ctl->done, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
    DAWN_CUDA(cudaStreamSynchronize(stream));
    if (done) break;
  }
  return DAWN_OK;
}

}  // namespace dawn
