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
// Neither writes distances during the traversal: the level at which a bit
// first appears is recorded in bit-sliced level words (slice k holds bit k
// of the level of every (source, vertex) pair, 64 sources per word), and a
// final pass expands them into the nsrc x n distance block with full-line
// coalesced stores, writing -1 for pairs never reached.
#include "dawn_device.cuh"

namespace dawn {
namespace {

struct BsCtl {
  int32_t aq_size[3];          // active (frontier) list sizes, rotating by level % 3
  int32_t pad0;
  unsigned long long alpack[3]; // active long rows: (vertices << 32) | segments
  int32_t tq_size;             // push: vertices touched this level
  int32_t ul_size[2];          // unfinished-vertex lists (pull work lists)
  int32_t ul_cur;              // list the next pull reads: -1 = the graph's static list
  int32_t level, mode, done, policy, batch, nsrc, n_push, n_pull;
  int32_t push_ratio;          // push while push_ratio * frontier edges < unfinished edges
  int32_t work;                // dynamic work counter of the current level (light rows)
  int32_t hwork;               // dynamic work counter of the heavy-row segments
  int32_t dense;               // push level: fire-and-forget scatter + dense update sweep
  int32_t nbits;               // level slices available
  int32_t pad3;
  unsigned long long mf[3];    // out-degree sums of the active lists
  long long mu;                // in-degree sum of vertices not yet finished
  long long mu_dec;            // in-degree of vertices finished this level
  unsigned long long reached;  // TEPS numerator of the batch
  unsigned long long full;     // this batch's source bits
  int32_t* dist_base;
  const int32_t* sources;
  unsigned long long total_reached;
  int32_t total_levels, total_push, total_pull, pad2;
};

using u64 = unsigned long long;

__device__ __forceinline__ u64 warp_or64(u64 x) {
  const unsigned lo = __reduce_or_sync(kFull, (unsigned)x);
  const unsigned hi = __reduce_or_sync(kFull, (unsigned)(x >> 32));
  return ((u64)hi << 32) | lo;
}

constexpr int kSlicesCleared = 8;
constexpr int kPullHeavy = 2048;  // in-degree from which a pull row is cut into segments
constexpr int kPullSeg = 1024;    // entries per heavy-row segment  // slices zeroed per batch; higher ones on first use

// Records the level of newly reached (source, vertex) pairs: slice k of
// vertex u gains nw for every set bit k of the level.  The caller owns u.
__device__ __forceinline__ void record_level(u64* __restrict__ slices, int32_t n, int32_t u, u64 nw, int32_t level) {
  for (unsigned L = (unsigned)level; L; L &= L - 1) {
    u64* w = slices + (size_t)(__ffs(L) - 1) * n + u;
    *w |= nw;
  }
}

// Level L is the last one before slice log2(L + 1) is first used: clear it.
__device__ __forceinline__ void clear_next_slice(u64* __restrict__ slices, int32_t n, int32_t level, int nbits) {
  const unsigned next = (unsigned)level + 1;
  if (next & (next - 1)) return;
  const int b = __ffs(next) - 1;
  if (b < kSlicesCleared || b >= nbits) return;
  u64* w = slices + (size_t)b * n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride) w[i] = 0ull;
}

// Zero the frontier words listed in a stale active list and its segment
// list (grid-stride).
__device__ __forceinline__ void clear_listed(u64* __restrict__ fr, const int32_t* __restrict__ list, int cnt,
                                             const Seg* __restrict__ segs, int nsegs) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)cnt; i += stride) fr[list[i]] = 0ull;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)nsegs; i += stride)
    fr[segs[i].v] = 0ull;
}

__global__ void __launch_bounds__(kBlock) bs_clear(u64* __restrict__ words, size_t count) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  ulonglong2* w2 = reinterpret_cast<ulonglong2*>(words);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count / 2; i += stride)
    w2[i] = make_ulonglong2(0ull, 0ull);
  if (blockIdx.x == 0 && threadIdx.x == 0 && (count & 1)) words[count - 1] = 0;
}

__global__ void bs_init(BsCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                        const int32_t* __restrict__ t_row_ptr, u64* __restrict__ visit, u64* __restrict__ fr0,
                        int32_t* __restrict__ aq0, Seg* __restrict__ segs0, int32_t n, long long m) {
  __shared__ u64 s_mf, s_reached, s_dec;
  const int b = threadIdx.x;
  const int batch = ctl->batch;
  const int nb = min(64, ctl->nsrc - batch * 64);
  if (b == 0) {
    s_mf = 0;
    s_reached = 0;
    s_dec = 0;
    for (int i = 0; i < 3; i++) {
      ctl->aq_size[i] = 0;
      ctl->alpack[i] = 0;
    }
    ctl->tq_size = 0;
    ctl->ul_size[0] = 0;
    ctl->ul_size[1] = 0;
    ctl->ul_cur = -1;
    ctl->work = 0;
    ctl->hwork = 0;
    ctl->dense = 0;
    ctl->full = nb == 64 ? ~0ull : ((1ull << nb) - 1ull);
  }
  __syncthreads();
  int32_t s = -1;
  bool first = false;
  if (b < nb) {
    s = ctl->sources[batch * 64 + b];
    const u64 bit = 1ull << b;
    atomicOr(visit + s, bit);
    first = atomicOr(fr0 + s, bit) == 0ull;
    atomicAdd(&s_reached, (u64)(row_ptr[s + 1] - row_ptr[s]));
  }
  __syncthreads();
  if (first) {
    const int rs = row_ptr[s], deg = row_ptr[s + 1] - rs;
    if (deg >= kLongRow) {
      const int nseg = (deg + kSeg - 1) / kSeg;
      const u64 old = atomicAdd(&ctl->alpack[0], (1ull << 32) | (unsigned)nseg);
      for (int j = 0; j < nseg; j++) segs0[(uint32_t)old + j] = Seg{s, rs + j * kSeg};
    } else {
      aq0[atomicAdd(&ctl->aq_size[0], 1)] = s;
    }
    atomicAdd(&s_mf, (u64)deg);
    if (visit[s] == ctl->full) atomicAdd(&s_dec, (u64)(t_row_ptr[s + 1] - t_row_ptr[s]));
  }
  __syncthreads();
  if (b == 0) {
    for (int i = 0; i < 3; i++) ctl->mf[i] = 0;
    ctl->mf[0] = s_mf;
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
  u64 mf = 0, reached = 0, dec = 0;
  __device__ __forceinline__ void add(u64 out_deg, u64 in_deg, u64 nw, bool finished) {
    mf += out_deg;
    reached += out_deg * (u64)__popcll(nw);
    if (finished) dec += in_deg;
  }
  __device__ __forceinline__ void flush(BsCtl* ctl, int slot) {
    mf = warp_sum(mf);
    reached = warp_sum(reached);
    dec = warp_sum(dec);
    if (lane_id() == 0) {
      if (mf) atomicAdd(&ctl->mf[slot], mf);
      if (reached) atomicAdd(&ctl->reached, reached);
      if (dec) atomicAdd(reinterpret_cast<u64*>(&ctl->mu_dec), dec);
    }
  }
};

// Pull: every vertex of the unfinished list ORs the frontier words of its
// in-neighbours.  Rows of >= 32 entries are swept by the whole warp (coalesced
// col loads, early exit once no missing bit is left); shorter rows are
// concatenated across the warp and OR-ed into per-lane shared-memory slots.
// The vertex then owns its words: no global atomics.  The list is filtered
// into the next unfinished list as it goes.
__global__ void __launch_bounds__(kBlock, 5) bs_pull(const int32_t* __restrict__ row_ptr,
                                                     const int32_t* __restrict__ t_row_ptr,
                                                     const int32_t* __restrict__ t_col, BsCtl* __restrict__ ctl,
                                                     u64* __restrict__ visit, u64* __restrict__ fr,
                                                     u64* __restrict__ slices, int32_t* __restrict__ aq,
                                                     Seg* __restrict__ segs, size_t segcap,
                                                     const int32_t* __restrict__ ul_static, int32_t ul_static_size,
                                                     int32_t* __restrict__ ul, const int32_t* __restrict__ hv_static,
                                                     const int32_t* __restrict__ hv_segoff, u64* __restrict__ hv_acc,
                                                     int32_t hv_count, int32_t hv_segs, int32_t n) {
  __shared__ int s_excl[kBlock / 32][32];
  __shared__ int s_rs[kBlock / 32][32];
  __shared__ u64 s_acc[kBlock / 32][32];
  __shared__ int32_t s_qa[kBlock / 32][kWarpQueue];
  __shared__ int32_t s_qu[kBlock / 32][kWarpQueue];
  if (ctl->done || ctl->mode != kModePull) return;
  const int L = ctl->level;
  const u64* __restrict__ fin = fr + (size_t)((L - 1) % 3) * n;
  u64* __restrict__ fout = fr + (size_t)(L % 3) * n;
  int32_t* aq_out = aq + (size_t)(L % 3) * n;
  Seg* seg_out = segs + (size_t)(L % 3) * segcap;
  int32_t* aq_count = &ctl->aq_size[L % 3];
  u64* al_pack = &ctl->alpack[L % 3];
  clear_listed(fr + (size_t)((L + 1) % 3) * n, aq + (size_t)((L + 1) % 3) * n, ctl->aq_size[(L + 1) % 3],
               segs + (size_t)((L + 1) % 3) * segcap, seg_count(ctl->alpack[(L + 1) % 3]));
  clear_next_slice(slices, n, L, ctl->nbits);
  const int cur = ctl->ul_cur;
  const int32_t* ul_in = cur < 0 ? ul_static : ul + (size_t)cur * n;
  const int un = cur < 0 ? ul_static_size : ctl->ul_size[cur];
  const int nxt = cur < 0 ? 0 : cur ^ 1;
  int32_t* ul_out = ul + (size_t)nxt * n;
  int32_t* ul_count = &ctl->ul_size[nxt];
  const u64 full = ctl->full;
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  LevelAcc acc;
  WarpQueue qa(s_qa[wib], aq_out, aq_count);
  WarpQueue qu(s_qu[wib], ul_out, ul_count);
  // Heavy rows first, one kPullSeg-entry segment per warp task.  Each
  // segment ORs its gathers into the row's accumulator; the warp finishing
  // the row's last segment folds the accumulator into the vertex.  Only
  // that warp writes the vertex's words, so every segment sees the same
  // visited word for the whole level.
  for (;;) {
    int sidx = 0;
    if (lane == 0) sidx = atomicAdd(&ctl->hwork, 1);
    sidx = __shfl_sync(kFull, sidx, 0);
    if (sidx >= hv_segs) break;
    int lo = 0, hi = hv_count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(hv_segoff + mid) <= sidx) lo = mid; else hi = mid - 1;
    }
    const int32_t u = __ldg(hv_static + lo);
    const u64 vis = visit[u];
    if (vis == full) continue;
    const int s0 = __ldg(hv_segoff + lo);
    const int nseg = __ldg(hv_segoff + lo + 1) - s0;
    const int rbeg = t_row_ptr[u], rend = t_row_ptr[u + 1];
    const int ks = rbeg + (sidx - s0) * kPullSeg, ke = min(ks + kPullSeg, rend);
    u64* hacc = hv_acc + 2 * (size_t)lo;
    u64 w = 0;
    for (int k0 = ks; k0 < ke; k0 += 128) {
      const int k = k0 + lane;
      const int32_t v0 = k < ke ? __ldg(t_col + k) : -1;
      const int32_t v1 = k + 32 < ke ? __ldg(t_col + k + 32) : -1;
      const int32_t v2 = k + 64 < ke ? __ldg(t_col + k + 64) : -1;
      const int32_t v3 = k + 96 < ke ? __ldg(t_col + k + 96) : -1;
      const u64 x0 = v0 >= 0 ? __ldg(fin + v0) : 0ull;
      const u64 x1 = v1 >= 0 ? __ldg(fin + v1) : 0ull;
      const u64 x2 = v2 >= 0 ? __ldg(fin + v2) : 0ull;
      const u64 x3 = v3 >= 0 ? __ldg(fin + v3) : 0ull;
      w |= x0 | x1 | x2 | x3;
      if ((warp_or64(w) | vis | __ldcg(hacc)) == full) break;
    }
    w = warp_or64(w);
    int last = 0;
    if (lane == 0) {
      if (w) atomicOr(hacc, w);
      __threadfence();
      last = atomicAdd(hacc + 1, 1ull) == (u64)(nseg - 1);
    }
    last = __shfl_sync(kFull, last, 0);
    if (!last) continue;
    u64 nw = 0;
    int odeg = 0, ors = 0;
    if (lane == 0) {
      __threadfence();
      const u64 got = atomicOr(hacc, 0ull);
      hacc[0] = 0ull;
      hacc[1] = 0ull;
      nw = got & ~vis;
      if (nw) {
        visit[u] = vis | nw;
        fout[u] = nw;
        record_level(slices, n, u, nw, L);
        ors = row_ptr[u];
        odeg = row_ptr[u + 1] - ors;
        acc.add((u64)odeg, (u64)(rend - rbeg), nw, (vis | nw) == full);
      }
    }
    emit_routed(nw != 0ull, u, odeg, ors, qa, seg_out, al_pack);
  }
  // Light rows: warps take 32 list entries at a time from a shared counter
  // (row lengths differ widely; static striding does not balance them).
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&ctl->work, 32);
    base = __shfl_sync(kFull, base, 0);
    if (base >= un) break;
    const int idx = base + lane;
    int32_t u = -1;
    u64 vis = full;
    if (idx < un) {
      u = ul_in[idx];
      vis = visit[u];
    }
    const bool active = vis != full;
    int rs = 0, re = 0;
    if (active) {
      rs = t_row_ptr[u];
      re = t_row_ptr[u + 1];
    }
    const int deg = re - rs;
    u64 got = 0;
    uint32_t big = __ballot_sync(kFull, deg >= kWarpRow);
    while (big) {
      const int leader = __ffs(big) - 1;
      big &= big - 1;
      const int s = __shfl_sync(kFull, rs, leader), e = __shfl_sync(kFull, re, leader);
      const u64 lvis = __shfl_sync(kFull, vis, leader);
      u64 w = 0;
      // Four independent gathers in flight per lane, one early-exit test
      // per 128 entries.
      for (int k0 = s; k0 < e; k0 += 128) {
        const int k = k0 + lane;
        const int32_t v0 = k < e ? __ldg(t_col + k) : -1;
        const int32_t v1 = k + 32 < e ? __ldg(t_col + k + 32) : -1;
        const int32_t v2 = k + 64 < e ? __ldg(t_col + k + 64) : -1;
        const int32_t v3 = k + 96 < e ? __ldg(t_col + k + 96) : -1;
        const u64 x0 = v0 >= 0 ? __ldg(fin + v0) : 0ull;
        const u64 x1 = v1 >= 0 ? __ldg(fin + v1) : 0ull;
        const u64 x2 = v2 >= 0 ? __ldg(fin + v2) : 0ull;
        const u64 x3 = v3 >= 0 ? __ldg(fin + v3) : 0ull;
        w |= x0 | x1 | x2 | x3;
        if ((warp_or64(w) | lvis) == full) break;
      }
      w = warp_or64(w);
      if (lane == leader) got = w;
    }
    const int sdeg = deg < kWarpRow ? deg : 0;
    const int incl = warp_incl_scan(sdeg);
    const int total = __shfl_sync(kFull, incl, 31);
    s_excl[wib][lane] = incl - sdeg;
    s_rs[wib][lane] = rs;
    s_acc[wib][lane] = 0ull;
    __syncwarp();
    // Two edges per lane per pass: both searches and both gathers are
    // independent, so their latencies overlap.
    for (int e0 = 0; e0 < total; e0 += 64) {
      const int ea = e0 + lane, eb = ea + 32;
      int la = 0, lb = 0;
      {
        int lo = 0, hi = 31, lo2 = 0, hi2 = 31;
#pragma unroll
        for (int it = 0; it < 5; it++) {
          const int mid = (lo + hi + 1) >> 1, mid2 = (lo2 + hi2 + 1) >> 1;
          if (s_excl[wib][mid] <= ea) lo = mid; else hi = mid - 1;
          if (s_excl[wib][mid2] <= eb) lo2 = mid2; else hi2 = mid2 - 1;
        }
        la = lo;
        lb = lo2;
      }
      const int32_t va = ea < total ? __ldg(t_col + s_rs[wib][la] + (ea - s_excl[wib][la])) : -1;
      const int32_t vb = eb < total ? __ldg(t_col + s_rs[wib][lb] + (eb - s_excl[wib][lb])) : -1;
      const u64 xa = va >= 0 ? __ldg(fin + va) : 0ull;
      const u64 xb = vb >= 0 ? __ldg(fin + vb) : 0ull;
      if (xa) atomicOr(&s_acc[wib][la], xa);
      if (xb) atomicOr(&s_acc[wib][lb], xb);
    }
    __syncwarp();
    if (sdeg > 0) got = s_acc[wib][lane];
    __syncwarp();
    const u64 nw = active ? (got & ~vis) : 0ull;
    const bool still = active && ((vis | nw) != full);
    int odeg = 0, ors = 0;
    if (nw) {
      visit[u] = vis | nw;
      fout[u] = nw;
      record_level(slices, n, u, nw, L);
      ors = row_ptr[u];
      odeg = row_ptr[u + 1] - ors;
      acc.add((u64)odeg, (u64)deg, nw, !still);
    }
    qu.push(still, u);
    emit_routed(nw != 0ull, u, odeg, ors, qa, seg_out, al_pack);
  }
  qa.flush();
  qu.flush();
  acc.flush(ctl, L % 3);
}

// Push, phase 1: the active vertices' rows (short rows warp-cooperatively,
// long rows as segments) are dealt to warps; bits new to a target are
// atomicOr-ed into `next` unless `next` already holds them.  In list mode
// the first toucher (old word 0) queues the target for phase 2; in dense
// mode (large frontiers) the atomic result is not needed and phase 2 sweeps
// all vertices instead.
__global__ void __launch_bounds__(kBlock) bs_push_scatter(const int32_t* __restrict__ row_ptr,
                                                          const int32_t* __restrict__ col, BsCtl* __restrict__ ctl,
                                                          const u64* __restrict__ visit, u64* __restrict__ fr,
                                                          u64* __restrict__ nxt, u64* __restrict__ slices,
                                                          int32_t* __restrict__ aq, const Seg* __restrict__ segs,
                                                          size_t segcap, int32_t* __restrict__ tq, int32_t n) {
  __shared__ int s_excl[kBlock / 32][32];
  __shared__ int s_rs[kBlock / 32][32];
  __shared__ int s_v[kBlock / 32][32];
  __shared__ int32_t s_q[kBlock / 32][kWarpQueue];
  if (ctl->done || ctl->mode != kModePush) return;
  const int L = ctl->level;
  const u64* __restrict__ fin = fr + (size_t)((L - 1) % 3) * n;
  const int32_t* aq_in = aq + (size_t)((L - 1) % 3) * n;
  const Seg* seg_in = segs + (size_t)((L - 1) % 3) * segcap;
  const int qn = ctl->aq_size[(L - 1) % 3];
  const int ln = seg_count(ctl->alpack[(L - 1) % 3]);
  const bool dense = ctl->dense != 0;
  clear_listed(fr + (size_t)((L + 1) % 3) * n, aq + (size_t)((L + 1) % 3) * n, ctl->aq_size[(L + 1) % 3],
               segs + (size_t)((L + 1) % 3) * segcap, seg_count(ctl->alpack[(L + 1) % 3]));
  clear_next_slice(slices, n, L, ctl->nbits);
  const int wib = threadIdx.x >> 5;
  WarpQueue wq(s_q[wib], tq, &ctl->tq_size);
  auto op = [&](int32_t v, int k, bool valid) {
    bool first = false;
    int32_t u = -1;
    if (valid) {
      u = __ldg(col + k);
      u64 bits = __ldg(fin + v) & ~__ldcg(visit + u);
      if (bits) bits &= ~__ldcg(nxt + u);
      if (bits) {
        if (dense)
          atomicOr(nxt + u, bits);
        else
          first = atomicOr(nxt + u, bits) == 0ull;
      }
    }
    if (!dense) wq.push(first, u);
  };
  seg_expand(row_ptr, seg_in, ln, op);
  warp_expand(row_ptr, aq_in, qn, s_excl[wib], s_rs[wib], s_v[wib], op);
  wq.flush();
}

// Push, phase 2: fold `next` into visited / frontier / level slices, over
// the touched list (list mode) or over every vertex (dense mode).
__global__ void __launch_bounds__(kBlock) bs_push_update(const int32_t* __restrict__ row_ptr,
                                                         const int32_t* __restrict__ t_row_ptr,
                                                         BsCtl* __restrict__ ctl, u64* __restrict__ visit,
                                                         u64* __restrict__ fr, u64* __restrict__ nxt,
                                                         u64* __restrict__ slices, int32_t* __restrict__ aq,
                                                         Seg* __restrict__ segs, size_t segcap,
                                                         const int32_t* __restrict__ tq, int32_t n) {
  __shared__ int32_t s_q[kBlock / 32][kWarpQueue];
  if (ctl->done || ctl->mode != kModePush) return;
  const int L = ctl->level;
  u64* __restrict__ fout = fr + (size_t)(L % 3) * n;
  int32_t* aq_out = aq + (size_t)(L % 3) * n;
  Seg* seg_out = segs + (size_t)(L % 3) * segcap;
  const u64 full = ctl->full;
  const bool dense = ctl->dense != 0;
  WarpQueue wq(s_q[threadIdx.x >> 5], aq_out, &ctl->aq_size[L % 3]);
  const int tn = dense ? n : ctl->tq_size;
  LevelAcc acc;
  const int total = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < tn; base += total) {
    const int i = base + threadIdx.x;
    u64 nw = 0;
    int32_t u = -1;
    int odeg = 0, ors = 0;
    if (i < tn) {
      u = dense ? i : tq[i];
      const u64 x = nxt[u];
      if (x) {
        nxt[u] = 0ull;
        const u64 vis = visit[u];
        nw = x & ~vis;
        if (nw) {
          visit[u] = vis | nw;
          fout[u] = nw;
          record_level(slices, n, u, nw, L);
          ors = row_ptr[u];
          odeg = row_ptr[u + 1] - ors;
          acc.add((u64)odeg, (u64)(t_row_ptr[u + 1] - t_row_ptr[u]), nw, (vis | nw) == full);
        }
      }
    }
    emit_routed(nw != 0ull, u, odeg, ors, wq, seg_out, &ctl->alpack[L % 3]);
  }
  wq.flush();
  acc.flush(ctl, L % 3);
}

// Expands the level slices of one batch into its distance rows: thread per
// vertex, one store per source, consecutive vertices per warp (full lines).
// NB is the number of level bits in use (template for the common <= 8).
template <int NB>
__device__ __forceinline__ void emit_vertex(int32_t* __restrict__ dist, int32_t n, int nb_src, size_t u, u64 vis,
                                            const u64* __restrict__ slices, int nbits) {
  u64 w[NB > 0 ? NB : 1];
#pragma unroll
  for (int k = 0; k < NB; k++) w[k] = slices[(size_t)k * n + u];
  for (int s = 0; s < nb_src; s++) {
    int32_t v = -1;
    if ((vis >> s) & 1ull) {
      v = 0;
#pragma unroll
      for (int k = 0; k < NB; k++) v |= (int32_t)((w[k] >> s) & 1ull) << k;
      for (int k = NB; k < nbits; k++) v |= (int32_t)((slices[(size_t)k * n + u] >> s) & 1ull) << k;
    }
    dist[(size_t)s * n + u] = v;
  }
}

__global__ void __launch_bounds__(kBlock) bs_emit_dist(const BsCtl* __restrict__ ctl, const u64* __restrict__ visit,
                                                       const u64* __restrict__ slices, int32_t n) {
  const int batch = ctl->batch;
  const int nb = min(64, ctl->nsrc - batch * 64);
  const int nbits = 32 - __clz(max(ctl->level, 1));
  int32_t* dist = ctl->dist_base + (size_t)batch * 64 * n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < (size_t)n; u += stride) {
    const u64 vis = visit[u];
    switch (nbits) {
      case 1: emit_vertex<1>(dist, n, nb, u, vis, slices, nbits); break;
      case 2: emit_vertex<2>(dist, n, nb, u, vis, slices, nbits); break;
      case 3: emit_vertex<3>(dist, n, nb, u, vis, slices, nbits); break;
      case 4: emit_vertex<4>(dist, n, nb, u, vis, slices, nbits); break;
      case 5: emit_vertex<5>(dist, n, nb, u, vis, slices, nbits); break;
      case 6: emit_vertex<6>(dist, n, nb, u, vis, slices, nbits); break;
      case 7: emit_vertex<7>(dist, n, nb, u, vis, slices, nbits); break;
      default: emit_vertex<8>(dist, n, nb, u, vis, slices, nbits); break;
    }
  }
}

__global__ void bs_decide(BsCtl* __restrict__ ctl, int32_t n, cudaGraphConditionalHandle loop, int in_graph) {
  if (threadIdx.x != 0) return;
  if (ctl->done) {
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  const int L = ctl->level;
  if (ctl->mode == kModePush) {
    ctl->n_push++;
  } else {
    ctl->n_pull++;
    ctl->ul_cur = ctl->ul_cur < 0 ? 0 : ctl->ul_cur ^ 1;
    ctl->ul_size[ctl->ul_cur ^ 1] = 0;
  }
  ctl->mu -= ctl->mu_dec;
  ctl->mu_dec = 0;
  ctl->tq_size = 0;
  ctl->work = 0;
  ctl->hwork = 0;
  const int nf = ctl->aq_size[L % 3] + long_vertices(ctl->alpack[L % 3]);
  if (nf == 0 || L >= n) {
    ctl->done = 1;
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  // Level L+1 writes list (L+1)%3, whose stale frontier words level L cleared.
  ctl->aq_size[(L + 1) % 3] = 0;
  ctl->alpack[(L + 1) % 3] = 0;
  ctl->mf[(L + 1) % 3] = 0;
  int mode;
  if (ctl->policy == DAWN_VARIANT_PUSH)
    mode = kModePush;
  else
    mode = (long long)ctl->mf[L % 3] * ctl->push_ratio < ctl->mu ? kModePush : kModePull;
  // A push whose frontier edges reach n/16 touches enough vertices that a
  // dense update sweep beats queueing every first touch.
  ctl->dense = (long long)ctl->mf[L % 3] * 16 >= (long long)n;
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
  const int pin = (c->level - 1) % 3;
  out->level = c->level;
  out->mode = c->mode;
  out->done = c->done;
  out->frontier = c->aq_size[pin] + (int64_t)(c->alpack[pin] >> 32);
  out->frontier_edges = (int64_t)c->mf[pin];
  out->unvisited_edges = c->mu;
}

// Static pull lists.  Light rows (0 < in-degree < kPullHeavy) are swept in
// id order, 32 per warp task; heavy rows are cut into kPullSeg-entry
// segments, one warp task each, so a hub row that cannot stop early is
// spread over many warps instead of holding one warp for the whole level.
__global__ void flag_rows(const int32_t* __restrict__ t_row_ptr, int32_t n, int heavy, int64_t* __restrict__ flags,
                          int64_t* __restrict__ segs) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride) {
    const int d = t_row_ptr[i + 1] - t_row_ptr[i];
    const bool h = d >= kPullHeavy;
    flags[i] = heavy ? h : (d > 0 && !h);
    if (segs) segs[i] = h ? (d + kPullSeg - 1) / kPullSeg : 0;
  }
}

__global__ void scatter_flagged(const int64_t* __restrict__ flags, const int64_t* __restrict__ pos, int32_t n,
                                int32_t* __restrict__ out, const int64_t* __restrict__ segpos,
                                int32_t* __restrict__ segoff) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride)
    if (flags[i]) {
      out[pos[i]] = (int32_t)i;
      if (segoff) segoff[pos[i]] = (int32_t)segpos[i];
    }
}

dawn_status build_static_list(dawn_graph* g) {
  if (g->ul_static.p) return DAWN_OK;
  const int32_t n = g->n;
  const size_t n1 = (size_t)n + 1;
  int64_t* tmp = nullptr;
  DAWN_CUDA(cudaMallocAsync(&tmp, sizeof(int64_t) * 4 * n1, g->stream));
  int64_t *flags = tmp, *pos = tmp + n1, *segs = tmp + 2 * n1, *segpos = tmp + 3 * n1;
  int64_t cnt[2] = {0, 0}, nseg = 0;
  DAWN_CHECK(ensure(g->ul_static, sizeof(int32_t) * (size_t)n, g->stream));
  DAWN_CHECK(ensure(g->hv_static, sizeof(int32_t) * (size_t)n, g->stream));
  DAWN_CHECK(ensure(g->hv_segoff, sizeof(int32_t) * n1, g->stream));
  for (int heavy = 0; heavy < 2; heavy++) {
    flag_rows<<<g->geo.sms * 4, kBlock, 0, g->stream>>>(g->t_row_ptr, n, heavy, flags, heavy ? segs : nullptr);
    DAWN_CUDA(cudaGetLastError());
    DAWN_CUDA(cudaMemsetAsync(flags + n, 0, sizeof(int64_t), g->stream));
    DAWN_CHECK(exclusive_scan_i64(flags, pos, (int64_t)n1, g->stream));
    if (heavy) {
      DAWN_CUDA(cudaMemsetAsync(segs + n, 0, sizeof(int64_t), g->stream));
      DAWN_CHECK(exclusive_scan_i64(segs, segpos, (int64_t)n1, g->stream));
    }
    scatter_flagged<<<g->geo.sms * 4, kBlock, 0, g->stream>>>(
        flags, pos, n, heavy ? g->hv_static.as<int32_t>() : g->ul_static.as<int32_t>(), heavy ? segpos : nullptr,
        heavy ? g->hv_segoff.as<int32_t>() : nullptr);
    DAWN_CUDA(cudaGetLastError());
    DAWN_CUDA(cudaMemcpyAsync(&cnt[heavy], pos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, g->stream));
    if (heavy) DAWN_CUDA(cudaMemcpyAsync(&nseg, segpos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, g->stream));
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
  }
  // closing offset of the heavy segment prefix
  const int32_t total = (int32_t)nseg;
  DAWN_CUDA(cudaMemcpyAsync(g->hv_segoff.as<int32_t>() + cnt[1], &total, sizeof(int32_t), cudaMemcpyHostToDevice,
                            g->stream));
  DAWN_CHECK(ensure(g->hv_acc, 16 * (size_t)(cnt[1] > 0 ? cnt[1] : 1), g->stream));
  DAWN_CUDA(cudaMemsetAsync(g->hv_acc.p, 0, 16 * (size_t)(cnt[1] > 0 ? cnt[1] : 1), g->stream));
  DAWN_CUDA(cudaFreeAsync(tmp, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  g->ul_static_size = (int32_t)cnt[0];
  g->hv_count = (int32_t)cnt[1];
  g->hv_segs = (int32_t)nseg;
  return DAWN_OK;
}

}  // namespace

dawn_status bfs_bitset(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_dist) {
  const int32_t n = g->n;
  const size_t nn = (size_t)n;
  DAWN_CHECK(build_static_list(g));
  // words: visit | fr[3] | nxt | level slices[nbits] ; lists: aq[3] | tq | ul[2] ; segments[3]
  const int nbits = 32 - __builtin_clz((unsigned)n);  // levels never exceed n
  DAWN_CHECK(ensure(g->bs_words, sizeof(u64) * (5 + (size_t)nbits) * nn, g->stream));
  DAWN_CHECK(ensure(g->bs_queues, sizeof(int32_t) * 6 * nn, g->stream));
  const size_t segcap = seg_capacity(n, g->m);
  DAWN_CHECK(ensure(g->bs_segs, sizeof(Seg) * 3 * segcap, g->stream));
  DAWN_CHECK(ensure(g->bs_ctl, sizeof(BsCtl), g->stream));
  DAWN_CHECK(ensure(g->bs_sources, sizeof(int32_t) * (size_t)nsrc, g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->bs_sources.p, sources, sizeof(int32_t) * nsrc, cudaMemcpyHostToDevice,
                            g->stream));
  BsCtl c = {};
  c.nsrc = nsrc;
  c.policy = DAWN_VARIANT_BITSET;
  c.push_ratio = g->bs_push_ratio;
  c.nbits = nbits;
  c.dist_base = d_dist;
  c.sources = g->bs_sources.as<int32_t>();
  DAWN_CUDA(cudaMemcpyAsync(g->bs_ctl.p, &c, sizeof(BsCtl), cudaMemcpyHostToDevice, g->stream));

  struct {
    BsCtl* ctl;
    const int32_t *row_ptr, *col, *t_row_ptr, *t_col, *ul_static;
    u64 *words, *visit, *fr, *fr0, *nxt, *slices;
    int32_t *aq, *aq0, *tq, *ul;
    Seg* segs;
    size_t segcap;
    int32_t ul_static_size, hv_count, hv_segs;
    const int32_t *hv_static, *hv_segoff;
    u64* hv_acc;
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
  a.ul_static = g->ul_static.as<int32_t>();
  a.ul_static_size = g->ul_static_size;
  a.hv_static = g->hv_static.as<int32_t>();
  a.hv_segoff = g->hv_segoff.as<int32_t>();
  a.hv_acc = g->hv_acc.as<u64>();
  a.hv_count = g->hv_count;
  a.hv_segs = g->hv_segs;
  a.words = g->bs_words.as<u64>();
  a.visit = a.words;
  a.fr = a.words + nn;
  a.fr0 = a.fr;
  a.nxt = a.words + 4 * nn;
  a.slices = a.words + 5 * nn;
  a.aq = g->bs_queues.as<int32_t>();
  a.aq0 = a.aq;
  a.tq = a.aq + 3 * nn;
  a.ul = a.aq + 4 * nn;
  a.segs = g->bs_segs.as<Seg>();
  a.segcap = segcap;
  a.nwords = (5 + (size_t)(nbits < kSlicesCleared ? nbits : kSlicesCleared)) * nn;
  a.n = n;
  a.m = g->m;
  a.handle = 0;
  a.in_graph = 0;
  void* clear_args[] = {&a.words, &a.nwords};
  void* init_args[] = {&a.ctl, &a.row_ptr, &a.t_row_ptr, &a.visit, &a.fr0, &a.aq0, &a.segs, &a.n, &a.m};
  void* pull_args[] = {&a.row_ptr, &a.t_row_ptr, &a.t_col, &a.ctl, &a.visit, &a.fr, &a.slices, &a.aq, &a.segs,
                       &a.segcap, &a.ul_static, &a.ul_static_size, &a.ul, &a.hv_static, &a.hv_segoff,
                       &a.hv_acc, &a.hv_count, &a.hv_segs, &a.n};
  void* scatter_args[] = {&a.row_ptr, &a.col, &a.ctl, &a.visit, &a.fr, &a.nxt, &a.slices, &a.aq, &a.segs,
                          &a.segcap, &a.tq, &a.n};
  void* update_args[] = {&a.row_ptr, &a.t_row_ptr, &a.ctl, &a.visit, &a.fr, &a.nxt, &a.slices, &a.aq, &a.segs,
                         &a.segcap, &a.tq, &a.n};
  void* emit_args[] = {&a.ctl, &a.visit, &a.slices, &a.n};
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
  fam.npost = 2;
  fam.post[0] = {(const void*)bs_emit_dist, emit_args, dim3(sms * 8), dim3(kBlock), "bs_emit_dist"};
  fam.post[1] = {(const void*)bs_next, next_args, dim3(1), dim3(32), "bs_next"};
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
