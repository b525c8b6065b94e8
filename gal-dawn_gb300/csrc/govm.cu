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
//   * stretches of levels with small frontiers run inside one launch of a
//     thread-block cluster (sssp_small), as the boolean expand's do;
//   * levels whose frontier out-edges exceed m run as a pull instead: every vertex with in-edges takes the minimum of d[u] + w over
//     its in-edges from last level's frontier (a bitmap test per in-edge,
//     the gathers only for frontier tails), so the dense levels need no
//     atomics on light rows; rows of at least 2 x pull_seg in-edges are cut
//     into warp tasks combined with atomicMin.
// Any relaxation order reaches the same fixed point (the minimum over paths
// of the path sums, which rounding leaves monotone), so push, pull and
// their mix give the distances of the reference CPU path.
#include <cooperative_groups.h>
#include <climits>

#include "cluster_levels.cuh"
#include "dawn_device.cuh"
#include "selector.cuh"

namespace dawn {
namespace {

__device__ __forceinline__ int32_t relax_sum(int32_t dv, int k, const int32_t* __restrict__ wi,
                                             const float* __restrict__ wf, bool is_float) {
  if (is_float) return __float_as_int(__fadd_rn(__int_as_float(dv), __ldg(wf + k)));
  return dv + __ldg(wi + k);
}

// Pull when a level's frontier out-edges exceed m, a full in-edge scan.  On
// RMAT scale 22 the pull was not faster than the push at any level (1.05 vs
// 1.08 ms at the 126M-edge level, 0.84 vs 0.43 ms at the 58M-edge one), so
// it is kept for frontiers heavier than the graph.
constexpr long long kPullRatio = 1;

// Frontier bitmaps rotate over three slots: level L reads slot (L-1)%3 (the
// vertices level L-1 improved), writes slot L%3 and clears slot (L+1)%3,
// which no kernel of level L reads or writes.
__device__ __forceinline__ uint32_t* slot_of(uint32_t* bm, int i, int32_t nwords) {
  return bm + (size_t)(i % 3) * nwords;
}

__device__ __forceinline__ void clear_slot(uint32_t* __restrict__ w, int32_t nwords) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)nwords; i += stride) w[i] = 0;
}

__global__ void __launch_bounds__(kBlock) sssp_clear(SsCtl* __restrict__ ctl, uint32_t* __restrict__ inq,
                                                     int32_t n, int32_t nwords, int32_t inf) {
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride) dist[i] = inf;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)3 * nwords; i += stride) inq[i] = 0;
}

// One CTA: resolve the source row (last CSR entry of a repeated neighbour
// wins), seed the first frontier, then set the source to 0.
__global__ void __launch_bounds__(kBlock) sssp_init(SsCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                                                    const int32_t* __restrict__ col, const int32_t* __restrict__ wi,
                                                    const float* __restrict__ wf, int is_float,
                                                    unsigned long long* __restrict__ last, int32_t* __restrict__ q,
                                                    Seg* __restrict__ segs, uint32_t* __restrict__ inq, int32_t n) {
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
    ctl->mf[0] = 0;
    ctl->mf[1] = 0;
    ctl->work = 0;
    ctl->hwork = 0;
    ctl->mode = ctl->force - 1 == kVarPull ? kModePull : kModePush;
  }
  for (int k = rs + threadIdx.x; k < re; k += blockDim.x) last[col[k]] = 0;
  __syncthreads();
  for (int k = rs + threadIdx.x; k < re; k += blockDim.x) atomicMax(last + col[k], (unsigned long long)(k + 1));
  __syncthreads();
  for (int k = rs + threadIdx.x; k < re; k += blockDim.x) {
    const int32_t u = col[k];
    if (last[u] == (unsigned long long)(k + 1)) {
      dist[u] = is_float ? __float_as_int(__ldg(wf + k)) : __ldg(wi + k);
      // winners are unique; the bit marks u in the level-0 frontier slot
      atomicOr(inq + (u >> 5), 1u << (u & 31));
      const int urs = row_ptr[u], udeg = row_ptr[u + 1] - urs;
      atomicAdd(&ctl->mf[0], (unsigned long long)udeg);
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

__device__ __forceinline__ void push_level(int* s_excl, int* s_rs, int* s_v, int32_t* s_q,
                                           const int32_t* __restrict__ row_ptr,
                                                     const int32_t* __restrict__ col, const int32_t* __restrict__ wi,
                                                     const float* __restrict__ wf, int is_float,
                                                     SsCtl* __restrict__ ctl, int32_t* __restrict__ q,
                                                     Seg* __restrict__ segs, size_t segcap,
                                                     uint32_t* __restrict__ inq, int32_t n, int32_t nwords) {
  const int L = ctl->level;
  const int pin = (L - 1) & 1, pout = L & 1;
  const int32_t* qin = q + (size_t)pin * n;
  const Seg* sin = segs + (size_t)pin * segcap;
  int32_t* qout = q + (size_t)pout * n;
  Seg* sout = segs + (size_t)pout * segcap;
  unsigned long long* lpack = &ctl->lpack[pout];
  const int ln = seg_count(ctl->lpack[pin]);
  uint32_t* inq_out = slot_of(inq, L, nwords);
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  int32_t* qcount = &ctl->qsize[pout];
  const int32_t source = ctl->source;
  const int qn = ctl->qsize[pin];
  const int wib = threadIdx.x >> 5;

  clear_slot(slot_of(inq, L + 1, nwords), nwords);

  unsigned long long my_mf = 0;
  WarpQueue wq(s_q, qout, qcount);
  auto op = [&](int32_t v, int k, bool valid) {
    bool found = false;
    int32_t u = -1;
    if (valid) {
      u = __ldg(col + k);
      if (u != source) {
        const int32_t nd = relax_sum(__ldcg(dist + v), k, wi, wf, is_float != 0);
        if (nd < __ldcg(dist + u)) {
          // Improvement is judged against the distance just read, and the
          // minimum is a reduction without a return value (no round trip):
          // a target another warp lowered further in the meantime is only
          // queued once more, and its next expansion relaxes nothing new.
          // The target was just lowered, so its bit is rarely set yet:
          // claim it with the OR alone, without a look first.
          atomicMin(dist + u, nd);
          const uint32_t bit = 1u << (u & 31);
          found = !(atomicOr(inq_out + (u >> 5), bit) & bit);
        }
      }
    }
    int deg = 0, rs = 0;
    if (found) {
      rs = row_ptr[u];
      deg = row_ptr[u + 1] - rs;
      my_mf += (unsigned long long)deg;
    }
    emit_routed(found, u, deg, rs, wq, sout, lpack);
  };
  seg_expand(row_ptr, sin, ln, op);
  warp_expand(row_ptr, qin, qn, s_excl, s_rs, s_v, op);
  wq.flush();
  my_mf = warp_sum(my_mf);
  if (lane_id() == 0 && my_mf) atomicAdd(&ctl->mf[pout], my_mf);
}

// Pull level: every vertex with in-edges takes the minimum of d[u] + w over
// in-edges whose tail u is in last level's frontier.  Heavy rows (>= 2 x
// pull_seg in-edges) come first as pull_seg-entry warp tasks, combined by
// atomicMin on the distance; light rows follow, 32 vertices per warp task,
// each owned by its warp (plain store): rows of >= 32 in-edges swept by the
// whole warp, shorter ones concatenated across the lanes and combined with
// shared-memory atomicMin.  Improved vertices form the next frontier (queue
// and bitmap slot), long rows as segments.
__device__ __forceinline__ void pull_level(int* s_excl, int* s_rs, int32_t* s_min, int32_t* s_q,
                                           const int32_t* __restrict__ row_ptr,
                                                    const int32_t* __restrict__ t_row_ptr,
                                                    const int32_t* __restrict__ t_col,
                                                    const int32_t* __restrict__ t_wi, const float* __restrict__ t_wf,
                                                    int is_float, SsCtl* __restrict__ ctl, int32_t* __restrict__ q,
                                                    Seg* __restrict__ segs, size_t segcap,
                                                    uint32_t* __restrict__ inq, const int32_t* __restrict__ ul,
                                                    int32_t ul_n, const int32_t* __restrict__ hv,
                                                    const int32_t* __restrict__ hv_segoff, int32_t hv_count,
                                                    int32_t hv_segs, int32_t pull_seg, int32_t n, int32_t nwords) {
  const int L = ctl->level;
  const int pout = L & 1;
  const uint32_t* fin = slot_of(inq, L - 1, nwords);
  uint32_t* fout = slot_of(inq, L, nwords);
  clear_slot(slot_of(inq, L + 1, nwords), nwords);
  int32_t* qout = q + (size_t)pout * n;
  Seg* sout = segs + (size_t)pout * segcap;
  unsigned long long* lpack = &ctl->lpack[pout];
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const bool fl = is_float != 0;
  unsigned long long my_mf = 0;
  WarpQueue wq(s_q, qout, &ctl->qsize[pout]);

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
    const int32_t v = __ldg(hv + lo);
    const int rbeg = t_row_ptr[v], rend = t_row_ptr[v + 1];
    const int ks = rbeg + (sidx - __ldg(hv_segoff + lo)) * pull_seg, ke = min(ks + pull_seg, rend);
    int32_t best = 0x7fffffff;
    for (int k = ks + lane; k < ke; k += 32) {
      const int32_t u = __ldg(t_col + k);
      if ((__ldcg(fin + (u >> 5)) >> (u & 31)) & 1u) best = min(best, relax_sum(__ldcg(dist + u), k, t_wi, t_wf, fl));
    }
    best = __reduce_min_sync(kFull, best);
    bool found = false;
    int deg = 0, rs = 0;
    if (lane == 0 && best < __ldcg(dist + v)) {
      const int32_t old = atomicMin(dist + v, best);
      if (best < old && claim_bit(fout, v)) {
        found = true;
        rs = row_ptr[v];
        deg = row_ptr[v + 1] - rs;
        my_mf += (unsigned long long)deg;
      }
    }
    emit_routed(found, v, deg, rs, wq, sout, lpack);
  }

  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&ctl->work, 32);
    base = __shfl_sync(kFull, base, 0);
    if (base >= ul_n) break;
    const int idx = base + lane;
    int32_t v = -1;
    int rs = 0, re = 0;
    if (idx < ul_n) {
      v = __ldg(ul + idx);
      rs = t_row_ptr[v];
      re = t_row_ptr[v + 1];
    }
    const int deg = re - rs;
    int32_t best = 0x7fffffff;
    uint32_t big = __ballot_sync(kFull, deg >= kWarpRow);
    while (big) {
      const int leader = __ffs(big) - 1;
      big &= big - 1;
      const int s = __shfl_sync(kFull, rs, leader), e = __shfl_sync(kFull, re, leader);
      int32_t b = 0x7fffffff;
      for (int k = s + lane; k < e; k += 32) {
        const int32_t u = __ldg(t_col + k);
        if ((__ldcg(fin + (u >> 5)) >> (u & 31)) & 1u) b = min(b, relax_sum(__ldcg(dist + u), k, t_wi, t_wf, fl));
      }
      b = __reduce_min_sync(kFull, b);
      if (lane == leader) best = b;
    }
    const int sdeg = deg < kWarpRow ? deg : 0;
    const int incl = warp_incl_scan(sdeg);
    const int total = __shfl_sync(kFull, incl, 31);
    s_excl[lane] = incl - sdeg;
    s_rs[lane] = rs;
    s_min[lane] = 0x7fffffff;
    __syncwarp();
    for (int e = lane; e < total; e += 32) {
      int lo = 0, hi = 31;
#pragma unroll
      for (int it = 0; it < 5; it++) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_excl[mid] <= e) lo = mid; else hi = mid - 1;
      }
      const int k = s_rs[lo] + (e - s_excl[lo]);
      const int32_t u = __ldg(t_col + k);
      if ((__ldcg(fin + (u >> 5)) >> (u & 31)) & 1u)
        atomicMin(&s_min[lo], relax_sum(__ldcg(dist + u), k, t_wi, t_wf, fl));
    }
    __syncwarp();
    if (sdeg > 0) best = s_min[lane];
    __syncwarp();
    bool found = false;
    int odeg = 0, ors = 0;
    if (v >= 0 && best < __ldcg(dist + v)) {
      dist[v] = best;  // this warp owns v's light row
      atomicOr(fout + (v >> 5), 1u << (v & 31));
      found = true;
      ors = row_ptr[v];
      odeg = row_ptr[v + 1] - ors;
      my_mf += (unsigned long long)odeg;
    }
    emit_routed(found, v, odeg, ors, wq, sout, lpack);
  }
  wq.flush();
  my_mf = warp_sum(my_mf);
  if (lane == 0 && my_mf) atomicAdd(&ctl->mf[pout], my_mf);
}

// One level: the push or the pull body, as the decide kernel chose, in one
// launch per level.
__global__ void __launch_bounds__(kBlock, 6) sssp_step(const int32_t* __restrict__ row_ptr,
                                                    const int32_t* __restrict__ col, const int32_t* __restrict__ wi,
                                                    const float* __restrict__ wf, int is_float,
                                                    SsCtl* __restrict__ ctl, int32_t* __restrict__ q,
                                                    Seg* __restrict__ segs, size_t segcap,
                                                    uint32_t* __restrict__ inq, int32_t n, int32_t nwords,
                                                    const int32_t* __restrict__ t_row_ptr,
                                                    const int32_t* __restrict__ t_col,
                                                    const int32_t* __restrict__ t_wi, const float* __restrict__ t_wf,
                                                    const int32_t* __restrict__ ul, int32_t ul_n,
                                                    const int32_t* __restrict__ hv,
                                                    const int32_t* __restrict__ hv_segoff, int32_t hv_count,
                                                    int32_t hv_segs, int32_t pull_seg) {
  __shared__ int s_excl[kBlock / 32][32];
  __shared__ int s_rs[kBlock / 32][32];
  __shared__ int32_t s_aux[kBlock / 32][32];
  __shared__ int32_t s_q[kBlock / 32][kWarpQueue];
  if (ctl->done || ctl->mode == kModeSmall) return;
  const int wib = threadIdx.x >> 5;
  if (ctl->mode == kModePush)
    push_level(s_excl[wib], s_rs[wib], s_aux[wib], s_q[wib], row_ptr, col, wi, wf, is_float, ctl, q, segs, segcap,
               inq, n, nwords);
  else
    pull_level(s_excl[wib], s_rs[wib], s_aux[wib], s_q[wib], row_ptr, t_row_ptr, t_col, t_wi, t_wf, is_float, ctl,
               q, segs, segcap, inq, ul, ul_n, hv, hv_segoff, hv_count, hv_segs, pull_seg, n, nwords);
}

// Small frontiers, weighted: one cluster runs push levels one after another
// in one launch, like bfs_small.  A level relaxes the rows of the previous
// level's slices (each row with its vertex's current distance) with
// atomicMin; a target it improves is claimed in the level's frontier bitmap
// slot (the same three rotating slots as the per-level kernels, so nothing
// needs rebuilding when they take over) and, if first, appended to the
// CTA's slice.  One cluster barrier per level; every warp reads the eight
// slices' counters after it and takes the same decision.  The loop stops
// after a level whose frontier is empty, holds a long row, outgrows a limit
// or a slice (entries past it went to the global queue at once), at level
// n - 1, or after kSmallMaxLevels levels, and that level is handed back as
// a push level: slices -> global queue and segments, and its counters.
__global__ void __cluster_dims__(kSmallCtas, 1, 1) __launch_bounds__(kSmallBlock)
    sssp_small(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
               const int32_t* __restrict__ wi, const float* __restrict__ wf, int is_float, SsCtl* ctl, int32_t* q,
               Seg* segs, size_t segcap, uint32_t* inq, int32_t n, int32_t nwords) {
  __shared__ SmallSlice s_sl[2];
  __shared__ int32_t s_cnt[2], s_nlong[2];
  __shared__ uint32_t s_mf[2];
  if (ctl->done || ctl->mode != kModeSmall) return;
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  constexpr int kWarps = kSmallBlock / 32;
  const int cwarp = rank * kWarps + wib;
  const size_t tid = (size_t)rank * kSmallBlock + threadIdx.x;
  const size_t stride = (size_t)kSmallCtas * kSmallBlock;
  int32_t* dist = ctl->dist_base + (size_t)ctl->src_idx * n;
  const int32_t source = ctl->source;
  const bool fl = is_float != 0;
  if (threadIdx.x < 2) {
    s_cnt[threadIdx.x] = 0;
    s_nlong[threadIdx.x] = 0;
    s_mf[threadIdx.x] = 0;
  }
  __syncthreads();

  int L = ctl->level;
  int pre = INT_MAX, tot = 0;  // dealing of the previous level's slices (lane r < kSmallCtas: slice r)
  int nlev = 0;
  unsigned long long mf = 0;
  for (int iter = 0;; iter++) {
    const int p = L & 1;
    uint32_t* inq_out = inq + (size_t)(L % 3) * nwords;
    {
      uint32_t* clr = inq + (size_t)((L + 1) % 3) * nwords;  // claimed two levels ago; nobody reads it now
      for (size_t i = tid; i < (size_t)nwords; i += stride) clr[i] = 0;
    }
    uint32_t my_mf = 0;
    bool my_long = false;
    auto op = [&](int k, bool valid, int32_t dv) {
      int32_t u = valid ? __ldg(col + k) : -1;
      bool found = false;
      int rs = 0, deg = 0;
      if (valid && u != source) {
        const int32_t nd = relax_sum(dv, k, wi, wf, fl);
        rs = __ldg(row_ptr + u);
        const int re = __ldg(row_ptr + u + 1);
        if (nd < atomicMin(dist + u, nd)) {
          const uint32_t bit = 1u << (u & 31);
          found = !(atomicOr(inq_out + (u >> 5), bit) & bit);
        }
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
      if (__any_sync(kFull, spill))
        emit_routed(spill, u, deg, rs, q + (size_t)p * n, &ctl->qsize[p], segs + (size_t)p * segcap, &ctl->lpack[p]);
    };
    if (iter == 0) {
      // the previous level in the global format
      const int pin = p ^ 1;
      const int32_t* qin = q + (size_t)pin * n;
      const int qn = ctl->qsize[pin], ln = seg_count(ctl->lpack[pin]);
      const Seg* sin = segs + (size_t)pin * segcap;
      seg_expand(row_ptr, sin, ln, [&](int32_t v, int k, bool valid) { op(k, valid, valid ? __ldcg(dist + v) : 0); });
      const int bs = batch_rows(qn);
      for (int b = cwarp * bs; b < qn; b += kSmallCtas * kWarps * bs) {
        const int i = b + lane;
        const bool ok = lane < bs && i < qn;
        int rs = 0, deg = 0;
        int32_t dv = 0;
        if (ok) {
          const int32_t v = qin[i];
          rs = row_ptr[v];
          deg = row_ptr[v + 1] - rs;
          dv = __ldcg(dist + v);
        }
        expand_rows(ok, rs, deg, dv, op);
      }
    } else {
      // the previous level's slices, across the cluster
      const int bs = batch_rows(tot);
      for (int b = cwarp * bs; b < tot; b += kSmallCtas * kWarps * bs) {
        const int e = lane < bs ? b + lane : INT_MAX;
        int r = 0;
#pragma unroll
        for (int step = kSmallCtas / 2; step; step >>= 1) {
          const int ex = __shfl_sync(kFull, pre, r + step);
          if (ex <= e) r += step;
        }
        const int off = e - __shfl_sync(kFull, pre, r);
        int rs = 0, deg = 0;
        int32_t dv = 0;
        if (e < tot) {
          const SmallSlice* src = cluster.map_shared_rank(&s_sl[p ^ 1], r);
          rs = src->rs[off];
          deg = src->deg[off];
          dv = __ldcg(dist + src->u[off]);
        }
        expand_rows(e < tot, rs, deg, dv, op);
      }
    }
    my_mf = __reduce_add_sync(kFull, my_mf);
    my_long = __any_sync(kFull, my_long);
    if (lane == 0) {
      if (my_mf) atomicAdd(&s_mf[p], my_mf);
      if (my_long) s_nlong[p] = 1;
    }
    cluster.sync();
    int cnt = 0, nl = 0;
    uint32_t mr = 0;
    if (lane < kSmallCtas) {
      cnt = *cluster.map_shared_rank(&s_cnt[p], lane);
      nl = *cluster.map_shared_rank(&s_nlong[p], lane);
      mr = *cluster.map_shared_rank(&s_mf[p], lane);
    }
    const int kept = cnt < kSmallCap ? cnt : kSmallCap;
    int incl = kept;
#pragma unroll
    for (int d = 1; d < kSmallCtas; d <<= 1) {
      const int t = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl += t;
    }
    const int nf = (int)__reduce_add_sync(kFull, (uint32_t)cnt);
    mf = __reduce_add_sync(kFull, mr);
    const bool longs = __any_sync(kFull, nl != 0);
    const bool over = __any_sync(kFull, cnt > kSmallCap);
    const bool stop = nf == 0 || longs || over || nf > kSmallFrontier || (long long)mf > kSmallEdges ||
                      L + 1 >= n || iter + 1 == kSmallMaxLevels;
    if (stop) break;
    pre = lane < kSmallCtas ? incl - kept : INT_MAX;
    tot = __shfl_sync(kFull, incl, kSmallCtas - 1);
    nlev++;
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
    emit_routed(ok, ok ? s_sl[p].u[i] : 0, ok ? s_sl[p].deg[i] : 0, ok ? s_sl[p].rs[i] : 0, q + (size_t)p * n,
                &ctl->qsize[p], segs + (size_t)p * segcap, &ctl->lpack[p]);
  }
  if (rank == 0 && threadIdx.x == 0) {
    ctl->mf[p] = mf;
    ctl->n_push += nlev;
    ctl->level = L;
  }
  // No CTA may exit while another still reads its counters or slices
  // through distributed shared memory.
  cluster.sync();
}

__global__ void sssp_decide(SsCtl* __restrict__ ctl, int32_t n, int can_pull, cudaGraphConditionalHandle loop,
                            int in_graph) {
  if (threadIdx.x != 0) return;
  if (ctl->done) {
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  const int L = ctl->level, pout = L & 1;
  if (ctl->mode == kModePull) ctl->n_pull++; else ctl->n_push++;  // cluster levels are push levels
  // The reference stops after n levels at most (src/algorithm/cpu/sssp.cpp:34);
  // with non-negative weights the queue empties long before.
  if ((ctl->qsize[pout] == 0 && ctl->lpack[pout] == 0) || L >= n) {
    ctl->done = 1;
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  ctl->qsize[pout ^ 1] = 0;
  ctl->lpack[pout ^ 1] = 0;
  ctl->mf[pout ^ 1] = 0;
  ctl->work = 0;
  ctl->hwork = 0;
  int mode = (long long)ctl->mf[pout] * kPullRatio > ctl->m ? kModePull : kModePush;
  if (ctl->force) mode = ctl->force - 1 == kVarPull ? kModePull : kModePush;
  if (!can_pull) mode = kModePush;
  if (mode == kModePush && ctl->small && !ctl->force && ctl->qsize[pout] <= kSmallFrontier &&
      ctl->lpack[pout] == 0 && (long long)ctl->mf[pout] <= kSmallEdges)
    mode = kModeSmall;
  ctl->mode = mode;
  ctl->level = L + 1;
}

__global__ void sssp_next(SsCtl* __restrict__ ctl) {
  if (threadIdx.x != 0) return;
  ctl->total_levels += ctl->level;
  ctl->total_push += ctl->n_push;
  ctl->total_pull += ctl->n_pull;
  ctl->src_idx += 1;
}

void probe_sssp(const void* p, LevelProbe* out) {
  const SsCtl* c = static_cast<const SsCtl*>(p);
  out->level = c->level;
  out->mode = c->mode;
  out->done = c->done;
  out->frontier = c->qsize[(c->level - 1) & 1] + (int64_t)(c->lpack[(c->level - 1) & 1] >> 32);
  out->frontier_edges = (int64_t)c->mf[(c->level - 1) & 1];
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
  // pull levels read in-edges with their weights and the in-degree lists
  if (g->static_seg != g->pull_seg && g->sssp_exec) {
    cudaGraphExecDestroy(g->sssp_exec);  // its pull launch holds the old list sizes
    g->sssp_exec = nullptr;
  }
  DAWN_CHECK(build_weighted_in_edges(g));
  DAWN_CHECK(build_static_list(g));
  DAWN_CUDA(cudaMemcpyAsync(g->ss_sources.p, sources, sizeof(int32_t) * nsrc, cudaMemcpyHostToDevice,
                            g->stream));
  const int is_float = g->wtype == DAWN_W_F32;
  SsCtl c = {};
  c.policy = DAWN_VARIANT_PUSH;
  c.force = g->force_variant == 3 ? 1 + kVarPush : g->force_variant;
  c.small = g->small_levels && cluster_fits((const void*)sssp_small, kSmallCtas, kSmallBlock) ? 1 : 0;
  c.m = g->m;
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
    const int32_t *t_row_ptr, *t_col, *t_wi, *ul, *hv, *hv_segoff;
    const float* t_wf;
    int32_t ul_n, hv_count, hv_segs, pull_seg, can_pull;
  } a;
  a.t_row_ptr = g->t_row_ptr;
  a.t_col = g->wt_col.as<int32_t>();
  a.t_wi = is_float ? nullptr : g->wt_val.as<int32_t>();
  a.t_wf = is_float ? g->wt_val.as<float>() : nullptr;
  a.ul = g->ul_static.as<int32_t>();
  a.hv = g->hv_static.as<int32_t>();
  a.hv_segoff = g->hv_segoff.as<int32_t>();
  a.ul_n = g->ul_static_size;
  a.hv_count = g->hv_count;
  a.hv_segs = g->hv_segs;
  a.pull_seg = g->pull_seg;
  a.can_pull = 1;
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
  void* init_args[] = {&a.ctl, &a.row_ptr, &a.col, &a.wi, &a.wf, &a.is_float, &a.last, &a.q, &a.segs, &a.inq, &a.n};
  void* step_args[] = {&a.row_ptr, &a.col, &a.wi, &a.wf, &a.is_float, &a.ctl, &a.q, &a.segs, &a.segcap,
                       &a.inq, &a.n, &a.nwords, &a.t_row_ptr, &a.t_col, &a.t_wi, &a.t_wf, &a.ul, &a.ul_n, &a.hv,
                       &a.hv_segoff, &a.hv_count, &a.hv_segs, &a.pull_seg};
  void* small_args[] = {&a.row_ptr, &a.col, &a.wi, &a.wf, &a.is_float, &a.ctl, &a.q, &a.segs, &a.segcap,
                        &a.inq, &a.n, &a.nwords};
  void* decide_args[] = {&a.ctl, &a.n, &a.can_pull, &a.handle, &a.in_graph};
  void* next_args[] = {&a.ctl};

  const int sms = g->geo.sms;
  SsFamily fam;
  fam.npre = 2;
  fam.pre[0] = {(const void*)sssp_clear, clear_args, dim3(sms * 4), dim3(kBlock)};
  fam.pre[1] = {(const void*)sssp_init, init_args, dim3(1), dim3(kBlock)};
  fam.nbody = 3;
  fam.body[0] = {(const void*)sssp_step, step_args,
                 dim3(persistent_blocks((const void*)sssp_step, kBlock, 0, g->blocks_per_sm)), dim3(kBlock),
                 "sssp_step"};
  fam.body[1] = {(const void*)sssp_small, small_args, dim3(kSmallCtas), dim3(kSmallBlock), "sssp_small", kModeSmall};
  fam.body[2] = {(const void*)sssp_decide, decide_args, dim3(1), dim3(32), "sssp_decide"};
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
