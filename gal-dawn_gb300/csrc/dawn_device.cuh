// Device-side helpers shared by the frontier kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dawn_internal.cuh"

namespace dawn {

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ int warp_incl_scan(int x) {
  const int lane = lane_id();
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  return x;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long x) {
#pragma unroll
  for (int d = 16; d; d >>= 1) x += __shfl_xor_sync(kFull, x, d);
  return x;
}

__device__ __forceinline__ unsigned long long warp_or(unsigned long long x) {
#pragma unroll
  for (int d = 16; d; d >>= 1) x |= __shfl_xor_sync(kFull, x, d);
  return x;
}

// Warp-aggregated append: one atomicAdd per warp.  Must be reached by all
// 32 lanes.  Returns the slot of a lane with pred set, -1 otherwise.
__device__ __forceinline__ int warp_append(bool pred, int32_t* count) {
  const uint32_t m = __ballot_sync(kFull, pred);
  if (m == 0) return -1;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane_id() == leader) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(kFull, base, leader);
  return pred ? base + __popc(m & lanemask_lt()) : -1;
}

// Claims vertex u in a visited bitmap; true for exactly one caller.
__device__ __forceinline__ bool claim_bit(uint32_t* bm, int32_t u) {
  const uint32_t bit = 1u << (u & 31);
  if (__ldcg(bm + (u >> 5)) & bit) return false;
  return !(atomicOr(bm + (u >> 5), bit) & bit);
}

__device__ __forceinline__ bool test_bit(const uint32_t* bm, int32_t u) {
  return (__ldg(bm + (u >> 5)) >> (u & 31)) & 1u;
}

__device__ __forceinline__ int global_warp() {
  return (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}
__device__ __forceinline__ int num_warps() {
  return (int)((gridDim.x * blockDim.x) >> 5);
}

}  // namespace dawn

namespace dawn {

constexpr int kWarpRow = 32;  // rows with at least this many entries use the whole warp

// Deals the out-edges of a vertex queue to the lanes of every warp of the
// grid.  Rows of >= kWarpRow entries are swept by the whole warp with
// coalesced col loads; shorter rows are concatenated through a warp scan and
// dealt 32 edges at a time.  op(v, k, valid) runs on all 32 lanes in
// lockstep (it may use warp collectives); when valid, k is a CSR position in
// the row of vertex v.  s_excl / s_rs / s_v are this warp's 32-entry
// shared-memory scratch.  kCoherent reads the queue through L2 (a queue
// written earlier in the same launch must not come from the read-only path).
// A warp task is 32 queue entries, or fewer when the queue cannot give every
// warp 32: the smallest power of two that still covers the queue in one
// round of the grid, so a short queue is spread over all warps instead of
// being walked by a few (64 rows of 16 edges: 64 warps, not two).
template <bool kCoherent = false, class Op>
__device__ __forceinline__ void warp_expand(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ qin,
                                            int qn, int* s_excl, int* s_rs, int* s_v, Op&& op) {
  const int lane = lane_id();
  const int nw = num_warps();
  int per = 32;
  while (per > 1 && (long long)(per >> 1) * nw >= qn) per >>= 1;
  for (int base = global_warp() * per; base < qn; base += nw * per) {
    const int idx = base + lane;
    int32_t v = -1;
    int rs = 0, re = 0;
    if (lane < per && idx < qn) {
      v = kCoherent ? __ldcg(qin + idx) : qin[idx];
      rs = row_ptr[v];
      re = row_ptr[v + 1];
    }
    const int deg = re - rs;
    uint32_t big = __ballot_sync(kFull, deg >= kWarpRow);
    while (big) {
      const int leader = __ffs(big) - 1;
      big &= big - 1;
      const int32_t lv = __shfl_sync(kFull, v, leader);
      const int s = __shfl_sync(kFull, rs, leader), e = __shfl_sync(kFull, re, leader);
      for (int k0 = s; k0 < e; k0 += 32) op(lv, k0 + lane, k0 + lane < e);
    }
    const int sdeg = deg < kWarpRow ? deg : 0;
    const int incl = warp_incl_scan(sdeg);
    const int total = __shfl_sync(kFull, incl, 31);
    s_excl[lane] = incl - sdeg;
    s_rs[lane] = rs;
    s_v[lane] = v;
    __syncwarp();
    for (int e0 = 0; e0 < total; e0 += 32) {
      const int e = e0 + lane;
      int32_t ov = -1;
      int k = 0;
      if (e < total) {
        int lo = 0, hi = 31;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_excl[mid] <= e) lo = mid; else hi = mid - 1;
        }
        ov = s_v[lo];
        k = s_rs[lo] + (e - s_excl[lo]);
      }
      op(ov, k, e < total);
    }
    __syncwarp();
  }
}

}  // namespace dawn

namespace dawn {

// Rows of at least kLongRow entries leave the vertex queues: when such a
// vertex is discovered it is entered as ceil(deg / kSeg) segments of at most
// kSeg consecutive CSR positions, and the next expansion deals segments to
// warps, so a hub's row is spread over many warps instead of one.
constexpr int kSeg = 128;
constexpr int kLongRow = kSeg;

struct Seg {
  int32_t v;   // vertex
  int32_t k0;  // first CSR position of the segment
};

// Capacity of one level's segment list.  A vertex enters a level's list at
// most once and a row of d >= kLongRow entries adds ceil(d / kSeg) <=
// d / kSeg + 1 <= 2 d / kSeg segments, so 2 m / kSeg bounds the list.
__host__ __device__ inline size_t seg_capacity(int32_t n, long long m) {
  (void)n;
  return 2 * (size_t)(m / kSeg) + 64;
}

// Writes the segments of every lane in lm (nseg segments of lane l's row
// from CSR position rs, at list index first).  A lane writes up to
// kOwnSegs of its own; the whole warp writes a longer row's, so a hub's
// thousands of segments go out 32 per store instead of from one lane.
constexpr int kOwnSegs = 16;
__device__ __forceinline__ void write_segments(uint32_t lm, int32_t u, int rs, int nseg, uint32_t first,
                                               Seg* __restrict__ segs) {
  const int lane = lane_id();
  if (nseg <= kOwnSegs)
    for (int j = 0; j < nseg; j++) segs[first + j] = Seg{u, rs + j * kSeg};
  lm &= __ballot_sync(kFull, nseg > kOwnSegs);
  while (lm) {
    const int l = __ffs(lm) - 1;
    lm &= lm - 1;
    const int32_t lu = __shfl_sync(kFull, u, l);
    const int lrs = __shfl_sync(kFull, rs, l), ln = __shfl_sync(kFull, nseg, l);
    const uint32_t lf = __shfl_sync(kFull, first, l);
    for (int j = lane; j < ln; j += 32) segs[lf + j] = Seg{lu, lrs + j * kSeg};
  }
}

// Queues a discovered vertex: short rows as a vertex, long rows as segments.
// lpack packs (long vertices << 32 | segments) so one atomicAdd per warp
// reserves the warp's segment slots.  All 32 lanes must call it.
__device__ __forceinline__ void emit_routed(bool found, int32_t u, int deg, int rs, int32_t* __restrict__ q_short,
                                            int32_t* short_count, Seg* __restrict__ segs,
                                            unsigned long long* lpack) {
  const bool is_long = found && deg >= kLongRow;
  const bool is_short = found && !is_long;
  const int p = warp_append(is_short, short_count);
  if (is_short) q_short[p] = u;
  const uint32_t lm = __ballot_sync(kFull, is_long);
  if (lm) {
    const int nseg = is_long ? (deg + kSeg - 1) / kSeg : 0;
    const int incl = warp_incl_scan(nseg);
    const int tot = __shfl_sync(kFull, incl, 31);
    unsigned long long base = 0;
    if (lane_id() == 0) base = atomicAdd(lpack, ((unsigned long long)__popc(lm) << 32) | (unsigned)tot);
    const uint32_t b = (uint32_t)__shfl_sync(kFull, base, 0);
    write_segments(lm, u, rs, nseg, b + incl - nseg, segs);
  }
}

__device__ __forceinline__ int seg_count(unsigned long long lpack) { return (int)(uint32_t)lpack; }
__device__ __forceinline__ int long_vertices(unsigned long long lpack) { return (int)(lpack >> 32); }

// Deals segments to warps (one segment per warp at a time, one lane per
// edge).  op(v, k, valid) as in warp_expand; kCoherent as there.
template <bool kCoherent = false, class Op>
__device__ __forceinline__ void seg_expand(const int32_t* __restrict__ row_ptr, const Seg* __restrict__ segs,
                                           int nsegs, Op&& op) {
  const int lane = lane_id();
  for (int i = global_warp(); i < nsegs; i += num_warps()) {
    Seg sg;
    if (kCoherent) {
      sg.v = __ldcg(&segs[i].v);
      sg.k0 = __ldcg(&segs[i].k0);
    } else {
      sg = segs[i];
    }
    const int e = min(sg.k0 + kSeg, row_ptr[sg.v + 1]);
    for (int k0 = sg.k0; k0 < e; k0 += 32) op(sg.v, k0 + lane, k0 + lane < e);
  }
}

}  // namespace dawn

namespace dawn {

// Per-warp staging of queue appends in shared memory.  Appending straight
// to a global queue costs one atomicAdd on the queue's single counter per
// warp step; with thousands of warps those same-address atomics serialise.
// Here a warp collects up to kCap entries (warp-synchronously, no atomics)
// and reserves global space once per full buffer.  All 32 lanes must make
// every call; flush() must run before the warp exits.  The unweighted
// traversals stage kWarpQueueBig entries (a quarter of the counter's
// atomics: RMAT-22 x 64 batched 1.66 -> 1.64 ms, 64 single-source
// traversals 18.0 -> 17.5 ms); the batched min-plus kernel lost 4.5% with
// the larger buffer and keeps kWarpQueue.
constexpr int kWarpQueue = 64;
constexpr int kWarpQueueBig = 256;

template <int kCap = kWarpQueue>
struct WarpQueueT {
  int32_t* buf;      // this warp's kCap shared-memory slots
  int32_t* out;      // global queue
  int32_t* count;    // global queue length
  int n = 0;         // staged entries (warp-uniform)

  __device__ __forceinline__ WarpQueueT(int32_t* sbuf, int32_t* q, int32_t* cnt) : buf(sbuf), out(q), count(cnt) {}

  __device__ __forceinline__ void flush() {
    if (n == 0) return;
    int base = 0;
    if (lane_id() == 0) base = atomicAdd(count, n);
    base = __shfl_sync(kFull, base, 0);
    __syncwarp();
    for (int i = lane_id(); i < n; i += 32) out[base + i] = buf[i];
    __syncwarp();
    n = 0;
  }

  __device__ __forceinline__ void push(bool pred, int32_t v) {
    const uint32_t m = __ballot_sync(kFull, pred);
    if (m == 0) return;
    const int c = __popc(m);
    if (n + c > kCap) flush();
    if (pred) buf[n + __popc(m & lanemask_lt())] = v;
    n += c;
  }
};

using WarpQueue = WarpQueueT<>;
using WarpQueueBig = WarpQueueT<kWarpQueueBig>;

// emit_routed with the short-row queue staged through a WarpQueueT.
template <int kCap>
__device__ __forceinline__ void emit_routed(bool found, int32_t u, int deg, int rs, WarpQueueT<kCap>& q_short,
                                            Seg* __restrict__ segs, unsigned long long* lpack) {
  const bool is_long = found && deg >= kLongRow;
  q_short.push(found && !is_long, u);
  const uint32_t lm = __ballot_sync(kFull, is_long);
  if (lm) {
    const int nseg = is_long ? (deg + kSeg - 1) / kSeg : 0;
    const int incl = warp_incl_scan(nseg);
    const int tot = __shfl_sync(kFull, incl, 31);
    unsigned long long base = 0;
    if (lane_id() == 0) base = atomicAdd(lpack, ((unsigned long long)__popc(lm) << 32) | (unsigned)tot);
    const uint32_t b = (uint32_t)__shfl_sync(kFull, base, 0);
    write_segments(lm, u, rs, nseg, b + incl - nseg, segs);
  }
}

}  // namespace dawn
