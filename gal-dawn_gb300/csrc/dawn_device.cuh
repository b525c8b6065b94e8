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
// shared-memory scratch.
template <class Op>
__device__ __forceinline__ void warp_expand(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ qin,
                                            int qn, int* s_excl, int* s_rs, int* s_v, Op&& op) {
  const int lane = lane_id();
  for (int base = global_warp() * 32; base < qn; base += num_warps() * 32) {
    const int idx = base + lane;
    int32_t v = -1;
    int rs = 0, re = 0;
    if (idx < qn) {
      v = qin[idx];
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

constexpr int kLongRow = 2048;  // rows this long are dealt to the whole grid
constexpr int kLongTile = 1024; // long rows staged per shared-memory tile

// Shared-memory staging of a tile of long rows for grid_expand_long.
struct LongTile {
  int v[kLongTile];
  int rs[kLongTile];
  long long off[kLongTile + 1];
};

// Deals the edges of a list of long rows over every warp of the grid: each
// CTA stages up to kLongTile rows (vertex, row start, exclusive edge offset)
// in shared memory, then warp w takes edges [32 c, 32 c + 32) of the
// concatenated rows for c = w, w + warps, ...  One lane per edge, coalesced
// within a row.  op(v, k, valid) as in warp_expand.  Every thread of the CTA
// must call this (it synchronises the CTA).
template <class Op>
__device__ __forceinline__ void grid_expand_long(const int32_t* __restrict__ row_ptr,
                                                 const int32_t* __restrict__ list, int cnt, LongTile& t,
                                                 Op&& op) {
  const int lane = lane_id();
  for (int tile = 0; tile < cnt; tile += kLongTile) {
    const int tc = min(kLongTile, cnt - tile);
    __syncthreads();
    // Block-wide exclusive scan of the row lengths (blockDim.x == kBlock).
    constexpr int kPer = kLongTile / kBlock;
    long long local[kPer];
    long long sum = 0;
#pragma unroll
    for (int j = 0; j < kPer; j++) {
      const int i = threadIdx.x * kPer + j;
      long long d = 0;
      if (i < tc) {
        const int32_t v = list[tile + i];
        const int rs = row_ptr[v];
        t.v[i] = v;
        t.rs[i] = rs;
        d = row_ptr[v + 1] - rs;
      }
      local[j] = sum;
      sum += d;
    }
    __shared__ long long s_warp[kBlock / 32];
    long long incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const long long y = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl += y;
    }
    if (lane == 31) s_warp[threadIdx.x >> 5] = incl;
    __syncthreads();
    long long before = incl - sum;
    for (int w = 0; w < (int)(threadIdx.x >> 5); w++) before += s_warp[w];
#pragma unroll
    for (int j = 0; j < kPer; j++) {
      const int i = threadIdx.x * kPer + j;
      if (i < tc) t.off[i] = before + local[j];
    }
    if (threadIdx.x == blockDim.x - 1) t.off[tc] = before + sum;
    __syncthreads();
    const long long total = t.off[tc];
    for (long long e0 = (long long)global_warp() * 32; e0 < total; e0 += (long long)num_warps() * 32) {
      const long long e = e0 + lane;
      int32_t v = -1;
      int k = 0;
      if (e < total) {
        int lo = 0, hi = tc - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (t.off[mid] <= e) lo = mid; else hi = mid - 1;
        }
        v = t.v[lo];
        k = t.rs[lo] + (int)(e - t.off[lo]);
      }
      op(v, k, e < total);
    }
  }
}

}  // namespace dawn

namespace dawn {

// Appends a discovered vertex to the short-row or the long-row list by its
// out-degree.  All 32 lanes must call it.
__device__ __forceinline__ void emit_routed(bool found, int32_t u, int deg, int32_t* __restrict__ q_short,
                                            int32_t* short_count, int32_t* __restrict__ q_long,
                                            int32_t* long_count) {
  const bool is_long = found && deg >= kLongRow;
  const bool is_short = found && !is_long;
  int p = warp_append(is_short, short_count);
  if (is_short) q_short[p] = u;
  p = warp_append(is_long, long_count);
  if (is_long) q_long[p] = u;
}

}  // namespace dawn
