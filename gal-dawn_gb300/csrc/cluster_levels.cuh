// Shared pieces of the small-frontier cluster kernels (bfs_small,
// sssp_small): one cluster of kSmallCtas CTAs runs level after level of a
// single-source traversal inside one launch, each CTA keeping the vertices
// its warps add to the next frontier in a shared-memory slice that the
// whole cluster reads at the next level through distributed shared memory.
#pragma once

#include "dawn_device.cuh"

namespace dawn {

// Small-frontier levels: one cluster of kSmallCtas CTAs runs
// push levels back to back while the frontier stays within kSmallFrontier
// vertices, kSmallEdges out-edges and kSmallCap vertices per CTA, at most
// kSmallMaxLevels levels per launch.
constexpr int kSmallCtas = 8;
constexpr int kSmallBlock = 1024;
constexpr int kSmallCap = 1536;
constexpr int kSmallFrontier = 8192;
constexpr long long kSmallEdges = 32768;
constexpr int kSmallMaxLevels = 512;

// Expands one warp batch of frontier rows: lane i holds row (rs, deg) when
// valid, and a value of its row (the row vertex's distance, for instance).
// Rows of >= kWarpRow entries are swept by the whole warp, shorter ones are
// concatenated through a warp scan and dealt 32 edges at a time (the owning
// lane is found by a binary search over the lanes' exclusive offsets,
// through shuffles).  op(k, valid, value of k's row) runs on all 32 lanes.
template <class Op>
__device__ __forceinline__ void expand_rows(bool valid, int rs, int deg, int32_t val, Op&& op) {
  const int lane = lane_id();
  if (!valid) deg = 0;
  uint32_t big = __ballot_sync(kFull, deg >= kWarpRow);
  while (big) {
    const int leader = __ffs(big) - 1;
    big &= big - 1;
    const int s = __shfl_sync(kFull, rs, leader), d = __shfl_sync(kFull, deg, leader);
    const int32_t lv = __shfl_sync(kFull, val, leader);
    for (int k0 = 0; k0 < d; k0 += 32) op(s + k0 + lane, k0 + lane < d, lv);
  }
  const int sdeg = deg < kWarpRow ? deg : 0;
  const int incl = warp_incl_scan(sdeg);
  const int excl = incl - sdeg;
  const int total = __shfl_sync(kFull, incl, 31);
  for (int e0 = 0; e0 < total; e0 += 32) {
    const int e = e0 + lane;
    int lo = 0;  // last lane whose offset is <= e
#pragma unroll
    for (int step = 16; step; step >>= 1) {
      const int ex = __shfl_sync(kFull, excl, lo + step);
      if (ex <= e) lo += step;
    }
    const int k = __shfl_sync(kFull, rs, lo) + (e - __shfl_sync(kFull, excl, lo));
    op(k, e < total, __shfl_sync(kFull, val, lo));
  }
}

// Rows per warp batch in bfs_small: the level's rows spread over all the
// cluster's warps (fewer than 32 per warp when the frontier is small), so
// that each warp's chain of dependent loads is short.
__device__ __forceinline__ int batch_rows(int rows) {
  constexpr int kLanes = kSmallCtas * kSmallBlock;
  if (rows >= kLanes) return 32;
  const int bs = (rows + kLanes / 32 - 1) / (kLanes / 32);
  return bs < 1 ? 1 : bs;
}

// One CTA's share of one level's frontier in bfs_small: discovered vertices
// with their row start and degree.
struct SmallSlice {
  int32_t u[kSmallCap];
  int32_t rs[kSmallCap];
  int32_t deg[kSmallCap];
};

}  // namespace dawn
