// BCDAWN betweenness on sm_103a.
//
// The reference computes it on the CPU only (src/algorithm/cpu/bc.cpp:9-191;
// include/dawn/algorithm/gpu/bc.cuh is empty), one source at a time.  Its
// dependency for a source s, with levels counted from s:
//   * a vertex c at level >= 2 has amount(c) predecessor entries: CSR
//     entries j -> c with level(j) = level(c) - 1 (duplicates count);
//   * delta(v) = sum over v's entries v -> c with level(c) = level(v) + 1 of
//     1 / amount(c) + delta(c);
//   * the betweenness of v is the sum of delta(v) over the sources.
// Here 64 sources go together:
//   1. the batched bitset traversal writes every vertex's 64 levels as one
//      row (and the vertex's lowest and highest level);
//   2. bc_amount: a warp per vertex walks its in-edges, reading one 256-byte
//      level row per edge, and stores 1 / amount per source (0 where the
//      vertex is unreached or at level 0 or 1);
//   3. bc_sweep, from the deepest level up: for level l, a warp per vertex
//      with a source at level l sums, per such source, term(c) = 1 / amount
//      (c) + delta(c) over its out-edges to level l + 1, adds the sum to its
//      own term (which now holds 1 / amount + delta), and adds the finished
//      delta of those sources to the vertex's betweenness.  Terms of level
//      l + 1 are final when level l runs, and every (vertex, source) slot is
//      written by one warp in one sweep, so no atomics are needed.
// Terms are float (the reference's bc_temp is float); the sums over
// sources are double.  The additions group as (1 / amount + delta) per
// entry rather than the reference's two separate additions, so values agree
// with it to float rounding, not bit for bit.
#include <cstring>

#include "dawn_device.cuh"

namespace dawn {
namespace {

constexpr int kLanes = 64;
constexpr int kUnroll = 4;

// 1 / amount for every (vertex, source) slot.
__global__ void __launch_bounds__(kBlock) bc_amount(const int32_t* __restrict__ t_row_ptr,
                                                    const int32_t* __restrict__ t_col,
                                                    const int32_t* __restrict__ L, float* __restrict__ T,
                                                    int32_t n) {
  const int lane = lane_id();
  for (int c = global_warp(); c < n; c += num_warps()) {
    const int32_t* Lc = L + (size_t)c * kLanes;
    const int32_t la = Lc[lane], lb = Lc[lane + 32];
    const bool wa = la >= 2, wb = lb >= 2;
    int ca = 0, cb = 0;
    if (__any_sync(kFull, wa || wb)) {
      const int k0 = t_row_ptr[c], k1 = t_row_ptr[c + 1];
      for (int kb = k0; kb < k1; kb += 32) {
        const int k = kb + lane;
        const int32_t jv = k < k1 ? __ldg(t_col + k) : -1;
        const int cnt = min(32, k1 - kb);
        for (int j0 = 0; j0 < cnt; j0 += kUnroll) {
          int32_t ra[kUnroll], rb[kUnroll];
#pragma unroll
          for (int i = 0; i < kUnroll; i++) {
            const int32_t j = __shfl_sync(kFull, jv, (j0 + i) & 31);
            const bool ok = j0 + i < cnt;
            const int32_t* Lj = L + (size_t)(ok ? j : 0) * kLanes;
            ra[i] = ok && wa ? __ldcg(Lj + lane) : -2;
            rb[i] = ok && wb ? __ldcg(Lj + lane + 32) : -2;
          }
#pragma unroll
          for (int i = 0; i < kUnroll; i++) {
            ca += ra[i] == la - 1;
            cb += rb[i] == lb - 1;
          }
        }
      }
    }
    float* Tc = T + (size_t)c * kLanes;
    Tc[lane] = wa && ca ? 1.0f / (float)ca : 0.0f;
    Tc[lane + 32] = wb && cb ? 1.0f / (float)cb : 0.0f;
  }
}

// Level l of the backward sweep (see the file comment).
__global__ void __launch_bounds__(kBlock) bc_sweep(const int32_t* __restrict__ row_ptr,
                                                   const int32_t* __restrict__ col,
                                                   const int32_t* __restrict__ L, const int32_t* __restrict__ range,
                                                   float* __restrict__ T, double* __restrict__ bc, int32_t n,
                                                   int32_t level) {
  const int lane = lane_id();
  for (int v = global_warp(); v < n; v += num_warps()) {
    if (level < range[2 * v] || level > range[2 * v + 1]) continue;  // warp-uniform
    const int32_t* Lv = L + (size_t)v * kLanes;
    const bool wa = Lv[lane] == level, wb = Lv[lane + 32] == level;
    if (!__any_sync(kFull, wa || wb)) continue;
    float sa = 0.0f, sb = 0.0f;
    const int k0 = row_ptr[v], k1 = row_ptr[v + 1];
    for (int kb = k0; kb < k1; kb += 32) {
      const int k = kb + lane;
      const int32_t cv = k < k1 ? __ldg(col + k) : -1;
      const int cnt = min(32, k1 - kb);
      for (int j0 = 0; j0 < cnt; j0 += kUnroll) {
        int32_t la[kUnroll], lb[kUnroll];
        float ta[kUnroll], tb[kUnroll];
#pragma unroll
        for (int i = 0; i < kUnroll; i++) {
          const int32_t c = __shfl_sync(kFull, cv, (j0 + i) & 31);
          const bool ok = j0 + i < cnt;
          const size_t row = (size_t)(ok ? c : 0) * kLanes;
          la[i] = ok && wa ? __ldcg(L + row + lane) : -2;
          lb[i] = ok && wb ? __ldcg(L + row + lane + 32) : -2;
          ta[i] = ok && wa ? __ldcg(T + row + lane) : 0.0f;
          tb[i] = ok && wb ? __ldcg(T + row + lane + 32) : 0.0f;
        }
#pragma unroll
        for (int i = 0; i < kUnroll; i++) {
          if (la[i] == level + 1) sa += ta[i];
          if (lb[i] == level + 1) sb += tb[i];
        }
      }
    }
    float* Tv = T + (size_t)v * kLanes;
    if (wa) Tv[lane] += sa;
    if (wb) Tv[lane + 32] += sb;
    double part = (wa ? (double)sa : 0.0) + (wb ? (double)sb : 0.0);
#pragma unroll
    for (int d = 16; d; d >>= 1) part += __shfl_xor_sync(kFull, part, d);
    if (lane == 0 && part != 0.0) bc[v] += part;  // this warp alone touches bc[v] in this sweep
  }
}

}  // namespace

dawn_status betweenness(dawn_graph* g, const int32_t* sources, int32_t nsrc, double* d_bc, dawn_stats* st) {
  const size_t nn = (size_t)g->n;
  DAWN_CHECK(ensure(g->bc_levels, sizeof(int32_t) * kLanes * nn, g->stream));
  DAWN_CHECK(ensure(g->bc_terms, sizeof(float) * kLanes * nn, g->stream));
  DAWN_CHECK(ensure(g->bc_range, sizeof(int32_t) * 2 * nn, g->stream));
  DAWN_CUDA(cudaMemsetAsync(d_bc, 0, sizeof(double) * nn, g->stream));
  int32_t* L = g->bc_levels.as<int32_t>();
  float* T = g->bc_terms.as<float>();
  int32_t* R = g->bc_range.as<int32_t>();
  const int grid = persistent_blocks((const void*)bc_sweep, kBlock, 0, g->blocks_per_sm);
  // the level pass runs the plain batched traversal (direction heuristic)
  DAWN_CHECK(call_selector(g, DAWN_VARIANT_BITSET, &g->sel_call));
  int64_t levels = 0;
  for (int32_t b0 = 0; b0 < nsrc; b0 += kLanes) {
    const int32_t k = nsrc - b0 < kLanes ? nsrc - b0 : kLanes;
    int32_t deepest = 0;
    DAWN_CHECK(bfs_bitset_levels(g, sources + b0, k, L, R, &deepest));
    levels += deepest;
    bc_amount<<<grid, kBlock, 0, g->stream>>>(g->t_row_ptr, g->t_col, L, T, g->n);
    DAWN_CUDA(cudaGetLastError());
    for (int32_t l = deepest - 1; l >= 1; l--) {
      bc_sweep<<<grid, kBlock, 0, g->stream>>>(g->row_ptr, g->col, L, R, T, d_bc, g->n, l);
      DAWN_CUDA(cudaGetLastError());
    }
  }
  if (st) {
    std::memset(st, 0, sizeof(*st));
    st->levels = (int32_t)levels;
    st->batches = (nsrc + kLanes - 1) / kLanes;
  }
  return DAWN_OK;
}

}  // namespace dawn
