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
// Rows of at least kHeavy entries (the hubs of power-law graphs) would keep
// one warp busy for thousands of dependent row loads while the rest of the
// grid idles, so they are cut into kBcSeg-entry segments, each a warp task
// of its own: in-row segments add their counts to a per-row counter
// (integers, so the order does not matter), out-row segments write their
// partial sums to a slot of their own, and a second kernel per pass finishes
// the heavy rows, adding the partials in segment order.
// Terms are float (the reference's bc_temp is float); the sums over
// sources are double.  The additions group as (1 / amount + delta) per
// entry, and a heavy row's sum by segments, rather than the reference's
// sequence, so values agree with it to float rounding, not bit for bit.
#include <algorithm>
#include <cstring>
#include <vector>

#include "dawn_device.cuh"

namespace dawn {
namespace {

constexpr int kLanes = 64;
constexpr int kUnroll = 4;
constexpr int kHeavy = 128;  // rows of at least this many entries are cut into segments
constexpr int kBcSeg = 64;   // entries per segment

// Rows cut into segments: vertex ids and the prefix of their segment counts.
struct HeavyRows {
  const int32_t* v;    // count entries
  const int32_t* off;  // count + 1 entries, off[count] = segs
  int32_t count, segs;
};

// The heavy row holding segment seg (binary search over the prefix).
__device__ __forceinline__ int heavy_of(const HeavyRows& h, int seg) {
  int lo = 0, hi = h.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(h.off + mid) <= seg) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Warp task t: vertices 0..n-1 whose rows are short, then the segments of
// the heavy rows.  Sets the vertex, the CSR range and the heavy row index
// (-1 for a short row); false for a heavy vertex's own task (its segments
// cover it).
__device__ __forceinline__ bool task_range(int t, int32_t n, const int32_t* __restrict__ rp, const HeavyRows& h,
                                           int32_t& v, int& ks, int& ke, int& hidx, int& seg) {
  if (t < n) {
    v = t;
    ks = rp[t];
    ke = rp[t + 1];
    hidx = -1;
    seg = -1;
    return ke - ks < kHeavy;
  }
  seg = t - n;
  hidx = heavy_of(h, seg);
  v = __ldg(h.v + hidx);
  const int rb = rp[v], re = rp[v + 1];
  ks = rb + (seg - __ldg(h.off + hidx)) * kBcSeg;
  ke = min(ks + kBcSeg, re);
  return true;
}

// Per lane, the entries j -> c in [ks, ke) whose level row holds la - 1
// (lanes 0-31) and lb - 1 (lanes 32-63 of the row).
__device__ __forceinline__ void count_preds(const int32_t* __restrict__ t_col, const int32_t* __restrict__ L,
                                            int ks, int ke, bool wa, bool wb, int32_t la, int32_t lb, int& ca,
                                            int& cb) {
  const int lane = lane_id();
  for (int kb = ks; kb < ke; kb += 32) {
    const int k = kb + lane;
    const int32_t jv = k < ke ? __ldg(t_col + k) : -1;
    const int cnt = min(32, ke - kb);
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

// Per lane, the sum of term(c) over entries v -> c in [ks, ke) with c at
// level + 1 for the lane's sources.
__device__ __forceinline__ void sum_terms(const int32_t* __restrict__ col, const int32_t* __restrict__ L,
                                          const float* __restrict__ T, int ks, int ke, bool wa, bool wb,
                                          int32_t level, float& sa, float& sb) {
  const int lane = lane_id();
  for (int kb = ks; kb < ke; kb += 32) {
    const int k = kb + lane;
    const int32_t cv = k < ke ? __ldg(col + k) : -1;
    const int cnt = min(32, ke - kb);
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
}

// 1 / amount for every (vertex, source) slot of the short in-rows; heavy
// in-rows' segments add their counts to cnt (one 64-entry row per heavy row).
__global__ void __launch_bounds__(kBlock) bc_amount(const int32_t* __restrict__ t_row_ptr,
                                                    const int32_t* __restrict__ t_col,
                                                    const int32_t* __restrict__ L, float* __restrict__ T,
                                                    int32_t n, HeavyRows h, int32_t* __restrict__ cnt) {
  const int lane = lane_id();
  for (int t = global_warp(); t < n + h.segs; t += num_warps()) {
    int32_t c;
    int ks, ke, hidx, seg;
    if (!task_range(t, n, t_row_ptr, h, c, ks, ke, hidx, seg)) continue;  // warp-uniform
    const int32_t* Lc = L + (size_t)c * kLanes;
    const int32_t la = Lc[lane], lb = Lc[lane + 32];
    const bool wa = la >= 2, wb = lb >= 2;
    int ca = 0, cb = 0;
    if (__any_sync(kFull, wa || wb)) count_preds(t_col, L, ks, ke, wa, wb, la, lb, ca, cb);
    if (hidx < 0) {
      float* Tc = T + (size_t)c * kLanes;
      Tc[lane] = wa && ca ? 1.0f / (float)ca : 0.0f;
      Tc[lane + 32] = wb && cb ? 1.0f / (float)cb : 0.0f;
    } else {
      if (ca) atomicAdd(cnt + (size_t)hidx * kLanes + lane, ca);
      if (cb) atomicAdd(cnt + (size_t)hidx * kLanes + lane + 32, cb);
    }
  }
}

// Heavy in-rows: 1 / amount from the summed counts, which are cleared for
// the next batch.
__global__ void __launch_bounds__(kBlock) bc_amount_heavy(const int32_t* __restrict__ L, float* __restrict__ T,
                                                          HeavyRows h, int32_t* __restrict__ cnt) {
  const int lane = lane_id();
  for (int hidx = global_warp(); hidx < h.count; hidx += num_warps()) {
    const int32_t c = __ldg(h.v + hidx);
    const int32_t la = L[(size_t)c * kLanes + lane], lb = L[(size_t)c * kLanes + lane + 32];
    int32_t* cr = cnt + (size_t)hidx * kLanes;
    const int ca = cr[lane], cb = cr[lane + 32];
    cr[lane] = 0;
    cr[lane + 32] = 0;
    float* Tc = T + (size_t)c * kLanes;
    Tc[lane] = la >= 2 && ca ? 1.0f / (float)ca : 0.0f;
    Tc[lane + 32] = lb >= 2 && cb ? 1.0f / (float)cb : 0.0f;
  }
}

// Level l of the backward sweep (see the file comment) over the short
// out-rows; heavy out-rows' segments leave their partial sums in part.
__global__ void __launch_bounds__(kBlock) bc_sweep(const int32_t* __restrict__ row_ptr,
                                                   const int32_t* __restrict__ col,
                                                   const int32_t* __restrict__ L, const int32_t* __restrict__ range,
                                                   float* __restrict__ T, double* __restrict__ bc, int32_t n,
                                                   int32_t level, HeavyRows h, float* __restrict__ part) {
  const int lane = lane_id();
  for (int t = global_warp(); t < n + h.segs; t += num_warps()) {
    int32_t v;
    int ks, ke, hidx, seg;
    if (!task_range(t, n, row_ptr, h, v, ks, ke, hidx, seg)) continue;  // warp-uniform
    if (level < range[2 * v] || level > range[2 * v + 1]) continue;      // warp-uniform
    const int32_t* Lv = L + (size_t)v * kLanes;
    const bool wa = Lv[lane] == level, wb = Lv[lane + 32] == level;
    if (!__any_sync(kFull, wa || wb)) continue;
    float sa = 0.0f, sb = 0.0f;
    sum_terms(col, L, T, ks, ke, wa, wb, level, sa, sb);
    if (hidx >= 0) {
      part[(size_t)seg * kLanes + lane] = sa;
      part[(size_t)seg * kLanes + lane + 32] = sb;
      continue;
    }
    float* Tv = T + (size_t)v * kLanes;
    if (wa) Tv[lane] += sa;
    if (wb) Tv[lane + 32] += sb;
    double pd = (wa ? (double)sa : 0.0) + (wb ? (double)sb : 0.0);
#pragma unroll
    for (int d = 16; d; d >>= 1) pd += __shfl_xor_sync(kFull, pd, d);
    if (lane == 0 && pd != 0.0) bc[v] += pd;  // this warp alone touches bc[v] in this sweep
  }
}

// Level l for the heavy out-rows: their segments' partial sums, added in
// segment order.
__global__ void __launch_bounds__(kBlock) bc_sweep_heavy(const int32_t* __restrict__ L,
                                                         const int32_t* __restrict__ range, float* __restrict__ T,
                                                         double* __restrict__ bc, int32_t level, HeavyRows h,
                                                         const float* __restrict__ part) {
  const int lane = lane_id();
  for (int hidx = global_warp(); hidx < h.count; hidx += num_warps()) {
    const int32_t v = __ldg(h.v + hidx);
    if (level < range[2 * v] || level > range[2 * v + 1]) continue;
    const int32_t* Lv = L + (size_t)v * kLanes;
    const bool wa = Lv[lane] == level, wb = Lv[lane + 32] == level;
    if (!__any_sync(kFull, wa || wb)) continue;
    float sa = 0.0f, sb = 0.0f;
    const int s1 = __ldg(h.off + hidx + 1);
    for (int sg = __ldg(h.off + hidx); sg < s1; sg++) {
      sa += part[(size_t)sg * kLanes + lane];
      sb += part[(size_t)sg * kLanes + lane + 32];
    }
    float* Tv = T + (size_t)v * kLanes;
    if (wa) Tv[lane] += sa;
    if (wb) Tv[lane + 32] += sb;
    double pd = (wa ? (double)sa : 0.0) + (wb ? (double)sb : 0.0);
#pragma unroll
    for (int d = 16; d; d >>= 1) pd += __shfl_xor_sync(kFull, pd, d);
    if (lane == 0 && pd != 0.0) bc[v] += pd;
  }
}

// Heavy-row lists of one CSR (host side): rows of at least kHeavy entries
// and the prefix of their segment counts.
void heavy_rows(const std::vector<int32_t>& rp, std::vector<int32_t>& ids, std::vector<int32_t>& off) {
  ids.clear();
  off.assign(1, 0);
  for (size_t v = 0; v + 1 < rp.size(); v++) {
    const int deg = rp[v + 1] - rp[v];
    if (deg < kHeavy) continue;
    ids.push_back((int32_t)v);
    off.push_back(off.back() + (deg + kBcSeg - 1) / kBcSeg);
  }
}

// Builds the heavy-row lists once per handle (out-rows for the sweeps,
// in-rows for the amounts; one list when the graph is symmetric) and the
// partial-sum scratch.
dawn_status prepare_heavy(dawn_graph* g) {
  if (g->bc_hout >= 0) return DAWN_OK;
  const size_t nn = (size_t)g->n;
  std::vector<int32_t> rp(nn + 1), out_ids, out_off, in_ids, in_off;
  DAWN_CUDA(cudaMemcpyAsync(rp.data(), g->row_ptr, sizeof(int32_t) * (nn + 1), cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  heavy_rows(rp, out_ids, out_off);
  if (g->t_row_ptr == g->row_ptr) {
    in_ids = out_ids;
    in_off = out_off;
  } else {
    DAWN_CUDA(cudaMemcpyAsync(rp.data(), g->t_row_ptr, sizeof(int32_t) * (nn + 1), cudaMemcpyDeviceToHost,
                              g->stream));
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    heavy_rows(rp, in_ids, in_off);
  }
  std::vector<int32_t> all;
  all.insert(all.end(), out_ids.begin(), out_ids.end());
  all.insert(all.end(), out_off.begin(), out_off.end());
  all.insert(all.end(), in_ids.begin(), in_ids.end());
  all.insert(all.end(), in_off.begin(), in_off.end());
  DAWN_CHECK(ensure(g->bc_heavy, sizeof(int32_t) * all.size(), g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->bc_heavy.p, all.data(), sizeof(int32_t) * all.size(), cudaMemcpyHostToDevice,
                            g->stream));
  // partial sums of the out-row segments, then the in-row counters, which
  // start at zero (bc_amount_heavy clears them after use)
  const int32_t segs_out = out_off.back();
  const size_t words = ((size_t)segs_out + in_ids.size()) * kLanes + 1;
  DAWN_CHECK(ensure(g->bc_part, sizeof(float) * words, g->stream));
  DAWN_CUDA(cudaMemsetAsync(g->bc_part.p, 0, sizeof(float) * words, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  g->bc_segs_out = segs_out;
  g->bc_hin = (int32_t)in_ids.size();
  g->bc_segs_in = in_off.back();
  g->bc_hout = (int32_t)out_ids.size();
  return DAWN_OK;
}

}  // namespace

dawn_status betweenness(dawn_graph* g, const int32_t* sources, int32_t nsrc, double* d_bc, dawn_stats* st) {
  const size_t nn = (size_t)g->n;
  // Level rows and ranges are double-buffered: the traversal of batch b runs
  // while the host waits for batch b - 1's depth, so the stream always has
  // work queued (traversal b, then the sweeps of b - 1).  The terms need one
  // buffer: the amount and sweep passes of the batches follow one another.
  DAWN_CHECK(ensure(g->bc_levels, sizeof(int32_t) * kLanes * nn * 2, g->stream));
  DAWN_CHECK(ensure(g->bc_terms, sizeof(float) * kLanes * nn, g->stream));
  DAWN_CHECK(ensure(g->bc_range, sizeof(int32_t) * 2 * nn * 2, g->stream));
  DAWN_CHECK(prepare_heavy(g));
  if (!g->bc_h_level) DAWN_CHECK(pinned_slot((void**)&g->bc_h_level));
  DAWN_CUDA(cudaMemsetAsync(d_bc, 0, sizeof(double) * nn, g->stream));
  int32_t* const Ls[2] = {g->bc_levels.as<int32_t>(), g->bc_levels.as<int32_t>() + kLanes * nn};
  int32_t* const Rs[2] = {g->bc_range.as<int32_t>(), g->bc_range.as<int32_t>() + 2 * nn};
  float* T = g->bc_terms.as<float>();
  const int32_t* hv = g->bc_heavy.as<int32_t>();
  HeavyRows hout{hv, hv + g->bc_hout, g->bc_hout, g->bc_segs_out};
  const int32_t* hin_base = hv + 2 * g->bc_hout + 1;
  HeavyRows hin{hin_base, hin_base + g->bc_hin, g->bc_hin, g->bc_segs_in};
  float* part = g->bc_part.as<float>();
  int32_t* cnt = g->bc_part.as<int32_t>() + (size_t)g->bc_segs_out * kLanes;
  const int grid = persistent_blocks((const void*)bc_sweep, kBlock, 0, g->blocks_per_sm);
  // the level pass runs the plain batched traversal (direction heuristic)
  DAWN_CHECK(call_selector(g, DAWN_VARIANT_BITSET, &g->sel_call));
  cudaEvent_t done[2] = {nullptr, nullptr};
  dawn_status status = DAWN_OK;
  int64_t levels = 0;
  const int32_t nb = (nsrc + kLanes - 1) / kLanes;
  for (int i = 0; i < 2; i++)
    if (cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) != cudaSuccess) {
      set_error("betweenness: cudaEventCreate failed");
      status = DAWN_ERR_CUDA;
    }
  for (int32_t b = 0; b <= nb && status == DAWN_OK; b++) {
    if (b < nb) {
      const int32_t b0 = b * kLanes, k = nsrc - b0 < kLanes ? nsrc - b0 : kLanes;
      status = bfs_bitset_levels(g, sources + b0, k, Ls[b & 1], Rs[b & 1], g->bc_h_level + (b & 1));
      if (status == DAWN_OK && cudaEventRecord(done[b & 1], g->stream) != cudaSuccess) {
        set_error("betweenness: cudaEventRecord failed");
        status = DAWN_ERR_CUDA;
      }
      if (status != DAWN_OK) break;
    }
    if (b == 0) continue;
    // the dependency passes of batch b - 1, once its depth is known
    const int p = (b - 1) & 1;
    if (cudaEventSynchronize(done[p]) != cudaSuccess) {
      set_error("betweenness: %s", cudaGetErrorString(cudaGetLastError()));
      status = DAWN_ERR_CUDA;
      break;
    }
    const int32_t deepest = g->bc_h_level[p] - 1;  // the batch ended on an empty level
    levels += deepest;
    const int32_t* L = Ls[p];
    const int32_t* R = Rs[p];
    bc_amount<<<grid, kBlock, 0, g->stream>>>(g->t_row_ptr, g->t_col, L, T, g->n, hin, cnt);
    if (hin.count) bc_amount_heavy<<<grid, kBlock, 0, g->stream>>>(L, T, hin, cnt);
    for (int32_t l = deepest - 1; l >= 1; l--) {
      bc_sweep<<<grid, kBlock, 0, g->stream>>>(g->row_ptr, g->col, L, R, T, d_bc, g->n, l, hout, part);
      if (hout.count) bc_sweep_heavy<<<grid, kBlock, 0, g->stream>>>(L, R, T, d_bc, l, hout, part);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("betweenness: %s", cudaGetErrorString(e));
      status = DAWN_ERR_CUDA;
    }
  }
  for (cudaEvent_t e : done)
    if (e) cudaEventDestroy(e);
  DAWN_CHECK(status);
  if (st) {
    std::memset(st, 0, sizeof(*st));
    st->levels = (int32_t)levels;
    st->batches = nb;
  }
  return DAWN_OK;
}

}  // namespace dawn
