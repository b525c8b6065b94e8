// Batched min-plus relax: weighted distances from up to 64 sources in one
// traversal, on sm_103a.
//
// The reference computes weighted multi-source distances one source at a
// time (MSSP_GPU::run_Weighted, src/algorithm/gpu/mssp.cu:53-102), each a
// full GOVM traversal that re-reads the CSR and pays one atomic per
// improving edge.  Here a batch of up to 64 sources shares one traversal:
//   * distances live vertex-major, 64 int32 words per vertex (int32 weights
//     natively, float32 through their bit pattern, which orders like the
//     value for the non-negative floats the upload admits), so the 64
//     distances of an edge's head are one 256-byte row;
//   * the frontier is a queue of vertices with a 64-bit mask per vertex of
//     the sources whose distance improved at the last level (three mask
//     slots rotate by level % 3: level L reads (L-1)%3, writes L%3, clears
//     (L+1)%3);
//   * a warp takes one frontier vertex (rows of >= 128 entries one
//     128-entry segment at a time), or, for vertices active for at most
//     kSparse sources, a lane takes one (vertex, source) pair; in the warp
//     form lane i owns sources i and i + 32.  The
//     warp loads 32 of the row's targets and weights in one coalesced read,
//     then for each edge every lane relaxes its two sources against the
//     target's distance row (fetched for four edges at a time) and issues a
//     return-free atomicMin where it improves on the fetched value;
//     the improved sources are OR-ed into the target's next mask, and the
//     first setter queues the target;
//   * a final pass transposes the block into the caller's source-major rows
//     and counts the reached edges.
// Each source's first frontier is resolved as the single-source path does
// (the reference CPU path, src/algorithm/cpu/sssp.cpp:41-46): each distinct
// neighbour takes the weight of its last CSR entry, the source is set to 0
// and is relaxed again only through a self loop.  Any relaxation order
// reaches the same fixed point, so the distances equal the single-source
// traversal's.
#include "dawn_device.cuh"

namespace dawn {
namespace {

constexpr int kBatch = 64;  // sources per batch (two per lane)
constexpr int kUnroll = 4;  // edges whose distance rows are fetched together
constexpr int kInitBlock = 1024;  // threads per source in mw_init (hub rows)

struct MwCtl {
  int32_t qsize[2];
  unsigned long long lpack[2];
  unsigned long long mf[2];
  int32_t level, done, batch, nsrc;
  int32_t mode;                 // kModePush or kModePull for the next level
  int32_t force;                // 0 = decide per level; 2 = every level a pull, other values a push
  int32_t work, hwork;          // pull: dynamic work counters (light rows, heavy-row segments)
  int32_t n_pull;
  int32_t n_push, inits;       // inits: mw_init CTAs finished
  unsigned long long reached;   // TEPS numerator of all batches so far
  int32_t* dist_base;           // nsrc x n output (source-major)
  const int32_t* sources;
  int32_t total_levels, total_push, total_pull;
};

__device__ __forceinline__ int32_t relax(int32_t d, int32_t w, bool is_float) {
  if (is_float) return __float_as_int(__fadd_rn(__int_as_float(d), __int_as_float(w)));
  return d + w;
}

// Fills the block with "unreached", clears the mask slots and resets the
// level counters for the batch.
__global__ void __launch_bounds__(kBlock) mw_clear(MwCtl* __restrict__ ctl, int32_t* __restrict__ D, size_t words,
                                                   int32_t inf, unsigned long long* __restrict__ masks,
                                                   size_t nmask) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->qsize[0] = ctl->qsize[1] = 0;
    ctl->lpack[0] = ctl->lpack[1] = 0;
    ctl->mf[0] = ctl->mf[1] = 0;
    ctl->level = 1;
    ctl->done = 0;
    ctl->n_push = 0;
    ctl->n_pull = 0;
    ctl->inits = 0;
    ctl->mode = ctl->force == 2 ? kModePull : kModePush;
    ctl->work = 0;
    ctl->hwork = 0;
  }
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  int4* d4 = reinterpret_cast<int4*>(D);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < words / 4; i += stride)
    d4[i] = make_int4(inf, inf, inf, inf);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nmask; i += stride) masks[i] = 0ull;
}

// One CTA per source b of the batch (kBatch CTAs; those past the batch's
// end only check in).  Each distinct neighbour takes the weight of its last
// CSR entry: the entries first lower the neighbour's block word for b to
// -(k + 1) with atomicMin, so the largest position k wins, and the winner
// then stores its weight there (weights are non-negative, so no later test
// mistakes a weight for a marker).  Column b of the block is this CTA's
// alone.  A winner enters the level-0 mask with bit b and is queued by its
// first setter; then the source's own entry is set to 0.  The last CTA to
// check in decides whether the first frontier is empty.
__global__ void __launch_bounds__(kInitBlock) mw_init(MwCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                                                      const int32_t* __restrict__ col,
                                                      const int32_t* __restrict__ w, int32_t* __restrict__ D,
                                                      unsigned long long* __restrict__ mask0,
                                                      int32_t* __restrict__ q, Seg* __restrict__ segs) {
  const int batch = ctl->batch;
  const int nb = min(kBatch, ctl->nsrc - batch * kBatch);
  const int b = blockIdx.x;
  if (b < nb) {
    const int32_t s = ctl->sources[batch * kBatch + b];
    const int rs = row_ptr[s], re = row_ptr[s + 1];
    for (int k = rs + threadIdx.x; k < re; k += blockDim.x) atomicMin(D + (size_t)col[k] * kBatch + b, -(k + 1));
    __syncthreads();
    for (int k = rs + threadIdx.x; k < re; k += blockDim.x) {
      const int32_t u = col[k];
      int32_t* du = D + (size_t)u * kBatch + b;
      if (__ldcg(du) != -(k + 1)) continue;
      *du = __ldg(w + k);
      const unsigned long long old = atomicOr(mask0 + u, 1ull << b);
      if (old == 0ull) {
        const int urs = row_ptr[u], udeg = row_ptr[u + 1] - urs;
        atomicAdd(&ctl->mf[0], (unsigned long long)udeg);
        if (udeg >= kLongRow) {
          const int nseg = (udeg + kSeg - 1) / kSeg;
          const unsigned long long o = atomicAdd(&ctl->lpack[0], (1ull << 32) | (unsigned)nseg);
          for (int j = 0; j < nseg; j++) segs[(uint32_t)o + j] = Seg{u, urs + j * kSeg};
        } else {
          q[atomicAdd(&ctl->qsize[0], 1)] = u;
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) D[(size_t)s * kBatch + b] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ctl->inits, 1) == (int)gridDim.x - 1) {
      __threadfence();
      ctl->done = __ldcg(&ctl->qsize[0]) == 0 && __ldcg(&ctl->lpack[0]) == 0ull;
    }
  }
}

// The row [k0, k1) of frontier vertex u relaxed by one warp: lane i owns
// sources i and i + 32 of the batch.  The warp loads 32 targets and weights
// in one coalesced read; for each edge every lane relaxes its two sources
// against the target's distance row (fetched for kUnroll edges at a time)
// and issues a return-free atomicMin where it improves on the fetched
// value.  Lane j collects the improved sources of edge kb + j, so the
// next-mask update and the queue append run once per 32 edges.  All 32
// lanes call it with the same arguments.
__device__ __forceinline__ void relax_row(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                          const int32_t* __restrict__ w, bool fl, int32_t* __restrict__ D,
                                          unsigned long long* __restrict__ m_out, int32_t u, int k0, int k1,
                                          unsigned long long mask, WarpQueue& wq, Seg* __restrict__ sout,
                                          unsigned long long* lpack, unsigned long long& my_mf) {
  const int lane = lane_id();
  const bool actA = (mask >> lane) & 1ull, actB = (mask >> (lane + 32)) & 1ull;
  const int32_t* du = D + (size_t)u * kBatch;
  const int32_t dA = __ldcg(du + lane), dB = __ldcg(du + lane + 32);
  for (int kb = k0; kb < k1; kb += 32) {
    const int k = kb + lane;
    const int32_t cv = k < k1 ? __ldg(col + k) : -1;
    const int32_t cw = k < k1 ? __ldg(w + k) : 0;
    const int cnt = min(32, k1 - kb);
    unsigned long long mybits = 0ull;
    for (int j0 = 0; j0 < cnt; j0 += kUnroll) {
      int32_t v[kUnroll], wv[kUnroll], curA[kUnroll], curB[kUnroll];
#pragma unroll
      for (int i = 0; i < kUnroll; i++) {
        v[i] = __shfl_sync(kFull, cv, (j0 + i) & 31);
        wv[i] = __shfl_sync(kFull, cw, (j0 + i) & 31);
        if (j0 + i >= cnt) v[i] = -1;
      }
#pragma unroll
      for (int i = 0; i < kUnroll; i++) {
        const int32_t* dv = D + (size_t)(v[i] < 0 ? 0 : v[i]) * kBatch;
        curA[i] = (v[i] >= 0 && actA) ? __ldcg(dv + lane) : 0;
        curB[i] = (v[i] >= 0 && actB) ? __ldcg(dv + lane + 32) : 0;
      }
      bool impA[kUnroll], impB[kUnroll];
#pragma unroll
      for (int i = 0; i < kUnroll; i++) {
        impA[i] = impB[i] = false;
        if (v[i] < 0) continue;
        int32_t* dv = D + (size_t)v[i] * kBatch;
        // Improvement is judged against the row fetched above and the
        // minimum is a reduction without a return value: a target whose
        // entry another warp lowered further in the meantime is only
        // relaxed once more at the next level, which leaves the fixed
        // point unchanged.
        if (actA) {
          const int32_t c = relax(dA, wv[i], fl);
          if (c < curA[i]) {
            atomicMin(dv + lane, c);
            impA[i] = true;
          }
        }
        if (actB) {
          const int32_t c = relax(dB, wv[i], fl);
          if (c < curB[i]) {
            atomicMin(dv + lane + 32, c);
            impB[i] = true;
          }
        }
      }
#pragma unroll
      for (int i = 0; i < kUnroll; i++) {
        const unsigned long long bits = (unsigned long long)__ballot_sync(kFull, impA[i]) |
                                        ((unsigned long long)__ballot_sync(kFull, impB[i]) << 32);
        if (lane == j0 + i) mybits = bits;
      }
    }
    bool first = false;
    int deg = 0, rs = 0;
    if (mybits) {
      first = atomicOr(m_out + cv, mybits) == 0ull;
      if (first) {
        rs = row_ptr[cv];
        deg = row_ptr[cv + 1] - rs;
        my_mf += (unsigned long long)deg;
      }
    }
    emit_routed(first, cv, deg, rs, wq, sout, lpack);
  }
}

// A long-row segment (at most kSeg entries) of a vertex active for few
// sources: the lanes take 32 consecutive edges at a time and relax each of
// the vertex's active sources along them, so a segment costs
// ceil(len / 32) rounds per source instead of the len / kUnroll rounds of
// the warp-per-edge form, whose lanes mostly idle on such a mask (the hubs
// next to the sources at the first levels).  All 32 lanes call it with the
// same arguments.
__device__ __forceinline__ void relax_seg_sparse(const int32_t* __restrict__ row_ptr,
                                                 const int32_t* __restrict__ col, const int32_t* __restrict__ w,
                                                 bool fl, int32_t* __restrict__ D,
                                                 unsigned long long* __restrict__ m_out, int32_t u, int k0, int k1,
                                                 unsigned long long mask, WarpQueue& wq, Seg* __restrict__ sout,
                                                 unsigned long long* lpack, unsigned long long& my_mf) {
  const int lane = lane_id();
  const int32_t* du = D + (size_t)u * kBatch;
  for (int kb = k0; kb < k1; kb += 32) {
    const int k = kb + lane;
    const int32_t v = k < k1 ? __ldg(col + k) : -1;
    const int32_t wv = k < k1 ? __ldg(w + k) : 0;
    const int32_t* dv = D + (size_t)(v < 0 ? 0 : v) * kBatch;
    unsigned long long mine = 0ull;
    for (unsigned long long m = mask; m; m &= m - 1) {
      const int src = __ffsll((long long)m) - 1;
      const int32_t dsu = __ldcg(du + src);
      if (v >= 0) {
        const int32_t c = relax(dsu, wv, fl);
        if (c < __ldcg(dv + src)) {
          atomicMin(D + (size_t)v * kBatch + src, c);
          mine |= 1ull << src;
        }
      }
    }
    bool first = false;
    int deg = 0, rs = 0;
    if (mine) {
      first = atomicOr(m_out + v, mine) == 0ull;
      if (first) {
        rs = row_ptr[v];
        deg = row_ptr[v + 1] - rs;
        my_mf += (unsigned long long)deg;
      }
    }
    emit_routed(first, v, deg, rs, wq, sout, lpack);
  }
}

// Frontier vertices whose mask holds at most kSparse sources (the waves of
// different sources crossing a high-diameter graph: most vertices are
// active for one or two of the 64 at a time) go through pairs instead of a
// warp per vertex: one lane per (vertex, improved source), relaxing that
// source along the vertex's row with kUnroll targets in flight.
constexpr int kSparse = 16;
// Long-row segments go edge-parallel up to this many active sources.
// RMAT scale 22 x 64, int32, same host: 22.4 -> 21.2 ms (level 1, the
// sources' hub neighbours, 1.86 -> 0.87 ms); thresholds 2, 8 and 16 within
// 0.1%.
constexpr int kSparseSeg = 8;

// One level.  Warp tasks: the long-row segments (a warp each), then the
// input queue 32 vertices at a time: the vertices with dense masks get the
// warp one after another, the sparse ones are dealt as (vertex, source)
// pairs across the lanes.
__global__ void __launch_bounds__(kBlock, 4) mw_push(const int32_t* __restrict__ row_ptr,
                                                  const int32_t* __restrict__ col, const int32_t* __restrict__ w,
                                                  int is_float, MwCtl* __restrict__ ctl, int32_t* __restrict__ D,
                                                  unsigned long long* __restrict__ masks, int32_t* __restrict__ q,
                                                  Seg* __restrict__ segs, size_t segcap, int32_t n) {
  __shared__ int32_t s_q[kBlock / 32][kWarpQueue];
  if (ctl->done || ctl->mode != kModePush) return;
  const int L = ctl->level;
  const int pin = (L - 1) & 1, pout = L & 1;
  const unsigned long long* __restrict__ m_in = masks + (size_t)((L - 1) % 3) * n;
  unsigned long long* m_out = masks + (size_t)(L % 3) * n;
  {
    unsigned long long* m_clr = masks + (size_t)((L + 1) % 3) * n;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride) m_clr[i] = 0ull;
  }
  const int32_t* qin = q + (size_t)pin * n;
  const Seg* sin = segs + (size_t)pin * segcap;
  const int qn = ctl->qsize[pin];
  const int ln = seg_count(ctl->lpack[pin]);
  const int ngroups = (qn + 31) / 32;
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const bool fl = is_float != 0;
  WarpQueue wq(s_q[wib], q + (size_t)pout * n, &ctl->qsize[pout]);
  Seg* sout = segs + (size_t)pout * segcap;
  unsigned long long* lpack = &ctl->lpack[pout];
  unsigned long long my_mf = 0;

  for (int t = global_warp(); t < ln + ngroups; t += num_warps()) {
    if (t < ln) {
      const Seg sg = sin[t];
      const int k1 = min(sg.k0 + kSeg, row_ptr[sg.v + 1]);
      const unsigned long long sm = __ldcg(m_in + sg.v);
      if (__popcll(sm) <= kSparseSeg)
        relax_seg_sparse(row_ptr, col, w, fl, D, m_out, sg.v, sg.k0, k1, sm, wq, sout, lpack, my_mf);
      else
        relax_row(row_ptr, col, w, fl, D, m_out, sg.v, sg.k0, k1, sm, wq, sout, lpack, my_mf);
      continue;
    }
    const int i = (t - ln) * 32 + lane;
    int32_t u = -1;
    int k0 = 0, k1 = 0;
    unsigned long long mask = 0ull;
    if (i < qn) {
      u = qin[i];
      k0 = row_ptr[u];
      k1 = row_ptr[u + 1];
      mask = __ldcg(m_in + u);
    }
    const int pc = __popcll(mask);
    const bool sparse = pc <= kSparse;
    uint32_t dense = __ballot_sync(kFull, !sparse);
    while (dense) {
      const int l = __ffs(dense) - 1;
      dense &= dense - 1;
      relax_row(row_ptr, col, w, fl, D, m_out, __shfl_sync(kFull, u, l), __shfl_sync(kFull, k0, l),
                __shfl_sync(kFull, k1, l), __shfl_sync(kFull, mask, l), wq, sout, lpack, my_mf);
    }
    // (vertex, source) pairs of the sparse lanes, 32 at a time
    const int np = sparse && k1 > k0 ? pc : 0;
    const int incl = warp_incl_scan(np);
    const int excl = incl - np;
    const int total = __shfl_sync(kFull, incl, 31);
    for (int e0 = 0; e0 < total; e0 += 32) {
      const int e = e0 + lane;
      int lo = 0;  // last lane whose first pair is <= e
#pragma unroll
      for (int step = 16; step; step >>= 1) {
        const int ex = __shfl_sync(kFull, excl, lo + step);
        if (ex <= e) lo += step;
      }
      const bool ok = e < total;
      const int r = e - __shfl_sync(kFull, excl, lo);
      unsigned long long m = __shfl_sync(kFull, mask, lo);
      const int32_t pu = __shfl_sync(kFull, u, lo);
      const int pk0 = __shfl_sync(kFull, k0, lo), pk1 = __shfl_sync(kFull, k1, lo);
      int src = 0, nd = 0;
      int32_t dsu = 0;
      if (ok) {
        for (int c = 0; c < r; c++) m &= m - 1;  // drop the r lowest sources
        src = __ffsll((long long)m) - 1;
        dsu = __ldcg(D + (size_t)pu * kBatch + src);
        nd = pk1 - pk0;
      }
      const int maxd = (int)__reduce_max_sync(kFull, (unsigned)nd);
      for (int j0 = 0; j0 < maxd; j0 += kUnroll) {
        int32_t v[kUnroll], wv[kUnroll], cur[kUnroll];
#pragma unroll
        for (int x = 0; x < kUnroll; x++) {
          const bool act = j0 + x < nd;
          v[x] = act ? __ldg(col + pk0 + j0 + x) : -1;
          wv[x] = act ? __ldg(w + pk0 + j0 + x) : 0;
        }
#pragma unroll
        for (int x = 0; x < kUnroll; x++) cur[x] = v[x] >= 0 ? __ldcg(D + (size_t)v[x] * kBatch + src) : 0;
#pragma unroll
        for (int x = 0; x < kUnroll; x++) {
          bool first = false;
          int deg = 0, rs = 0;
          if (v[x] >= 0) {
            const int32_t c = relax(dsu, wv[x], fl);
            if (c < cur[x]) {
              atomicMin(D + (size_t)v[x] * kBatch + src, c);
              first = atomicOr(m_out + v[x], 1ull << src) == 0ull;
              if (first) {
                rs = row_ptr[v[x]];
                deg = row_ptr[v[x] + 1] - rs;
                my_mf += (unsigned long long)deg;
              }
            }
          }
          emit_routed(first, v[x], deg, rs, wq, sout, lpack);
        }
      }
    }
  }
  wq.flush();
  my_mf = warp_sum(my_mf);
  if (lane == 0 && my_mf) atomicAdd(&ctl->mf[pout], my_mf);
}

// Pull level (frontiers whose out-edges reach half the graph): every vertex
// v takes, per source, the minimum of D[u][s] + w over its in-edges (u, w)
// from tails whose source s improved at the last level, and keeps it where
// it beats D[v][s].  A warp owns a light row (in-degree below 2 x pull_seg)
// and writes its row of D and its next mask with plain stores: no atomics
// per edge, and one improved-source mask per vertex instead of per edge.
// Heavy rows are cut into pull_seg-entry segment tasks, each a warp, which
// lower the row with return-free atomicMin where they improve on it and
// OR their improved sources into the next mask (the first setter queues
// the vertex).  A tail row (256 bytes) is read by a group of kRowLanes
// lanes, kPullSrc sources (16 or 32 bytes) per lane, so one warp-wide load
// brings kRowGroups rows.  Tails are read 32 at a time (vertex coalesced,
// mask gathered once per lane); the live ones (mask not empty) are packed
// with their weights into a per-warp shared-memory stage, and the groups
// walk the stage kPullUnroll rows each, fetching those rows before any is
// used.  Per-source minima stay in registers; the groups' minima are folded
// at the end of the vertex and group 0 holds the result.
// Reading a row that another warp lowers in the same level is harmless:
// every value a row holds is the length of some path, and a value lowered
// now is relaxed again at the next level through the mask it sets.
// Eight sources per lane (four rows per warp-wide load) and three rows per
// group in flight: 64 registers, four CTAs per SM.  RMAT scale 22 x 64
// sources, int32: 29.3 ms with two sources per lane (one row per load,
// tails passed by shuffles), 29.7 ms with four (two rows per load), 22.6
// with eight and two rows per group, 22.3 with three; four rows per group
// at three CTAs per SM 24.4 ms.
constexpr int kPullSrc = 8;                 // sources per lane (4 or 8)
constexpr int kPullUnroll = 3;              // rows per lane group fetched together
constexpr int kRowLanes = kBatch / kPullSrc;  // lanes reading one tail row
constexpr int kRowGroups = 32 / kRowLanes;    // tail rows per warp-wide load
constexpr int kQuads = kPullSrc / 4;          // 16-byte pieces per lane and row
static_assert(kPullSrc == 4 || kPullSrc == 8, "a lane reads whole 16-byte pieces of a row");

// Quad q of lane `sub` of a group: sources quad_base(sub, q) .. + 3 (with
// eight sources per lane the second quad sits in the row's upper half, so
// each load instruction of a group covers 128 contiguous bytes).
__device__ __forceinline__ int quad_base(int sub, int q) { return 4 * sub + q * (kBatch / kQuads); }

__device__ __forceinline__ void pull_min(const int32_t* __restrict__ t_col, const int32_t* __restrict__ t_w,
                                         const unsigned long long* __restrict__ m_in,
                                         const int32_t* __restrict__ D, bool fl, int k0, int k1,
                                         int4* __restrict__ stage, int32_t (&mn)[kPullSrc]) {
  const int lane = lane_id(), grp = lane / kRowLanes, sub = lane % kRowLanes;
  for (int kb = k0; kb < k1; kb += 32) {
    const int k = kb + lane;
    const int32_t cu = k < k1 ? __ldg(t_col + k) : -1;
    const unsigned long long cm = cu >= 0 ? __ldcg(m_in + cu) : 0ull;
    const unsigned live = __ballot_sync(kFull, cm != 0ull);
    if (cm)
      stage[__popc(live & lanemask_lt())] =
          make_int4(cu, __ldg(t_w + k), (int)(unsigned)cm, (int)(unsigned)(cm >> 32));
    __syncwarp();
    const int cnt = __popc(live);
    for (int r0 = 0; r0 < cnt; r0 += kRowGroups * kPullUnroll) {
      int4 e[kPullUnroll];
      unsigned bits[kPullUnroll];
      int4 d[kPullUnroll][kQuads];
#pragma unroll
      for (int i = 0; i < kPullUnroll; i++) {
        const int r = r0 + i * kRowGroups + grp;
        e[i] = r < cnt ? stage[r] : make_int4(0, 0, 0, 0);
        bits[i] = 0u;
#pragma unroll
        for (int q = 0; q < kQuads; q++) {
          const int base = quad_base(sub, q);
          const unsigned word = base >= 32 ? (unsigned)e[i].w : (unsigned)e[i].z;
          bits[i] |= ((word >> (base & 31)) & 15u) << (4 * q);
        }
      }
#pragma unroll
      for (int i = 0; i < kPullUnroll; i++) {
        const int4* du = reinterpret_cast<const int4*>(D + (size_t)e[i].x * kBatch);
#pragma unroll
        for (int q = 0; q < kQuads; q++)
          d[i][q] = ((bits[i] >> (4 * q)) & 15u) ? __ldcg(du + quad_base(sub, q) / 4) : make_int4(0, 0, 0, 0);
      }
#pragma unroll
      for (int i = 0; i < kPullUnroll; i++) {
#pragma unroll
        for (int q = 0; q < kQuads; q++) {
          const unsigned b = bits[i] >> (4 * q);
          if (b & 1u) mn[4 * q + 0] = min(mn[4 * q + 0], relax(d[i][q].x, e[i].y, fl));
          if (b & 2u) mn[4 * q + 1] = min(mn[4 * q + 1], relax(d[i][q].y, e[i].y, fl));
          if (b & 4u) mn[4 * q + 2] = min(mn[4 * q + 2], relax(d[i][q].z, e[i].y, fl));
          if (b & 8u) mn[4 * q + 3] = min(mn[4 * q + 3], relax(d[i][q].w, e[i].y, fl));
        }
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int off = kRowLanes; off < 32; off <<= 1)
#pragma unroll
    for (int t = 0; t < kPullSrc; t++) mn[t] = min(mn[t], __shfl_xor_sync(kFull, mn[t], off));
}

// The pulled minima of vertex v against its row: group 0 lowers the row
// (plain stores where the warp owns the row, atomicMin on heavy-row
// segments) and the warp returns the 64-bit mask of improved sources.
template <bool kAtomic>
__device__ __forceinline__ unsigned long long pull_store(int32_t* __restrict__ D, int32_t v,
                                                         const int32_t (&mn)[kPullSrc]) {
  const int lane = lane_id(), sub = lane % kRowLanes;
  unsigned lo = 0u, hi = 0u;
  if (lane < kRowLanes) {
    int4* dv = reinterpret_cast<int4*>(D + (size_t)v * kBatch);
#pragma unroll
    for (int q = 0; q < kQuads; q++) {
      const int base = quad_base(sub, q);
      const int4 cur = __ldcg(dv + base / 4);
      const int32_t* m = mn + 4 * q;
      const unsigned imp = (unsigned)(m[0] < cur.x) | (unsigned)(m[1] < cur.y) << 1 |
                           (unsigned)(m[2] < cur.z) << 2 | (unsigned)(m[3] < cur.w) << 3;
      if (imp) {
        if (kAtomic) {
          int32_t* p = D + (size_t)v * kBatch + base;
          if (imp & 1u) atomicMin(p + 0, m[0]);
          if (imp & 2u) atomicMin(p + 1, m[1]);
          if (imp & 4u) atomicMin(p + 2, m[2]);
          if (imp & 8u) atomicMin(p + 3, m[3]);
        } else {
          dv[base / 4] = make_int4(imp & 1u ? m[0] : cur.x, imp & 2u ? m[1] : cur.y, imp & 4u ? m[2] : cur.z,
                                   imp & 8u ? m[3] : cur.w);
        }
      }
      if (base >= 32) hi |= imp << (base & 31);
      else lo |= imp << base;
    }
  }
  lo = __reduce_or_sync(kFull, lo);
  hi = __reduce_or_sync(kFull, hi);
  return (unsigned long long)hi << 32 | lo;
}

__global__ void __launch_bounds__(kBlock, 4) mw_pull(const int32_t* __restrict__ row_ptr,
                                                  const int32_t* __restrict__ t_row_ptr,
                                                  const int32_t* __restrict__ t_col, const int32_t* __restrict__ t_w,
                                                  int is_float, MwCtl* __restrict__ ctl, int32_t* __restrict__ D,
                                                  unsigned long long* __restrict__ masks, int32_t* __restrict__ q,
                                                  Seg* __restrict__ segs, size_t segcap,
                                                  const int32_t* __restrict__ ul, int32_t ul_n,
                                                  const int32_t* __restrict__ hv, const int32_t* __restrict__ hv_segoff,
                                                  int32_t hv_count, int32_t hv_segs, int32_t pull_seg, int32_t n) {
  __shared__ int32_t s_q[kBlock / 32][kWarpQueue];
  __shared__ int4 s_stage[kBlock / 32][32];
  if (ctl->done || ctl->mode != kModePull) return;
  const int L = ctl->level;
  const int pout = L & 1;
  const unsigned long long* __restrict__ m_in = masks + (size_t)((L - 1) % 3) * n;
  unsigned long long* m_out = masks + (size_t)(L % 3) * n;
  {
    unsigned long long* m_clr = masks + (size_t)((L + 1) % 3) * n;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride) m_clr[i] = 0ull;
  }
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const bool fl = is_float != 0;
  int4* stage = s_stage[wib];
  WarpQueue wq(s_q[wib], q + (size_t)pout * n, &ctl->qsize[pout]);
  Seg* sout = segs + (size_t)pout * segcap;
  unsigned long long* lpack = &ctl->lpack[pout];
  unsigned long long my_mf = 0;

  // heavy rows: segment tasks
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
    int32_t mn[kPullSrc];
#pragma unroll
    for (int t = 0; t < kPullSrc; t++) mn[t] = 0x7fffffff;
    pull_min(t_col, t_w, m_in, D, fl, ks, ke, stage, mn);
    const unsigned long long bits = pull_store<true>(D, v, mn);
    bool first = false;
    int deg = 0, rs = 0;
    if (bits && lane == 0) {
      first = atomicOr(m_out + v, bits) == 0ull;
      if (first) {
        rs = row_ptr[v];
        deg = row_ptr[v + 1] - rs;
        my_mf += (unsigned long long)deg;
      }
    }
    emit_routed(first, v, deg, rs, wq, sout, lpack);
  }

  // light rows: 32 list entries per warp task, one vertex after another
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&ctl->work, 32);
    base = __shfl_sync(kFull, base, 0);
    if (base >= ul_n) break;
    const int cnt = min(32, ul_n - base);
    const int32_t mine = lane < cnt ? __ldg(ul + base + lane) : -1;
    for (int j = 0; j < cnt; j++) {
      const int32_t v = __shfl_sync(kFull, mine, j);
      const int k0 = t_row_ptr[v], k1 = t_row_ptr[v + 1];
      int32_t mn[kPullSrc];
#pragma unroll
      for (int t = 0; t < kPullSrc; t++) mn[t] = 0x7fffffff;
      pull_min(t_col, t_w, m_in, D, fl, k0, k1, stage, mn);
      const unsigned long long bits = pull_store<false>(D, v, mn);
      int deg = 0, rs = 0;
      if (bits) {
        if (lane == 0) m_out[v] = bits;
        rs = row_ptr[v];
        deg = row_ptr[v + 1] - rs;
        if (lane == 0) my_mf += (unsigned long long)deg;
      }
      emit_routed(bits != 0ull && lane == 0, v, deg, rs, wq, sout, lpack);
    }
  }
  wq.flush();
  my_mf = warp_sum(my_mf);
  if (lane == 0 && my_mf) atomicAdd(&ctl->mf[pout], my_mf);
}

__global__ void mw_decide(MwCtl* __restrict__ ctl, int32_t n, long long m, int can_pull,
                          cudaGraphConditionalHandle loop, int in_graph) {
  if (threadIdx.x != 0) return;
  if (ctl->done) {
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  const int L = ctl->level, pout = L & 1;
  if (ctl->mode == kModePull) ctl->n_pull++; else ctl->n_push++;
  if ((ctl->qsize[pout] == 0 && ctl->lpack[pout] == 0) || L >= n) {
    ctl->done = 1;
    if (in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  // a frontier whose out-edges reach half the graph is relaxed by a pull
  if (ctl->force) ctl->mode = ctl->force == 2 ? kModePull : kModePush;
  else ctl->mode = can_pull && 2 * (long long)ctl->mf[pout] >= m ? kModePull : kModePush;
  ctl->work = 0;
  ctl->hwork = 0;
  ctl->qsize[pout ^ 1] = 0;
  ctl->lpack[pout ^ 1] = 0;
  ctl->mf[pout ^ 1] = 0;
  ctl->level = L + 1;
}

// Block -> the batch's source-major rows; each vertex adds its out-degree
// once per source that reached it (TEPS numerator).  A warp takes 32
// consecutive vertices: their 32 rows are 8 KB of the block in one piece,
// read with coalesced 16-byte loads (512 bytes per warp load, all sixteen
// issued before the first is waited on), transposed through a padded
// shared-memory tile and written as one 128-byte run per source row.
constexpr int kEmitBlock = 128;
constexpr int kEmitPitch = kBatch + 1;  // words per tile row: column reads hit 32 banks

__global__ void __launch_bounds__(kEmitBlock) mw_emit(MwCtl* __restrict__ ctl, const int32_t* __restrict__ D,
                                                      const int32_t* __restrict__ row_ptr, int32_t inf, int32_t n) {
  __shared__ int32_t s_tile[kEmitBlock / 32][32 * kEmitPitch];
  const int batch = ctl->batch;
  const int nb = min(kBatch, ctl->nsrc - batch * kBatch);
  int32_t* dist = ctl->dist_base + (size_t)batch * kBatch * n;
  int32_t* tile = s_tile[threadIdx.x >> 5];
  const int lane = lane_id();
  constexpr int kVecs = 32 * kBatch / 4;  // 16-byte pieces of 32 rows
  unsigned long long reached = 0;
  const size_t nwarps = (size_t)gridDim.x * (kEmitBlock / 32);
  for (size_t v0 = ((size_t)blockIdx.x * (kEmitBlock / 32) + (threadIdx.x >> 5)) * 32; v0 < (size_t)n;
       v0 += nwarps * 32) {
    const int rows = (int)min((size_t)32, (size_t)n - v0);
    const int4* src = reinterpret_cast<const int4*>(D + v0 * kBatch);
    int4 x[kVecs / 32];
#pragma unroll
    for (int i = 0; i < kVecs / 32; i++) {
      const int j = i * 32 + lane;  // piece j: row j / 16, words 4 (j % 16) ..
      x[i] = j / (kBatch / 4) < rows ? __ldcs(src + j) : make_int4(inf, inf, inf, inf);
    }
#pragma unroll
    for (int i = 0; i < kVecs / 32; i++) {
      const int j = i * 32 + lane;
      int32_t* t = tile + (j / (kBatch / 4)) * kEmitPitch + (j % (kBatch / 4)) * 4;
      t[0] = x[i].x;
      t[1] = x[i].y;
      t[2] = x[i].z;
      t[3] = x[i].w;
    }
    __syncwarp();
    int cnt = 0;
    const bool own = lane < rows;
    for (int c = 0; c < nb; c++) {
      const int32_t d = tile[lane * kEmitPitch + c];
      if (own) {
        dist[(size_t)c * n + v0 + lane] = d;
        cnt += d != inf;
      }
    }
    if (own) reached += (unsigned long long)cnt * (unsigned long long)(row_ptr[v0 + lane + 1] - row_ptr[v0 + lane]);
    __syncwarp();
  }
  reached = warp_sum(reached);
  if (lane == 0 && reached) atomicAdd(&ctl->reached, reached);
}

__global__ void mw_next(MwCtl* __restrict__ ctl) {
  if (threadIdx.x != 0) return;
  ctl->total_levels += ctl->level;
  ctl->total_push += ctl->n_push;
  ctl->total_pull += ctl->n_pull;
  ctl->batch += 1;
}

void probe_mw(const void* p, LevelProbe* out) {
  const MwCtl* c = static_cast<const MwCtl*>(p);
  const int pin = (c->level - 1) & 1;
  out->level = c->level;
  out->mode = c->mode;
  out->done = c->done;
  out->frontier = c->qsize[pin] + (int64_t)(c->lpack[pin] >> 32);
  out->frontier_edges = (int64_t)c->mf[pin];
  out->unvisited_edges = 0;
}

}  // namespace

dawn_status sssp_batched(dawn_graph* g, const int32_t* sources, int32_t nsrc, void* d_dist) {
  const int32_t n = g->n;
  const size_t nn = (size_t)n;
  const int is_float = g->wtype == DAWN_W_F32;
  const size_t segcap = seg_capacity(n, g->m);
  DAWN_CHECK(ensure(g->mw_block, sizeof(int32_t) * kBatch * nn, g->stream));
  DAWN_CHECK(ensure(g->mw_masks, sizeof(unsigned long long) * 3 * nn, g->stream));
  DAWN_CHECK(ensure(g->ss_queues, sizeof(int32_t) * 2 * nn, g->stream));
  DAWN_CHECK(ensure(g->ss_segs, sizeof(Seg) * 2 * segcap, g->stream));
  DAWN_CHECK(ensure(g->mw_ctl, sizeof(MwCtl), g->stream));
  DAWN_CHECK(ensure(g->mw_sources, sizeof(int32_t) * (size_t)nsrc, g->stream));
  // pull levels read in-edges with their weights and the in-degree lists
  DAWN_CHECK(build_weighted_in_edges(g));
  DAWN_CHECK(build_static_list(g));
  DAWN_CUDA(cudaMemcpyAsync(g->mw_sources.p, sources, sizeof(int32_t) * nsrc, cudaMemcpyHostToDevice,
                            g->stream));
  MwCtl c = {};
  c.force = g->force_variant;
  c.nsrc = nsrc;
  c.dist_base = static_cast<int32_t*>(d_dist);
  c.sources = g->mw_sources.as<int32_t>();
  DAWN_CUDA(cudaMemcpyAsync(g->mw_ctl.p, &c, sizeof(MwCtl), cudaMemcpyHostToDevice, g->stream));

  struct {
    MwCtl* ctl;
    const int32_t *row_ptr, *col, *w;
    int is_float;
    int32_t* D;
    unsigned long long* masks;
    int32_t* q;
    Seg* segs;
    size_t segcap, words, nmask;
    int32_t n, inf;
    cudaGraphConditionalHandle handle;
    int in_graph;
    const int32_t *t_row_ptr, *t_col, *t_w, *ul, *hv, *hv_segoff;
    int32_t ul_n, hv_count, hv_segs, pull_seg, can_pull;
    long long m;
  } a;
  a.t_row_ptr = g->t_row_ptr;
  a.t_col = g->wt_col.as<int32_t>();
  a.t_w = g->wt_val.as<int32_t>();  // int32 weights or float32 bit patterns, in in-edge order
  a.ul = g->ul_static.as<int32_t>();
  a.hv = g->hv_static.as<int32_t>();
  a.hv_segoff = g->hv_segoff.as<int32_t>();
  a.ul_n = g->ul_static_size;
  a.hv_count = g->hv_count;
  a.hv_segs = g->hv_segs;
  a.pull_seg = g->pull_seg;
  a.can_pull = 1;
  a.m = g->m;
  a.ctl = g->mw_ctl.as<MwCtl>();
  a.row_ptr = g->row_ptr;
  a.col = g->col;
  a.w = static_cast<const int32_t*>(g->val);  // int32 weights or float32 bit patterns
  a.is_float = is_float;
  a.D = g->mw_block.as<int32_t>();
  a.masks = g->mw_masks.as<unsigned long long>();
  a.q = g->ss_queues.as<int32_t>();
  a.segs = g->ss_segs.as<Seg>();
  a.segcap = segcap;
  a.words = kBatch * nn;
  a.nmask = 3 * nn;
  a.n = n;
  a.inf = is_float ? 0x7f7fffff : 0x7fffffff;  // FLT_MAX bits / INT32_MAX
  a.handle = 0;
  a.in_graph = 0;
  void* clear_args[] = {&a.ctl, &a.D, &a.words, &a.inf, &a.masks, &a.nmask};
  void* init_args[] = {&a.ctl, &a.row_ptr, &a.col, &a.w, &a.D, &a.masks, &a.q, &a.segs};
  void* push_args[] = {&a.row_ptr, &a.col, &a.w, &a.is_float, &a.ctl, &a.D, &a.masks, &a.q, &a.segs, &a.segcap,
                       &a.n};
  void* pull_args[] = {&a.row_ptr, &a.t_row_ptr, &a.t_col, &a.t_w, &a.is_float, &a.ctl, &a.D, &a.masks, &a.q,
                       &a.segs, &a.segcap, &a.ul, &a.ul_n, &a.hv, &a.hv_segoff, &a.hv_count, &a.hv_segs,
                       &a.pull_seg, &a.n};
  void* decide_args[] = {&a.ctl, &a.n, &a.m, &a.can_pull, &a.handle, &a.in_graph};
  void* emit_args[] = {&a.ctl, &a.D, &a.row_ptr, &a.inf, &a.n};
  void* next_args[] = {&a.ctl};
  const int sms = g->geo.sms;
  SsFamily fam;
  fam.npre = 2;
  fam.pre[0] = {(const void*)mw_clear, clear_args, dim3(sms * 8), dim3(kBlock), "mw_clear"};
  fam.pre[1] = {(const void*)mw_init, init_args, dim3(kBatch), dim3(kInitBlock), "mw_init"};
  fam.nbody = 3;
  fam.body[0] = {(const void*)mw_push, push_args,
                 dim3(persistent_blocks((const void*)mw_push, kBlock, 0, g->blocks_per_sm)), dim3(kBlock),
                 "mw_push", kModePush};
  fam.body[1] = {(const void*)mw_pull, pull_args,
                 dim3(persistent_blocks((const void*)mw_pull, kBlock, 0, g->blocks_per_sm)), dim3(kBlock),
                 "mw_pull", kModePull};
  fam.body[2] = {(const void*)mw_decide, decide_args, dim3(1), dim3(32), "mw_decide"};
  fam.npost = 2;
  fam.post[0] = {(const void*)mw_emit, emit_args, dim3(sms * 8), dim3(kEmitBlock), "mw_emit"};
  fam.post[1] = {(const void*)mw_next, next_args, dim3(1), dim3(32), "mw_next"};
  fam.ctl = a.ctl;
  fam.ctl_bytes = sizeof(MwCtl);
  fam.probe = probe_mw;
  fam.handle = &a.handle;
  fam.in_graph = &a.in_graph;
  fam.done_flag = &a.ctl->done;
  if (g->mw_exec && g->mw_exec_float != is_float) {
    cudaGraphExecDestroy(g->mw_exec);
    g->mw_exec = nullptr;
  }
  g->mw_exec_float = is_float;
  return ss_run(g, fam, (nsrc + kBatch - 1) / kBatch, &g->mw_exec);
}

dawn_status sssp_batched_stats(dawn_graph* g, dawn_stats* st, int32_t nsrc) {
  MwCtl h;
  DAWN_CUDA(cudaMemcpyAsync(&h, g->mw_ctl.p, sizeof(MwCtl), cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  st->edges_traversed = (int64_t)h.reached;
  st->levels = h.total_levels;
  st->push_levels = h.total_push;
  st->pull_levels = h.total_pull;
  st->batches = (nsrc + kBatch - 1) / kBatch;
  return DAWN_OK;
}

}  // namespace dawn
