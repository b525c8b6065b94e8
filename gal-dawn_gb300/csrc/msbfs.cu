// Batched boolean expand over bitset frontiers on sm_103a.
//
// The reference runs multi-source and all-pairs BFS as a serial loop of
// single-source traversals (src/algorithm/gpu/mssp.cu:26-43,
// src/algorithm/gpu/apsp.cu:81-100), re-reading the whole CSR once per
// source.  Here up to 64*W sources share one traversal: every vertex carries
// W uint64 words per state (visited, frontier, next), bit b of word i
// standing for source 64*i + b of the batch, so one pass over an adjacency
// row serves all of them.  The W words of a vertex are contiguous, so a
// gather of a neighbour's frontier is one 8W-byte load (one 32-byte sector
// for W = 4).  Hop distances come out identical to separate traversals: a
// source's bit appears at a vertex at level L exactly when that source
// first reaches it at L.
//
// A level runs in one of two directions, chosen on the device:
//   pull: each unfinished vertex (some source has not reached it) ORs the
//         frontier words of its in-neighbours, stopping early once every
//         missing bit is found; the vertex owns its words, so no atomics.
//         Heavy rows are cut into segments combined by the last finisher;
//   push: the active vertices' rows are dealt to warps; new bits are
//         atomicOr-ed into `next`, and an update pass folds `next` into
//         visited / frontier (over the touched list, or densely for large
//         frontiers).
// Below level kDeepLevel neither writes distances: the level at which a bit
// first appears is recorded in bit-sliced level words (slice k holds bit k
// of the level of every (source, vertex) pair), and a final pass expands
// them into the distance block with full-line coalesced stores, writing -1
// for pairs never reached.  From kDeepLevel on (high-diameter graphs, whose
// vertices gain their bits one source at a time over thousands of levels) a
// new bit is written out directly instead: one store per (source, vertex)
// pair rather than a read-modify-write of every set bit's slice, and the
// final pass leaves those entries alone.
#include <algorithm>

#include "dawn_device.cuh"
#include "selector.cuh"

namespace dawn {
namespace {

using u64 = unsigned long long;
constexpr int kMaxW = 4;

struct BsCtl {
  int32_t aq_size[3];           // active (frontier) list sizes, rotating by level % 3
  int32_t pad0;
  unsigned long long alpack[3]; // active long rows: (vertices << 32) | segments
  int32_t tq_size;              // push: vertices touched this level
  int32_t ul_size[2];           // unfinished-vertex lists (pull work lists)
  int32_t ul_cur;               // list the next pull reads: -1 = the graph's static list
  int32_t level, mode, done, policy, batch, nsrc, n_push, n_pull;
  int32_t push_ratio;           // push while push_ratio * frontier edges < unfinished edges
  int32_t work;                 // dynamic work counter of the current level (light rows)
  int32_t hwork;                // dynamic work counter of the heavy-row segments
  int32_t hs_size[2];           // heavy-segment task lists: segments of rows still unfinished
  int32_t hs_cur;               // list the next pull reads: -1 = every segment of the graph
  int32_t dense;                // push level: fire-and-forget scatter + dense update sweep
  int32_t nbits;                // level slices available
  int32_t width;                // W: words per vertex and state
  unsigned long long mf[3];     // out-degree sums of the active lists
  long long mu;                 // in-degree sum of vertices not yet finished
  long long mu_dec;             // in-degree of vertices finished this level
  unsigned long long reached;   // TEPS numerator of the batch
  unsigned long long full[kMaxW];  // this batch's source bits, less those of sources without out-edges
  int32_t* dist_base;
  const int32_t* sources;
  int32_t* lv_block;            // level mode: n x 64 levels, vertex-major (else NULL)
  int32_t* lv_range;            // level mode: per vertex, lowest and highest level reached
  unsigned long long* cc_sum;   // closeness mode: per source, sum of hop distances (else NULL)
  unsigned long long* cc_cnt;   // closeness mode: per source, vertices reached besides itself
  int32_t use_sel;              // decide with the handle's selector weights
  float sel_margin;             // log2 margin by which the selector must beat the heuristic
  int32_t force;                // 0 = decide per level; 1 + variant = always that variant
  int32_t prev_nf;              // frontier size entering the current level
  int32_t pad3;
  long long m;                  // CSR entries (selector input)
  unsigned long long total_reached;
  int32_t total_levels, total_push, total_pull, pad2;
  // 1 = the level that wrote this slot's frontier words kept no active list
  // (a dense push update: the next level is then a pull, which needs none,
  // and the slot is cleared densely when it goes stale); aq_size holds the
  // count only
  int32_t unlisted[3], pad5;
};

constexpr int kSlicesCleared = 4;  // slices zeroed per batch; higher ones on first use
// Pull rows below this many in-edges are walked by one lane each; longer
// ones are swept by the whole warp.  Packing short rows across the lanes
// (a warp scan, a shared-memory search and a shared-memory OR per edge)
// measured 4-10% slower: the pull is bound by its L1/TEX traffic, and the
// lane walk adds none beyond the column loads and the gathers.
constexpr int kPullLaneMax = 64;
constexpr int kDeepLevel = 32;     // levels from here on are written out directly
constexpr int kShallowBits = 5;    // level slices kept: the bits of levels below kDeepLevel
static_assert(kDeepLevel == 1 << kShallowBits, "slices hold exactly the levels below kDeepLevel");
// Heavy pull rows: a row of at least 2 x seg in-edges (seg = the handle's
// pull segment, 1024 by default) is cut into seg-entry warp tasks.

// Words per heavy-row accumulator: W bits and a finished-segment counter,
// rounded up to an even count so the W words start 16-byte aligned for
// the vectorised loads.
__host__ __device__ constexpr int acc_stride(int w) { return (w + 2) & ~1; }

__device__ __forceinline__ u64 warp_or64(u64 x) {
  const unsigned lo = __reduce_or_sync(kFull, (unsigned)x);
  const unsigned hi = __reduce_or_sync(kFull, (unsigned)(x >> 32));
  return ((u64)hi << 32) | lo;
}

// 32 x 32 bit transpose across a warp: lane i holds row i on entry and
// column i on exit (bit j of lane i's result = bit i of lane j's input).
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
  const int lane = lane_id();
  const uint32_t left[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int t = 0; t < 5; t++) {
    const int s = 16 >> t;
    const uint32_t y = __shfl_xor_sync(kFull, x, s);
    x = (lane & s) ? ((x & ~left[t]) | ((y & ~left[t]) >> s)) : ((x & left[t]) | ((y & left[t]) << s));
  }
  return x;
}

// W words of one vertex.
template <int W>
struct Bits {
  u64 w[W];
  __device__ __forceinline__ static Bits zero() {
    Bits b;
#pragma unroll
    for (int i = 0; i < W; i++) b.w[i] = 0ull;
    return b;
  }
  __device__ __forceinline__ static Bits full_of(const BsCtl* ctl) {
    Bits b;
#pragma unroll
    for (int i = 0; i < W; i++) b.w[i] = ctl->full[i];
    return b;
  }
  // Vectorised loads: W = 2 is one 16-byte load, W = 4 one 32-byte load
  // (a gather then asks L1/TEX for its sector once, not twice).  The
  // vertex's words start on a 32-byte boundary: slots are n x 32 bytes
  // apart from an aligned base.
  __device__ __forceinline__ static Bits ldg(const u64* p) {
    Bits b;
    if constexpr (W == 4) {
      asm("ld.global.nc.v4.u64 {%0,%1,%2,%3}, [%4];" : "=l"(b.w[0]), "=l"(b.w[1]), "=l"(b.w[2]), "=l"(b.w[3])
          : "l"(p));
    } else if (W == 1) {
      b.w[0] = __ldg(p);
    } else {
#pragma unroll
      for (int i = 0; i < W; i += 2) {
        const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p + i));
        b.w[i] = v.x;
        b.w[i + 1] = v.y;
      }
    }
    return b;
  }
  __device__ __forceinline__ static Bits ldcg(const u64* p) {
    Bits b;
    if (W == 1) {
      b.w[0] = __ldcg(p);
    } else {
#pragma unroll
      for (int i = 0; i < W; i += 2) {
        const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2*>(p + i));
        b.w[i] = v.x;
        b.w[i + 1] = v.y;
      }
    }
    return b;
  }
  __device__ __forceinline__ static Bits ld(const u64* p) {
    Bits b;
    if (W == 1) {
      b.w[0] = *p;
    } else {
#pragma unroll
      for (int i = 0; i < W; i += 2) {
        const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p + i);
        b.w[i] = v.x;
        b.w[i + 1] = v.y;
      }
    }
    return b;
  }
  __device__ __forceinline__ void st(u64* p) const {
    if (W == 1) {
      *p = w[0];
    } else {
#pragma unroll
      for (int i = 0; i < W; i += 2) *reinterpret_cast<ulonglong2*>(p + i) = make_ulonglong2(w[i], w[i + 1]);
    }
  }
  __device__ __forceinline__ Bits operator|(const Bits& o) const {
    Bits b;
#pragma unroll
    for (int i = 0; i < W; i++) b.w[i] = w[i] | o.w[i];
    return b;
  }
  __device__ __forceinline__ Bits andnot(const Bits& o) const {  // this & ~o
    Bits b;
#pragma unroll
    for (int i = 0; i < W; i++) b.w[i] = w[i] & ~o.w[i];
    return b;
  }
  __device__ __forceinline__ bool operator==(const Bits& o) const {
    bool e = true;
#pragma unroll
    for (int i = 0; i < W; i++) e &= w[i] == o.w[i];
    return e;
  }
  __device__ __forceinline__ bool any() const {
    u64 x = 0;
#pragma unroll
    for (int i = 0; i < W; i++) x |= w[i];
    return x != 0ull;
  }
  __device__ __forceinline__ int popc() const {
    int c = 0;
#pragma unroll
    for (int i = 0; i < W; i++) c += __popcll(w[i]);
    return c;
  }
  __device__ __forceinline__ Bits warp_or() const {
    Bits b;
#pragma unroll
    for (int i = 0; i < W; i++) b.w[i] = warp_or64(w[i]);
    return b;
  }
  __device__ __forceinline__ Bits shfl(int src) const {
    Bits b;
#pragma unroll
    for (int i = 0; i < W; i++) b.w[i] = __shfl_sync(kFull, w[i], src);
    return b;
  }
};

// Records the level of newly reached (source, vertex) pairs.  Below
// kDeepLevel slice k of vertex u gains nw for every set bit k of the level.
// From kDeepLevel on the level is stored at once: in the batch's distance
// rows, or in u's level row (level mode); closeness mode sums it per source
// instead (add_deep_sums).  The caller owns u.
template <int W>
__device__ __forceinline__ void record_level(const BsCtl* __restrict__ ctl, u64* __restrict__ slices, int32_t n,
                                             int32_t u, const Bits<W>& nw, int32_t level) {
  if (level < kDeepLevel) {
    for (unsigned L = (unsigned)level; L; L &= L - 1) {
      u64* p = slices + ((size_t)(__ffs(L) - 1) * n + u) * W;
      (Bits<W>::ld(p) | nw).st(p);
    }
    return;
  }
  if (ctl->cc_sum) return;
  if (ctl->lv_block) {
    int32_t* row = ctl->lv_block + (size_t)u * 64;
    for (u64 b = nw.w[0]; b; b &= b - 1) row[__ffsll((long long)b) - 1] = level;
    return;
  }
  int32_t* dist = ctl->dist_base + (size_t)ctl->batch * 64 * W * n;
#pragma unroll
  for (int i = 0; i < W; i++)
    for (u64 b = nw.w[i]; b; b &= b - 1) dist[(size_t)(64 * i + __ffsll((long long)b) - 1) * n + u] = level;
}

// Closeness mode from kDeepLevel on: adds the levels of the warp's new bits
// to the batch's per-source sums.  The warp's 32 new-bit words are
// transposed so lane j counts the bits of sources 64i + j and 64i + 32 + j
// with popc; one atomic per lane and nonzero sum.  All 32 lanes call it (nw
// zero where a lane has no vertex).
template <int W>
__device__ __forceinline__ void add_deep_sums(const BsCtl* __restrict__ ctl, const Bits<W>& nw, int32_t level) {
  const size_t row0 = (size_t)ctl->batch * 64 * W;
  const int lane = lane_id();
#pragma unroll
  for (int i = 0; i < W; i++) {
    if (!__any_sync(kFull, nw.w[i] != 0ull)) continue;
    const unsigned lo = __popc(warp_transpose32((uint32_t)nw.w[i]));
    const unsigned hi = __popc(warp_transpose32((uint32_t)(nw.w[i] >> 32)));
    if (lo) atomicAdd(ctl->cc_sum + row0 + 64 * i + lane, (unsigned long long)lo * (unsigned)level);
    if (hi) atomicAdd(ctl->cc_sum + row0 + 64 * i + 32 + lane, (unsigned long long)hi * (unsigned)level);
  }
}

// Level L is the last one before slice log2(L + 1) is first used: clear it.
template <int W>
__device__ __forceinline__ void clear_next_slice(u64* __restrict__ slices, int32_t n, int32_t level, int nbits) {
  const unsigned next = (unsigned)level + 1;
  if (next & (next - 1)) return;
  const int b = __ffs(next) - 1;
  if (b < kSlicesCleared || b >= nbits) return;
  u64* p = slices + (size_t)b * n * W;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n * W; i += stride) p[i] = 0ull;
}

template <int W>
__device__ __forceinline__ void clear_listed(u64* __restrict__ fr, const int32_t* __restrict__ list, int cnt,
                                             const Seg* __restrict__ segs, int nsegs);

// Column loads of the pull.  The in-edge columns stream through once per
// level, so they bypass L1 and are marked first to leave L2 (the frontier
// words they index are what L1 and L2 should keep).  A lane reads its short
// row 32 bytes at a time: one sector per load where two 16-byte loads
// cost two sector lookups in L1/TEX, whose sector throughput bounds the
// pull (one sector per in-edge for the gather of its frontier word).
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ int32_t ld_col(const int32_t* p, uint64_t pol) {
  int32_t v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
// p must be 32-byte aligned; the eight entries may run up to 28 bytes past
// the row (the column arrays carry 32 spare bytes).
__device__ __forceinline__ void ld_col8(const int32_t* p, uint64_t pol, int32_t (&c)[8]) {
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
      : "=r"(c[0]), "=r"(c[1]), "=r"(c[2]), "=r"(c[3]), "=r"(c[4]), "=r"(c[5]), "=r"(c[6]), "=r"(c[7])
      : "l"(p), "l"(pol));
}

// Zero the frontier words of a stale active list and its segment list
// (grid-stride).  A list that covers more than a quarter of the vertices is
// cleared as the whole slot instead: n coalesced word stores cost less than
// that many scattered partial-sector writes.
template <int W>
__device__ __forceinline__ void clear_stale(u64* __restrict__ fr, int32_t n, const int32_t* __restrict__ list,
                                            int cnt, const Seg* __restrict__ segs, int nsegs, bool unlisted) {
  if (!unlisted && (long long)cnt * 4 <= n) {
    clear_listed<W>(fr, list, cnt, segs, nsegs);
    return;
  }
  // 8-byte stores: a slot starts on an 8-byte boundary only (n * W words
  // per slot, n odd possible), and a warp's 32 of them still fill two lines.
  const size_t words = (size_t)n * W, stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < words; i += stride) fr[i] = 0ull;
}

// Zero the frontier words listed in a stale active list and its segment
// list (grid-stride).
template <int W>
__device__ __forceinline__ void clear_listed(u64* __restrict__ fr, const int32_t* __restrict__ list, int cnt,
                                             const Seg* __restrict__ segs, int nsegs) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)cnt; i += stride)
    Bits<W>::zero().st(fr + (size_t)list[i] * W);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)nsegs; i += stride)
    Bits<W>::zero().st(fr + (size_t)segs[i].v * W);
}

__global__ void __launch_bounds__(kBlock) bs_clear(u64* __restrict__ words, size_t count) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  ulonglong2* w2 = reinterpret_cast<ulonglong2*>(words);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count / 2; i += stride)
    w2[i] = make_ulonglong2(0ull, 0ull);
  if (blockIdx.x == 0 && threadIdx.x == 0 && (count & 1)) words[count - 1] = 0;
}

// One CTA of 64 W threads: thread b seeds source b of the batch.
template <int W>
__global__ void bs_init(BsCtl* __restrict__ ctl, const int32_t* __restrict__ row_ptr,
                        const int32_t* __restrict__ t_row_ptr, u64* __restrict__ visit, u64* __restrict__ fr0,
                        int32_t* __restrict__ aq0, Seg* __restrict__ segs0, int32_t n, long long m) {
  __shared__ u64 s_mf, s_reached, s_dec;
  const int b = threadIdx.x;
  const int batch = ctl->batch;
  const int per = 64 * W;
  const int nb = min(per, ctl->nsrc - batch * per);
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
    ctl->unlisted[0] = ctl->unlisted[1] = ctl->unlisted[2] = 0;
    ctl->hs_size[0] = 0;
    ctl->hs_size[1] = 0;
    ctl->hs_cur = -1;
    ctl->work = 0;
    ctl->hwork = 0;
    ctl->dense = 0;
    for (int i = 0; i < kMaxW; i++) {
      const int bits = min(64, max(0, nb - 64 * i));
      ctl->full[i] = i >= W ? 0ull : (bits == 64 ? ~0ull : ((1ull << bits) - 1ull));
    }
  }
  __syncthreads();
  int32_t s = -1;
  if (b < nb) {
    s = ctl->sources[batch * per + b];
    const u64 bit = 1ull << (b & 63);
    atomicOr(visit + (size_t)s * W + (b >> 6), bit);
    atomicOr(fr0 + (size_t)s * W + (b >> 6), bit);
    const int deg = row_ptr[s + 1] - row_ptr[s];
    atomicAdd(&s_reached, (u64)deg);
    // A source without out-edges reaches no vertex but itself.  Its bit is
    // left out of `full`, so the other vertices still finish (and leave
    // the pull lists) once every other source has reached them; a batch
    // of all vertices as sources holds many such sources.
    if (deg == 0) atomicAnd(&ctl->full[b >> 6], ~bit);
  }
  __syncthreads();
  // A vertex that is the source of several bits is queued once, by the
  // thread of its lowest bit.
  bool lowest = b < nb;
  if (lowest) {
    for (int i = 0; i < (b >> 6); i++) lowest &= fr0[(size_t)s * W + i] == 0ull;
    const u64 below = fr0[(size_t)s * W + (b >> 6)] & ((1ull << (b & 63)) - 1ull);
    lowest &= below == 0ull;
  }
  if (lowest) {
    const int rs = row_ptr[s], deg = row_ptr[s + 1] - rs;
    if (deg >= kLongRow) {
      const int nseg = (deg + kSeg - 1) / kSeg;
      const u64 old = atomicAdd(&ctl->alpack[0], (1ull << 32) | (unsigned)nseg);
      for (int j = 0; j < nseg; j++) segs0[(uint32_t)old + j] = Seg{s, rs + j * kSeg};
    } else {
      aq0[atomicAdd(&ctl->aq_size[0], 1)] = s;
    }
    atomicAdd(&s_mf, (u64)deg);
    if (Bits<W>::ld(visit + (size_t)s * W) == Bits<W>::full_of(ctl))
      atomicAdd(&s_dec, (u64)(t_row_ptr[s + 1] - t_row_ptr[s]));
  }
  __syncthreads();
  if (b == 0) {
    for (int i = 0; i < 3; i++) ctl->mf[i] = 0;
    ctl->mf[0] = s_mf;
    ctl->reached = s_reached;
    ctl->mu = m - (long long)s_dec;
    ctl->mu_dec = 0;
    ctl->level = 1;
    ctl->mode = ctl->force - 1 == kVarPull ? kModePull : kModePush;
    ctl->dense = ctl->force - 1 == kVarDense;
    ctl->prev_nf = 0;
    ctl->done = 0;
    ctl->n_push = 0;
    ctl->n_pull = 0;
  }
}

// Per-thread accumulators of a level, flushed once per warp.
struct LevelAcc {
  u64 mf = 0, reached = 0, dec = 0;
  __device__ __forceinline__ void add(u64 out_deg, u64 in_deg, int new_pairs, bool finished) {
    mf += out_deg;
    reached += out_deg * (u64)new_pairs;
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
// in-neighbours.  Heavy rows (>= 2 x pull_seg in-edges) come first, one
// pull_seg-entry segment per warp task, OR-ed into the row's accumulator;
// the warp finishing a row's last segment folds the accumulator into the
// vertex, so only one warp writes a vertex's words and every segment sees
// the same visited words for the whole level.  Light rows follow, 32 list
// entries per warp task from a shared counter: rows of >= kPullLaneMax
// entries are swept by the whole warp (4 gathers in flight per lane, early
// exit once no missing bit is left), shorter ones are walked by one lane
// each.  The list is filtered into the next unfinished list as it goes.
template <int W>
__global__ void __launch_bounds__(kBlock, W == 1 ? 5 : 4) bs_pull(const int32_t* __restrict__ row_ptr,
                                                     const int32_t* __restrict__ t_row_ptr,
                                                     const int32_t* __restrict__ t_col, BsCtl* __restrict__ ctl,
                                                     u64* __restrict__ visit, u64* __restrict__ fr,
                                                     u64* __restrict__ slices, int32_t* __restrict__ aq,
                                                     Seg* __restrict__ segs, size_t segcap,
                                                     const int32_t* __restrict__ ul_static, int32_t ul_static_size,
                                                     int32_t* __restrict__ ul, const int32_t* __restrict__ hv_static,
                                                     const int32_t* __restrict__ hv_segoff, u64* __restrict__ hv_acc,
                                                     int2* __restrict__ hv_tasks, int32_t hv_count, int32_t hv_segs,
                                                     int32_t pull_seg, int32_t n) {
  using B = Bits<W>;
  __shared__ int32_t s_qa[kBlock / 32][kWarpQueueBig];
  __shared__ int32_t s_qu[kBlock / 32][kWarpQueueBig];
  if (ctl->done || ctl->mode != kModePull) return;
  const int L = ctl->level;
  const u64* __restrict__ fin = fr + (size_t)((L - 1) % 3) * n * W;
  u64* __restrict__ fout = fr + (size_t)(L % 3) * n * W;
  int32_t* aq_out = aq + (size_t)(L % 3) * n;
  Seg* seg_out = segs + (size_t)(L % 3) * segcap;
  int32_t* aq_count = &ctl->aq_size[L % 3];
  u64* al_pack = &ctl->alpack[L % 3];
  clear_stale<W>(fr + (size_t)((L + 1) % 3) * n * W, n, aq + (size_t)((L + 1) % 3) * n, ctl->aq_size[(L + 1) % 3],
                 segs + (size_t)((L + 1) % 3) * segcap, seg_count(ctl->alpack[(L + 1) % 3]),
                 ctl->unlisted[(L + 1) % 3] != 0);
  const uint64_t pol = evict_first_policy();
  clear_next_slice<W>(slices, n, L, ctl->nbits);
  const int cur = ctl->ul_cur;
  const int32_t* ul_in = cur < 0 ? ul_static : ul + (size_t)cur * n;
  const int un = cur < 0 ? ul_static_size : ctl->ul_size[cur];
  const int nxt = cur < 0 ? 0 : cur ^ 1;
  int32_t* ul_out = ul + (size_t)nxt * n;
  int32_t* ul_count = &ctl->ul_size[nxt];
  const B full = B::full_of(ctl);
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  LevelAcc acc;
  WarpQueueBig qa(s_qa[wib], aq_out, aq_count);
  WarpQueueBig qu(s_qu[wib], ul_out, ul_count);
  const bool deep_cc = ctl->cc_sum && L >= kDeepLevel;
  // A pull level entered with a frontier of at least n / 16 vertices keeps
  // no active list: its output frontier is counted, the next level is made
  // a pull (which reads frontier words), and the slot is cleared densely
  // when it goes stale.  Smaller levels queue their output for a push.
  const long long nf_in = (long long)ctl->aq_size[(L - 1) % 3] + long_vertices(ctl->alpack[(L - 1) % 3]);
  const bool lazy = !ctl->force && nf_in * 16 >= n;
  int my_nf = 0;
  // Heavy-row segments: the first pull level deals every segment of the
  // graph (finding its row by binary search); the finisher of a row that
  // stays unfinished re-lists the row's segments as (row, segment) tasks,
  // and later pull levels deal only those.
  const int hcur = ctl->hs_cur;
  const int hn = hcur < 0 ? hv_segs : ctl->hs_size[hcur];
  const int2* __restrict__ hs_in = hv_tasks + (size_t)(hcur < 0 ? 0 : hcur) * hv_segs;
  int2* hs_out = hv_tasks + (size_t)(hcur < 0 ? 0 : hcur ^ 1) * hv_segs;
  int32_t* hs_count = &ctl->hs_size[hcur < 0 ? 0 : hcur ^ 1];

  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(&ctl->hwork, 1);
    t = __shfl_sync(kFull, t, 0);
    if (t >= hn) break;
    int lo = 0, sidx = t;
    if (hcur < 0) {
      int hi = hv_count - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(hv_segoff + mid) <= sidx) lo = mid; else hi = mid - 1;
      }
    } else {
      const int2 e = hs_in[t];
      lo = e.x;
      sidx = e.y;
    }
    const int32_t u = __ldg(hv_static + lo);
    const B vis = B::ld(visit + (size_t)u * W);
    if (vis == full) continue;
    const int s0 = __ldg(hv_segoff + lo);
    const int nseg = __ldg(hv_segoff + lo + 1) - s0;
    const int rbeg = t_row_ptr[u], rend = t_row_ptr[u + 1];
    const int ks = rbeg + (sidx - s0) * pull_seg, ke = min(ks + pull_seg, rend);
    u64* hacc = hv_acc + (size_t)lo * acc_stride(W);
    B w = B::zero();
    for (int k0 = ks; k0 < ke; k0 += 128) {
      const int k = k0 + lane;
      const int32_t v0 = k < ke ? ld_col(t_col + k, pol) : -1;
      const int32_t v1 = k + 32 < ke ? ld_col(t_col + k + 32, pol) : -1;
      const int32_t v2 = k + 64 < ke ? ld_col(t_col + k + 64, pol) : -1;
      const int32_t v3 = k + 96 < ke ? ld_col(t_col + k + 96, pol) : -1;
      if (v0 >= 0) w = w | B::ldg(fin + (size_t)v0 * W);
      if (v1 >= 0) w = w | B::ldg(fin + (size_t)v1 * W);
      if (v2 >= 0) w = w | B::ldg(fin + (size_t)v2 * W);
      if (v3 >= 0) w = w | B::ldg(fin + (size_t)v3 * W);
      if ((w.warp_or() | vis | B::ldcg(hacc)) == full) break;
    }
    w = w.warp_or();
    int last = 0;
    if (lane == 0) {
#pragma unroll
      for (int i = 0; i < W; i++)
        if (w.w[i]) atomicOr(hacc + i, w.w[i]);
      __threadfence();
      last = atomicAdd(hacc + W, 1ull) == (u64)(nseg - 1);
    }
    last = __shfl_sync(kFull, last, 0);
    if (!last) continue;
    B nw = B::zero();
    int odeg = 0, ors = 0;
    if (lane == 0) {
      __threadfence();
      B got;
#pragma unroll
      for (int i = 0; i < W; i++) {
        got.w[i] = atomicOr(hacc + i, 0ull);
        hacc[i] = 0ull;
      }
      hacc[W] = 0ull;
      nw = got.andnot(vis);
      if (nw.any()) {
        (vis | nw).st(visit + (size_t)u * W);
        nw.st(fout + (size_t)u * W);
        record_level<W>(ctl, slices, n, u, nw, L);
        ors = row_ptr[u];
        odeg = row_ptr[u + 1] - ors;
        acc.add((u64)odeg, (u64)(rend - rbeg), nw.popc(), (vis | nw) == full);
      }
    }
    // a row still missing bits keeps its segments for the next pull level
    const B nw0 = nw.shfl(0);
    if (!((vis | nw0) == full)) {
      int base = 0;
      if (lane == 0) base = atomicAdd(hs_count, nseg);
      base = __shfl_sync(kFull, base, 0);
      for (int j = lane; j < nseg; j += 32) hs_out[base + j] = make_int2(lo, s0 + j);
    }
    if (deep_cc) add_deep_sums<W>(ctl, nw, L);
    if (lazy)
      my_nf += __popc(__ballot_sync(kFull, nw.any()));
    else
      emit_routed(nw.any(), u, odeg, ors, qa, seg_out, al_pack);
  }

  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&ctl->work, 32);
    base = __shfl_sync(kFull, base, 0);
    if (base >= un) break;
    const int idx = base + lane;
    int32_t u = -1;
    B vis = full;
    if (idx < un) {
      u = ul_in[idx];
      vis = B::ld(visit + (size_t)u * W);
    }
    const bool active = !(vis == full);
    int rs = 0, re = 0;
    if (active) {
      rs = t_row_ptr[u];
      re = t_row_ptr[u + 1];
    }
    const int deg = re - rs;
    B got = B::zero();
    uint32_t big = __ballot_sync(kFull, deg >= kPullLaneMax);
    while (big) {
      const int leader = __ffs(big) - 1;
      big &= big - 1;
      const int s = __shfl_sync(kFull, rs, leader), e = __shfl_sync(kFull, re, leader);
      const B lvis = vis.shfl(leader);
      B w = B::zero();
      for (int k0 = s; k0 < e; k0 += 128) {
        const int k = k0 + lane;
        const int32_t v0 = k < e ? ld_col(t_col + k, pol) : -1;
        const int32_t v1 = k + 32 < e ? ld_col(t_col + k + 32, pol) : -1;
        const int32_t v2 = k + 64 < e ? ld_col(t_col + k + 64, pol) : -1;
        const int32_t v3 = k + 96 < e ? ld_col(t_col + k + 96, pol) : -1;
        if (v0 >= 0) w = w | B::ldg(fin + (size_t)v0 * W);
        if (v1 >= 0) w = w | B::ldg(fin + (size_t)v1 * W);
        if (v2 >= 0) w = w | B::ldg(fin + (size_t)v2 * W);
        if (v3 >= 0) w = w | B::ldg(fin + (size_t)v3 * W);
        if ((w.warp_or() | lvis) == full) break;
      }
      w = w.warp_or();
      if (lane == leader) got = w;
    }
    // Short rows: each lane walks its own row, four in-neighbours in
    // flight, and stops once its missing bits are all found.  No shared
    // memory and no search per edge: the L1/TEX path carries only the
    // column loads and the gathers.
    if (active && deg < kPullLaneMax) {
      // The row is read in 32-byte aligned chunks of eight entries, one
      // 32-byte load each (from before the row start when it is not
      // aligned; in-edge arrays carry 32 spare bytes, so no load passes
      // their end), so a lane issues one column load per eight gathers.
      B w = B::zero();
      for (int a = rs & ~7; a < re; a += 8) {
        int32_t c[8];
        ld_col8(t_col + a, pol, c);
#pragma unroll
        for (int j = 0; j < 8; j++)
          if (a + j >= rs && a + j < re) w = w | B::ldg(fin + (size_t)c[j] * W);
        if ((w | vis) == full) break;
      }
      got = w;
    }
    const B nw = active ? got.andnot(vis) : B::zero();
    const bool has = nw.any();
    const bool still = active && !((vis | nw) == full);
    int odeg = 0, ors = 0;
    if (has) {
      (vis | nw).st(visit + (size_t)u * W);
      nw.st(fout + (size_t)u * W);
      record_level<W>(ctl, slices, n, u, nw, L);
      ors = row_ptr[u];
      odeg = row_ptr[u + 1] - ors;
      acc.add((u64)odeg, (u64)deg, nw.popc(), !still);
    }
    if (deep_cc) add_deep_sums<W>(ctl, nw, L);
    qu.push(still, u);
    if (lazy)
      my_nf += __popc(__ballot_sync(kFull, has));
    else
      emit_routed(has, u, odeg, ors, qa, seg_out, al_pack);
  }
  qa.flush();
  qu.flush();
  acc.flush(ctl, L % 3);
  if (lazy) {
    if (lane == 0 && my_nf) atomicAdd(aq_count, my_nf);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->unlisted[L % 3] = 1;
  }
}

// Push, phase 1: the active vertices' rows (short rows warp-cooperatively,
// long rows as segments) are dealt to warps; bits new to a target are
// atomicOr-ed into `next` (not visited yet at that source).  In list mode
// the first toucher (claiming the target in a touched bitmap) queues it for
// phase 2; in dense mode (large frontiers) no queue is kept and phase 2
// sweeps all vertices instead.
template <int W>
__global__ void __launch_bounds__(kBlock) bs_push_scatter(const int32_t* __restrict__ row_ptr,
                                                          const int32_t* __restrict__ col, BsCtl* __restrict__ ctl,
                                                          const u64* __restrict__ visit, u64* __restrict__ fr,
                                                          u64* __restrict__ nxt, u64* __restrict__ slices,
                                                          int32_t* __restrict__ aq, const Seg* __restrict__ segs,
                                                          size_t segcap, int32_t* __restrict__ tq,
                                                          uint32_t* __restrict__ tbm, int32_t n) {
  using B = Bits<W>;
  __shared__ int s_excl[kBlock / 32][32];
  __shared__ int s_rs[kBlock / 32][32];
  __shared__ int s_v[kBlock / 32][32];
  __shared__ int32_t s_q[kBlock / 32][kWarpQueueBig];
  if (ctl->done || ctl->mode != kModePush) return;
  const int L = ctl->level;
  const u64* __restrict__ fin = fr + (size_t)((L - 1) % 3) * n * W;
  const int32_t* aq_in = aq + (size_t)((L - 1) % 3) * n;
  const Seg* seg_in = segs + (size_t)((L - 1) % 3) * segcap;
  const int qn = ctl->aq_size[(L - 1) % 3];
  const int ln = seg_count(ctl->alpack[(L - 1) % 3]);
  const bool dense = ctl->dense != 0;
  clear_stale<W>(fr + (size_t)((L + 1) % 3) * n * W, n, aq + (size_t)((L + 1) % 3) * n, ctl->aq_size[(L + 1) % 3],
                 segs + (size_t)((L + 1) % 3) * segcap, seg_count(ctl->alpack[(L + 1) % 3]),
                 ctl->unlisted[(L + 1) % 3] != 0);
  clear_next_slice<W>(slices, n, L, ctl->nbits);
  const int wib = threadIdx.x >> 5;
  // The first two levels expand the sources and their neighbours, whose
  // targets are almost never visited yet: there the visited words are not
  // read (one random load per edge fewer), and the update drops the few
  // visited bits.  Later levels filter first, which saves the atomics of
  // edges back into the visited region (half of a wavefront's edges on a
  // mesh).
  const bool filter = L > 2;
  WarpQueueBig wq(s_q[wib], tq, &ctl->tq_size);
  auto op = [&](int32_t v, int k, bool valid) {
    bool first = false;
    int32_t u = -1;
    if (valid) {
      u = __ldg(col + k);
      // No look at `next` first: its bits are OR-ed in whether or not they
      // are there, which saves a random load per edge (the scatter is bound
      // by the L1/TEX traffic of its random accesses).
      B bits = B::ldg(fin + (size_t)v * W);
      if (filter) bits = bits.andnot(B::ldcg(visit + (size_t)u * W));
      if (bits.any()) {
        if (W == 1 && !dense) {
          // one word: the OR that finds it empty is the first touch (no
          // touched bitmap to claim in and clear again)
          first = atomicOr(nxt + u, bits.w[0]) == 0ull;
        } else {
#pragma unroll
          for (int i = 0; i < W; i++)
            if (bits.w[i]) atomicOr(nxt + (size_t)u * W + i, bits.w[i]);
          if (!dense) first = claim_bit(tbm, u);
        }
      }
    }
    if (!dense) wq.push(first, u);
  };
  seg_expand(row_ptr, seg_in, ln, op);
  warp_expand(row_ptr, aq_in, qn, s_excl[wib], s_rs[wib], s_v[wib], op);
  wq.flush();
}

// Push, phase 2: fold `next` into visited / frontier / level slices, over
// the touched list (list mode, clearing the touched bitmap) or over every
// vertex (dense mode).
template <int W>
__global__ void __launch_bounds__(kBlock) bs_push_update(const int32_t* __restrict__ row_ptr,
                                                         const int32_t* __restrict__ t_row_ptr,
                                                         BsCtl* __restrict__ ctl, u64* __restrict__ visit,
                                                         u64* __restrict__ fr, u64* __restrict__ nxt,
                                                         u64* __restrict__ slices, int32_t* __restrict__ aq,
                                                         Seg* __restrict__ segs, size_t segcap,
                                                         const int32_t* __restrict__ tq, uint32_t* __restrict__ tbm,
                                                         int32_t n) {
  using B = Bits<W>;
  __shared__ int32_t s_q[kBlock / 32][kWarpQueueBig];
  if (ctl->done || ctl->mode != kModePush) return;
  const int L = ctl->level;
  u64* __restrict__ fout = fr + (size_t)(L % 3) * n * W;
  int32_t* aq_out = aq + (size_t)(L % 3) * n;
  Seg* seg_out = segs + (size_t)(L % 3) * segcap;
  const B full = B::full_of(ctl);
  const bool dense = ctl->dense != 0;
  const int tn = dense ? n : ctl->tq_size;
  // A dense level's output frontier is large enough that the next level is
  // a pull (the decide kernel makes it one), which reads frontier words,
  // not an active list: the sweep then only counts the frontier instead of
  // queueing it and cutting its long rows into segments.  Forced-variant
  // runs keep the list (a forced push reads it).
  const bool lazy = dense && !ctl->force;
  int my_nf = 0;
  WarpQueueBig wq(s_q[threadIdx.x >> 5], aq_out, &ctl->aq_size[L % 3]);
  LevelAcc acc;
  const bool deep_cc = ctl->cc_sum && L >= kDeepLevel;
  const int total = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < tn; base += total) {
    const int i = base + threadIdx.x;
    B nw = B::zero();
    int32_t u = -1;
    int odeg = 0, ors = 0;
    if (i < tn) {
      u = dense ? i : tq[i];
      if (!dense && W > 1) atomicAnd(tbm + (u >> 5), ~(1u << (u & 31)));
      const B x = B::ld(nxt + (size_t)u * W);
      if (x.any()) {
        B::zero().st(nxt + (size_t)u * W);
        const B vis = B::ld(visit + (size_t)u * W);
        nw = x.andnot(vis);
        if (nw.any()) {
          (vis | nw).st(visit + (size_t)u * W);
          nw.st(fout + (size_t)u * W);
          record_level<W>(ctl, slices, n, u, nw, L);
          ors = row_ptr[u];
          odeg = row_ptr[u + 1] - ors;
          acc.add((u64)odeg, (u64)(t_row_ptr[u + 1] - t_row_ptr[u]), nw.popc(), (vis | nw) == full);
        }
      }
    }
    if (deep_cc) add_deep_sums<W>(ctl, nw, L);
    if (lazy)
      my_nf += __popc(__ballot_sync(kFull, nw.any()));
    else
      emit_routed(nw.any(), u, odeg, ors, wq, seg_out, &ctl->alpack[L % 3]);
  }
  wq.flush();
  acc.flush(ctl, L % 3);
  if (lazy) {
    if (lane_id() == 0 && my_nf) atomicAdd(&ctl->aq_size[L % 3], my_nf);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->unlisted[L % 3] = 1;
  }
}

// Expands the level slices of one batch into its distance rows: thread per
// vertex, one store per source, consecutive vertices per warp (full lines).
// NB is the number of level bits in use (<= kShallowBits).  src is the
// batch's source list when the traversal went past kDeepLevel, else NULL:
// then a reached pair whose slice bits are all zero is either the source
// itself (level 0) or was written out during the traversal, and is kept.
template <int W, int NB>
__device__ __forceinline__ void emit_vertex(int32_t* __restrict__ dist, int32_t n, int nb_src, size_t u,
                                            const u64* __restrict__ visit, const u64* __restrict__ slices,
                                            const int32_t* __restrict__ src) {
#pragma unroll
  for (int i = 0; i < W; i++) {
    if (64 * i >= nb_src) break;
    const u64 vis = visit[u * W + i];
    u64 w[NB];
    u64 any = 0ull;
#pragma unroll
    for (int k = 0; k < NB; k++) {
      w[k] = slices[((size_t)k * n + u) * W + i];
      any |= w[k];
    }
    const int cnt = min(64, nb_src - 64 * i);
    for (int s = 0; s < cnt; s++) {
      int32_t v = -1;
      if ((vis >> s) & 1ull) {
        if (src && !((any >> s) & 1ull) && src[64 * i + s] != (int32_t)u) continue;  // written at its level
        v = 0;
#pragma unroll
        for (int k = 0; k < NB; k++) v |= (int32_t)((w[k] >> s) & 1ull) << k;
      }
      dist[(size_t)(64 * i + s) * n + u] = v;
    }
  }
}

// emit_vertex4 without deep levels (no pair was written during the
// traversal): the level of source s at vertex j is assembled from the level
// slices eight sources at a time.  Byte c of slices 0-3 goes into one word
// (slice k in byte k); for source 8c + i, ((word >> i) & 0x01010101) holds
// the four level bits at bits 0, 8, 16, 24, and multiplying by 0x01020408
// moves them to bits 24-27 without carries (every partial product lands on
// a distinct bit, and only the four wanted ones land in bits 24-31).  A
// fifth slice adds its bit separately; an unreached pair becomes -1 by
// OR-ing (bit - 1).  About 8 instructions per (source, vertex) instead of
// 19 with a shift and mask per slice.
template <int W, int NB>
__device__ __forceinline__ void emit_vertex4_packed(int32_t* __restrict__ dist, int32_t n, int nb_src, size_t u0,
                                                    const u64* __restrict__ visit,
                                                    const u64* __restrict__ slices) {
#pragma unroll
  for (int i = 0; i < W; i++) {
    if (64 * i >= nb_src) break;
    u64 vis[4], w[NB][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      vis[j] = visit[(u0 + j) * W + i];
#pragma unroll
      for (int k = 0; k < NB; k++) w[k][j] = slices[((size_t)k * n + u0 + j) * W + i];
    }
    const int cnt = min(64, nb_src - 64 * i);
    int32_t* row0 = dist + (size_t)(64 * i) * n + u0;
    for (int c = 0; c < 8 && 8 * c < cnt; c++) {
      uint32_t packed[4], five[4], vb[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        uint32_t x = 0;
#pragma unroll
        for (int k = 0; k < (NB < 4 ? NB : 4); k++) x |= (uint32_t)((w[k][j] >> (8 * c)) & 0xffull) << (8 * k);
        packed[j] = x;
        five[j] = NB > 4 ? (uint32_t)(w[NB > 4 ? 4 : 0][j] >> (8 * c)) & 0xffu : 0u;
        vb[j] = (uint32_t)(vis[j] >> (8 * c)) & 0xffu;
      }
      const int lim = min(8, cnt - 8 * c);
      for (int b = 0; b < lim; b++) {
        int32_t v[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          uint32_t x = (((packed[j] >> b) & 0x01010101u) * 0x01020408u) >> 24;
          if (NB > 4) x |= ((five[j] >> b) & 1u) << 4;
          v[j] = (int32_t)(x | (((vb[j] >> b) & 1u) - 1u));
        }
        *reinterpret_cast<int4*>(row0 + (size_t)(8 * c + b) * n) = make_int4(v[0], v[1], v[2], v[3]);
      }
    }
  }
}

// Four consecutive vertices u0..u0+3 per thread: every source row gets one
// 16-byte store, so a warp writes 512 contiguous bytes per row (needs n and
// the output base 16-byte aligned, which the caller checks).  Rows holding a
// pair written during the traversal (see emit_vertex) get scalar stores for
// the other three.
template <int W, int NB>
__device__ __forceinline__ void emit_vertex4(int32_t* __restrict__ dist, int32_t n, int nb_src, size_t u0,
                                             const u64* __restrict__ visit, const u64* __restrict__ slices,
                                             const int32_t* __restrict__ src) {
#pragma unroll
  for (int i = 0; i < W; i++) {
    if (64 * i >= nb_src) break;
    u64 vis[4], any[4];
    u64 w[NB][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      vis[j] = visit[(u0 + j) * W + i];
      any[j] = 0ull;
#pragma unroll
      for (int k = 0; k < NB; k++) {
        w[k][j] = slices[((size_t)k * n + u0 + j) * W + i];
        any[j] |= w[k][j];
      }
    }
    const int cnt = min(64, nb_src - 64 * i);
    for (int s = 0; s < cnt; s++) {
      int32_t v[4];
      bool keep[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        v[j] = -1;
        keep[j] = false;
        if ((vis[j] >> s) & 1ull) {
          int32_t x = 0;
#pragma unroll
          for (int k = 0; k < NB; k++) x |= (int32_t)((w[k][j] >> s) & 1ull) << k;
          v[j] = x;
          keep[j] = src && !((any[j] >> s) & 1ull) && src[64 * i + s] != (int32_t)(u0 + j);
        }
      }
      int32_t* row = dist + (size_t)(64 * i + s) * n + u0;
      if (!(keep[0] | keep[1] | keep[2] | keep[3])) {
        *reinterpret_cast<int4*>(row) = make_int4(v[0], v[1], v[2], v[3]);
      } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (!keep[j]) row[j] = v[j];
      }
    }
  }
}

// Closeness mode of the final pass: per source of the batch, the sum of its
// hop distances (sum over level bits k of 2^k x the vertices whose slice k
// holds the source's bit) and the vertices it reached besides itself,
// without writing distances.  Each warp transposes the words of 32
// consecutive vertices so lane j holds bit j (and j + 32) of all of them and
// counts them with popc; CTA totals go to the batch's rows with one atomic
// per source.
template <int W>
__device__ __forceinline__ void emit_closeness(const BsCtl* __restrict__ ctl, const u64* __restrict__ visit,
                                               const u64* __restrict__ slices, int32_t n, int nb, int nbits) {
  __shared__ unsigned long long s_sum[64 * W], s_cnt[64 * W];
  for (int t = threadIdx.x; t < 64 * W; t += blockDim.x) {
    s_sum[t] = 0;
    s_cnt[t] = 0;
  }
  __syncthreads();
  const int lane = lane_id();
#pragma unroll
  for (int i = 0; i < W; i++) {
    if (64 * i >= nb) break;
    unsigned long long sum_lo = 0, sum_hi = 0, cnt_lo = 0, cnt_hi = 0;
    for (int base = global_warp() * 32; base < n; base += num_warps() * 32) {
      const int u = base + lane;
      const bool in = u < n;
      const u64 vis = in ? visit[(size_t)u * W + i] : 0ull;
      cnt_lo += __popc(warp_transpose32((uint32_t)vis));
      cnt_hi += __popc(warp_transpose32((uint32_t)(vis >> 32)));
      for (int k = 0; k < nbits; k++) {
        const u64 x = in ? slices[((size_t)k * n + u) * W + i] : 0ull;
        sum_lo += (unsigned long long)__popc(warp_transpose32((uint32_t)x)) << k;
        sum_hi += (unsigned long long)__popc(warp_transpose32((uint32_t)(x >> 32))) << k;
      }
    }
    if (cnt_lo | sum_lo) {
      atomicAdd(&s_cnt[64 * i + lane], cnt_lo);
      atomicAdd(&s_sum[64 * i + lane], sum_lo);
    }
    if (cnt_hi | sum_hi) {
      atomicAdd(&s_cnt[64 * i + 32 + lane], cnt_hi);
      atomicAdd(&s_sum[64 * i + 32 + lane], sum_hi);
    }
  }
  __syncthreads();
  const size_t row0 = (size_t)ctl->batch * 64 * W;
  for (int t = threadIdx.x; t < nb; t += blockDim.x) {
    if (s_sum[t]) atomicAdd(ctl->cc_sum + row0 + t, s_sum[t]);
    if (s_cnt[t]) atomicAdd(ctl->cc_cnt + row0 + t, s_cnt[t]);
  }
}

// Level mode of the final pass (one-word batches): each vertex's levels for
// the batch's sources as one 64-word row (-1 where unreached), and the
// lowest and highest level among them (INT_MAX / -1 when none).  Entries
// written during the traversal (src set, as in emit_vertex) are kept.
template <int W>
__device__ __forceinline__ void emit_levels(const BsCtl* __restrict__ ctl, const u64* __restrict__ visit,
                                            const u64* __restrict__ slices, int32_t n, int nb, int nbits,
                                            const int32_t* __restrict__ src) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < (size_t)n; u += stride) {
    const u64 vis = visit[u * W];
    u64 any = 0ull;
    for (int k = 0; k < nbits; k++) any |= slices[((size_t)k * n + u) * W];
    int lo = 0x7fffffff, hi = -1;
    int4* row = reinterpret_cast<int4*>(ctl->lv_block + u * 64);
    for (int s0 = 0; s0 < 64; s0 += 4) {
      int32_t v[4];
      int4 old = make_int4(0, 0, 0, 0);
      if (src && (vis & ~any & (0xfull << s0))) old = row[s0 / 4];
      const int32_t kept[4] = {old.x, old.y, old.z, old.w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int s = s0 + j;
        v[j] = -1;
        if (s < nb && ((vis >> s) & 1ull)) {
          int32_t x = 0;
          if (src && !((any >> s) & 1ull) && src[s] != (int32_t)u) {
            x = kept[j];
          } else {
            for (int k = 0; k < nbits; k++) x |= (int32_t)((slices[((size_t)k * n + u) * W] >> s) & 1ull) << k;
          }
          v[j] = x;
          lo = min(lo, x);
          hi = max(hi, x);
        }
      }
      row[s0 / 4] = make_int4(v[0], v[1], v[2], v[3]);
    }
    ctl->lv_range[2 * u] = lo;
    ctl->lv_range[2 * u + 1] = hi;
  }
}

template <int W>
__global__ void __launch_bounds__(kBlock) bs_emit_dist(const BsCtl* __restrict__ ctl, const u64* __restrict__ visit,
                                                       const u64* __restrict__ slices, int32_t n) {
  const int batch = ctl->batch;
  const int per = 64 * W;
  const int nb = min(per, ctl->nsrc - batch * per);
  // levels below kDeepLevel are in the slices; deeper ones were written out
  const int nbits = min(32 - __clz(max(ctl->level, 1)), kShallowBits);
  const int32_t* src = ctl->level >= kDeepLevel ? ctl->sources + (size_t)batch * per : nullptr;
  if (ctl->lv_block) {
    if (W == 1) emit_levels<W>(ctl, visit, slices, n, min(64, ctl->nsrc - batch * 64), nbits, src);
    return;
  }
  if (ctl->cc_sum) {
    emit_closeness<W>(ctl, visit, slices, n, nb, nbits);
    return;
  }
  int32_t* dist = ctl->dist_base + (size_t)batch * per * n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if ((n & 3) == 0 && (reinterpret_cast<uintptr_t>(dist) & 15) == 0 && !src) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < (size_t)n / 4; q += stride) {
      switch (nbits) {
        case 1: emit_vertex4_packed<W, 1>(dist, n, nb, 4 * q, visit, slices); break;
        case 2: emit_vertex4_packed<W, 2>(dist, n, nb, 4 * q, visit, slices); break;
        case 3: emit_vertex4_packed<W, 3>(dist, n, nb, 4 * q, visit, slices); break;
        case 4: emit_vertex4_packed<W, 4>(dist, n, nb, 4 * q, visit, slices); break;
        default: emit_vertex4_packed<W, 5>(dist, n, nb, 4 * q, visit, slices); break;
      }
    }
    return;
  }
  if ((n & 3) == 0 && (reinterpret_cast<uintptr_t>(dist) & 15) == 0) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < (size_t)n / 4; q += stride) {
      switch (nbits) {
        case 1: emit_vertex4<W, 1>(dist, n, nb, 4 * q, visit, slices, src); break;
        case 2: emit_vertex4<W, 2>(dist, n, nb, 4 * q, visit, slices, src); break;
        case 3: emit_vertex4<W, 3>(dist, n, nb, 4 * q, visit, slices, src); break;
        case 4: emit_vertex4<W, 4>(dist, n, nb, 4 * q, visit, slices, src); break;
        default: emit_vertex4<W, 5>(dist, n, nb, 4 * q, visit, slices, src); break;
      }
    }
    return;
  }
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < (size_t)n; u += stride) {
    switch (nbits) {
      case 1: emit_vertex<W, 1>(dist, n, nb, u, visit, slices, src); break;
      case 2: emit_vertex<W, 2>(dist, n, nb, u, visit, slices, src); break;
      case 3: emit_vertex<W, 3>(dist, n, nb, u, visit, slices, src); break;
      case 4: emit_vertex<W, 4>(dist, n, nb, u, visit, slices, src); break;
      default: emit_vertex<W, 5>(dist, n, nb, u, visit, slices, src); break;
    }
  }
}

// One warp.  Ends the batch when the frontier is empty, otherwise picks
// the next level's variant: the forced one if set, else the learned
// selector if weights are loaded, else push while
// push_ratio x frontier edges < unfinished in-edges, dense once the
// frontier's edges reach n.
__global__ void bs_decide(BsCtl* __restrict__ ctl, int32_t n, const float* __restrict__ sel_w,
                          cudaGraphConditionalHandle loop, int in_graph) {
  const int lane = threadIdx.x;
  if (sel_w) sel_prefetch(sel_w);
  // every lane reads the control block before lane 0 changes it
  const int done = ctl->done;
  const int L = ctl->level;
  const int cur_mode = ctl->mode, ul_cur = ctl->ul_cur, hs_cur = ctl->hs_cur;
  const long long mu = ctl->mu - ctl->mu_dec;
  const int nf = ctl->aq_size[L % 3] + long_vertices(ctl->alpack[L % 3]);
  const bool unlisted = ctl->unlisted[L % 3] != 0;
  const long long mf = (long long)ctl->mf[L % 3];
  const int policy = ctl->policy, ratio = ctl->push_ratio, force = ctl->force, prev_nf = ctl->prev_nf;
  const bool sel = ctl->use_sel && sel_w;
  const float sel_margin = ctl->sel_margin;
  const long long m = ctl->m;
  const int per = 64 * ctl->width;
  const int nb = min(per, ctl->nsrc - ctl->batch * per);
  __syncwarp();
  if (done) {
    if (lane == 0 && in_graph) cudaGraphSetConditional(loop, 0);
    return;
  }
  if (lane == 0) {
    if (cur_mode == kModePush) {
      ctl->n_push++;
    } else {
      ctl->n_pull++;
      ctl->ul_cur = ul_cur < 0 ? 0 : ul_cur ^ 1;
      ctl->ul_size[(ul_cur < 0 ? 0 : ul_cur ^ 1) ^ 1] = 0;
      ctl->hs_cur = hs_cur < 0 ? 0 : hs_cur ^ 1;
      ctl->hs_size[(hs_cur < 0 ? 0 : hs_cur ^ 1) ^ 1] = 0;
    }
    ctl->mu = mu;
    ctl->mu_dec = 0;
    ctl->tq_size = 0;
    ctl->work = 0;
    ctl->hwork = 0;
  }
  if (nf == 0 || L >= n) {
    if (lane == 0) {
      ctl->done = 1;
      if (in_graph) cudaGraphSetConditional(loop, 0);
    }
    return;
  }
  int variant;
  if (policy == DAWN_VARIANT_PUSH || mf * ratio < mu) {
    // A push whose frontier edges reach n touches enough vertices that a
    // dense update sweep beats queueing every first touch (at n/16 the
    // sweeps of a 2048x2048 grid cost 35% more than the lists, and 6% more
    // on a kNN graph at n/1.5).
    variant = mf >= (long long)n ? kVarDense : kVarPush;
  } else {
    variant = kVarPull;
  }
  if (force) {
    variant = force - 1;
  } else if (sel) {
    float x[kSelIn];
    sel_features(x, (float)n, (float)m, (float)nf, (float)mf, (float)mu, (float)(L + 1), (float)prev_nf,
                 (float)nb);
    const unsigned allowed = policy == DAWN_VARIANT_PUSH ? (1u << kVarPush) | (1u << kVarDense) : 7u;
    variant = sel_pick(sel_w, x, allowed, variant, sel_margin);
  }
  if (unlisted) variant = kVarPull;  // no active list to push from (never with a forced variant)
  if (lane == 0) {
    // Level L+1 writes list (L+1)%3, whose stale frontier words level L cleared.
    ctl->aq_size[(L + 1) % 3] = 0;
    ctl->alpack[(L + 1) % 3] = 0;
    ctl->mf[(L + 1) % 3] = 0;
    ctl->unlisted[(L + 1) % 3] = 0;
    ctl->dense = variant == kVarDense;
    ctl->mode = variant == kVarPull ? kModePull : kModePush;
    ctl->prev_nf = nf;
    ctl->level = L + 1;
  }
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

// Static pull lists.  Light rows (0 < in-degree < 2 x seg) are swept in
// id order, 32 per warp task; heavy rows are cut into seg-entry
// segments, one warp task each, so a hub row that cannot stop early is
// spread over many warps instead of holding one warp for the whole level.
__global__ void flag_rows(const int32_t* __restrict__ t_row_ptr, int32_t n, int heavy, int seg,
                          int64_t* __restrict__ flags, int64_t* __restrict__ segs) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n; i += stride) {
    const int d = t_row_ptr[i + 1] - t_row_ptr[i];
    const bool h = d >= 2 * seg;
    flags[i] = heavy ? h : (d > 0 && !h);
    if (segs) segs[i] = h ? (d + seg - 1) / seg : 0;
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

}  // namespace

// Static pull lists of the in-edge CSR (shared with the weighted pull).
dawn_status build_static_list(dawn_graph* g) {
  if (g->ul_static.p && g->static_seg == g->pull_seg) return DAWN_OK;
  // Captured traversal graphs (bitset and weighted single-source) hold these
  // lists' addresses and sizes; a rebuild for a new segment size may move
  // or resize them.
  if (g->ul_static.p) drop_graphs(g);
  const int seg = g->pull_seg;
  const int32_t n = g->n;
  const size_t n1 = (size_t)n + 1;
  int64_t* tmp = nullptr;
  DAWN_CHECK(pool_alloc((void**)&tmp, sizeof(int64_t) * 4 * n1, g->stream));
  int64_t *flags = tmp, *pos = tmp + n1, *segs = tmp + 2 * n1, *segpos = tmp + 3 * n1;
  int64_t cnt[2] = {0, 0}, nseg = 0;
  DAWN_CHECK(ensure(g->ul_static, sizeof(int32_t) * (size_t)n, g->stream));
  DAWN_CHECK(ensure(g->hv_static, sizeof(int32_t) * (size_t)n, g->stream));
  DAWN_CHECK(ensure(g->hv_segoff, sizeof(int32_t) * n1, g->stream));
  for (int heavy = 0; heavy < 2; heavy++) {
    flag_rows<<<g->geo.sms * 4, kBlock, 0, g->stream>>>(g->t_row_ptr, n, heavy, seg, flags, heavy ? segs : nullptr);
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
  const size_t acc_bytes = sizeof(u64) * acc_stride(kMaxW) * (size_t)(cnt[1] > 0 ? cnt[1] : 1);
  DAWN_CHECK(ensure(g->hv_acc, acc_bytes, g->stream));
  DAWN_CHECK(ensure(g->hv_tasks, sizeof(int2) * 2 * (size_t)(nseg > 0 ? nseg : 1), g->stream));
  DAWN_CUDA(cudaMemsetAsync(g->hv_acc.p, 0, acc_bytes, g->stream));
  pool_free(tmp, g->stream);
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  g->ul_static_size = (int32_t)cnt[0];
  g->hv_count = (int32_t)cnt[1];
  g->hv_segs = (int32_t)nseg;
  g->static_seg = seg;
  return DAWN_OK;
}

namespace {

template <int W>
dawn_status run_width(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_dist,
                      unsigned long long* cc_sum, unsigned long long* cc_cnt, int32_t* lv_block = nullptr,
                      int32_t* lv_range = nullptr) {
  const int32_t n = g->n;
  const size_t nn = (size_t)n;
  const int wi = W == 1 ? 0 : (W == 2 ? 1 : 2);
  if (g->static_seg != g->pull_seg) {
    // the pull lists are rebuilt for a new segment size; the captured
    // graphs hold the old list sizes
    for (cudaGraphExec_t& e : g->bs_exec)
      if (e) {
        cudaGraphExecDestroy(e);
        e = nullptr;
      }
  }
  DAWN_CHECK(build_static_list(g));
  if (reinterpret_cast<uintptr_t>(g->t_col) % 32 != 0) {  // the pull's 256-bit column loads
    set_error("in-edge column array is not 32-byte aligned");
    return DAWN_ERR_CUDA;
  }
  // words (per vertex W each): visit | fr[3] | nxt | level slices[nbits]
  // lists: aq[3] | tq | ul[2] | touched bitmap ; segments[3]
  // Levels never exceed n, and levels from kDeepLevel on bypass the slices.
  const int nbits = std::min(32 - __builtin_clz((unsigned)n), kShallowBits);
  // The cached graphs hold the word buffer's address: a wider batch that
  // grows the buffer makes the narrower widths' graphs stale.
  const void* words_before = g->bs_words.p;
  DAWN_CHECK(ensure(g->bs_words, sizeof(u64) * W * (5 + (size_t)nbits) * nn, g->stream));
  if (g->bs_words.p != words_before)
    for (cudaGraphExec_t& e : g->bs_exec)
      if (e) {
        cudaGraphExecDestroy(e);
        e = nullptr;
      }
  DAWN_CHECK(ensure(g->bs_queues, sizeof(int32_t) * 6 * nn + sizeof(uint32_t) * (nn / 32 + 1), g->stream));
  const size_t segcap = seg_capacity(n, g->m);
  DAWN_CHECK(ensure(g->bs_segs, sizeof(Seg) * 3 * segcap, g->stream));
  DAWN_CHECK(ensure(g->bs_ctl, sizeof(BsCtl), g->stream));
  DAWN_CHECK(ensure(g->bs_sources, sizeof(int32_t) * (size_t)nsrc, g->stream));
  DAWN_CUDA(cudaMemcpyAsync(g->bs_sources.p, sources, sizeof(int32_t) * nsrc, cudaMemcpyHostToDevice,
                            g->stream));
  // The touched bitmap must start clear; list-mode updates clear what they set.
  DAWN_CUDA(cudaMemsetAsync(g->bs_queues.as<int32_t>() + 6 * nn, 0, sizeof(uint32_t) * (nn / 32 + 1), g->stream));
  BsCtl c = {};
  c.nsrc = nsrc;
  c.policy = DAWN_VARIANT_BITSET;
  c.push_ratio = g->bs_push_ratio;
  c.nbits = nbits;
  c.width = W;
  c.dist_base = d_dist;
  c.sources = g->bs_sources.as<int32_t>();
  c.cc_sum = cc_sum;
  c.cc_cnt = cc_cnt;
  c.lv_block = lv_block;
  c.lv_range = lv_range;
  c.use_sel = g->sel_call;
  c.sel_margin = g->sel_margin;
  c.force = g->force_variant;
  c.m = g->m;
  DAWN_CUDA(cudaMemcpyAsync(g->bs_ctl.p, &c, sizeof(BsCtl), cudaMemcpyHostToDevice, g->stream));

  struct {
    BsCtl* ctl;
    const int32_t *row_ptr, *col, *t_row_ptr, *t_col, *ul_static;
    u64 *words, *visit, *fr, *fr0, *nxt, *slices;
    int32_t *aq, *aq0, *tq, *ul;
    uint32_t* tbm;
    Seg* segs;
    size_t segcap;
    int32_t ul_static_size, hv_count, hv_segs, pull_seg;
    const int32_t *hv_static, *hv_segoff;
    u64* hv_acc;
    int2* hv_tasks;
    size_t nwords;
    int32_t n;
    long long m;
    cudaGraphConditionalHandle handle;
    int in_graph;
    const float* sel_w;
  } a;
  a.sel_w = g->sel_slot.as<float>();
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
  a.hv_tasks = g->hv_tasks.as<int2>();
  a.hv_count = g->hv_count;
  a.hv_segs = g->hv_segs;
  a.pull_seg = g->pull_seg;
  a.words = g->bs_words.as<u64>();
  a.visit = a.words;
  a.fr = a.words + W * nn;
  a.fr0 = a.fr;
  a.nxt = a.words + 4 * W * nn;
  a.slices = a.words + 5 * W * nn;
  a.aq = g->bs_queues.as<int32_t>();
  a.aq0 = a.aq;
  a.tq = a.aq + 3 * nn;
  a.ul = a.aq + 4 * nn;
  a.tbm = reinterpret_cast<uint32_t*>(a.aq + 6 * nn);
  a.segs = g->bs_segs.as<Seg>();
  a.segcap = segcap;
  a.nwords = W * (5 + (size_t)(nbits < kSlicesCleared ? nbits : kSlicesCleared)) * nn;
  a.n = n;
  a.m = g->m;
  a.handle = 0;
  a.in_graph = 0;
  void* clear_args[] = {&a.words, &a.nwords};
  void* init_args[] = {&a.ctl, &a.row_ptr, &a.t_row_ptr, &a.visit, &a.fr0, &a.aq0, &a.segs, &a.n, &a.m};
  void* pull_args[] = {&a.row_ptr, &a.t_row_ptr, &a.t_col, &a.ctl, &a.visit, &a.fr, &a.slices, &a.aq, &a.segs,
                       &a.segcap, &a.ul_static, &a.ul_static_size, &a.ul, &a.hv_static, &a.hv_segoff,
                       &a.hv_acc, &a.hv_tasks, &a.hv_count, &a.hv_segs, &a.pull_seg, &a.n};
  void* scatter_args[] = {&a.row_ptr, &a.col, &a.ctl, &a.visit, &a.fr, &a.nxt, &a.slices, &a.aq, &a.segs,
                          &a.segcap, &a.tq, &a.tbm, &a.n};
  void* update_args[] = {&a.row_ptr, &a.t_row_ptr, &a.ctl, &a.visit, &a.fr, &a.nxt, &a.slices, &a.aq, &a.segs,
                         &a.segcap, &a.tq, &a.tbm, &a.n};
  void* emit_args[] = {&a.ctl, &a.visit, &a.slices, &a.n};
  void* decide_args[] = {&a.ctl, &a.n, &a.sel_w, &a.handle, &a.in_graph};
  void* next_args[] = {&a.ctl};
  const int sms = g->geo.sms;
  SsFamily fam;
  fam.npre = 2;
  fam.pre[0] = {(const void*)bs_clear, clear_args, dim3(sms * 8), dim3(kBlock), "bs_clear"};
  fam.pre[1] = {(const void*)bs_init<W>, init_args, dim3(1), dim3(64 * W), "bs_init"};
  fam.nbody = 4;
  fam.body[0] = {(const void*)bs_pull<W>, pull_args, dim3(persistent_blocks((const void*)bs_pull<W>, kBlock, 0, g->blocks_per_sm)),
                 dim3(kBlock), "bs_pull", kModePull};
  fam.body[1] = {(const void*)bs_push_scatter<W>, scatter_args,
                 dim3(persistent_blocks((const void*)bs_push_scatter<W>, kBlock, 0, g->blocks_per_sm)), dim3(kBlock),
                 "bs_push_scatter", kModePush};
  fam.body[2] = {(const void*)bs_push_update<W>, update_args,
                 dim3(persistent_blocks((const void*)bs_push_update<W>, kBlock, 0, g->blocks_per_sm)), dim3(kBlock),
                 "bs_push_update", kModePush};
  fam.body[3] = {(const void*)bs_decide, decide_args, dim3(1), dim3(32), "bs_decide"};
  fam.npost = 2;
  fam.post[0] = {(const void*)bs_emit_dist<W>, emit_args, dim3(sms * 8), dim3(kBlock), "bs_emit_dist"};
  fam.post[1] = {(const void*)bs_next, next_args, dim3(1), dim3(32), "bs_next"};
  fam.ctl = a.ctl;
  fam.ctl_bytes = sizeof(BsCtl);
  fam.probe = probe_bs;
  if (g->l2_persist) {
    // the three rotating frontier slots: every pull level gathers from one
    fam.l2_base = a.fr;
    fam.l2_bytes = sizeof(u64) * 3 * W * nn;
  }
  fam.handle = &a.handle;
  fam.in_graph = &a.in_graph;
  fam.done_flag = &a.ctl->done;
  const int nbatches = (nsrc + 64 * W - 1) / (64 * W);
  return ss_run(g, fam, nbatches, &g->bs_exec[wi]);
}

}  // namespace

int bitset_width(const dawn_graph* g, int32_t nsrc) {
  if (g->bs_width > 0) return g->bs_width;
  if (nsrc > 128) return 4;
  if (nsrc > 64) return 2;
  return 1;
}

dawn_status bfs_bitset(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_dist,
                       unsigned long long* cc_sum, unsigned long long* cc_cnt) {
  const int w = bitset_width(g, nsrc);
  if (w == 4) return run_width<4>(g, sources, nsrc, d_dist, cc_sum, cc_cnt);
  if (w == 2) return run_width<2>(g, sources, nsrc, d_dist, cc_sum, cc_cnt);
  return run_width<1>(g, sources, nsrc, d_dist, cc_sum, cc_cnt);
}

dawn_status bfs_bitset_levels(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_levels,
                              int32_t* d_range, int32_t* h_level) {
  if (nsrc < 1 || nsrc > 64) {
    set_error("level mode takes 1 to 64 sources per call");
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CHECK(run_width<1>(g, sources, nsrc, nullptr, nullptr, nullptr, d_levels, d_range));
  // the level the batch ended on (an empty one), once the traversal is done
  DAWN_CUDA(cudaMemcpyAsync(h_level, &g->bs_ctl.as<BsCtl>()->level, sizeof(int32_t), cudaMemcpyDeviceToHost,
                            g->stream));
  return DAWN_OK;
}

dawn_status bfs_bitset_stats(dawn_graph* g, dawn_stats* st, int32_t nsrc) {
  BsCtl h;
  DAWN_CUDA(cudaMemcpyAsync(&h, g->bs_ctl.p, sizeof(BsCtl), cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  st->edges_traversed = (int64_t)h.total_reached;
  st->levels = h.total_levels;
  st->push_levels = h.total_push;
  st->pull_levels = h.total_pull;
  st->batches = (nsrc + 64 * h.width - 1) / (64 * h.width);
  return DAWN_OK;
}

}  // namespace dawn
