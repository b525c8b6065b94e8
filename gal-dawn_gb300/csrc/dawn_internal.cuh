// Internal declarations shared by the translation units of libdawn_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <vector>

#include "dawn_gb300.h"

namespace dawn {

void set_error(const char* fmt, ...);
void clear_error();

#define DAWN_CUDA(expr)                                                        \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ::dawn::set_error("%s: %s (%s:%d)", #expr, cudaGetErrorString(e_),       \
                        __FILE__, __LINE__);                                   \
      return e_ == cudaErrorMemoryAllocation ? DAWN_ERR_OOM : DAWN_ERR_CUDA;   \
    }                                                                          \
  } while (0)

#define DAWN_CHECK(expr)                                                       \
  do {                                                                         \
    dawn_status s_ = (expr);                                                   \
    if (s_ != DAWN_OK) return s_;                                              \
  } while (0)

constexpr uint32_t kFull = 0xffffffffu;
constexpr int kBlock = 256;  // threads per CTA of the frontier kernels

// Device buffer owned by a graph handle; grows on demand, never shrinks.
// Storage comes from the device's stream-ordered memory pool, which keeps
// freed blocks, so creating and destroying handles repeatedly does not go
// back to the driver each time.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};
dawn_status ensure(DevBuf& b, size_t bytes, cudaStream_t s);
void release(DevBuf& b);
dawn_status pool_alloc(void** p, size_t bytes, cudaStream_t s);
// Small page-locked host slots (up to kPinnedSlot bytes) for a handle's
// control-block copies, carved from chunks that live until the process
// exits: creating and destroying a handle then never calls cudaFreeHost,
// which waits for the whole device, so handles on other streams keep
// running while one is destroyed.
constexpr size_t kPinnedSlot = 512;
dawn_status pinned_slot(void** p);
void pinned_slot_release(void* p);
void pool_free(void* p, cudaStream_t s);

// --- single-source frontier traversal (BOVM push/pull, GOVM push) ---------

// kModeSmall: small frontiers, several push levels in one cluster launch
enum : int32_t { kModePush = 0, kModePull = 1, kModeSmall = 2 };
// Launch tag of a kernel that runs at push and at pull levels alike.
constexpr int32_t kModeStep = 3;

// Device-resident control block of one single-source traversal.  Every
// per-level kernel reads its parameters from here, so the same launches
// (and the same captured CUDA graph) serve every level and every source.
struct SsCtl {
  int32_t qsize[2];             // frontier queue sizes by level parity (short rows)
  unsigned long long lpack[2];  // long rows: (vertices << 32) | segments, by parity
  unsigned long long mf[2];     // out-degree sum of each queue
  long long mu;                 // degree sum of still-unvisited vertices
  unsigned long long reached;   // TEPS numerator of this source
  int32_t level;                // level the next kernels compute
  int32_t mode;                 // kModePush / kModePull for that level
  int32_t done;                 // set when the frontier is empty
  int32_t prev_nf;              // frontier size of the previous level
  int32_t n_push, n_pull;       // per-source mode counters
  int32_t src_idx;              // index into the source list
  int32_t source;               // current source vertex
  int32_t policy;               // DAWN_VARIANT_PUSH or DAWN_VARIANT_DO
  int32_t weighted;             // GOVM: 0 int32, 1 float32 distances
  int32_t err;                  // first device-side error code (0 = none)
  int32_t nsrc;                 // sources of the current call
  // per-call parameters (host-written before the first launch)
  int32_t* dist_base;           // nsrc x n output, row src_idx is current
  const int32_t* sources;       // device copy of the source list
  int32_t use_sel;              // decide with the handle's selector weights
  int32_t force;                // 0 = decide per level; 1 + variant = always that variant
  float sel_margin;             // log2 margin by which the selector must beat the heuristic
  int32_t work;                 // weighted pull: dynamic work counter (light rows)
  int32_t hwork;                // weighted pull: dynamic work counter (heavy-row segments)
  int32_t small;                // single-source BFS: 1 = small frontiers may run as cluster levels
  long long m;                  // CSR entries (selector input)
  // accumulated over all sources of the call
  unsigned long long total_reached;
  int32_t total_levels, total_push, total_pull;
  int32_t arrive;               // CTAs of the running level kernel that finished (last one resets it)
};

// Kernel launches of one frontier-traversal family.  The driver runs them as
// one CUDA graph per source (or per source batch):
//   pre[0] -> ... -> while(cond){ body[0] -> ... -> body[nbody-1] } -> post[0] -> ...
// where the last body kernel ("decide") ends the loop through
// cudaGraphSetConditional.  When conditional graphs are unavailable the
// same sequence runs from a host loop that polls the `done` word.
struct Launch {
  const void* fn = nullptr;
  void** args = nullptr;
  dim3 grid, block;
  const char* name = "";
  int mode = -1;  // traced form: launch only at levels of this mode (-1 always)
  size_t smem = 0;  // dynamic shared memory per CTA
};

// Frontier statistics a family exposes to the traced form (read from a
// host copy of its control block before every level).
struct LevelProbe {
  int32_t level, mode, done;
  int64_t frontier, frontier_edges, unvisited_edges;
};
struct SsFamily {
  Launch pre[2];
  int npre = 0;
  Launch body[5];
  int nbody = 0;
  // true: every body kernel ends its level with the bookkeeping itself;
  // false: the last body kernel is the decide kernel, run at every level
  bool decide_in_body = false;
  Launch post[2];
  int npost = 0;
  // the decide kernel (body[nbody-1]) takes these two arguments
  cudaGraphConditionalHandle* handle = nullptr;
  int* in_graph = nullptr;
  // device address of the int32 `done` flag polled by the host loop
  const void* done_flag = nullptr;
  // L2 persisting window for the body kernels (hot arrays re-read at every
  // level); l2_bytes = 0: none
  const void* l2_base = nullptr;
  size_t l2_bytes = 0;
  // traced form: the control block and how to read it
  const void* ctl = nullptr;
  size_t ctl_bytes = 0;
  void (*probe)(const void* ctl, LevelProbe* out) = nullptr;
};

// One task of the multi-graph traversal: up to 64 sources of one part.
struct PartTask {
  int32_t part;    // part index
  int32_t src0;    // first source, an index into the call's source list
  int32_t nsrc;    // sources in the task (1..64)
  int32_t pad;
  long long out0;  // output offset of the task's first distance row
};
// One distance row of the multi-graph output (closeness reduction).
struct PartRow {
  long long off;   // output offset
  int32_t len;     // the part's vertex count
  int32_t part;
};
constexpr int32_t kPartMaxVertices = DAWN_PART_MAX_VERTICES;

// Launch geometry for persistent grids on this device.
struct Geometry {
  int sms = 0;
  int blocks_push = 0, blocks_pull = 0, blocks_relax = 0, blocks_bitset = 0;
};

}  // namespace dawn

struct dawn_graph {
  int device = 0;
  int32_t n = 0;
  int64_t m = 0;
  uint32_t flags = 0;
  dawn_wtype wtype = DAWN_W_NONE;
  bool symmetric = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  dawn::Geometry geo;

  // CSR (out-edges) and in-edge CSR for pull sweeps (aliases when symmetric)
  int32_t* row_ptr = nullptr;
  int32_t* col = nullptr;
  void* val = nullptr;
  int32_t* t_row_ptr = nullptr;
  int32_t* t_col = nullptr;

  // single-source workspace
  dawn::DevBuf ss_queues;   // 2 x n int32 short-row queues
  dawn::DevBuf ss_segs;     // 2 x seg_capacity long-row segments
  dawn::DevBuf ss_bitmaps;  // visited + 3 frontier bitmaps (words)
  dawn::DevBuf ss_ctl;      // SsCtl
  dawn::DevBuf ss_sources;  // int32 source list of the current call
  dawn::DevBuf ss_scratch;  // n x u64 (GOVM source-row resolution)
  dawn::DevBuf bc_levels;   // betweenness: n x 64 int32 levels of a batch
  dawn::DevBuf bc_terms;    // n x 64 float (1 / amount + dependency)
  dawn::DevBuf bc_range;    // 2 x n int32 lowest / highest level per vertex
  dawn::DevBuf bc_out;      // n double (host-pointer calls)
  dawn::DevBuf bc_heavy;    // rows cut into segments: out-rows (ids, segment prefix), in-rows (same)
  dawn::DevBuf bc_part;     // per-segment partial sums (float) / per-heavy-row counts (int32), 64 each
  int32_t bc_hout = -1, bc_segs_out = 0, bc_hin = 0, bc_segs_in = 0;  // -1: lists not built
  int32_t* bc_h_level = nullptr;  // pinned: the end level of the two batches in flight
  dawn::DevBuf mw_block;    // batched weighted traversal: n x 64 int32 distances
  dawn::DevBuf mw_masks;    // 3 x n uint64 improved-source masks
  dawn::DevBuf mw_ctl;
  dawn::DevBuf mw_sources;
  dawn::DevBuf wt_col;      // weighted in-edge CSR (rows of t_row_ptr): tail vertex
  dawn::DevBuf wt_val;      // and weight of each in-edge, built on the first weighted pull
  dawn::SsCtl* h_ctl = nullptr;  // pinned: [0] upload staging, [1] download
  bool graphs_ok = true;         // conditional CUDA graphs usable

  // batched bitset workspace
  dawn::DevBuf bs_words;    // visit / frontier / next words
  dawn::DevBuf bs_queues;   // active + touched queues
  dawn::DevBuf bs_ctl;
  dawn::DevBuf bs_sources;
  dawn::DevBuf bs_segs;         // 3 x seg_capacity long-row segments
  dawn::DevBuf ul_static;       // light pull rows: 0 < in-degree < kPullHeavy, id order
  int32_t ul_static_size = 0;
  dawn::DevBuf hv_static;       // heavy pull rows: in-degree >= kPullHeavy, id order
  dawn::DevBuf hv_segoff;       // exclusive prefix of their segment counts (nh + 1)
  dawn::DevBuf hv_acc;          // per heavy row: OR accumulator + finished-segment count
  dawn::DevBuf hv_tasks;        // 2 x hv_segs (row, segment): segments of heavy rows still unfinished
  int32_t hv_count = 0, hv_segs = 0;
  int32_t bs_push_ratio = 4;    // push while ratio * frontier edges < unfinished edges
  int32_t bs_width = 0;         // words per vertex of the bitset traversal (0 = by source count)
  int32_t force_variant = 0;    // 0 = decide per level, else 1 + variant for every level
  int32_t blocks_per_sm = 0;    // CTAs per SM of the persistent traversal grids (0 = occupancy limit)
  int32_t pull_seg = 1024;      // heavy pull rows: in-edges per warp task (rows of >= 2x are cut)
  int32_t static_seg = 0;       // pull_seg the static pull lists were built with
  bool auto_learned = false;    // DAWN_VARIANT_AUTO batched calls use the learned selector
  bool l2_persist = false;      // DAWN_OPT_L2_PERSIST: persisting L2 window on the frontier words
  bool small_levels = true;     // DAWN_OPT_SMALL_LEVELS: small frontiers as cluster levels
  // Learned selector.  The decide kernels take the slot's address as a
  // launch argument (fixed for the handle's life, so captured graphs stay
  // valid) and prefetch it while they read the control block.
  dawn::DevBuf sel_slot;        // weights the next call evaluates
  int32_t sel_slot_state = 0;   // 0 nothing loaded, 1 the handle's own, 2 the library's defaults
  std::vector<float> sel_user;  // dawn_graph_set_selector weights (host copy)
  bool sel_on = false;
  int32_t sel_call = 0;         // the running call uses the slot
  float sel_margin = 0.0f;      // DAWN_OPT_SELECTOR_MARGIN / 1000

  // disjoint-union parts (dawn_graph_set_parts)
  std::vector<int32_t> pt_off;   // nparts + 1 vertex offsets (empty: no parts)
  std::vector<long long> pt_pos; // row_ptr at those offsets (edge positions)
  dawn::DevBuf pt_voff, pt_tasks, pt_sources, pt_ctl, pt_scratch, pt_rows;
  size_t pt_slot_words = 0;
  int32_t pt_slots = 0, pt_maxn = 0;
  int32_t pt_cluster = 1;  // CTAs per task of the multi-graph launch
  cudaGraphExec_t pt_exec = nullptr;

  // closeness reduction
  dawn::DevBuf cc_out;

  // distance staging for host-pointer calls
  dawn::DevBuf dist_stage;

  // captured single-source traversal graphs (one per kernel family)
  cudaGraphExec_t bfs_exec = nullptr;
  cudaGraphExec_t sssp_exec = nullptr;
  int32_t sssp_exec_weighted = -1;
  cudaGraphExec_t mw_exec = nullptr;  // batched weighted traversal
  int32_t mw_exec_float = -1;
  cudaGraphExec_t bs_exec[3] = {nullptr, nullptr, nullptr};  // bitset width 1, 2, 4

  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // per-level trace (dawn_trace_enable)
  bool trace = false;
  std::vector<dawn_trace_rec> trace_log;
  cudaEvent_t trace_ev[10] = {};
};

namespace dawn {

// bovm.cu
dawn_status bfs_single(dawn_graph* g, const int32_t* sources, int32_t nsrc,
                       int32_t* d_dist, int32_t policy);
// abi.cu: whether a call of this variant evaluates the learned selector
// (and loads its weights into the handle's slot); *use = 0 or 1.
dawn_status call_selector(dawn_graph* g, int32_t variant, int32_t* use);
void drop_graphs(dawn_graph* g);

// tune.cu
dawn_status autotune(dawn_graph* g, const int32_t* sources, int32_t nsrc,
                     uint32_t flags, dawn_tuning* out);
dawn_status tune_cache_save(const char* path);
dawn_status tune_cache_load(const char* path);

// msssp.cu: weighted distances of up to 64 sources per batched traversal
// (d_dist nsrc x n, the single-source encoding)
dawn_status sssp_batched(dawn_graph* g, const int32_t* sources, int32_t nsrc, void* d_dist);
dawn_status sssp_batched_stats(dawn_graph* g, dawn_stats* st, int32_t nsrc);

// bc.cu: BCDAWN betweenness summed over the sources into d_bc (n doubles).
dawn_status betweenness(dawn_graph* g, const int32_t* sources, int32_t nsrc, double* d_bc, dawn_stats* st);

// parts.cu
dawn_status parts_set(dawn_graph* g, int32_t nparts, const int32_t* offsets);
dawn_status parts_bfs(dawn_graph* g, const int32_t* source_offset,
                      const int32_t* sources, int32_t* d_dist,
                      std::vector<PartRow>* rows_out, dawn_stats* st);
dawn_status parts_row_reduce(dawn_graph* g, const int32_t* d_dist,
                             const std::vector<PartRow>& rows, long long* h_sum,
                             long long* h_cnt);

dawn_status bfs_static(const int32_t* row_ptr, const int32_t* col, int32_t n,
                       int64_t m, int32_t source, int32_t* dist, uint32_t flags,
                       cudaStream_t stream);
// msbfs.cu
// d_dist (nsrc x n) receives the distances; or, with cc_sum / cc_cnt set
// (zeroed by the caller, nsrc entries each), each source's hop-distance sum
// and reached count accumulate there and no distances are written.
dawn_status bfs_bitset(dawn_graph* g, const int32_t* sources, int32_t nsrc,
                       int32_t* d_dist, unsigned long long* cc_sum = nullptr,
                       unsigned long long* cc_cnt = nullptr);
dawn_status bfs_bitset_stats(dawn_graph* g, dawn_stats* st, int32_t nsrc);
// One batch of at most 64 sources: levels as n x 64 int32 rows (vertex-major,
// -1 unreached), per vertex the lowest and highest level (2 x n int32).
// Enqueued only: the level the batch ended on (the deepest level + 1) is
// copied to *h_level (pinned host memory) behind the traversal.
dawn_status bfs_bitset_levels(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_levels,
                              int32_t* d_range, int32_t* h_level);
int bitset_width(const dawn_graph* g, int32_t nsrc);
// govm.cu
dawn_status sssp_single(dawn_graph* g, const int32_t* sources, int32_t nsrc,
                        void* d_dist);
// runtime.cu
dawn_status ss_run(dawn_graph* g, SsFamily& fam, int32_t nsrc,
                   cudaGraphExec_t* exec_cache);
dawn_status upload_ctl(dawn_graph* g, const SsCtl& c);
dawn_status download_ctl(dawn_graph* g, SsCtl* out);
// CTAs of a persistent grid: the SM count times the resident CTAs per SM,
// capped at `cap` per SM when cap > 0.
int persistent_blocks(const void* fn, int block, size_t smem, int cap = 0);
// Whether one cluster of `ctas` CTAs of `threads` threads of kernel fn (its
// cluster shape fixed at compile time) can be resident on the current
// device; the answer is kept per kernel for the process.
bool cluster_fits(const void* fn, int ctas, int threads);
dawn_status build_transpose(dawn_graph* g);
// In-edge tails and weights in the row layout of t_row_ptr (g->wt_col, g->wt_val).
dawn_status build_weighted_in_edges(dawn_graph* g);
// msbfs.cu: light/heavy in-degree lists of the pull kernels (g->ul_static, g->hv_*).
dawn_status build_static_list(dawn_graph* g);
// Per-row reductions over a distance block (kind 0 hops, 1 int32, 2 float):
// with degree = 0, d_sum gets the exact sum of reached distances of v != s
// (int64 bits for kinds 0/1, float64 for kind 2) and d_cnt their count;
// with degree = 1, d_sum gets (int64 bits) the out-degree sum of the
// reached vertices, source included: the TEPS numerator.
dawn_status row_reduce(dawn_graph* g, const void* d_dist, int32_t nsrc,
                       const int32_t* d_sources, int kind, int degree,
                       double* d_sum, long long* d_cnt);
const char* last_error();
dawn_status validate_csr(dawn_graph* g);
dawn_status exclusive_scan_i64(const int64_t* d_in, int64_t* d_out, int64_t n,
                               cudaStream_t s);

}  // namespace dawn
