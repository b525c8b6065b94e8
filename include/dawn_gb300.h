/* dawn_gb300.h — C ABI of the GB300-native DAWN frontier path.
 *
 * These entry points replace the device side of GAL-DAWN's GPU algorithms.
 * They take plain pointers and sizes (no C++ or torch types), return a
 * status code on every call and keep device state behind an opaque graph
 * handle.  Citations are to the reference project's files.
 *
 * Encodings
 *   hop distance   int32, -1 = unreachable, 0 = the source itself.  The
 *                  reference stores 0 for both (src/algorithm/cpu/bfs.cpp:62);
 *                  the C++ host layer converts back for its text output.
 *   int32 weights  int32 distance, INT32_MAX = unreachable.
 *   float weights  float distance, FLT_MAX = unreachable, as the reference
 *                  (src/algorithm/cpu/sssp.cpp:36).
 *   dist arrays    row-major nsrc x n: row i belongs to sources[i].
 *
 * Threading: a graph handle is not thread safe; calls on one handle are
 * ordered on its CUDA stream.  Different handles may be used concurrently.
 */
#ifndef DAWN_GB300_H
#define DAWN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t dawn_status;
#define DAWN_OK 0
#define DAWN_ERR_INVALID_ARG 1 /* bad pointer, size, CSR or source id */
#define DAWN_ERR_OOM 2         /* device allocation failed */
#define DAWN_ERR_CUDA 3        /* a CUDA runtime call failed */
#define DAWN_ERR_TIMEOUT 4     /* a bounded device wait gave up */
#define DAWN_ERR_UNSUPPORTED 5 /* variant / weight type not available */

typedef enum dawn_wtype {
  DAWN_W_NONE = 0, /* unweighted */
  DAWN_W_I32 = 1,  /* int32 edge weights */
  DAWN_W_F32 = 2   /* float32 edge weights (non-negative) */
} dawn_wtype;

/* dawn_graph_create flags */
#define DAWN_GRAPH_SYMMETRIC 1u   /* every edge is stored in both directions */
#define DAWN_GRAPH_NO_VALIDATE 2u /* skip the O(n + m) CSR validation pass */

/* Traversal variants (the result never depends on the variant). */
#define DAWN_VARIANT_AUTO 0    /* library choice: BITSET for >= 2 sources */
#define DAWN_VARIANT_PUSH 1    /* single source, top-down queue every level */
#define DAWN_VARIANT_DO 2      /* single source, push/pull by heuristic */
#define DAWN_VARIANT_BITSET 3  /* batched: 64 sources per uint64 frontier word */
#define DAWN_VARIANT_LEARNED 4 /* batched; each level's variant picked by the learned
                                  selector (dawn_graph_set_selector weights,
                                  else the library's trained ones) */

typedef struct dawn_stats {
  int64_t edges_traversed; /* TEPS numerator: sum over sources of the CSR
                              entries whose tail vertex was reached */
  int32_t levels;          /* frontier iterations, summed over batches */
  int32_t push_levels;     /* iterations that ran a push (top-down) kernel */
  int32_t pull_levels;     /* iterations that ran a pull (bottom-up) kernel */
  int32_t batches;         /* source batches (single-source: = nsrc) */
  float device_ms;         /* CUDA-event time of the traversal only */
} dawn_stats;

typedef struct dawn_graph dawn_graph;

/* Uploads a host CSR (row_ptr[n+1], col[m], optional val[m]) to the current
 * CUDA device.  Replaces the per-call thrust::copy_n of the CSR in
 * BFS_GPU::run (src/algorithm/gpu/bfs.cu:115-118), SSSP_GPU::run
 * (src/algorithm/gpu/sssp.cu:139-144) and MSSP_GPU::run
 * (src/algorithm/gpu/mssp.cu:14-17, 58-63): the graph stays resident for
 * any number of traversals.  stream may be NULL (library-owned stream). */
dawn_status dawn_graph_create(const int32_t* row_ptr, const int32_t* col,
                              const void* val, dawn_wtype wtype, int32_t n,
                              int64_t m, uint32_t flags, void* stream,
                              dawn_graph** out);

/* As dawn_graph_create, from device-resident arrays (copied device to
 * device; the caller keeps ownership of its buffers). */
dawn_status dawn_graph_create_device(const int32_t* d_row_ptr,
                                     const int32_t* d_col, const void* d_val,
                                     dawn_wtype wtype, int32_t n, int64_t m,
                                     uint32_t flags, void* stream,
                                     dawn_graph** out);

/* Frees every device buffer of the handle.  Replaces the thrust
 * device_vector destructors at the end of each reference run(). */
dawn_status dawn_graph_destroy(dawn_graph* g);

/* Sets the CUDA stream later calls are ordered on (NULL = library stream). */
dawn_status dawn_graph_set_stream(dawn_graph* g, void* stream);

/* Waits for the handle's stream. */
dawn_status dawn_graph_synchronize(dawn_graph* g);

/* Hop distances from nsrc sources (host arrays; dist is nsrc x n int32).
 * Replaces BFS_GPU::kernel + SOVM (src/algorithm/gpu/bfs.cu:9-105) for one
 * source, and the per-source loops of MSSP_GPU::run
 * (src/algorithm/gpu/mssp.cu:9-51) and APSP_GPU::run
 * (src/algorithm/gpu/apsp.cu:62-111) for many.  Sources must lie in [0, n);
 * isolated sources are legal (their row holds only the 0 at the source).
 * dist may be NULL: the traversal runs and only the statistics come back
 * (the reference's MSSP/APSP drivers discard the distances the same way
 * unless printing).  stats may be NULL. */
dawn_status dawn_bfs(dawn_graph* g, const int32_t* sources, int32_t nsrc,
                     int32_t* dist, int32_t variant, dawn_stats* stats);

/* As dawn_bfs with dist in device memory (nsrc x n).  Asynchronous on the
 * handle's stream when stats is NULL. */
dawn_status dawn_bfs_device(dawn_graph* g, const int32_t* sources,
                            int32_t nsrc, int32_t* d_dist, int32_t variant,
                            dawn_stats* stats);

/* Single-source hop distances that allocate nothing (no counterpart in
 * the reference: every reference driver allocates its own device arrays per
 * call, src/algorithm/gpu/bfs.cu:36-46).  For callers that may not allocate
 * while they traverse: a serving loop whose device memory is owned entirely
 * by another allocator, or one that must not wait on an allocation, which
 * can synchronise the device or fail under fragmentation.
 *   row_ptr (n + 1), col (m) and dist (n) are memory of the calling
 *   thread's current device; no handle is needed.  dist receives the hop
 *   distance of every vertex from source, -1 where unreachable: the same
 *   values as dawn_bfs / dawn_bfs_device on a handle of the same CSR.
 *   Top-down (push) levels only.  flags: DAWN_GRAPH_NO_VALIDATE skips the
 *   CSR check that otherwise runs first.  stream orders the work (NULL: the
 *   default stream); the call returns once the traversal has finished.
 * Working memory is one fixed block of device memory per GPU, declared by
 * the library (about 12.5 MiB, held on each GPU once the library's
 * kernels are loaded there, until the process exits), so a graph is limited to
 * DAWN_STATIC_MAX_VERTICES vertices and DAWN_STATIC_MAX_EDGES edges; larger
 * ones are rejected with DAWN_ERR_INVALID_ARG.  The first call on a device
 * looks up that device's block.  Calls that overlap on one device (two host
 * threads, or two streams) share the block and race: serialise them. */
#define DAWN_STATIC_MAX_VERTICES (1 << 20)
#define DAWN_STATIC_MAX_EDGES (1LL << 24)
dawn_status dawn_bfs_static(const int32_t* row_ptr, const int32_t* col,
                            int32_t n, int64_t m, int32_t source,
                            int32_t* dist, uint32_t flags, void* stream);

/* BCDAWN betweenness: for each vertex, the sum over `sources` of the
 * reference's dependency (src/algorithm/cpu/bc.cpp:9-191, the CPU-only
 * BC_CPU::Betweenness_Centrality, which takes every vertex as a source).
 * With levels counted from a source s, a vertex c at level >= 2 splits 1
 * equally over its predecessor entries (CSR entries j -> c with level(j) =
 * level(c) - 1, duplicates counted), and each predecessor also receives
 * c's own dependency in full.  bc (host, n doubles) receives the sums;
 * pass every vertex as a source for the reference's result.  The terms are
 * float32 like the reference's; they agree with it to float rounding.
 * Sources go 64 per batched traversal. */
dawn_status dawn_betweenness(dawn_graph* g, const int32_t* sources,
                             int32_t nsrc, double* bc, dawn_stats* stats);
dawn_status dawn_betweenness_device(dawn_graph* g, const int32_t* sources,
                                    int32_t nsrc, double* d_bc,
                                    dawn_stats* stats);

/* Many independent graphs in one call (no counterpart in the reference,
 * which traverses one graph per MSSP_GPU::run, src/algorithm/gpu/mssp.cu:9-51).
 * The handle's graph is declared the disjoint union of nparts graphs:
 * part p owns the vertices [offsets[p], offsets[p+1]) (offsets: host,
 * nparts + 1 entries, from 0 to n) and no edge may leave its part (checked
 * unless the handle was created with DAWN_GRAPH_NO_VALIDATE).  A part holds
 * at most DAWN_PART_MAX_VERTICES vertices. */
#define DAWN_PART_MAX_VERTICES (1 << 18)
dawn_status dawn_graph_set_parts(dawn_graph* g, int32_t nparts,
                                 const int32_t* offsets);

/* Hop distances from the sources of every part, all parts in one
 * persistent launch.  source_offset (host, nparts + 1, from 0) delimits
 * each part's sources in `sources`, which hold part-local vertex ids.  dist
 * receives, part after part, a (sources of p) x (vertices of p) int32 block
 * in part-local ids, -1 where unreachable: the values dawn_bfs gives on
 * each part as a graph of its own.  stats->batches counts the
 * (part, 64-source) tasks. */
dawn_status dawn_multi_bfs(dawn_graph* g, const int32_t* source_offset,
                           const int32_t* sources, int32_t* dist,
                           dawn_stats* stats);
dawn_status dawn_multi_bfs_device(dawn_graph* g, const int32_t* source_offset,
                                  const int32_t* sources, int32_t* d_dist,
                                  dawn_stats* stats);

/* Closeness of each (part, source): (n_p - 1) / sum of the hop distances
 * to the vertices the source reaches in its part, as dawn_closeness
 * computes it on the part alone.  cc, dist_sum and reached are indexed like
 * `sources`; dist_sum and reached may be NULL. */
dawn_status dawn_multi_closeness(dawn_graph* g, const int32_t* source_offset,
                                 const int32_t* sources, double* cc,
                                 double* dist_sum, int64_t* reached,
                                 dawn_stats* stats);

/* Weighted shortest-path distances (min-plus relax).  dist is nsrc x n of
 * int32 (DAWN_W_I32 graphs) or float (DAWN_W_F32 graphs).  Replaces
 * SSSP_GPU::kernel + GOVM (src/algorithm/gpu/sssp.cu:18-129) and
 * MSSP_GPU::run_Weighted (src/algorithm/gpu/mssp.cu:53-102).  The source's
 * own row initialises its neighbours with the last CSR entry of a repeated
 * neighbour, as the reference CPU path does (src/algorithm/cpu/sssp.cpp:41-45).
 * As with dawn_bfs, a NULL dist returns only the statistics.
 * variant: DAWN_VARIANT_PUSH or DAWN_VARIANT_DO run one traversal per
 * source; any other value (AUTO) runs two or more sources 64 per batched
 * traversal (a vertex-major 64-distance block, one relaxation pass per
 * edge for all sources of the batch).  The distances are the same. */
dawn_status dawn_sssp(dawn_graph* g, const int32_t* sources, int32_t nsrc,
                      void* dist, int32_t variant, dawn_stats* stats);
dawn_status dawn_sssp_device(dawn_graph* g, const int32_t* sources,
                             int32_t nsrc, void* d_dist, int32_t variant,
                             dawn_stats* stats);

/* Closeness centrality of each source, (n - 1) / sum of d(s, v) over the
 * reached v != s, accumulated exactly (int64 for hops and int32 weights,
 * float64 for float weights) and divided in float64.  weighted = 0 uses hop
 * distances, 1 the graph's weights.  dist_sum / reached (nullable) return
 * the sum and the number of reached vertices other than s, from which the
 * reference's own integer-division value (src/algorithm/cpu/cc.cpp:77-78,
 * src/algorithm/gpu/cc.cu:92-94) can be recomputed.  Replaces
 * CC_GPU::kernel / kernel_Weighted (src/algorithm/gpu/cc.cu:32-202). */
dawn_status dawn_closeness(dawn_graph* g, const int32_t* sources,
                           int32_t nsrc, int32_t weighted, double* cc,
                           double* dist_sum, int64_t* reached,
                           dawn_stats* stats);

/* Tuning knobs of a handle (no counterpart in the reference, whose only
 * knobs are the block size and stream count hard-coded in its tools,
 * algorithm/gpu/mssp_gpu/mssp_gpu.cu:16-17).  The autotuner sets these;
 * results never depend on them.
 *   DAWN_OPT_BITSET_WIDTH  uint64 words per vertex of the batched traversal:
 *                          0 = chosen from the source count, or 1, 2, 4
 *                          (64, 128, 256 sources per batch)
 *   DAWN_OPT_PUSH_RATIO    a level pushes while ratio x frontier edges <
 *                          edges of unfinished vertices (default 4) */
#define DAWN_OPT_BITSET_WIDTH 1
#define DAWN_OPT_PUSH_RATIO 2
/*   DAWN_OPT_FORCE_VARIANT every level of BFS and SSSP traversals runs one
 *                          variant: 0 = decide per level (default), 1 =
 *                          sparse push, 2 = bitmap pull, 3 = dense push
 *                          (batched bitset only; the other traversals run
 *                          it as sparse push).  For recording the
 *                          per-variant level timings the selector is
 *                          trained on, and for tests; distances are
 *                          unchanged. */
#define DAWN_OPT_FORCE_VARIANT 3
/*   DAWN_OPT_SELECTOR_MARGIN the learned selector overrides the direction
 *                          heuristic only when it predicts the other variant
 *                          faster by this many thousandths of a log2 unit
 *                          (default 0: ties go to the heuristic; 250 asks
 *                          for a predicted gain of about 19%). */
#define DAWN_OPT_SELECTOR_MARGIN 4
/*   DAWN_OPT_PULL_SEGMENT  in-edges per warp task on heavy pull rows of the
 *                          batched traversal (rows of at least twice this
 *                          are spread over several warps); 128..65536,
 *                          default 1024
 *   DAWN_OPT_BLOCKS_PER_SM CTAs per SM of the persistent traversal grids:
 *                          0 = as many as fit (default), else 1..32
 *   DAWN_OPT_AUTO_LEARNED  1: DAWN_VARIANT_AUTO runs batched calls with the
 *                          learned selector (as DAWN_VARIANT_LEARNED), 0: with
 *                          the direction heuristic (default) */
#define DAWN_OPT_PULL_SEGMENT 5
#define DAWN_OPT_BLOCKS_PER_SM 6
#define DAWN_OPT_AUTO_LEARNED 7
/*   DAWN_OPT_L2_PERSIST    1: the batched traversal's frontier words are
 *                          marked persisting in L2 (an access-policy window on
 *                          its level kernels; the device's persisting carve-out
 *                          is set for the rest of this process), so the edge
 *                          arrays streaming through L2 do not evict them.
 *                          0 (default): no window.  Measured slower on RMAT
 *                          scale 22 (1.74 -> 2.25 ms per 64 sources: the
 *                          carve-out shrinks the L2 the gathers also use), even
 *                          at scales 21 and 24. */
#define DAWN_OPT_L2_PERSIST 8
/*   DAWN_OPT_SMALL_LEVELS  1 (default): single-source traversals (BFS with
 *                          DAWN_VARIANT_DO, weighted distances with
 *                          DAWN_VARIANT_DO / PUSH) run stretches of levels
 *                          whose frontier holds at most 8192 vertices and
 *                          32768 out-edges, and no row of 128 entries or
 *                          more, inside one launch of a thread-block cluster
 *                          (8 CTAs, one cluster barrier per level), instead
 *                          of two launches per level.  0: every level is its
 *                          own launch.  Distances are the same. */
#define DAWN_OPT_SMALL_LEVELS 9

/* Autotuner (no counterpart in the reference, whose launch shapes are fixed
 * in its tools, algorithm/gpu/mssp_gpu/mssp_gpu.cu:16-17).  Times the
 * traversal of a sample of `sources` (at most 256, distances not written)
 * under candidate settings, one option at a time: batch width (more than 64
 * sources), learned selector or heuristic, push ratio, pull segment and
 * CTAs per SM; keeps the fastest of each and sets them on the handle.
 * nsrc == 1 tunes the single-source traversal (CTAs per SM only).  The
 * result is also kept in a process-wide cache keyed by device and graph
 * class (log2 n, log2 average degree, symmetry, source-count class); with
 * DAWN_TUNE_USE_CACHE a cached entry is applied without measuring.
 * Results never depend on the settings. */
typedef struct dawn_tuning {
  int32_t bitset_width;   /* 1, 2 or 4 (0: not tuned) */
  int32_t push_ratio;
  int32_t pull_segment;
  int32_t blocks_per_sm;  /* 0: as many as fit */
  int32_t learned;        /* AUTO batched calls use the learned selector */
  int32_t from_cache;     /* 1: applied from the cache, nothing measured */
  float ms;               /* sample time with the chosen settings */
  float default_ms;       /* sample time with the defaults */
} dawn_tuning;
#define DAWN_TUNE_USE_CACHE 1
dawn_status dawn_autotune(dawn_graph* g, const int32_t* sources, int32_t nsrc,
                          uint32_t flags, dawn_tuning* out);
/* Writes / reads the process-wide tuning cache (text, one entry per line). */
dawn_status dawn_tune_cache_save(const char* path);
dawn_status dawn_tune_cache_load(const char* path);
dawn_status dawn_graph_set_option(dawn_graph* g, int32_t option, int64_t value);
dawn_status dawn_graph_get_option(const dawn_graph* g, int32_t option,
                                  int64_t* value);

/* Learned per-level variant selector (no counterpart in the reference).
 * weights: DAWN_SELECTOR_WEIGHTS floats of a 9 x 32 x 32 x 3 ReLU MLP,
 * row-major W1[32][9], b1[32], W2[32][32], b2[32], W3[3][32], b3[3], that
 * predicts log2 of a level's duration in microseconds for sparse push,
 * bitmap pull and dense push from nine frontier statistics.  The decide
 * kernel of each level (one warp, on the device) runs the variant with the
 * smallest prediction when it beats the direction heuristic's choice by
 * DAWN_OPT_SELECTOR_MARGIN, else the heuristic's choice: the heuristic is
 * both the fallback and the reference the selector must beat.  weights =
 * NULL (count 0) restores the heuristics alone.  Distances never depend on
 * the choice. */
#define DAWN_SELECTOR_WEIGHTS 1475
dawn_status dawn_graph_set_selector(dawn_graph* g, const float* weights,
                                    int32_t count);

/* Per-level trace.  No counterpart in the reference, which only times whole
 * runs with host std::chrono (src/algorithm/gpu/bfs.cu:70,93-95).  While
 * tracing is enabled on a handle, traversals run level by level from the
 * host instead of as one CUDA graph per source batch: before each level the
 * host reads the frontier statistics, launches only the kernels that level
 * uses, brackets each with CUDA events on the handle's stream, and appends
 * one record per kernel.  Results are identical; only speed differs.  The
 * records are the per-iteration timing log the variant selector trains on
 * and the per-kernel durations the roofline report divides by.
 * dawn_multi_* calls on a tracing handle run as usual and add one record
 * per (part, source batch) task, kernel "parts_task": run = part, level =
 * levels, mode = push levels, pad = SM, frontier = sources, frontier_edges
 * = the part's edges, unvisited_edges = task start in ns after the first
 * task's start, ms = task duration (device clock). */
typedef struct dawn_trace_rec {
  char kernel[24];          /* kernel name */
  int32_t run;              /* source index (single-source) or batch index */
  int32_t level;            /* 1-based frontier iteration */
  int32_t mode;             /* 0 push (top-down), 1 pull (bottom-up) */
  int32_t pad;
  int64_t frontier;         /* vertices in the frontier entering the level */
  int64_t frontier_edges;   /* out-degree sum of that frontier */
  int64_t unvisited_edges;  /* degree sum of vertices not yet finished */
  float ms;                 /* CUDA-event duration of the kernel */
  float pad2;
} dawn_trace_rec;

dawn_status dawn_trace_enable(dawn_graph* g, int32_t enable);
/* Copies up to cap records (oldest first) and removes them from the handle;
 * *count receives the number copied. */
dawn_status dawn_trace_read(dawn_graph* g, dawn_trace_rec* out, int64_t cap,
                            int64_t* count);

/* Message of the last failing call on this host thread ("" if none). */
const char* dawn_last_error(void);

/* Library version string. */
const char* dawn_version(void);

#ifdef __cplusplus
}
#endif
#endif /* DAWN_GB300_H */
