/* ORACLE — test infrastructure only.
 *
 * A plain-C restatement of GAL-DAWN's CPU frontier path, used by the tests,
 * by __graft_entry__.smoke() and by bench.py's CPU baseline leg as the
 * checker.  The product (libdawn_gb300.so) never links or calls this file.
 *
 * Distances are produced in the reference's own encoding unless a function
 * says otherwise: hop distance 0 means "unvisited" and the source is reset
 * to 0 at the end (src/algorithm/cpu/bfs.cpp:62,117); weighted distance
 * FLT_MAX means unreachable (src/algorithm/cpu/sssp.cpp:36).
 *
 * Parity of this file is pinned by tests/test_oracle.py against
 *   - the reference compiled from its own sources (oracle/_ref, when built),
 *   - the committed golden fixtures under tests/golden/ made by running the
 *     reference command-line tools (tests/golden/make_golden.py).
 */
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Serial queue expand: restates BFS_CPU::SOVM, src/algorithm/cpu/bfs.cpp:134-157.
 * Every unvisited neighbour of a queued vertex gets `level` and is appended
 * to the output queue in discovery order. */
static int32_t expand_queue(const int32_t* row_ptr, const int32_t* col,
                            const int32_t* q_in, int32_t n_in, int32_t* q_out,
                            int32_t* dist, int32_t level) {
  int32_t n_out = 0;
  for (int32_t j = 0; j < n_in; j++) {
    const int32_t v = q_in[j];
    for (int32_t k = row_ptr[v]; k < row_ptr[v + 1]; k++) {
      const int32_t u = col[k];
      if (dist[u] == 0) {
        dist[u] = level;
        q_out[n_out++] = u;
      }
    }
  }
  return n_out;
}

/* Queue BFS: restates BFS_CPU::BFS_kernel, src/algorithm/cpu/bfs.cpp:79-132.
 * The source's neighbours start at level 1, levels run 2..n-1, the loop
 * stops on an empty queue and the source is reset to 0.  Returns the number
 * of CSR entries whose tail was reached (source included), the TEPS unit. */
int64_t oracle_bfs_queue(const int32_t* row_ptr, const int32_t* col, int32_t n,
                         int32_t source, int32_t* dist) {
  int32_t* qa = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  int32_t* qb = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  memset(dist, 0, sizeof(int32_t) * (size_t)n);
  int32_t entry = 0;
  for (int32_t k = row_ptr[source]; k < row_ptr[source + 1]; k++) {
    dist[col[k]] = 1;
    qa[entry++] = col[k]; /* duplicates stay queued, as bfs.cpp:96-99 */
  }
  int32_t level = 1;
  while (level < n) {
    level++;
    if (level % 2 == 0)
      entry = expand_queue(row_ptr, col, qa, entry, qb, dist, level);
    else
      entry = expand_queue(row_ptr, col, qb, entry, qa, dist, level);
    if (entry == 0) break;
  }
  dist[source] = 0;
  int64_t edges = (int64_t)row_ptr[source + 1] - row_ptr[source];
  for (int32_t v = 0; v < n; v++)
    if (dist[v] > 0 && v != source) edges += row_ptr[v + 1] - row_ptr[v];
  free(qa);
  free(qb);
  return edges;
}

/* Bitmap expand: restates BFS_CPU::SOVMP, src/algorithm/cpu/bfs.cpp:159-185
 * (run single-threaded: every racing writer stores the same level, so the
 * OpenMP form has the same result). */
static int expand_bitmap(const int32_t* row_ptr, const int32_t* col, int32_t n,
                         uint8_t* in, uint8_t* out, int32_t* dist,
                         int32_t level) {
  int converged = 1;
  for (int32_t j = 0; j < n; j++) {
    if (!in[j]) continue;
    for (int32_t k = row_ptr[j]; k < row_ptr[j + 1]; k++) {
      const int32_t u = col[k];
      if (dist[u] == 0) {
        dist[u] = level;
        out[u] = 1;
        converged = 0;
      }
    }
    in[j] = 0;
  }
  return converged;
}

/* Bitmap BFS: restates BFS_CPU::BFS, src/algorithm/cpu/bfs.cpp:23-77. */
void oracle_bfs_bitmap(const int32_t* row_ptr, const int32_t* col, int32_t n,
                       int32_t source, int32_t* dist) {
  uint8_t* a = (uint8_t*)calloc((size_t)(n > 0 ? n : 1), 1);
  uint8_t* b = (uint8_t*)calloc((size_t)(n > 0 ? n : 1), 1);
  memset(dist, 0, sizeof(int32_t) * (size_t)n);
  for (int32_t k = row_ptr[source]; k < row_ptr[source + 1]; k++) {
    a[col[k]] = 1;
    dist[col[k]] = 1;
  }
  int32_t level = 1;
  while (level < n) {
    level++;
    int done = (level % 2 == 0)
                   ? expand_bitmap(row_ptr, col, n, a, b, dist, level)
                   : expand_bitmap(row_ptr, col, n, b, a, dist, level);
    if (done) break;
  }
  dist[source] = 0;
  free(a);
  free(b);
}

/* Min-plus relax over a bitmap frontier: restates SSSP_CPU::GOVMP,
 * src/algorithm/cpu/sssp.cpp:169-199, single-threaded (the OpenMP form
 * races on the min, see sssp.cpp:186-189).  Vertices relax in index order
 * and read distances updated earlier in the same sweep. */
static int relax_bitmap(const int32_t* row_ptr, const int32_t* col,
                        const float* val, int32_t n, uint8_t* in, uint8_t* out,
                        float* dist, int32_t source) {
  int converged = 1;
  for (int32_t j = 0; j < n; j++) {
    if (!in[j]) continue;
    for (int32_t k = row_ptr[j]; k < row_ptr[j + 1]; k++) {
      const int32_t u = col[k];
      const float t = dist[j] + val[k];
      if (dist[u] > t && u != source) {
        dist[u] = t;
        out[u] = 1;
        converged = 0;
      }
    }
    in[j] = 0;
  }
  return converged;
}

/* Weighted SSSP: restates SSSP_CPU::SSSP, src/algorithm/cpu/sssp.cpp:23-80.
 * The source row initialises its neighbours directly, the last CSR entry of
 * a repeated neighbour winning (sssp.cpp:43-46), the source is set to 0 and
 * is never relaxed.  Unreachable vertices keep FLT_MAX. */
void oracle_sssp(const int32_t* row_ptr, const int32_t* col, const float* val,
                 int32_t n, int32_t source, float* dist) {
  uint8_t* a = (uint8_t*)calloc((size_t)(n > 0 ? n : 1), 1);
  uint8_t* b = (uint8_t*)calloc((size_t)(n > 0 ? n : 1), 1);
  for (int32_t v = 0; v < n; v++) dist[v] = FLT_MAX;
  for (int32_t k = row_ptr[source]; k < row_ptr[source + 1]; k++) {
    dist[col[k]] = val[k];
    a[col[k]] = 1;
  }
  dist[source] = 0.0f;
  int32_t level = 1;
  while (level < n) {
    level++;
    int done = (level % 2 == 0)
                   ? relax_bitmap(row_ptr, col, val, n, a, b, dist, source)
                   : relax_bitmap(row_ptr, col, val, n, b, a, dist, source);
    if (done) break;
  }
  free(a);
  free(b);
}

/* Multi-source unweighted: restates MSSP_CPU::run, src/algorithm/cpu/mssp.cpp:9-32:
 * an OpenMP loop over the sources (taken modulo n), isolated sources skipped,
 * each source a serial queue BFS (BFS_kernel).  `threads` <= 0 keeps the
 * OpenMP default.  dist (nsrc x n, reference encoding) may be NULL; rows of
 * skipped sources are left all zero and skipped[i] is set when given.
 * Returns the summed TEPS edge count of the processed sources. */
int64_t oracle_mssp(const int32_t* row_ptr, const int32_t* col, int32_t n,
                    const int32_t* sources, int32_t nsrc, int32_t threads,
                    int32_t* dist, uint8_t* skipped) {
  int64_t edges = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for reduction(+ : edges)
  for (int32_t i = 0; i < nsrc; i++) {
    const int32_t s = sources[i] % n;
    int32_t* row = dist ? dist + (size_t)i * n : NULL;
    if (row_ptr[s] == row_ptr[s + 1]) {
      if (row) memset(row, 0, sizeof(int32_t) * (size_t)n);
      if (skipped) skipped[i] = 1;
      continue;
    }
    if (skipped) skipped[i] = 0;
    int32_t* scratch = row ? row : (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    edges += oracle_bfs_queue(row_ptr, col, n, s, scratch);
    if (!row) free(scratch);
  }
  return edges;
}

/* Weighted multi-source parity target: SSSP_CPU::SSSP per source (the
 * reference's weighted MSSP queue kernel indexes distance by queue slot,
 * src/algorithm/cpu/sssp.cpp:157, and is not a usable oracle). */
void oracle_msssp(const int32_t* row_ptr, const int32_t* col, const float* val,
                  int32_t n, const int32_t* sources, int32_t nsrc,
                  int32_t threads, float* dist) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t i = 0; i < nsrc; i++)
    oracle_sssp(row_ptr, col, val, n, sources[i] % n, dist + (size_t)i * n);
}

/* Closeness in float64: (n-1) / sum of d(s,v) over reached v != s.
 * Hop rows use the reference encoding (0 = unvisited); weighted rows skip
 * FLT_MAX.  The reference's own value divides int by int
 * (src/algorithm/cpu/cc.cpp:77-78); oracle_closeness_ref_int restates it. */
double oracle_closeness_hops(const int32_t* dist, int32_t n, int32_t source) {
  int64_t sum = 0;
  for (int32_t v = 0; v < n; v++)
    if (v != source && dist[v] > 0) sum += dist[v];
  return sum > 0 ? (double)(n - 1) / (double)sum : 0.0;
}

double oracle_closeness_weighted(const float* dist, int32_t n, int32_t source) {
  double sum = 0.0;
  for (int32_t v = 0; v < n; v++)
    if (v != source && dist[v] != FLT_MAX) sum += (double)dist[v];
  return sum > 0 ? (double)(n - 1) / sum : 0.0;
}

/* src/algorithm/cpu/cc.cpp:155-157: int (n-1) / int sum, converted to float. */
float oracle_closeness_ref_int(const int32_t* dist, int32_t n, int32_t source) {
  uint32_t acc = 0; /* int accumulate, wrapping like the reference's int sum */
  for (int32_t v = 0; v < n; v++)
    if (v != source) acc += (uint32_t)dist[v];
  const int32_t sum = (int32_t)acc;
  return sum ? (float)((n - 1) / sum) : 0.0f;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* --- BCDAWN betweenness (bc.cpp:9-191) --------------------------------------
 * Per source s (BC_CPU::SOVM + kernel + accumulate):
 *   * the first frontier is the set of s's out-neighbours (bc.cpp:57-62),
 *     which are also marked visited; s itself is never marked;
 *   * each step scans the frontier in vertex order and, for every CSR entry
 *     j -> c whose head c is unvisited, counts amount[c]++ and records the
 *     pair (j, c) (bc.cpp:126-140); then, pair by pair, c != s gets j
 *     appended to its predecessor list, j gains 1 / amount[c], c joins the
 *     next frontier and, the first time, the discovery order
 *     (bc.cpp:142-158);
 *   * finally, in reverse discovery order, every c adds its value to each of
 *     its predecessors, in the order they were appended (bc.cpp:173-191).
 * The result is the sum over the sources.  T selects the arithmetic: double
 * for the oracle, float to repeat the reference's float32 additions in its
 * order. */
#define BC_SOURCE(T, NAME)                                                                   \
  static void NAME(const int32_t* rp, const int32_t* col, int32_t n, int32_t s, T* delta,   \
                   uint8_t* alpha, uint8_t* beta, uint8_t* gamma, int32_t* amount,          \
                   int32_t* pj, int32_t* pc, int64_t* head, int64_t* tail, int64_t* nxt,    \
                   int32_t* order) {                                                         \
    memset(alpha, 0, (size_t)n);                                                             \
    memset(beta, 0, (size_t)n);                                                              \
    memset(gamma, 0, (size_t)n);                                                             \
    memset(amount, 0, sizeof(int32_t) * (size_t)n);                                          \
    for (int32_t v = 0; v < n; v++) head[v] = tail[v] = -1;                                  \
    for (int32_t k = rp[s]; k < rp[s + 1]; k++) alpha[col[k]] = gamma[col[k]] = 1;           \
    int64_t npairs_total = 0;                                                                \
    int32_t norder = 0;                                                                      \
    for (int32_t step = 1; step < n;) {                                                      \
      step++;                                                                                \
      uint8_t* in = (step % 2) ? beta : alpha;                                               \
      uint8_t* out = (step % 2) ? alpha : beta;                                              \
      int converged = 1;                                                                     \
      int64_t p0 = npairs_total;                                                             \
      for (int32_t j = 0; j < n; j++) {                                                      \
        if (!in[j]) continue;                                                                \
        for (int32_t k = rp[j]; k < rp[j + 1]; k++) {                                        \
          const int32_t c = col[k];                                                          \
          if (!gamma[c]) {                                                                   \
            amount[c] += 1;                                                                  \
            pj[npairs_total] = j;                                                            \
            pc[npairs_total] = c;                                                            \
            npairs_total++;                                                                  \
            converged = 0;                                                                   \
          }                                                                                  \
        }                                                                                    \
        in[j] = 0;                                                                           \
      }                                                                                      \
      for (int64_t p = p0; p < npairs_total; p++) {                                          \
        const int32_t j = pj[p], c = pc[p];                                                  \
        if (c == s || j == s) continue;                                                      \
        nxt[p] = -1;                                                                         \
        if (tail[c] < 0) head[c] = p; else nxt[tail[c]] = p;                                 \
        tail[c] = p;                                                                         \
        delta[j] += (T)1 / (T)amount[c];                                                     \
        out[c] = 1;                                                                          \
        if (!gamma[c]) {                                                                     \
          gamma[c] = 1;                                                                      \
          order[norder++] = c;                                                               \
        }                                                                                    \
      }                                                                                      \
      if (converged) break;                                                                  \
    }                                                                                        \
    for (int32_t i = norder - 1; i >= 0; i--) {                                              \
      const int32_t c = order[i];                                                            \
      for (int64_t p = head[c]; p >= 0; p = nxt[p]) delta[pj[p]] += delta[c];               \
    }                                                                                        \
  }

BC_SOURCE(double, bc_source_d)
BC_SOURCE(float, bc_source_f)

/* Betweenness summed over `sources`.  bc (double, may be NULL) from the
 * double restatement, sources in parallel; bcf (float, may be NULL) with
 * the reference's float32 arithmetic and order (sources in sequence, the
 * per-source values added as bc_values[j] += bc_temp[j], bc.cpp:24-27). */
void oracle_bc(const int32_t* rp, const int32_t* col, int32_t n, const int32_t* sources, int32_t nsrc,
               double* bc, float* bcf) {
  const int64_t m = rp[n];
  if (bc) {
    memset(bc, 0, sizeof(double) * (size_t)n);
#pragma omp parallel
    {
      double* acc = (double*)calloc((size_t)n, sizeof(double));
      double* delta = (double*)malloc(sizeof(double) * (size_t)n);
      uint8_t* a = (uint8_t*)malloc((size_t)n * 3);
      int32_t* amount = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
      int32_t* pj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m + 1));
      int32_t* pc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m + 1));
      int64_t* hd = (int64_t*)malloc(sizeof(int64_t) * (size_t)n * 2);
      int64_t* nx = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m + 1));
      int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
#pragma omp for schedule(dynamic, 1)
      for (int32_t i = 0; i < nsrc; i++) {
        memset(delta, 0, sizeof(double) * (size_t)n);
        bc_source_d(rp, col, n, sources[i], delta, a, a + n, a + 2 * (size_t)n, amount, pj, pc, hd, hd + n, nx,
                    order);
        for (int32_t v = 0; v < n; v++) acc[v] += delta[v];
      }
#pragma omp critical
      for (int32_t v = 0; v < n; v++) bc[v] += acc[v];
      free(acc); free(delta); free(a); free(amount); free(pj); free(pc); free(hd); free(nx); free(order);
    }
  }
  if (bcf) {
    memset(bcf, 0, sizeof(float) * (size_t)n);
    float* delta = (float*)malloc(sizeof(float) * (size_t)n);
    uint8_t* a = (uint8_t*)malloc((size_t)n * 3);
    int32_t* amount = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* pj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m + 1));
    int32_t* pc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m + 1));
    int64_t* hd = (int64_t*)malloc(sizeof(int64_t) * (size_t)n * 2);
    int64_t* nx = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m + 1));
    int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    for (int32_t i = 0; i < nsrc; i++) {
      memset(delta, 0, sizeof(float) * (size_t)n);
      bc_source_f(rp, col, n, sources[i], delta, a, a + n, a + 2 * (size_t)n, amount, pj, pc, hd, hd + n, nx,
                  order);
      for (int32_t v = 0; v < n; v++) bcf[v] += delta[v];
    }
    free(delta); free(a); free(amount); free(pj); free(pc); free(hd); free(nx); free(order);
  }
}
