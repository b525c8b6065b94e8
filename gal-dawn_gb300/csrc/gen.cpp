// Seeded synthetic graph generators for the DAWN frontier workloads.
//
// Every generator is a pure function of its arguments: random numbers come
// from a counter-based hash (splitmix64 finaliser applied to seed, stream and
// index), rows are sorted and deduplicated after the parallel scatter, and no
// floating point decides an edge.  The same call therefore returns the same
// CSR on x86_64 and aarch64 and for any OpenMP thread count.
//
// Output CSR follows the reference's container (include/dawn/matrix.hxx:7-12):
// int32 row_ptr[n+1], int32 col[m], sorted by (row, col); optional int32 and
// float32 weights holding the same integer values in [1, 63].

#include "dawn_gen.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint64_t kStreamRmat = 1, kStreamPerm = 2, kStreamErU = 3,
                   kStreamErV = 4, kStreamW = 5, kStreamPts = 6,
                   kStreamSrc = 7;

inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

inline uint64_t rnd(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
}

// Uniform integer in [0, n) from 32 high bits (multiply-shift, no division).
inline uint32_t below(uint64_t r, uint32_t n) {
  return (uint32_t)(((r >> 32) * (uint64_t)n) >> 32);
}

inline int32_t edge_weight(uint64_t seed, int32_t u, int32_t v) {
  uint64_t lo = (uint64_t)(uint32_t)std::min(u, v);
  uint64_t hi = (uint64_t)(uint32_t)std::max(u, v);
  return 1 + (int32_t)(rnd(seed, kStreamW, (hi << 32) | lo) % 63u);
}

void set_error(const char* msg) { std::fprintf(stderr, "dawn_gen: %s\n", msg); }

// Builds a sorted CSR from an edge list.  Self loops are dropped when
// DAWN_GEN_NO_SELF is set, every edge is mirrored under DAWN_GEN_SYMMETRIC,
// and equal (row, col) pairs collapse under DAWN_GEN_DEDUP.
int build_csr(int32_t n, const std::vector<int32_t>& src,
              const std::vector<int32_t>& dst, int flags, uint64_t seed,
              dawn_csr* out) {
  const bool sym = flags & DAWN_GEN_SYMMETRIC;
  const bool noself = flags & DAWN_GEN_NO_SELF;
  const int64_t e = (int64_t)src.size();
  std::vector<std::atomic<int64_t>> deg(n + 1);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i <= n; i++) deg[i].store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < e; i++) {
    int32_t u = src[i], v = dst[i];
    if (noself && u == v) continue;
    deg[u].fetch_add(1, std::memory_order_relaxed);
    if (sym && u != v) deg[v].fetch_add(1, std::memory_order_relaxed);
  }
  std::vector<int64_t> off(n + 1, 0);
  for (int32_t i = 0; i < n; i++) off[i + 1] = off[i] + deg[i].load();
  const int64_t total = off[n];
  std::vector<int32_t> tmp;
  try {
    tmp.resize(total);
  } catch (...) {
    set_error("out of memory");
    return 2;
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i <= n; i++) deg[i].store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < e; i++) {
    int32_t u = src[i], v = dst[i];
    if (noself && u == v) continue;
    tmp[off[u] + deg[u].fetch_add(1, std::memory_order_relaxed)] = v;
    if (sym && u != v)
      tmp[off[v] + deg[v].fetch_add(1, std::memory_order_relaxed)] = u;
  }
  std::vector<int64_t> keep(n + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t r = 0; r < n; r++) {
    int32_t* b = tmp.data() + off[r];
    int32_t* en = tmp.data() + off[r + 1];
    std::sort(b, en);
    if (flags & DAWN_GEN_DEDUP) en = std::unique(b, en);
    keep[r + 1] = en - b;
  }
  for (int32_t i = 0; i < n; i++) keep[i + 1] += keep[i];
  const int64_t m = keep[n];
  if (m > INT32_MAX) {
    set_error("edge count exceeds int32 CSR range");
    return 1;
  }
  out->n = n;
  out->m = m;
  out->row_ptr = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)(n + 1));
  out->col = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1));
  out->w_i32 = nullptr;
  out->w_f32 = nullptr;
  if (!out->row_ptr || !out->col) {
    set_error("out of memory");
    return 2;
  }
  for (int32_t i = 0; i <= n; i++) out->row_ptr[i] = (int32_t)keep[i];
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t r = 0; r < n; r++) {
    int64_t len = keep[r + 1] - keep[r];
    std::memcpy(out->col + keep[r], tmp.data() + off[r], sizeof(int32_t) * len);
  }
  if (flags & DAWN_GEN_WEIGHTS) {
    out->w_i32 = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1));
    out->w_f32 = (float*)std::malloc(sizeof(float) * (size_t)std::max<int64_t>(m, 1));
    if (!out->w_i32 || !out->w_f32) {
      set_error("out of memory");
      return 2;
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < n; r++) {
      for (int64_t k = keep[r]; k < keep[r + 1]; k++) {
        int32_t w = edge_weight(seed, (int32_t)r, out->col[k]);
        out->w_i32[k] = w;
        out->w_f32[k] = (float)w;
      }
    }
  }
  return 0;
}

struct Dsu {
  std::vector<int32_t> p;
  explicit Dsu(int32_t n) : p(n) { std::iota(p.begin(), p.end(), 0); }
  int32_t find(int32_t x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  }
  void unite(int32_t a, int32_t b) {
    a = find(a);
    b = find(b);
    if (a == b) return;
    if (a < b) std::swap(a, b);
    p[a] = b;
  }
};

}  // namespace

extern "C" {

void dawn_csr_free(dawn_csr* g) {
  if (!g) return;
  std::free(g->row_ptr);
  std::free(g->col);
  std::free(g->w_i32);
  std::free(g->w_f32);
  g->row_ptr = g->col = g->w_i32 = nullptr;
  g->w_f32 = nullptr;
}

int dawn_gen_rmat(int scale, int edgefactor, double a, double b, double c,
                  uint64_t seed, int flags, dawn_csr* out) {
  if (!out || scale < 1 || scale > 30 || edgefactor < 1 || a < 0 || b < 0 ||
      c < 0 || a + b + c > 1.0) {
    set_error("invalid RMAT arguments");
    return 1;
  }
  const int32_t n = (int32_t)1 << scale;
  const int64_t e = (int64_t)edgefactor << scale;
  const uint64_t ta = (uint64_t)(a * 4294967296.0);
  const uint64_t tab = (uint64_t)((a + b) * 4294967296.0);
  const uint64_t tabc = (uint64_t)((a + b + c) * 4294967296.0);
  std::vector<int32_t> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  if (flags & DAWN_GEN_PERMUTE) {
    for (int32_t i = n - 1; i > 0; i--) {
      uint32_t j = below(rnd(seed, kStreamPerm, (uint64_t)i), (uint32_t)i + 1);
      std::swap(perm[i], perm[j]);
    }
  }
  std::vector<int32_t> src(e), dst(e);
  const int words = (scale + 1) / 2;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < e; i++) {
    uint32_t u = 0, v = 0;
    for (int w = 0; w < words; w++) {
      uint64_t r = rnd(seed, kStreamRmat, (uint64_t)i * words + w);
      for (int h = 0; h < 2 && 2 * w + h < scale; h++) {
        uint64_t x = h ? (r >> 32) : (r & 0xffffffffull);
        uint32_t bu = 0, bv = 0;
        if (x < ta) {
        } else if (x < tab) {
          bv = 1;
        } else if (x < tabc) {
          bu = 1;
        } else {
          bu = 1;
          bv = 1;
        }
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
    }
    src[i] = perm[u];
    dst[i] = perm[v];
  }
  return build_csr(n, src, dst, flags, seed, out);
}

int dawn_gen_er(int32_t n, int64_t nedges, uint64_t seed, int flags,
                dawn_csr* out) {
  if (!out || n < 1 || nedges < 0) {
    set_error("invalid ER arguments");
    return 1;
  }
  std::vector<int32_t> src(nedges), dst(nedges);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nedges; i++) {
    src[i] = (int32_t)below(rnd(seed, kStreamErU, (uint64_t)i), (uint32_t)n);
    dst[i] = (int32_t)below(rnd(seed, kStreamErV, (uint64_t)i), (uint32_t)n);
  }
  return build_csr(n, src, dst, flags, seed, out);
}

int dawn_gen_grid(int32_t rows, int32_t cols, uint64_t seed, int flags,
                  dawn_csr* out) {
  if (!out || rows < 1 || cols < 1 || (int64_t)rows * cols > INT32_MAX) {
    set_error("invalid grid arguments");
    return 1;
  }
  const int32_t n = rows * cols;
  std::vector<int32_t> src, dst;
  src.reserve((size_t)2 * n);
  dst.reserve((size_t)2 * n);
  for (int32_t r = 0; r < rows; r++)
    for (int32_t c = 0; c < cols; c++) {
      int32_t v = r * cols + c;
      if (c + 1 < cols) {
        src.push_back(v);
        dst.push_back(v + 1);
      }
      if (r + 1 < rows) {
        src.push_back(v);
        dst.push_back(v + cols);
      }
    }
  return build_csr(n, src, dst, flags | DAWN_GEN_SYMMETRIC, seed, out);
}

int dawn_gen_knn(int32_t npts, int k, uint64_t seed, int flags, dawn_csr* out) {
  if (!out || npts < 2 || k < 1 || k >= npts) {
    set_error("invalid kNN arguments");
    return 1;
  }
  // Integer coordinates in [0, 2^30): squared distances are exact in uint64.
  std::vector<uint32_t> px(npts), py(npts);
  for (int32_t i = 0; i < npts; i++) {
    uint64_t r = rnd(seed, kStreamPts, (uint64_t)i);
    px[i] = (uint32_t)(r & 0x3fffffffu);
    py[i] = (uint32_t)((r >> 32) & 0x3fffffffu);
  }
  int32_t g = 1;
  while ((int64_t)g * g * 2 < npts) g <<= 1;
  const int shift = 30 - __builtin_ctz((unsigned)g);
  std::vector<int32_t> cell_start((size_t)g * g + 1, 0), order(npts);
  for (int32_t i = 0; i < npts; i++)
    cell_start[((size_t)(py[i] >> shift) * g + (px[i] >> shift)) + 1]++;
  for (size_t i = 0; i < (size_t)g * g; i++) cell_start[i + 1] += cell_start[i];
  {
    std::vector<int32_t> cur(cell_start.begin(), cell_start.end() - 1);
    for (int32_t i = 0; i < npts; i++)
      order[cur[(size_t)(py[i] >> shift) * g + (px[i] >> shift)]++] = i;
  }
  std::vector<int32_t> src((size_t)npts * k), dst((size_t)npts * k);
  const uint64_t cell = (uint64_t)1 << shift;
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t i = 0; i < npts; i++) {
    std::vector<std::pair<uint64_t, int32_t>> best;
    best.reserve(64);
    const int32_t cx = (int32_t)(px[i] >> shift), cy = (int32_t)(py[i] >> shift);
    for (int32_t ring = 0;; ring++) {
      for (int32_t yy = cy - ring; yy <= cy + ring; yy++) {
        if (yy < 0 || yy >= g) continue;
        for (int32_t xx = cx - ring; xx <= cx + ring; xx++) {
          if (xx < 0 || xx >= g) continue;
          if (std::max(std::abs(yy - cy), std::abs(xx - cx)) != ring) continue;
          size_t cidx = (size_t)yy * g + xx;
          for (int32_t t = cell_start[cidx]; t < cell_start[cidx + 1]; t++) {
            int32_t j = order[t];
            if (j == i) continue;
            int64_t dx = (int64_t)px[i] - px[j], dy = (int64_t)py[i] - py[j];
            best.push_back({(uint64_t)(dx * dx) + (uint64_t)(dy * dy), j});
          }
        }
      }
      if ((int)best.size() >= k) {
        std::partial_sort(best.begin(), best.begin() + k, best.end());
        // Every point outside the searched square is at least ring*cell away.
        uint64_t reach = (uint64_t)ring * cell;
        if (best[k - 1].first <= reach * reach || ring > g) break;
      }
      if (ring > g) break;
    }
    std::partial_sort(best.begin(), best.begin() + k, best.end());
    for (int t = 0; t < k; t++) {
      src[(size_t)i * k + t] = i;
      dst[(size_t)i * k + t] = best[t].second;
    }
  }
  return build_csr(npts, src, dst, flags, seed, out);
}

int dawn_gen_sources(const dawn_csr* gph, int32_t nsrc, uint64_t seed,
                     int from_lcc, int32_t* out) {
  if (!gph || !out || nsrc < 0 || gph->n < 1) {
    set_error("invalid source arguments");
    return 1;
  }
  const int32_t n = gph->n;
  std::vector<int32_t> pool;
  if (from_lcc) {
    Dsu d(n);
    for (int32_t u = 0; u < n; u++)
      for (int32_t k = gph->row_ptr[u]; k < gph->row_ptr[u + 1]; k++)
        d.unite(u, gph->col[k]);
    std::vector<int32_t> size(n, 0);
    for (int32_t u = 0; u < n; u++) size[d.find(u)]++;
    int32_t best = 0;
    for (int32_t u = 0; u < n; u++)
      if (size[u] > size[best]) best = u;
    for (int32_t u = 0; u < n; u++)
      if (d.find(u) == best) pool.push_back(u);
  } else {
    pool.resize(n);
    std::iota(pool.begin(), pool.end(), 0);
  }
  // Partial Fisher-Yates: distinct sources while the pool allows it.
  const int32_t p = (int32_t)pool.size();
  for (int32_t i = 0; i < nsrc; i++) {
    int32_t lim = p - (i % p);
    int32_t j = (i % p) + (int32_t)below(rnd(seed, kStreamSrc, (uint64_t)i), (uint32_t)lim);
    std::swap(pool[i % p], pool[j]);
    out[i] = pool[i % p];
  }
  return 0;
}

int dawn_write_mtx(const dawn_csr* gph, const char* path, int symmetric,
                   int weighted) {
  if (!gph || !path) return 1;
  FILE* f = std::fopen(path, "w");
  if (!f) {
    set_error("cannot open output file");
    return 1;
  }
  const int32_t n = gph->n;
  int64_t cnt = 0;
  for (int32_t u = 0; u < n; u++)
    for (int32_t k = gph->row_ptr[u]; k < gph->row_ptr[u + 1]; k++)
      if (!symmetric || gph->col[k] < u) cnt++;
  std::fprintf(f, "%%%%MatrixMarket matrix coordinate %s %s\n",
               weighted ? "integer" : "pattern", symmetric ? "symmetric" : "general");
  std::fprintf(f, "%d %d %lld\n", n, n, (long long)cnt);
  for (int32_t u = 0; u < n; u++)
    for (int32_t k = gph->row_ptr[u]; k < gph->row_ptr[u + 1]; k++) {
      int32_t v = gph->col[k];
      if (symmetric && v >= u) continue;
      if (weighted)
        std::fprintf(f, "%d %d %d\n", u + 1, v + 1, gph->w_i32 ? gph->w_i32[k] : 1);
      else
        std::fprintf(f, "%d %d\n", u + 1, v + 1);
    }
  std::fclose(f);
  return 0;
}

}  // extern "C"
