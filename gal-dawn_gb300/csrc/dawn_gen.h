/* Seeded synthetic graph generators (host only, OpenMP).
 *
 * These build the benchmark and test inputs: Erdos-Renyi, RMAT, 2D grid and
 * random-geometric kNN graphs as sorted int32 CSR.  They are workload tools,
 * not part of the drop-in boundary, so they live in their own library
 * (libdawn_gen.so) beside the kernels. */
#ifndef DAWN_GEN_H
#define DAWN_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  DAWN_GEN_SYMMETRIC = 1, /* mirror every edge (undirected graph) */
  DAWN_GEN_DEDUP = 2,     /* collapse equal (row, col) pairs */
  DAWN_GEN_NO_SELF = 4,   /* drop self loops */
  DAWN_GEN_WEIGHTS = 8,   /* attach int32 + float32 weights in [1, 63] */
  DAWN_GEN_PERMUTE = 16   /* seeded relabelling of RMAT vertex ids */
};

typedef struct dawn_csr {
  int32_t n;
  int64_t m;
  int32_t* row_ptr; /* n + 1 */
  int32_t* col;     /* m */
  int32_t* w_i32;   /* m or NULL */
  float* w_f32;     /* m or NULL, same integer values as w_i32 */
} dawn_csr;

int dawn_gen_rmat(int scale, int edgefactor, double a, double b, double c,
                  uint64_t seed, int flags, dawn_csr* out);
int dawn_gen_er(int32_t n, int64_t nedges, uint64_t seed, int flags,
                dawn_csr* out);
int dawn_gen_grid(int32_t rows, int32_t cols, uint64_t seed, int flags,
                  dawn_csr* out);
int dawn_gen_knn(int32_t npts, int k, uint64_t seed, int flags, dawn_csr* out);
/* nsrc sources, distinct while possible, uniform over the largest weakly
 * connected component (from_lcc != 0) or over all vertices. */
int dawn_gen_sources(const dawn_csr* g, int32_t nsrc, uint64_t seed,
                     int from_lcc, int32_t* out);
/* MatrixMarket coordinate file readable by the reference loader; symmetric
 * graphs are written as their strict lower triangle. */
int dawn_write_mtx(const dawn_csr* g, const char* path, int symmetric,
                   int weighted);
void dawn_csr_free(dawn_csr* g);

#ifdef __cplusplus
}
#endif
#endif
