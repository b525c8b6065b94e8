// COO -> CSR conversion and COO sorting (API of src/matrix.cpp in the
// reference project): the COO entries are sorted by (row, col[, val]) and
// the CSR keeps that order; duplicates are kept.
#include <dawn/matrix.hxx>

#include <parallel/algorithm>
#include <tuple>

namespace DAWN {
namespace Matrix {

static void build_row_ptr(int n, int nnz, const int* row, int* row_ptr) {
  std::vector<int> count(n, 0);
  for (int i = 0; i < nnz; i++) count[row[i]]++;
  row_ptr[0] = 0;
  for (int i = 0; i < n; i++) row_ptr[i + 1] = row_ptr[i] + count[i];
}

void coo2Csr(int n, int nnz, Csr_t& csr, Coo_t& coo) {
  csr.row_ptr = new int[n + 1];
  csr.col = new int[nnz > 0 ? nnz : 1];
  build_row_ptr(n, nnz, coo.row, csr.row_ptr);
  std::copy(coo.col, coo.col + nnz, csr.col);
}

void coo2Csr_Weighted(int n, int nnz, Csr_t& csr, Coo_t& coo) {
  csr.row_ptr = new int[n + 1];
  csr.col = new int[nnz > 0 ? nnz : 1];
  csr.val = new float[nnz > 0 ? nnz : 1];
  build_row_ptr(n, nnz, coo.row, csr.row_ptr);
  std::copy(coo.col, coo.col + nnz, csr.col);
  std::copy(coo.val, coo.val + nnz, csr.val);
}

void transpose(int nnz, Coo_t& coo) {
  std::vector<uint64_t> key(nnz);
  for (int i = 0; i < nnz; i++) key[i] = ((uint64_t)(uint32_t)coo.row[i] << 32) | (uint32_t)coo.col[i];
  __gnu_parallel::sort(key.begin(), key.end());
  for (int i = 0; i < nnz; i++) {
    coo.row[i] = (int)(key[i] >> 32);
    coo.col[i] = (int)(uint32_t)key[i];
  }
}

void transpose_Weighted(int nnz, Coo_t& coo) {
  std::vector<std::tuple<int, int, float>> t(nnz);
  for (int i = 0; i < nnz; i++) t[i] = std::make_tuple(coo.row[i], coo.col[i], coo.val[i]);
  __gnu_parallel::sort(t.begin(), t.end());
  for (int i = 0; i < nnz; i++) std::tie(coo.row[i], coo.col[i], coo.val[i]) = t[i];
}

}  // namespace Matrix
}  // namespace DAWN
