// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// CSR / COO containers and conversions, API of include/dawn/matrix.hxx in
// the reference project.
#pragma once
#include <dawn/include.hxx>

namespace DAWN {
namespace Matrix {

struct Csr_t {
 public:
  int* row_ptr = nullptr;
  int* col = nullptr;
  float* val = nullptr;
};

struct Coo_t {
 public:
  int* row = nullptr;
  int* col = nullptr;
  float* val = nullptr;
};

// Rows are counted from coo.row; coo must already be sorted by row.
void coo2Csr(int n, int nnz, Csr_t& csr, Coo_t& coo);
void coo2Csr_Weighted(int n, int nnz, Csr_t& csr, Coo_t& coo);
// Sorts the COO entries by (row, col) / (row, col, val).
void transpose(int nnz, Coo_t& coo);
void transpose_Weighted(int nnz, Coo_t& coo);

}  // namespace Matrix
}  // namespace DAWN
