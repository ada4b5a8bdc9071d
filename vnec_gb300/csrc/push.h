// Push-side SpMSpV (push.cu): A as CSC, y = A x for sparse x.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace vnec {

struct PushMatrix {
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  const int64_t* col_ptr = nullptr;  // n_cols + 1
  const int32_t* row = nullptr;      // nnz row indices, increasing within a column
  const void* val = nullptr;         // nnz values (double or float)
  int* status = nullptr;             // set when an x index is out of range
};

// y (n_rows, overwritten) = A x with x given by nx (index, value) pairs; with
// idx == nullptr, x is dense (xval has n_cols entries, index = position).
bool push_spmspv(const PushMatrix& m, bool fp64, long long nx, const int32_t* idx, const void* xval, void* y,
                 cudaStream_t s);

}  // namespace vnec
