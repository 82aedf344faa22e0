// Device descriptors of the split-precision GEMM shared by its own kernels
// (gemm_split.cu) and the persistent iteration program (program.cu).
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace gbx {

struct SplitRowSet {   // one operand of one problem for the split kernels
  const double* src;
  int64_t rows, K;     // source rows (M or N) and row length
  __nv_bfloat16* dst;  // slice 0, row 0
  int64_t slice_stride, Kp;
  int* exps;
  int64_t first_row;   // first (row, K chunk) work item of this set
  int64_t ld;          // source row stride (elements)
};

struct DevProblem {
  int M, N, K, nkb;
  int tiles_m, tiles_n;
  int ksplit, kb_per_split;  // K split into ranges of kb_per_split k-blocks
  const int* eA;
  const int* eB;
  double* C;        // ksplit == 1: output
  double* partial;  // ksplit > 1: ksplit x M x N raw contributions
  int64_t ldc;
};

}  // namespace gbx
