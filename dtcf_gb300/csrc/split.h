// Split-precision FP64 GEMM: FP64 operands split into exact integer slices
// held in bf16, products on the tcgen05 tensor cores with exact FP32
// accumulation chunks, recombined in FP64 (gemm_split.cu).
#pragma once
#include <cstdint>
#include <utility>
#include <vector>

#include "common.h"

namespace gbx {

// C[M x N] = A[M x K] * B[N x K]^T, all row-major FP64 (row strides lda,
// ldb, ldc; 0 means K for A and B, N for C).
struct SplitProblem {
  const double* A;
  const double* B;
  double* C;
  int64_t M, N, K;
  // the GEMM's A rows come from the plan's packed B operand (swapped
  // orientation); split_operands(plan_a, plan_b) maps accordingly
  bool a_is_plan_b = false;
  int64_t lda = 0, ldb = 0, ldc = 0;
  int width = 0;  // output tile width 32/64/128/256; 0 = the built-in model
};

struct SplitPlan;
// Memory of a split plan.  Slices of a constant plan operand (static_a /
// static_b) persist with the plan; everything rewritten by each run (the
// other operands' slices and exponents, split-K partial sums) lives in
// `arena` when given (split_plan_sizes bytes, 256-byte aligned, shared by
// plans that never run at the same time), else in the plan's own buffer.
struct SplitMem {
  bool static_a = false, static_b = false;
  unsigned char* arena = nullptr;
};
int split_plan_sizes(const std::vector<SplitProblem>& probs, int slices, bool static_a, bool static_b,
                     size_t* persist_bytes, size_t* arena_bytes);
int create_split_plan(const std::vector<SplitProblem>& probs, int slices, SplitPlan** out,
                      const SplitMem* mem = nullptr);
// plan_a / plan_b: re-split the operands that come from the plan's packed A /
// B (false when unchanged since the last run, e.g. constant integrals).
int run_split_plan(SplitPlan* sp, bool plan_a, bool plan_b, cudaStream_t st);
// Only the split kernels (for operands that stay constant afterwards).
int split_operands(SplitPlan* sp, bool plan_a, bool plan_b, cudaStream_t st);
void destroy_split_plan(SplitPlan* sp);
// Force the output tile width of plans created afterwards (0 = model).
int split_set_width(int bn);
double split_plan_bytes(const SplitPlan* sp);
// bf16 tensor flops one run issues (S(S+1)/2 slice products on padded tiles).
double split_plan_tensor_flops(const SplitPlan* sp);
// Error word of the GEMM kernel (0 = ok, else the wait that ran out); syncs.
int split_plan_error(SplitPlan* sp);

// GEMM launches of several plans merged into one launch per kernel (the
// persistent iteration program): launches of the same class run the same
// kernel with the same slice count, so their problems can share a launch.
int split_launch_class(const SplitPlan* sp, int launch);
struct SplitMerged;
// parts: (plan, launch index) pairs of one class; err: the merged launch's
// error word (bounded waits that run out).
int split_merge(const std::vector<std::pair<SplitPlan*, int>>& parts, int* err, SplitMerged** out);
int split_merged_run(const SplitMerged* m, cudaStream_t st);
void split_merged_destroy(SplitMerged* m);

}  // namespace gbx
