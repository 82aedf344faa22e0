// C-ABI plan entry points over RRR tensor descriptors (include/gbx.h).
#include <cstring>
#include <memory>

#include "plan.h"
#include "split.h"

using namespace gbx;

struct gbx_plan {
  std::unique_ptr<ContractionPlan> p;
};

namespace {

int layout_from_desc(const gbx_tensor_desc* t, int sign, TensorLayout& L) {
  if (!t || t->dims < 1 || t->dims > kMaxDims || !t->sym || (int)std::strlen(t->sym) != t->dims || !t->block_range ||
      !t->vgrid || t->num_tiles < 0 || (t->num_tiles > 0 && !t->tile_address))
    return fail(GBX_EINVAL, "bad tensor descriptor");
  L = TensorLayout();
  L.rank = t->dims;
  L.sign = sign;
  for (int d = 0; d < t->dims; ++d) {
    if (t->vgrid[d] < 1 || t->block_range[d] < 1) return fail(GBX_EINVAL, "bad block grid");
    L.dims.push_back(BlockDim::uniform(t->vgrid[d], t->block_range[d]));
    char c = t->sym[d];
    L.group.push_back((c == 'a' || c == 'A') ? 0 : (c == 'b' || c == 'B') ? 1 : -1);
  }
  for (int i = 0; i < t->num_tiles; ++i) {
    Coords c(t->tile_address + (int64_t)i * t->dims, t->tile_address + (int64_t)(i + 1) * t->dims);
    for (int d = 0; d < t->dims; ++d)
      if (c[d] < 0 || c[d] >= t->vgrid[d]) return fail(GBX_EINVAL, "tile address outside the block grid");
    if (L.find(c.data()) >= 0) return fail(GBX_EINVAL, "tile address repeated");
    L.add_tile(c);
  }
  return GBX_OK;
}

}  // namespace

extern "C" {

int gbx_plan_create(const gbx_tensor_desc* A, const gbx_tensor_desc* B, const gbx_tensor_desc* C, const char* idxA,
                    const char* idxB, const char* idxC, int mode, int sign, int slices, gbx_plan** plan) {
  if (!plan) return fail(GBX_EINVAL, "plan pointer is null");
  *plan = nullptr;
  if (sign != 1 && sign != -1) return fail(GBX_EINVAL, "sign must be +1 or -1");
  if (mode != GBX_MODE_FP64 && mode != GBX_MODE_SPLIT) return fail(GBX_EINVAL, "unknown mode %d", mode);
  TensorLayout LA, LB, LC;
  GBX_TRY(layout_from_desc(A, sign, LA));
  GBX_TRY(layout_from_desc(B, sign, LB));
  GBX_TRY(layout_from_desc(C, sign, LC));
  auto h = std::make_unique<gbx_plan>();
  GBX_TRY(plan_contraction(LA, LB, LC, split_labels(idxA), split_labels(idxB), split_labels(idxC),
                           mode == GBX_MODE_SPLIT ? Engine::Split : Engine::F64, slices, h->p));
  *plan = h.release();
  return GBX_OK;
}

int gbx_execute(gbx_plan* plan, const double* d_A, const double* d_B, double* d_C, double alpha, void* stream) {
  if (!plan || !plan->p) return fail(GBX_EINVAL, "null plan");
  return plan->p->execute(d_A, d_B, d_C, alpha, (cudaStream_t)stream);
}

double gbx_plan_flops(const gbx_plan* plan) { return (plan && plan->p) ? plan->p->flops : 0.0; }

int gbx_split_gemm(const double* d_A, const double* d_B, double* d_C, int64_t M, int64_t N, int64_t K, int slices,
                   void* stream) {
  if (M < 0 || N < 0 || K < 0) return fail(GBX_EINVAL, "negative extent");
  if (M == 0 || N == 0) return GBX_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (K == 0) {
    for (int64_t i = 0; i < M; ++i) GBX_CUDA(cudaMemsetAsync(d_C + i * N, 0, sizeof(double) * N, st));
    return GBX_OK;
  }
  SplitPlan* sp = nullptr;
  GBX_TRY(create_split_plan({SplitProblem{d_A, d_B, d_C, M, N, K}}, slices, &sp));
  int rc = run_split_plan(sp, true, true, st);
  if (rc == GBX_OK) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "split gemm", __FILE__, __LINE__);
  }
  if (rc == GBX_OK) {
    int err = split_plan_error(sp);
    if (err != 0) rc = fail(GBX_ETIMEOUT, "split GEMM: a bounded device wait ran out (stage %d)", err);
  }
  destroy_split_plan(sp);
  return rc;
}

int gbx_split_set_width(int width) { return split_set_width(width); }

int gbx_plan_destroy(gbx_plan* plan) {
  delete plan;
  return GBX_OK;
}

}  // extern "C"
