// Direct FP64 contraction engine: contractions with a small contracted extent
// per output element (an occupied index contracted with t1 or a Fock block,
// K ~ 6) are formed in place from the stored tiles.  On this GPU FP64
// instructions are the scarce resource (about 1.6 per clock per SM, for FMA
// and DMMA alike), so a contraction of K products per output element costs K
// FMAs here against the pack, split, GEMM and accumulate passes of the
// packed path, each of which streams the whole output-sized operand.
#include <algorithm>

#include "bodies.cuh"
#include "common.h"
#include "program.h"

namespace gbx {

namespace {
constexpr int kDirThreads = 512;
}  // namespace

// One CTA of 512 threads per work item (dev::direct_body).
template <bool kStore>
__global__ void __launch_bounds__(kDirThreads, 2)
    direct_contract_kernel(const DirItem* __restrict__ items, int nitems, const DirPair* __restrict__ pairs,
                           const double* __restrict__ A, const double* __restrict__ B, double* __restrict__ C,
                           double alpha) {
  __shared__ dev::DirSmem sm;
  dev::direct_body<kDirThreads, false, kStore>(items, nitems, pairs, A, B, C, alpha, blockIdx.x, gridDim.x, sm);
}

int run_direct(const DirItem* items, int nitems, const DirPair* pairs, const double* A, const double* B, double* C,
               double alpha, bool overwrite, cudaStream_t st) {
  if (nitems == 0) return GBX_OK;
  const int grid = std::min(nitems, 152 * 6);
  if (ProgRecorder* rec = prog_recording()) {
    ProgArgs a;
    a.direct = {items, pairs, A, B, C, alpha, nitems, overwrite ? 1 : 0};
    return prog_mem(rec, PK_DIRECT, (uint32_t)grid, a, {{A, false}, {B, false}, {C, true}});
  }
  if (overwrite) direct_contract_kernel<true><<<grid, kDirThreads, 0, st>>>(items, nitems, pairs, A, B, C, alpha);
  else direct_contract_kernel<false><<<grid, kDirThreads, 0, st>>>(items, nitems, pairs, A, B, C, alpha);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

}  // namespace gbx
