// Direct FP64 contraction engine: contractions with a small contracted extent
// per output element (an occupied index contracted with t1 or a Fock block,
// K ~ 6) are formed in place from the stored tiles.  On this GPU FP64
// instructions are the scarce resource (about 1.6 per clock per SM, for FMA
// and DMMA alike), so a contraction of K products per output element costs K
// FMAs here against the pack, split, GEMM and accumulate passes of the
// packed path, each of which streams the whole output-sized operand.
#include <algorithm>

#include "common.h"

namespace gbx {

namespace {
constexpr int kDirThreads = 512;
constexpr int kDirPer = kDirItemElems / kDirThreads;
static_assert(kDirPer * kDirThreads == kDirItemElems, "item size");
}  // namespace

// One CTA per work item (grid-stride).  Each thread holds kDirPer output
// elements in output order; for every tile pair it forms their operand base
// offsets, then walks the contracted indices with all kDirPer loads of A and
// of B in flight.  Consecutive lanes hold consecutive output elements, so the
// operand that carries the output's last dimension is read coalesced and the
// other one is (mostly) a broadcast.
__global__ void __launch_bounds__(kDirThreads, 2)
    direct_contract_kernel(const DirItem* __restrict__ items, int nitems, const DirPair* __restrict__ pairs,
                           const double* __restrict__ A, const double* __restrict__ B, double* __restrict__ C,
                           double alpha) {
  __shared__ DirItem s_item;
  __shared__ DirPair s_pairs[kDirMaxPairs];
  for (int i = blockIdx.x; i < nitems; i += gridDim.x) {
    __syncthreads();  // the previous item is finished with s_item and s_pairs
    if (threadIdx.x == 0) s_item = items[i];
    __syncthreads();
    const DirItem& it = s_item;
    if (threadIdx.x < it.npair) s_pairs[threadIdx.x] = pairs[it.pair0 + threadIdx.x];
    __syncthreads();
    const uint32_t e1 = it.f1.d, e2 = it.f2.d, e3 = it.f3.d;
    double acc[kDirPer];
#pragma unroll
    for (int k = 0; k < kDirPer; ++k) acc[k] = 0.0;
    for (uint32_t p = 0; p < it.npair; ++p) {
      const DirPair& pr = s_pairs[p];
      // offsets inside the operand tiles (a tile holds fewer than 2^31 elements)
      uint32_t ba[kDirPer], bb[kDirPer];
#pragma unroll
      for (int k = 0; k < kDirPer; ++k) {
        // lanes past the end repeat the last element (valid addresses, no store)
        const uint32_t f = it.f0 + min((uint32_t)(threadIdx.x + k * kDirThreads), it.n - 1);
        const uint32_t q3 = it.f3.div(f), c3 = f - q3 * e3;
        const uint32_t q2 = it.f2.div(q3), c2 = q3 - q2 * e2;
        const uint32_t c0 = it.f1.div(q2), c1 = q2 - c0 * e1;
        ba[k] = (uint32_t)(c0 * pr.sA[0] + c1 * pr.sA[1] + c2 * pr.sA[2] + c3 * pr.sA[3]);
        bb[k] = (uint32_t)(c0 * pr.sB[0] + c1 * pr.sB[1] + c2 * pr.sB[2] + c3 * pr.sB[3]);
      }
      // the pair's loop fields in registers; its sign flips the sign bit of
      // the A values on the integer pipe (written as a floating-point
      // negation it costs a second DFMA per product: both signs computed,
      // then selected)
      const uint32_t ek0 = pr.ek[0], ek1 = pr.ek[1];
      const int64_t sak0 = pr.sAk[0], sak1 = pr.sAk[1], sbk0 = pr.sBk[0], sbk1 = pr.sBk[1];
      const double* __restrict__ A0 = A + pr.offA;
      const double* __restrict__ B0 = B + pr.offB;
      const long long flip = pr.neg != 0 ? (long long)0x8000000000000000ull : 0ll;
      for (uint32_t k1 = 0; k1 < ek1; ++k1) {
        for (uint32_t k0 = 0; k0 < ek0; ++k0) {
          const double* __restrict__ pa = A0 + (int64_t)k0 * sak0 + (int64_t)k1 * sak1;
          const double* __restrict__ pb = B0 + (int64_t)k0 * sbk0 + (int64_t)k1 * sbk1;
          long long x[kDirPer];
          double y[kDirPer];
#pragma unroll
          for (int k = 0; k < kDirPer; ++k) {
            x[k] = __double_as_longlong(__ldg(pa + ba[k]));
            y[k] = __ldg(pb + bb[k]);
          }
#pragma unroll
          for (int k = 0; k < kDirPer; ++k) acc[k] = __fma_rn(__longlong_as_double(x[k] ^ flip), y[k], acc[k]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < kDirPer; ++k) {
      const uint32_t e = threadIdx.x + k * kDirThreads;
      if (e < it.n) {
        double* c = C + it.coff + e;
        *c = __fma_rn(alpha, acc[k], *c);
      }
    }
  }
}

int run_direct(const DirItem* items, int nitems, const DirPair* pairs, const double* A, const double* B, double* C,
               double alpha, cudaStream_t st) {
  if (nitems == 0) return GBX_OK;
  const int grid = std::min(nitems, 152 * 6);
  direct_contract_kernel<<<grid, kDirThreads, 0, st>>>(items, nitems, pairs, A, B, C, alpha);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

}  // namespace gbx
