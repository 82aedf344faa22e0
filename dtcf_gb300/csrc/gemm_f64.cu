// Grouped FP64 GEMM on the FP64 tensor pipe (DMMA, mma.sync m8n8k4 f64).
//
// C_p (+)= alpha_p * A_p * B_p^T for every problem p of a launch.  One
// persistent grid walks a device-side queue of 64x64 output tiles over all
// problems (an atomic ticket per CTA), so a whole contraction -- every block
// triple, every irrep -- is one launch.  Operands are read through generic
// element strides, which covers the transposed forms of local_contraction.
//
// On GB300 the FP64 pipe runs near 1 TFLOP/s (DMMA and FFMA alike), so this
// kernel is FP64-issue bound at any reasonable occupancy; the data path is
// kept simple (register-staged shared-memory tiles, double buffered).
#include <algorithm>

#include "common.h"

namespace gbx {

namespace {
constexpr int BM = kF64TileM, BN = kF64TileN, BK = 16;
constexpr int kThreads = 128;
constexpr int kPad = 1;  // pad rows to spread shared-memory banks
}  // namespace

int f64_tiles(int m, int n) { return ((m + BM - 1) / BM) * ((n + BN - 1) / BN); }

__device__ __forceinline__ void dmma884(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(kThreads) grouped_gemm_f64_kernel(const GemmProblem* __restrict__ probs, int nprob,
                                                                    const int* __restrict__ tile_first,
                                                                    int total_tiles, int* __restrict__ ticket) {
  // ticket == nullptr: static round-robin over tiles; otherwise a device
  // work queue (one atomic ticket per tile) balances uneven problem sizes.
  __shared__ double As[2][BM][BK + kPad];
  __shared__ double Bs[2][BN][BK + kPad];
  __shared__ int s_tile;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;  // 2x2 warps, 32x32 each

  for (int iter = 0;; ++iter) {
    if (ticket) {
      if (tid == 0) s_tile = atomicAdd(ticket, 1);
      __syncthreads();
    }
    const int tile = ticket ? s_tile : (int)blockIdx.x + iter * (int)gridDim.x;
    if (ticket) __syncthreads();
    if (tile >= total_tiles) break;
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (tile_first[mid] <= tile) lo = mid; else hi = mid - 1;
    }
    const GemmProblem p = probs[lo];
    const int local = tile - tile_first[lo];
    const int ntn = (p.n + BN - 1) / BN;
    const int m0 = (local / ntn) * BM, n0 = (local % ntn) * BN;

    double acc[4][4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    // register staging: each thread loads 8 A and 8 B elements per K step
    double ra[8], rb[8];
    auto load_regs = [&](int k0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        int e = tid + r * kThreads;  // 0..1023 over a 64 x 16 tile
        int row = e / BK, col = e % BK;
        int gm = m0 + row, gk = k0 + col, gn = n0 + row;
        ra[r] = (gm < p.m && gk < p.k) ? __ldg(p.A + (int64_t)gm * p.a_rs + (int64_t)gk * p.a_cs) : 0.0;
        rb[r] = (gn < p.n && gk < p.k) ? __ldg(p.B + (int64_t)gn * p.b_rs + (int64_t)gk * p.b_cs) : 0.0;
      }
    };
    auto store_regs = [&](int buf) {
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        int e = tid + r * kThreads;
        int row = e / BK, col = e % BK;
        As[buf][row][col] = ra[r];
        Bs[buf][row][col] = rb[r];
      }
    };

    const int nk = (p.k + BK - 1) / BK;
    if (nk > 0) {
      load_regs(0);
      store_regs(0);
    }
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
      const int buf = kt & 1;
      if (kt + 1 < nk) load_regs((kt + 1) * BK);
#pragma unroll
      for (int k4 = 0; k4 < BK; k4 += 4) {
        double af[4], bf[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) af[i] = As[buf][wm * 32 + i * 8 + (lane >> 2)][k4 + (lane & 3)];
#pragma unroll
        for (int j = 0; j < 4; ++j) bf[j] = Bs[buf][wn * 32 + j * 8 + (lane >> 2)][k4 + (lane & 3)];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) dmma884(acc[i][j], af[i], bf[j]);
      }
      if (kt + 1 < nk) store_regs(buf ^ 1);
      __syncthreads();
    }

    // epilogue: C (+)= alpha * acc
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gm = m0 + wm * 32 + i * 8 + (lane >> 2);
      if (gm >= p.m) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int gn = n0 + wn * 32 + j * 8 + (lane & 3) * 2 + h;
          if (gn >= p.n) continue;
          double* c = p.C + (int64_t)gm * p.c_rs + gn;
          double v = __dmul_rn(p.alpha, acc[i][j][h]);
          *c = p.accumulate ? __dadd_rn(*c, v) : v;
        }
      }
    }
  }
}

int grouped_gemm_f64(const GemmProblem* d_problems, int nprob, int total_tiles, const int* d_tile_first,
                     int* d_ticket, cudaStream_t st) {
  if (nprob <= 0 || total_tiles <= 0) return GBX_OK;
  if (d_ticket) GBX_CUDA(cudaMemsetAsync(d_ticket, 0, sizeof(int), st));
  int grid = std::min(total_tiles, 152 * 4);
  grouped_gemm_f64_kernel<<<grid, kThreads, 0, st>>>(d_problems, nprob, d_tile_first, total_tiles, d_ticket);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

}  // namespace gbx
