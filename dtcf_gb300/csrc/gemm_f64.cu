// Grouped FP64 GEMM on the FP64 tensor pipe (DMMA, mma.sync m8n8k4 f64).
//
// C_p (+)= alpha_p * A_p * B_p^T for every problem p of a launch.  One
// persistent grid walks a device-side queue of work items (an atomic ticket
// per CTA) over all problems, so a whole contraction -- every block triple,
// every irrep -- is one launch.  A work item is a 64x64 output tile and, for
// problems whose output is too small to fill the GPU, one K range of it
// (split-K): those write raw partial sums to a workspace that a second
// kernel reduces in a fixed order, so results are deterministic.  Operands
// are read through generic element strides, which covers the transposed
// forms of local_contraction.
//
// On GB300 the FP64 pipe runs near 1 TFLOP/s (DMMA and FFMA alike), so the
// kernel is FP64-issue bound at any reasonable occupancy; the data path is
// kept simple (register-staged shared-memory tiles, double buffered).
#include <algorithm>
#include <cstring>
#include <mutex>

#include "bodies.cuh"
#include "common.h"
#include "program.h"

namespace gbx {

namespace {
constexpr int BK = 16;
constexpr int kThreads = 128;
constexpr int kPad = 1;               // pad rows to spread shared-memory banks
constexpr int kFillTiles = 152 * 3;   // work items that keep every SM busy
constexpr int kMinChunk = 256;        // smallest K range of a split
constexpr int kRedThreads = dev::kRedThreads;
constexpr int kRedChunk = dev::kRedChunk;
constexpr int kThinN = 32, kThinK = 64, kThinMinWide = 16384;
constexpr int kSmallK = dev::kSmallK;
constexpr int kSmallKElems = dev::kSmallKElems;  // output elements per CTA
constexpr int kSmallOutDim = dev::kSmallOutDim;  // small outputs: at most 16 x 16 ...
constexpr int kSmallOutMinK = 4096;  // ... with at least this K
constexpr int kSmallOutChunk = 2048;  // K per work item
constexpr int kGemvDim = dev::kGemvDim;  // matrix-vector problems: one side at most this ...
constexpr int kGemvMinK = 64;         // ... with K above this
constexpr int kGemvItems = 152 * 4;   // work items that keep every SM busy
constexpr int kGemvMinChunk = 1024;   // smallest K range of a split
}  // namespace

// Tile shapes: 64x64 for large problems, 64x16 / 16x64 / 16x16 for skinny ones
// (output dimensions below 48), so small outputs do not waste the FP64 pipe.
// Thin problems (one output dimension <= 32, the other at least 4x larger,
// and either K <= 64 or at least 16384 wide rows to spread over the GPU) run
// on CUDA-core FP64 with exact shapes: variant 4 = one thread per row of C
// (N thin), variant 5 = one thread per column (M thin).
int f64_variant(int m, int n, int k) {
  // K <= 8 (outer products): one thread per output element
  if (k <= kSmallK) return 6;
  // one thread per wide row: only with enough rows to fill the GPU, or short K
  if (n <= kThinN && m >= 4 * n && (k <= kThinK || m >= kThinMinWide)) return 4;
  if (m <= kThinN && n >= 4 * m && (k <= kThinK || n >= kThinMinWide)) return 5;
  return (m < 48 ? 2 : 0) + (n < 48 ? 1 : 0);
}
int f64_variant(int m, int n) { return (m < 48 ? 2 : 0) + (n < 48 ? 1 : 0); }
// Planned launches also use variant 7: outputs of at most 16 x 16 with long
// K, one CTA per K chunk holding the whole output (reduced in a fixed order).
int f64_variant_planned(int m, int n, int k) {
  if (m <= kSmallOutDim && n <= kSmallOutDim && k >= kSmallOutMinK) return 7;
  // matrix-vector shapes (one side <= 2, K > 64): one warp per output of the
  // wide side, the wide operand's rows read once and coalesced
  if (k > kGemvMinK && ((m <= kGemvDim && n > kSmallOutDim) || (n <= kGemvDim && m > kSmallOutDim))) return 8;
  return f64_variant(m, n, k);
}
int f64_tile_m(int variant) { return (variant & 2) ? 16 : 64; }
int f64_tile_n(int variant) { return (variant & 1) ? 16 : 64; }
int f64_tiles(int m, int n) {
  const int v = f64_variant(m, n), tm = f64_tile_m(v), tn = f64_tile_n(v);
  return ((m + tm - 1) / tm) * ((n + tn - 1) / tn);
}

// One thread per row (variant 4) or per column (variant 5) of C; the thin
// operand (at most kThinN rows) is staged through shared memory kThinK
// columns at a time, so K is unbounded.  Each output is a k-ordered FMA
// chain, so results are deterministic.
template <bool kRows>
__global__ void __launch_bounds__(256) thin_gemm_f64_kernel(const GemmProblem* __restrict__ probs, int nprob,
                                                            const int* __restrict__ block_first, int total_blocks) {
  __shared__ double Ts[kThinN * kThinK];
  for (int blk = blockIdx.x; blk < total_blocks; blk += gridDim.x) {
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (block_first[mid] <= blk) lo = mid; else hi = mid - 1;
    }
    const GemmProblem& p = probs[lo];
    const int64_t i0 = (int64_t)(blk - block_first[lo]) * 256;
    // thin operand: B (N x K) for row mode, A (M x K) for column mode
    const int tn = kRows ? p.n : p.m;
    const double* T = kRows ? p.B : p.A;
    const int64_t trs = kRows ? p.b_rs : p.a_rs, tcs = kRows ? p.b_cs : p.a_cs;
    const int64_t i = i0 + threadIdx.x;
    const int64_t wide = kRows ? p.m : p.n;
    const double* W = kRows ? p.A + i * p.a_rs : p.B + i * p.b_rs;
    const int64_t wcs = kRows ? p.a_cs : p.b_cs;
    double acc[kThinN];
#pragma unroll
    for (int j = 0; j < kThinN; ++j) acc[j] = 0.0;
    for (int k0 = 0; k0 < p.k; k0 += kThinK) {
      const int kc = min(kThinK, p.k - k0);
      __syncthreads();
      for (int e = threadIdx.x; e < tn * kc; e += 256)
        Ts[e] = __ldg(T + (int64_t)(e / kc) * trs + (int64_t)(k0 + e % kc) * tcs);
      __syncthreads();
      if (i < wide) {
        for (int k = 0; k < kc; ++k) {
          const double w = __ldg(W + (int64_t)(k0 + k) * wcs);
#pragma unroll
          for (int j = 0; j < kThinN; ++j)
            if (j < tn) acc[j] = fma(w, Ts[j * kc + k], acc[j]);
        }
      }
    }
    if (i < wide) {
#pragma unroll
      for (int j = 0; j < kThinN; ++j) {
        if (j >= tn) break;
        double* c = kRows ? p.C + i * p.c_rs + j : p.C + (int64_t)j * p.c_rs + i;
        const double v = __dmul_rn(p.alpha, acc[j]);
        *c = p.accumulate ? __dadd_rn(*c, v) : v;
      }
    }
  }
}

// Matrix-vector shapes (variant 8): dev::gemv_body.
__global__ void __launch_bounds__(256) gemv_f64_kernel(const GemmProblem* __restrict__ probs, int nprob,
                                                       const int* __restrict__ block_first, int total_blocks) {
  dev::gemv_body<false>(probs, nprob, block_first, total_blocks, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void dmma884(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

template <int BM, int BN>
__global__ void __launch_bounds__(kThreads) grouped_gemm_f64_kernel(const GemmProblem* __restrict__ probs, int nprob,
                                                                    const int* __restrict__ tile_first,
                                                                    int total_tiles, int* __restrict__ ticket) {
  constexpr int WM = BM / 16, WN = BN / 16;  // m8n8 blocks per warp (2x2 warps)
  constexpr int LA = BM * BK / kThreads, LB = BN * BK / kThreads;
  // ticket == nullptr: static round-robin over work items; otherwise a device
  // work queue (one atomic ticket per item) balances uneven problem sizes.
  __shared__ double As[2][BM][BK + kPad];
  __shared__ double Bs[2][BN][BK + kPad];
  __shared__ int s_tile;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;  // 2x2 warps

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
    int local = tile - tile_first[lo];
    const int ntn = (p.n + BN - 1) / BN, ntm = (p.m + BM - 1) / BM;
    const int kc = local / (ntm * ntn);
    local -= kc * ntm * ntn;
    const int m0 = (local / ntn) * BM, n0 = (local % ntn) * BN;
    const int kbeg = kc * p.kchunk;
    const int kend = min(p.k, kbeg + p.kchunk);

    double acc[WM][WN][2];
#pragma unroll
    for (int i = 0; i < WM; ++i)
#pragma unroll
      for (int j = 0; j < WN; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    // register staging: each thread loads LA elements of A and LB of B per K step
    double ra[LA], rb[LB];
    auto load_regs = [&](int k0) {
#pragma unroll
      for (int r = 0; r < LA; ++r) {
        int e = tid + r * kThreads;
        int row = e / BK, col = e % BK;
        int gm = m0 + row, gk = k0 + col;
        ra[r] = (gm < p.m && gk < kend) ? __ldg(p.A + (int64_t)gm * p.a_rs + (int64_t)gk * p.a_cs) : 0.0;
      }
#pragma unroll
      for (int r = 0; r < LB; ++r) {
        int e = tid + r * kThreads;
        int row = e / BK, col = e % BK;
        int gn = n0 + row, gk = k0 + col;
        rb[r] = (gn < p.n && gk < kend) ? __ldg(p.B + (int64_t)gn * p.b_rs + (int64_t)gk * p.b_cs) : 0.0;
      }
    };
    auto store_regs = [&](int buf) {
#pragma unroll
      for (int r = 0; r < LA; ++r) {
        int e = tid + r * kThreads;
        As[buf][e / BK][e % BK] = ra[r];
      }
#pragma unroll
      for (int r = 0; r < LB; ++r) {
        int e = tid + r * kThreads;
        Bs[buf][e / BK][e % BK] = rb[r];
      }
    };

    const int nk = kend > kbeg ? (kend - kbeg + BK - 1) / BK : 0;
    if (nk > 0) {
      load_regs(kbeg);
      store_regs(0);
    }
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
      const int buf = kt & 1;
      if (kt + 1 < nk) load_regs(kbeg + (kt + 1) * BK);
#pragma unroll
      for (int k4 = 0; k4 < BK; k4 += 4) {
        double af[WM], bf[WN];
#pragma unroll
        for (int i = 0; i < WM; ++i) af[i] = As[buf][wm * (BM / 2) + i * 8 + (lane >> 2)][k4 + (lane & 3)];
#pragma unroll
        for (int j = 0; j < WN; ++j) bf[j] = Bs[buf][wn * (BN / 2) + j * 8 + (lane >> 2)][k4 + (lane & 3)];
#pragma unroll
        for (int i = 0; i < WM; ++i)
#pragma unroll
          for (int j = 0; j < WN; ++j) dmma884(acc[i][j], af[i], bf[j]);
      }
      if (kt + 1 < nk) store_regs(buf ^ 1);
      __syncthreads();
    }

    // epilogue: C (+)= alpha * acc, or the raw partial of this K range
    double* part = p.partial ? p.partial + (int64_t)kc * p.m * p.n : nullptr;
#pragma unroll
    for (int i = 0; i < WM; ++i) {
      const int gm = m0 + wm * (BM / 2) + i * 8 + (lane >> 2);
      if (gm >= p.m) continue;
#pragma unroll
      for (int j = 0; j < WN; ++j) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int gn = n0 + wn * (BN / 2) + j * 8 + (lane & 3) * 2 + h;
          if (gn >= p.n) continue;
          if (part) {
            part[(int64_t)gm * p.n + gn] = acc[i][j][h];
          } else {
            double* c = p.C + (int64_t)gm * p.c_rs + gn;
            double v = __dmul_rn(p.alpha, acc[i][j][h]);
            *c = p.accumulate ? __dadd_rn(*c, v) : v;
          }
        }
      }
    }
  }
}

// K <= 8 (dev::small_k_body).
__global__ void __launch_bounds__(256) small_k_gemm_f64_kernel(const GemmProblem* __restrict__ probs, int nprob,
                                                               const int* __restrict__ block_first, int total_blocks) {
  dev::small_k_body<false>(probs, nprob, block_first, total_blocks, blockIdx.x, gridDim.x);
}

// Small output, long K (variant 7, dev::small_out_body).
__global__ void __launch_bounds__(256) small_out_gemm_f64_kernel(const GemmProblem* __restrict__ probs, int nprob,
                                                                 const int* __restrict__ item_first, int total) {
  __shared__ dev::SmallOutSmem sm;
  dev::small_out_body<false>(probs, nprob, item_first, total, blockIdx.x, gridDim.x, sm);
}

// Fixed-order reduction of split-K partials into C.
__global__ void __launch_bounds__(kRedThreads) splitk_reduce_kernel(const GemmProblem* __restrict__ probs,
                                                                    const int* __restrict__ red_prob,
                                                                    const uint32_t* __restrict__ red_first, int nred,
                                                                    uint32_t nchunks) {
  dev::splitk_reduce_body<false>(probs, red_prob, red_first, nred, nchunks, blockIdx.x, gridDim.x);
}

void F64Gemm::release() {
  auto fr = [&](void* q) {
    if (!q) return;
    if (async_stream_set) cudaFreeAsync(q, async_stream); else dev_free(q);
  };
  for (auto& sb : subs) {
    fr(sb.d_probs);
    fr(sb.d_first);
    fr(sb.d_ticket);
  }
  subs.clear();
  fr(d_all);
  fr(d_partial);
  fr(d_red_prob);
  fr(d_red_first);
  d_all = nullptr;
  d_partial = nullptr;
  d_red_prob = nullptr;
  d_red_first = nullptr;
  nprob = nred = 0;
  red_chunks = 0;
}

namespace {
// K split of a DMMA problem: only when the output tiles of the whole launch
// leave the GPU idle; ranges are multiples of the K step.
void f64_ksplit(int k, int64_t out_tiles, int* ks_out, int* chunk_out) {
  int ks = 1;
  if (out_tiles < kFillTiles && k > 2 * kMinChunk) {
    int want = (int)((kFillTiles + out_tiles - 1) / out_tiles);
    ks = std::max(1, std::min(want, (k + kMinChunk - 1) / kMinChunk));
  }
  int chunk = (k + ks - 1) / ks;
  chunk = ((chunk + BK - 1) / BK) * BK;
  ks = std::max(1, (k + chunk - 1) / chunk);
  *ks_out = ks;
  *chunk_out = chunk;
}
}  // namespace

int64_t f64_partial_elems(const std::vector<GemmProblem>& probs) {
  int64_t out_tiles = 0, part = 0;
  for (auto& q : probs)
    if (q.m > 0 && q.n > 0) out_tiles += f64_tiles(q.m, q.n);
  for (auto& q : probs) {
    if (q.m <= 0 || q.n <= 0) continue;
    const int v = f64_variant_planned(q.m, q.n, q.k);
    if (v == 7) {
      const int64_t ks7 = (q.k + kSmallOutChunk - 1) / kSmallOutChunk;
      if (ks7 > 1) part += ks7 * q.m * q.n;
      continue;
    }
    if (v == 8) {
      const int64_t wide = q.m <= kGemvDim && q.m <= q.n ? q.n : q.m;
      const int64_t groups = (wide + 7) / 8;
      int64_t ks8 = 1;
      if (groups < kGemvItems && q.k > 2 * kGemvMinChunk)
        ks8 = std::min<int64_t>((kGemvItems + groups - 1) / groups, (q.k + kGemvMinChunk - 1) / kGemvMinChunk);
      int64_t chunk = (q.k + ks8 - 1) / ks8;
      chunk = (chunk + 31) / 32 * 32;
      ks8 = std::max<int64_t>(1, (q.k + chunk - 1) / chunk);
      if (ks8 > 1) part += ks8 * q.m * q.n;
      continue;
    }
    if (v >= 4) continue;
    int ks = 1, chunk = 0;
    f64_ksplit(q.k, out_tiles, &ks, &chunk);
    if (ks > 1) part += (int64_t)ks * q.m * q.n;
  }
  return part;
}

int F64Gemm::build(const std::vector<GemmProblem>& in, bool async, cudaStream_t st, const std::vector<int>* variants) {
  release();
  async_stream_set = async;
  async_stream = st;
  std::vector<GemmProblem> probs;
  std::vector<int> want;
  for (size_t i = 0; i < in.size(); ++i) {
    const GemmProblem& q = in[i];
    if (q.m <= 0 || q.n <= 0) continue;
    probs.push_back(q);
    int v = variants && i < variants->size() ? (*variants)[i] : -1;
    if (v < -1 || v > 8) return fail(GBX_EINVAL, "FP64 tile variant %d", v);
    // the thin kernels need their shape limits
    if ((v == 4 && q.n > kThinN) || (v == 5 && q.m > kThinN) || (v == 6 && q.k > kSmallK) ||
        (v == 7 && (q.m > kSmallOutDim || q.n > kSmallOutDim)) || (v == 8 && q.m > kGemvDim && q.n > kGemvDim))
      return fail(GBX_EINVAL, "FP64 tile variant %d does not fit %d x %d x %d", v, q.m, q.n, q.k);
    want.push_back(v);
  }
  nprob = (int)probs.size();
  if (nprob == 0) return GBX_OK;
  // total output tiles decide how much K splitting the small problems get
  int64_t out_tiles = 0;
  for (auto& q : probs) out_tiles += f64_tiles(q.m, q.n);
  int64_t part_elems = 0;
  std::vector<int> red;
  std::vector<uint32_t> red_first;
  uint64_t rc = 0;
  for (int i = 0; i < nprob; ++i) {
    GemmProblem& q = probs[i];
    int ks = 1;
    const int thin = want[i] >= 0 ? want[i] : f64_variant_planned(q.m, q.n, q.k);
    if (thin == 7) {  // small output: one work item per K chunk, fixed-order reduction
      ks = std::max(1, (q.k + kSmallOutChunk - 1) / kSmallOutChunk);
      q.ksplit = ks;
      q.kchunk = kSmallOutChunk;
      q.partial = nullptr;
      q.pad_ = 7;
      if (ks > 1) {
        q.partial = (double*)(intptr_t)(part_elems + 1);  // offset + 1, patched below
        part_elems += (int64_t)ks * q.m * q.n;
        red.push_back(i);
        red_first.push_back((uint32_t)rc);
        rc += ((uint64_t)q.m * q.n + kRedChunk - 1) / kRedChunk;
      }
      continue;
    }
    if (thin == 8) {  // matrix-vector: K ranges when the outputs are few
      const int64_t wide = q.m <= kGemvDim && q.m <= q.n ? q.n : q.m;
      const int64_t groups = (wide + 7) / 8;
      ks = 1;
      if (groups < kGemvItems && q.k > 2 * kGemvMinChunk)
        ks = (int)std::min<int64_t>((kGemvItems + groups - 1) / groups, (q.k + kGemvMinChunk - 1) / kGemvMinChunk);
      int chunk = (q.k + ks - 1) / ks;
      chunk = (chunk + 31) / 32 * 32;
      ks = std::max(1, (q.k + chunk - 1) / chunk);
      q.ksplit = ks;
      q.kchunk = chunk;
      q.partial = nullptr;
      q.pad_ = 8;
      if (ks > 1) {
        q.partial = (double*)(intptr_t)(part_elems + 1);  // offset + 1, patched below
        part_elems += (int64_t)ks * q.m * q.n;
        red.push_back(i);
        red_first.push_back((uint32_t)rc);
        rc += ((uint64_t)q.m * q.n + kRedChunk - 1) / kRedChunk;
      }
      continue;
    }
    if (thin >= 4) {  // thin and small-K kernels: no split-K
      q.ksplit = 1;
      q.kchunk = std::max(q.k, BK);
      q.partial = nullptr;
      q.pad_ = thin;
      continue;
    }
    int chunk = 0;
    f64_ksplit(q.k, out_tiles, &ks, &chunk);
    q.ksplit = ks;
    q.kchunk = std::max(chunk, BK);
    q.partial = nullptr;
    q.pad_ = want[i] >= 0 ? want[i] : f64_variant(q.m, q.n);
    if (ks > 1) {
      q.partial = (double*)(intptr_t)(part_elems + 1);  // offset + 1, patched below
      part_elems += (int64_t)ks * q.m * q.n;
      red.push_back(i);
      red_first.push_back((uint32_t)rc);
      rc += ((uint64_t)q.m * q.n + kRedChunk - 1) / kRedChunk;
    }
  }
  nred = (int)red.size();
  red_chunks = (uint32_t)rc;
  auto alloc = [&](void** q, size_t bytes) -> int {
    if (bytes == 0) {
      *q = nullptr;
      return GBX_OK;
    }
    if (async) {
      GBX_CUDA(cudaMallocAsync(q, bytes, st));
      return GBX_OK;
    }
    return dev_alloc(q, bytes);
  };
  auto copy = [&](void* dst, const void* src, size_t bytes) -> int {
    if (bytes == 0) return GBX_OK;
    if (async) GBX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    else GBX_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return GBX_OK;
  };
  GBX_TRY(alloc((void**)&d_partial, sizeof(double) * part_elems));
  for (auto& q : probs)
    if (q.partial) q.partial = d_partial + ((intptr_t)q.partial - 1);
  // one launch per tile shape
  for (int v = 0; v < 9; ++v) {
    std::vector<GemmProblem> vp;
    std::vector<int> first;
    int64_t tiles = 0;
    for (auto& q : probs) {
      if (q.pad_ != v) continue;
      vp.push_back(q);
      first.push_back((int)tiles);
      if (v == 4) tiles += (q.m + 255) / 256;
      else if (v == 5) tiles += (q.n + 255) / 256;
      else if (v == 6) tiles += ((int64_t)q.m * q.n + kSmallKElems - 1) / kSmallKElems;
      else if (v == 7) tiles += q.ksplit;
      else if (v == 8) tiles += ((q.m <= kGemvDim && q.m <= q.n ? (int64_t)q.n : (int64_t)q.m) + 7) / 8 * q.ksplit;
      else tiles += (int64_t)((q.m + f64_tile_m(v) - 1) / f64_tile_m(v)) * ((q.n + f64_tile_n(v) - 1) / f64_tile_n(v)) * q.ksplit;
    }
    if (vp.empty()) continue;
    if (tiles >= (1ll << 31)) return fail(GBX_EUNSUPPORTED, "grouped GEMM has too many work items");
    Sub sb;
    sb.variant = v;
    sb.nprob = (int)vp.size();
    sb.total_tiles = (int)tiles;
    GBX_TRY(alloc((void**)&sb.d_probs, sizeof(GemmProblem) * vp.size()));
    GBX_TRY(alloc((void**)&sb.d_first, sizeof(int) * vp.size()));
    GBX_TRY(alloc((void**)&sb.d_ticket, sizeof(int)));
    GBX_TRY(copy(sb.d_probs, vp.data(), sizeof(GemmProblem) * vp.size()));
    GBX_TRY(copy(sb.d_first, first.data(), sizeof(int) * vp.size()));
    sb.first = first;
    sb.first.push_back((int)tiles);
    subs.push_back(sb);
  }
  if (nred) {
    GBX_TRY(alloc((void**)&d_all, sizeof(GemmProblem) * nprob));
    GBX_TRY(copy(d_all, probs.data(), sizeof(GemmProblem) * nprob));
    GBX_TRY(alloc((void**)&d_red_prob, sizeof(int) * nred));
    GBX_TRY(alloc((void**)&d_red_first, sizeof(uint32_t) * nred));
    GBX_TRY(copy(d_red_prob, red.data(), sizeof(int) * nred));
    GBX_TRY(copy(d_red_first, red_first.data(), sizeof(uint32_t) * nred));
  }
  workspace_bytes = (double)part_elems * 8.0;
  return GBX_OK;
}

int F64Gemm::run(cudaStream_t st) const {
  if (nprob == 0) return GBX_OK;
  if (ProgRecorder* rec = prog_recording()) {
    // the CUDA-core shapes become records of the persistent program (static
    // schedule over their work items); the DMMA tile shapes and the thin
    // kernels keep their own launches
    for (const Sub& sb : subs) {
      const int kind = sb.variant == 6 ? PK_SMALLK : sb.variant == 7 ? PK_SMALLOUT : sb.variant == 8 ? PK_GEMV : -1;
      if (kind >= 0) {
        ProgArgs a;
        a.gemm = {sb.d_probs, sb.d_first, sb.nprob, sb.total_tiles};
        GBX_TRY(prog_mem(rec, kind, (uint32_t)std::min(sb.total_tiles, 152 * 8), a, {}));
        continue;
      }
      const Sub* psb = &sb;
      GBX_TRY(prog_ext(rec, [psb](cudaStream_t s2) { return run_sub(*psb, s2); }, {}));
    }
    if (nred) {
      ProgArgs a;
      a.kred = {d_all, d_red_prob, d_red_first, nred, red_chunks};
      GBX_TRY(prog_mem(rec, PK_SPLITKRED, std::min<uint32_t>(red_chunks, 152u * 8u), a, {}));
    }
    return GBX_OK;
  }
  for (const Sub& sb : subs) GBX_TRY(run_sub(sb, st));
  if (nred) {
    int rg = (int)std::min<uint32_t>(red_chunks, 152u * 8u);
    splitk_reduce_kernel<<<rg, kRedThreads, 0, st>>>(d_all, d_red_prob, d_red_first, nred, red_chunks);
    GBX_CUDA(cudaGetLastError());
  }
  return GBX_OK;
}

int F64Gemm::run_sub(const Sub& sb, cudaStream_t st) {
  GBX_CUDA(cudaMemsetAsync(sb.d_ticket, 0, sizeof(int), st));
  int grid = std::min(sb.total_tiles, 152 * 4);
  switch (sb.variant) {
    case 0:
      grouped_gemm_f64_kernel<64, 64><<<grid, kThreads, 0, st>>>(sb.d_probs, sb.nprob, sb.d_first, sb.total_tiles,
                                                                 sb.d_ticket);
      break;
    case 1:
      grouped_gemm_f64_kernel<64, 16><<<grid, kThreads, 0, st>>>(sb.d_probs, sb.nprob, sb.d_first, sb.total_tiles,
                                                                 sb.d_ticket);
      break;
    case 2:
      grouped_gemm_f64_kernel<16, 64><<<grid, kThreads, 0, st>>>(sb.d_probs, sb.nprob, sb.d_first, sb.total_tiles,
                                                                 sb.d_ticket);
      break;
    case 3:
      grouped_gemm_f64_kernel<16, 16><<<grid, kThreads, 0, st>>>(sb.d_probs, sb.nprob, sb.d_first, sb.total_tiles,
                                                                 sb.d_ticket);
      break;
    case 4:
      thin_gemm_f64_kernel<true><<<std::min(sb.total_tiles, 152 * 8), 256, 0, st>>>(sb.d_probs, sb.nprob, sb.d_first,
                                                                                    sb.total_tiles);
      break;
    case 6:
      small_k_gemm_f64_kernel<<<std::min(sb.total_tiles, 152 * 8), 256, 0, st>>>(sb.d_probs, sb.nprob, sb.d_first,
                                                                                 sb.total_tiles);
      break;
    case 7:
      small_out_gemm_f64_kernel<<<std::min(sb.total_tiles, 152 * 8), 256, 0, st>>>(sb.d_probs, sb.nprob,
                                                                                   sb.d_first, sb.total_tiles);
      break;
    case 8:
      gemv_f64_kernel<<<std::min(sb.total_tiles, 152 * 8), 256, 0, st>>>(sb.d_probs, sb.nprob, sb.d_first,
                                                                         sb.total_tiles);
      break;
    default:
      thin_gemm_f64_kernel<false><<<std::min(sb.total_tiles, 152 * 8), 256, 0, st>>>(sb.d_probs, sb.nprob,
                                                                                     sb.d_first, sb.total_tiles);
      break;
  }
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}


namespace {
// A single-problem launch of variant v over work items [0, tiles).
int launch_one(int v, const GemmProblem* prob, const int* zero, int tiles, cudaStream_t st) {
  const int grid = std::min(tiles, 152 * 4), tgrid = std::min(tiles, 152 * 8);
  switch (v) {
    case 0: grouped_gemm_f64_kernel<64, 64><<<grid, kThreads, 0, st>>>(prob, 1, zero, tiles, nullptr); break;
    case 1: grouped_gemm_f64_kernel<64, 16><<<grid, kThreads, 0, st>>>(prob, 1, zero, tiles, nullptr); break;
    case 2: grouped_gemm_f64_kernel<16, 64><<<grid, kThreads, 0, st>>>(prob, 1, zero, tiles, nullptr); break;
    case 3: grouped_gemm_f64_kernel<16, 16><<<grid, kThreads, 0, st>>>(prob, 1, zero, tiles, nullptr); break;
    case 4: thin_gemm_f64_kernel<true><<<tgrid, 256, 0, st>>>(prob, 1, zero, tiles); break;
    case 6: small_k_gemm_f64_kernel<<<tgrid, 256, 0, st>>>(prob, 1, zero, tiles); break;
    case 7: small_out_gemm_f64_kernel<<<tgrid, 256, 0, st>>>(prob, 1, zero, tiles); break;
    case 8: gemv_f64_kernel<<<tgrid, 256, 0, st>>>(prob, 1, zero, tiles); break;
    default: thin_gemm_f64_kernel<false><<<tgrid, 256, 0, st>>>(prob, 1, zero, tiles); break;
  }
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}
}  // namespace

int F64Gemm::run_each(cudaStream_t st) const {
  if (nprob == 0) return GBX_OK;
  for (const Sub& sb : subs) {
    // d_first[0] is 0: problem i is launched as a one-problem group whose
    // first-work-item table is that zero
    for (int i = 0; i < sb.nprob; ++i)
      GBX_TRY(launch_one(sb.variant, sb.d_probs + i, sb.d_first, sb.first[i + 1] - sb.first[i], st));
  }
  if (nred) {
    int rg = (int)std::min<uint32_t>(red_chunks, 152u * 8u);
    splitk_reduce_kernel<<<rg, kRedThreads, 0, st>>>(d_all, d_red_prob, d_red_first, nred, red_chunks);
    GBX_CUDA(cudaGetLastError());
  }
  return GBX_OK;
}
}  // namespace gbx

// ---- allocation-free local contraction ----------------------------------
//
// Some callers cannot let a library allocate device memory: a framework that
// has handed nearly all of the device's memory to its own caching pool (a
// library cudaMalloc then fails, or forces the pool to give memory back), and
// latency-bound loops that keep other streams busy (cudaFree synchronises the
// device and stalls them).  For them gbx_local_contraction_noalloc runs the
// same FP64 GEMM with its descriptor and split-K partial sums in one
// file-scope device array of kNoAllocBytes, which every GPU that loads the
// library holds until the process exits.  What must start at zero: the
// work-queue ticket, written (with the whole descriptor, by a one-thread
// kernel on the caller's stream) by every call before its GEMM runs.  The
// partial-sum slabs need no clearing: every split-K range overwrites its slab
// in full before the reduction reads it.
namespace gbx {
namespace {
constexpr size_t kNoAllocHeader = 4096;                   // descriptor, schedule words
constexpr size_t kNoAllocPartialBytes = 32ull << 20;      // split-K partial sums
constexpr size_t kNoAllocBytes = kNoAllocHeader + kNoAllocPartialBytes;
constexpr int64_t kNoAllocMaxElems = (int64_t)(kNoAllocPartialBytes / sizeof(double));

struct NoAllocHeader {
  GemmProblem prob;
  int first;         // first work item of the problem (always 0)
  int ticket;        // work-queue counter, reset by every call
  int red_prob;      // split-K reduction: problem index (0)
  uint32_t red_first;
};
static_assert(sizeof(NoAllocHeader) <= kNoAllocHeader, "header does not fit");
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Writes the call's descriptor (ticket 0 included) into the scratch array
// ahead of the GEMM on the same stream: the descriptor travels as a kernel
// argument, so the call needs no host staging buffer and never waits for the
// stream.
__global__ void noalloc_header_kernel(NoAllocHeader h, NoAllocHeader* dst) { *dst = h; }

// Device address of the scratch array, looked up once per device (the host
// symbol is only a stand-in for it).
static int noalloc_scratch(unsigned char** out) {
  static std::mutex mu;
  static unsigned char* addr[256] = {nullptr};
  int dev = 0;
  GBX_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return fail(GBX_EUNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
    addr[dev] = (unsigned char*)p;
  }
  *out = addr[dev];
  return GBX_OK;
}

}  // namespace gbx

extern "C" int gbx_local_contraction_noalloc(int n_a, int n_b, int n_k, const double* d_A, const double* d_B,
                                             double* d_C, int at, int bt, double alpha, void* stream) {
  using namespace gbx;
  if (n_a < 0 || n_b < 0 || n_k < 0) return fail(GBX_EINVAL, "negative extent");
  if (n_a == 0 || n_b == 0) return GBX_OK;
  if ((int64_t)n_a * n_b > kNoAllocMaxElems)
    return fail(GBX_EINVAL, "output of %lld elements exceeds the allocation-free workspace (max %lld elements)",
                (long long)n_a * n_b, (long long)kNoAllocMaxElems);
  unsigned char* scratch = nullptr;
  GBX_TRY(noalloc_scratch(&scratch));
  cudaStream_t st = (cudaStream_t)stream;
  NoAllocHeader h;
  std::memset(&h, 0, sizeof(h));
  GemmProblem& p = h.prob;
  p.A = d_A;
  p.B = d_B;
  p.C = d_C;
  p.a_rs = at ? 1 : n_k;
  p.a_cs = at ? n_a : 1;
  p.b_rs = bt ? n_k : 1;
  p.b_cs = bt ? 1 : n_b;
  p.c_rs = n_b;
  p.m = n_a;
  p.n = n_b;
  p.k = n_k;
  p.alpha = alpha;
  p.accumulate = 1;
  // same schedule as the allocating path, split-K capped by the workspace
  const int variant = f64_variant(n_a, n_b, n_k);
  int ks = 1;
  const int out_tiles = f64_tiles(n_a, n_b);
  if (variant < 4 && out_tiles < kFillTiles && n_k > 2 * kMinChunk) {
    int want = (kFillTiles + out_tiles - 1) / out_tiles;
    ks = std::max(1, std::min(want, (n_k + kMinChunk - 1) / kMinChunk));
    ks = (int)std::min<int64_t>(ks, kNoAllocMaxElems / ((int64_t)n_a * n_b));
  }
  int chunk = (n_k + ks - 1) / ks;
  chunk = ((chunk + BK - 1) / BK) * BK;
  ks = std::max(1, (n_k + chunk - 1) / chunk);
  p.ksplit = ks;
  p.kchunk = std::max(chunk, BK);
  p.pad_ = variant;
  p.partial = ks > 1 ? (double*)(scratch + kNoAllocHeader) : nullptr;
  h.first = 0;
  h.ticket = 0;
  h.red_prob = 0;
  h.red_first = 0;
  NoAllocHeader* dh = (NoAllocHeader*)scratch;
  // the descriptor is written on the stream by a one-thread kernel; the ticket starts at 0
  noalloc_header_kernel<<<1, 1, 0, st>>>(h, dh);
  GBX_CUDA(cudaGetLastError());
  int tiles;
  if (variant == 4) tiles = (n_a + 255) / 256;
  else if (variant == 5) tiles = (n_b + 255) / 256;
  else if (variant == 6) tiles = (int)(((int64_t)n_a * n_b + kSmallKElems - 1) / kSmallKElems);
  else tiles = f64_tiles(n_a, n_b) * ks;
  const GemmProblem* dp = &dh->prob;
  const int* df = &dh->first;
  int* dt = &dh->ticket;
  const int grid = std::min(tiles, 152 * 4);
  switch (variant) {
    case 0: grouped_gemm_f64_kernel<64, 64><<<grid, kThreads, 0, st>>>(dp, 1, df, tiles, dt); break;
    case 1: grouped_gemm_f64_kernel<64, 16><<<grid, kThreads, 0, st>>>(dp, 1, df, tiles, dt); break;
    case 2: grouped_gemm_f64_kernel<16, 64><<<grid, kThreads, 0, st>>>(dp, 1, df, tiles, dt); break;
    case 3: grouped_gemm_f64_kernel<16, 16><<<grid, kThreads, 0, st>>>(dp, 1, df, tiles, dt); break;
    case 4: thin_gemm_f64_kernel<true><<<std::min(tiles, 152 * 8), 256, 0, st>>>(dp, 1, df, tiles); break;
    case 6: small_k_gemm_f64_kernel<<<std::min(tiles, 152 * 8), 256, 0, st>>>(dp, 1, df, tiles); break;
    default: thin_gemm_f64_kernel<false><<<std::min(tiles, 152 * 8), 256, 0, st>>>(dp, 1, df, tiles); break;
  }
  GBX_CUDA(cudaGetLastError());
  if (ks > 1) {
    const uint32_t chunks = (uint32_t)(((int64_t)n_a * n_b + kRedChunk - 1) / kRedChunk);
    const int rg = (int)std::min<uint32_t>(chunks, 152u * 8u);
    splitk_reduce_kernel<<<rg, kRedThreads, 0, st>>>(dp, &dh->red_prob, &dh->red_first, 1, chunks);
    GBX_CUDA(cudaGetLastError());
  }
  return GBX_OK;
}
