// Split-precision FP64 GEMM on the tcgen05 tensor cores.
//
// C = A * B^T with A (M x K) and B (N x K) row-major FP64.
//
// Split.  Row i of A is scaled by 2^-e_i, e_i the smallest exponent with
// max_k |A_ik| < 2^e_i, and the scaled row is rounded to a fixed-point
// integer X = round(A_ik 2^(F - e_i)), F = 7 + 8 (S - 1).  X is cut into S
// balanced base-256 digits d_1..d_S (d_1 in [-128, 128], the rest in
// [-128, 127]) so that A_ik ~ 2^e_i sum_s d_s 2^-(7 + 8 (s - 1)).  Every digit
// is an integer that bf16 holds exactly.  The split is pure integer
// arithmetic on the FP64 bit pattern (no FP64 instructions); subnormal
// inputs count as zero.  B is split by rows the same way (exponents f_j).
//
// Products.  C_ij = 2^(e_i + f_j - 14) sum_l 2^(-8 l) X_l with
// X_l = sum_{s + t - 2 = l} (D^A_s D^B_t^T)_ij, kept for levels l <= S - 1
// (S (S + 1) / 2 slice products).  Each product runs on tcgen05.mma
// (kind::f16, bf16 operands from TMA-loaded 128B-swizzled shared memory,
// FP32 accumulator in TMEM).  |d_A d_B| <= 2^14, so a TMEM accumulation over
// at most 1024 K-elements stays below 2^24 and is exact; the kernel drains
// the accumulator after every such chunk into int32 registers (exact), folds
// the int32 sums into an FP64 Horner accumulator at each level change
// (acc = acc * 2^-8 + X, levels from S - 1 down to 0), and writes
// 2^(e_i + f_j - 14) * acc.  Only the fold and the final scale are FP64.
//
// Kernel roles (one or two CTAs per SM, persistent over 128 x BN output
// tiles of all problems): warp 0 issues TMA loads into a ring of shared-
// memory stages, warp 1 allocates TMEM and issues the MMAs (one elected
// lane), the drain warps (one per TMEM lane quarter and 64 columns) empty
// the accumulators.  Two to eight TMEM accumulator buffers let the drain of
// one chunk overlap the MMAs of the next.  Every mbarrier wait is bounded (about a second); on timeout the
// kernel records an error, stops issuing work, waits (bounded) for its own
// TMA copies and MMAs in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <memory>

#include "bodies.cuh"
#include "program.h"
#include "split.h"
#include "split_dev.h"

namespace gbx {

namespace {

constexpr int BM = 128;
constexpr int BK = 64;             // bf16 elements per 128-byte swizzled row
constexpr int kChunkKb = 16;       // k-blocks per exact FP32 chunk (16 * 64 = 1024)
constexpr int kFoldChunks = 127;   // int32 drain sums fold into FP64 before overflow

constexpr long long kWaitCycles = 2000000000ll;  // ~1 s at 2 GHz
constexpr int kSplitFill = 152 * 2;  // work items that keep every SM busy

using dev::kMidRow;
using dev::kShortRow;
using dev::kSplitChunk;

struct GemmParams {
  const DevProblem* probs;
  const int* tile_first;
  const CUtensorMap* maps;  // 2 per problem: A, B
  int nprob, total_tiles, S, L;
  int* err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; false (and the error word set) when it ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code,
                                          long long limit = kWaitCycles) {
  if (mbar_try_wait(bar, parity)) return true;
  long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit) {
      atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of
// 1024 bytes stacked along M/N (stride byte offset 1024).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)2 << 61;              // 128-byte swizzle
  return d;
}

// 64-byte swizzled rows (32 bf16 of K): 8-row groups 512 bytes apart
__device__ __forceinline__ uint64_t sdesc64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;     // stride byte offset
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)4 << 61;              // 64-byte swizzle
  return d;
}

template <int BN>
__device__ __forceinline__ constexpr uint32_t idesc_bf16() {
  return (1u << 4)                  // D: f32
         | (1u << 7)                // A: bf16
         | (1u << 10)               // B: bf16
         | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

// The same with the output width N (a multiple of 16, at most 256) as a value.
__device__ __forceinline__ constexpr uint32_t idesc_bf16_n(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

struct TileInfo {
  int p, m0, n0, kb0, nkb, kc;
};

template <int BN>
__device__ __forceinline__ TileInfo decode_tile(const GemmParams& P, int tile) {
  TileInfo t;
  int p = 0, hi = P.nprob - 1;
  while (p < hi) {
    const int mid = (p + hi + 1) >> 1;
    if (P.tile_first[mid] <= tile) p = mid; else hi = mid - 1;
  }
  const DevProblem& pr = P.probs[p];
  int local = tile - P.tile_first[p];
  const int per_k = pr.tiles_m * pr.tiles_n;
  t.kc = local / per_k;
  local -= t.kc * per_k;
  t.p = p;
  t.m0 = (local / pr.tiles_n) * BM;
  t.n0 = (local % pr.tiles_n) * BN;
  t.kb0 = t.kc * pr.kb_per_split;
  t.nkb = min(pr.nkb, t.kb0 + pr.kb_per_split) - t.kb0;
  return t;
}

// Number of slice pairs (s, t), 1 <= s, t <= S, on level l = s + t - 2.
__device__ __forceinline__ int level_pairs(int l, int S) {
  int lo = max(1, l + 2 - S), hi = min(S, l + 1);
  return hi >= lo ? hi - lo + 1 : 0;
}

template <int BN>
struct SplitCfg {
  static constexpr int kStageBytes = (BM + BN) * BK * 2;
  // narrow tiles: two CTAs per SM (half the shared memory each) and deeper
  // TMEM buffering, since their chunks are short and drains come often
  static constexpr int kCtasPerSm = BN <= 64 ? 2 : 1;
  static constexpr int kSmemBudget = (BN <= 64 ? 100 : 200) * 1024;
  static constexpr int kStages = (kSmemBudget / kStageBytes) < 8 ? (kSmemBudget / kStageBytes) : 8;
  static constexpr int kAccBufs = BN <= 32 ? 8 : (BN <= 64 ? 4 : 2);
  static constexpr uint32_t kTmemCols = (kAccBufs * BN <= 32) ? 32 : (kAccBufs * BN <= 64) ? 64
                                        : (kAccBufs * BN <= 128) ? 128 : (kAccBufs * BN <= 256) ? 256 : 512;
  // drain warps: 4 per 64 columns (one per TMEM lane quarter), at least 4
  static constexpr int kDrainWarps = BN >= 64 ? 4 * (BN / 64) : 4;
  static constexpr int kCols = BN >= 64 ? 64 : BN;  // columns per drain thread
  static constexpr int kThreads = 64 + 32 * kDrainWarps;
};

template <int BN>
struct Smem {
  alignas(1024) __nv_bfloat16 a[SplitCfg<BN>::kStages][BM * BK];
  alignas(1024) __nv_bfloat16 b[SplitCfg<BN>::kStages][BN * BK];
  uint64_t full[SplitCfg<BN>::kStages], empty[SplitCfg<BN>::kStages], accfull[SplitCfg<BN>::kAccBufs],
      accempty[SplitCfg<BN>::kAccBufs], done;
  uint32_t tmem_base;
};

// Warp roles: 0 TMA producer, 1 TMEM owner + MMA issuer, 2.. drain.  A drain
// thread owns one row (its TMEM lane) and up to 64 columns; its exact int32 sums
// fold into an FP64 Horner accumulator kept in the output tile itself (or the
// split-K partial), which stays in L2 between the few folds of a tile.
template <int BN>
__global__ void __launch_bounds__(SplitCfg<BN>::kThreads, SplitCfg<BN>::kCtasPerSm)
    split_gemm_kernel(const GemmParams P) {
  using Cfg = SplitCfg<BN>;
  constexpr int kAcc = Cfg::kAccBufs;
  constexpr int kStagesN = Cfg::kStages;
  constexpr int kCols = Cfg::kCols;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  Smem<BN>& sm = *reinterpret_cast<Smem<BN>*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr uint32_t kTxBytes = (BM + BN) * BK * 2;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStagesN; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < kAcc; ++b) {
      mbar_init(&sm.accfull[b], 1);
      mbar_init(&sm.accempty[b], Cfg::kDrainWarps);
    }
    mbar_init(&sm.done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(Cfg::kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  const int S = P.S, L = P.L;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < P.total_tiles && ok; tile += gridDim.x) {
        const TileInfo ti = decode_tile<BN>(P, tile);
        const CUtensorMap* ma = P.maps + 2 * ti.p;
        const CUtensorMap* mb = P.maps + 2 * ti.p + 1;
        for (int l = L; l >= 0 && ok; --l)
          for (int s = max(1, l + 2 - S); s <= min(S, l + 1) && ok; ++s) {
            const int t = l + 2 - s;
            for (int kb = ti.kb0; kb < ti.kb0 + ti.nkb; ++kb) {
              if (!mbar_wait(&sm.empty[stage], phase ^ 1, P.err, 1)) {
                ok = false;
                break;
              }
              mbar_expect_tx(&sm.full[stage], kTxBytes);
              tma_load_3d(sm.a[stage], ma, &sm.full[stage], kb * BK, ti.m0, s - 1);
              tma_load_3d(sm.b[stage], mb, &sm.full[stage], kb * BK, ti.n0, t - 1);
              if (++stage == kStagesN) {
                stage = 0;
                phase ^= 1;
              }
            }
          }
      }
      // wait (bounded) for the copies this warp issued to land before leaving
      for (int i = 0; i < kStagesN; ++i) {
        if (--stage < 0) {
          stage = kStagesN - 1;
          phase ^= 1;
        }
        long long t0 = clock64();
        while (!mbar_try_wait(&sm.full[stage], phase) && !mbar_try_wait(&sm.empty[stage], phase)) {
          if (clock64() - t0 > kWaitCycles) {
            atomicCAS(P.err, 0, 5);
            break;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int stage = 0, buf = 0;
      uint32_t phase = 0, aphase = 0;
      bool ok = true;
      constexpr uint32_t idesc = idesc_bf16<BN>();
      for (int tile = blockIdx.x; tile < P.total_tiles && ok; tile += gridDim.x) {
        const int nkb = decode_tile<BN>(P, tile).nkb;
        for (int l = L; l >= 0 && ok; --l) {
          const int items = level_pairs(l, S) * nkb;
          int item = 0;
          for (int s = max(1, l + 2 - S); s <= min(S, l + 1) && ok; ++s) {
            for (int kb = 0; kb < nkb && ok; ++kb, ++item) {
              const int in_chunk = item % kChunkKb;
              if (in_chunk == 0 && !mbar_wait(&sm.accempty[buf], aphase ^ 1, P.err, 2)) {
                ok = false;
                break;
              }
              if (!mbar_wait(&sm.full[stage], phase, P.err, 3)) {
                ok = false;
                break;
              }
              tc_fence_after();
              const uint32_t d = tmem + (uint32_t)(buf * BN);
              const uint64_t a0 = sdesc(smem_u32(sm.a[stage]));
              const uint64_t b0 = sdesc(smem_u32(sm.b[stage]));
#pragma unroll
              for (int k = 0; k < BK / 16; ++k)
                umma(d, a0 + (uint64_t)(k * 2), b0 + (uint64_t)(k * 2), idesc, (in_chunk > 0 || k > 0) ? 1u : 0u);
              umma_commit(&sm.empty[stage]);
              if (++stage == kStagesN) {
                stage = 0;
                phase ^= 1;
              }
              if (in_chunk == kChunkKb - 1 || item == items - 1) {
                umma_commit(&sm.accfull[buf]);
                if (++buf == kAcc) {
                  buf = 0;
                  aphase ^= 1;
                }
              }
            }
          }
        }
      }
      // all MMAs issued by this thread complete before TMEM is released
      umma_commit(&sm.done);
      mbar_wait(&sm.done, 0, P.err, 6);
    }
  } else {
    // ---------------- drain / fold (warps 2..) ----------------
    const int quarter = warp & 3;
    const int group = (warp - 2) >> 2;
    const int row_in_tile = quarter * 32 + lane;
    const uint32_t lane_addr = (uint32_t)(quarter * 32) << 16;
    const int col0 = group * kCols;
    int buf = 0;
    uint32_t aphase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < P.total_tiles && ok; tile += gridDim.x) {
      const TileInfo ti = decode_tile<BN>(P, tile);
      const DevProblem& pr = P.probs[ti.p];
      const int row = ti.m0 + row_in_tile;
      const bool row_ok = row < pr.M;
      double* crow = nullptr;
      double scale[1] = {0.0};
      if (row_ok) {
        crow = pr.ksplit > 1 ? pr.partial + ((int64_t)ti.kc * pr.M + row) * pr.N : pr.C + (int64_t)row * pr.ldc;
        scale[0] = (double)pr.eA[row];  // biased row exponent, combined per column below
      }
      int32_t X[kCols];
#pragma unroll
      for (int j = 0; j < kCols; ++j) X[j] = 0;
      bool first_fold = true;
      for (int l = L; l >= 0 && ok; --l) {
        const int items = level_pairs(l, S) * ti.nkb;
        const int chunks = (items + kChunkKb - 1) / kChunkKb;
        bool scale_pending = l != L;  // Horner: acc = acc * 2^-8 + X_l at the first fold of level l
        int since_fold = 0;
        for (int c = 0; c < chunks; ++c) {
          // one lane waits, the warp follows (tcgen05.ld must stay warp-uniform)
          int w_ok = lane == 0 ? (int)mbar_wait(&sm.accfull[buf], aphase, P.err, 4) : 1;
          w_ok = __shfl_sync(0xffffffffu, w_ok, 0);
          if (!w_ok) {
            ok = false;
            break;
          }
          __syncwarp();
          tc_fence_after();
#pragma unroll
          for (int j0 = 0; j0 < kCols; j0 += 16) {
            uint32_t r[16];
            tmem_ld16(tmem + lane_addr + (uint32_t)(buf * BN + col0 + j0), r);
            tmem_wait_ld();
#pragma unroll
            for (int q = 0; q < 16; ++q) X[j0 + q] += __float2int_rn(__uint_as_float(r[q]));
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&sm.accempty[buf]);
          if (++buf == kAcc) {
            buf = 0;
            aphase ^= 1;
          }
          const bool last = (l == 0 && c == chunks - 1);
          if (++since_fold == kFoldChunks || c == chunks - 1) {
            if (row_ok) {
#pragma unroll
              for (int j = 0; j < kCols; ++j) {
                const int col = ti.n0 + col0 + j;
                if (col < pr.N) {
                  double acc = first_fold ? 0.0 : crow[col];
                  if (scale_pending) acc *= 0x1.0p-8;  // exact
                  acc += (double)X[j];
                  if (last) {
                    // row scale 2^(eA - 1022), column 2^(eB - 1022), digit weights 2^-14
                    int ex = (int)scale[0] + pr.eB[col] - 2 * 1022 - 14 + 1023;
                    ex = ex < 1 ? 1 : (ex > 2046 ? 2046 : ex);
                    acc *= __longlong_as_double((long long)ex << 52);
                  }
                  crow[col] = acc;
                }
              }
            }
#pragma unroll
            for (int j = 0; j < kCols; ++j) X[j] = 0;
            first_fold = false;
            scale_pending = false;
            since_fold = 0;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::kTmemCols));
  }
}

// ---- thin-K kernel: K <= 64, N <= 32 -----------------------------------
//
// One k-block per problem, so every slice is loaded once per 128-row tile
// and all S(S+1)/2 slice products go into per-level TMEM accumulators
// (level l at columns l*32 of a buffer; two buffers alternate between tiles).
// A level sums at most S products of 64 K-elements, below 2^24, so no drains
// are needed mid-tile: the drain warps read the levels from S-1 down to 0 and
// recombine them with FP64 Horner steps directly.  The k-block is TBK = 64
// (128-byte swizzled rows) or, for K <= 32, TBK = 32 (64-byte rows): slices
// are padded to the k-block, so short K (a virtual block of ~30 orbitals)
// streams half the bytes with the narrow block.
constexpr int kThinBN = 32;
constexpr int kThinBufs = 3;        // accumulator buffers (at most; S (S <= 5) levels of 32 columns each)
constexpr int kThinDrainWarps = 4 * kThinBufs;  // one group of four (one per TMEM lane quarter) per buffer
constexpr int kThinThreads = 64 + 32 * kThinDrainWarps;

template <int TBK>
struct ThinSmem {
  static constexpr int kSlots = 10 * (BK / TBK);  // ring of (A slice, B slice) pairs, 200 KB of them
  alignas(1024) __nv_bfloat16 a[kSlots][BM * TBK];
  alignas(1024) __nv_bfloat16 b[kSlots][kThinBN * TBK];
  uint64_t full[kSlots], empty[kSlots], accfull[kThinBufs], accempty[kThinBufs], done;
  uint32_t tmem_base;
};

// Drain of one thin tile, first NC columns (NC covers ncol): Horner over the
// levels in exact int64 fixed point, Y = sum_l X_l 2^(8 (L - l)), from level
// 0 up (|X_l| <= 7 * 64 * 2^14 < 2^23, so |Y| < 2^63 for L <= 5; S = 7 keeps
// the FP64 recombination); the accumulator buffer is released before the
// scaled results are stored.
// ea: the row's exponent, eb8: the first 8 column exponents, both loaded
// by the caller before it waited for the accumulator (their latency hidden
// behind the wait); columns past 8 are read here.
// Stores of one drained row: v[j] * 2^(its exponent), columns < ncol.
template <int NC>
__device__ __forceinline__ void thin_store(const double (&v)[NC], int L, int ncol, const DevProblem& pr, int row,
                                           int ea, const int* eb8) {
  if (row >= pr.M) return;
  double* crow = pr.C + (int64_t)row * pr.ldc;
  const int lshift = L <= 5 ? 8 * L : 0;  // the int64 path carries 2^(8L)
#pragma unroll
  for (int j = 0; j < NC; ++j) {
    if (j < ncol) {
      int ex = ea + (j < 8 ? eb8[j] : pr.eB[j]) - 2 * 1022 - 14 - lshift + 1023;
      ex = ex < 1 ? 1 : (ex > 2046 ? 2046 : ex);
      crow[j] = v[j] * __longlong_as_double((long long)ex << 52);
    }
  }
}

template <int NC>
__device__ __forceinline__ void thin_drain(uint32_t tb, int L, int ncol, const DevProblem& pr, int row,
                                           uint64_t* accempty, int lane, int ea, const int* eb8) {
  double v[NC];
  if (L <= 5) {
    long long Y[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) Y[j] = 0;
    if (NC == 8 && L <= 3) {
      // at most four levels of 8 columns (the usual thin tile: an occupied
      // block of about 6): every load issued, then one wait
      uint32_t rb[4][8];
#pragma unroll
      for (int l = 0; l < 4; ++l)
        if (l <= L) tmem_ld8(tb + (uint32_t)(l * kThinBN), rb[l]);
      tmem_wait_ld();
#pragma unroll
      for (int l = 0; l < 4; ++l)
        if (l <= L) {
#pragma unroll
          for (int j = 0; j < 8; ++j)
            if (j < ncol) Y[j] = Y[j] * 256 + (long long)__float2int_rn(__uint_as_float(rb[l][j]));
        }
    } else {
      for (int l = 0; l <= L; ++l) {
        uint32_t r[NC];
        if (NC == 8) {
          tmem_ld8(tb + (uint32_t)(l * kThinBN), r);
        } else {
#pragma unroll
          for (int h = 0; h < NC / 16; ++h)
            tmem_ld16(tb + (uint32_t)(l * kThinBN + 16 * h), *reinterpret_cast<uint32_t(*)[16]>(r + 16 * h));
        }
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < NC; ++j)
          if (j < ncol) Y[j] = Y[j] * 256 + (long long)__float2int_rn(__uint_as_float(r[j]));
      }
    }
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(accempty);
#pragma unroll
    for (int j = 0; j < NC; ++j) v[j] = (double)Y[j];
  } else {
#pragma unroll
    for (int j = 0; j < NC; ++j) v[j] = 0.0;
    for (int l = L; l >= 0; --l) {
      uint32_t r[NC];
      if (NC == 8) {
        tmem_ld8(tb + (uint32_t)(l * kThinBN), r);
      } else {
#pragma unroll
        for (int h = 0; h < NC / 16; ++h)
          tmem_ld16(tb + (uint32_t)(l * kThinBN + 16 * h), *reinterpret_cast<uint32_t(*)[16]>(r + 16 * h));
      }
      tmem_wait_ld();
#pragma unroll
      for (int j = 0; j < NC; ++j)
        if (j < ncol) v[j] = v[j] * 0x1.0p-8 + (double)__uint_as_float(r[j]);
    }
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(accempty);
  }
  thin_store<NC>(v, L, ncol, pr, row, ea, eb8);
}

template <int TBK>
__global__ void __launch_bounds__(kThinThreads, 1) split_thin_kernel(const GemmParams P) {
  static_assert(TBK == 32 || TBK == 64, "thin k-block");
  using Sm = ThinSmem<TBK>;
  constexpr int kThinSlots = Sm::kSlots;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  Sm& sm = *reinterpret_cast<Sm*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = P.S, L = P.L;
  // a stage holds one tile's S (A slice, B slice) pairs, the B slices back
  // to back, behind one full and one empty barrier
  const int stages = kThinSlots / S;
  constexpr uint32_t kTx = (BM + kThinBN) * TBK * 2;
  constexpr uint32_t kCols = 512;
  if (threadIdx.x == 0) {
    for (int i = 0; i < stages; ++i) {
      mbar_init(&sm.full[i], 1);
      mbar_init(&sm.empty[i], 1);
    }
    for (int b = 0; b < kThinBufs; ++b) {
      mbar_init(&sm.accfull[b], 1);
      mbar_init(&sm.accempty[b], 4);
    }
    mbar_init(&sm.done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  const uint32_t buf_cols = (uint32_t)(S * kThinBN);
  // accumulator buffers in the 512 columns: three for S <= 5, two above
  const int nbuf = min(kThinBufs, (int)(kCols / buf_cols));

  if (warp == 0) {
    if (lane == 0) {
      int st = 0;
      uint32_t phase = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < P.total_tiles && ok; tile += gridDim.x) {
        const TileInfo ti = decode_tile<kThinBN>(P, tile);
        const CUtensorMap* ma = P.maps + 2 * ti.p;
        const CUtensorMap* mb = P.maps + 2 * ti.p + 1;
        if (!mbar_wait(&sm.empty[st], phase ^ 1, P.err, 11)) {
          ok = false;
          break;
        }
        mbar_expect_tx(&sm.full[st], (uint32_t)S * kTx);
        for (int s = 0; s < S; ++s) {
          tma_load_3d(sm.a[st * S + s], ma, &sm.full[st], 0, ti.m0, s);
          tma_load_3d(sm.b[st * S + s], mb, &sm.full[st], 0, ti.n0, s);
        }
        if (++st == stages) {
          st = 0;
          phase ^= 1;
        }
      }
      for (int i = 0; i < stages; ++i) {
        if (--st < 0) {
          st = stages - 1;
          phase ^= 1;
        }
        long long t0 = clock64();
        while (!mbar_try_wait(&sm.full[st], phase) && !mbar_try_wait(&sm.empty[st], phase)) {
          if (clock64() - t0 > kWaitCycles) {
            atomicCAS(P.err, 0, 15);
            break;
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int st = 0, buf = 0;
      uint32_t phase = 0, aphase = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < P.total_tiles && ok; tile += gridDim.x) {
        if (!mbar_wait(&sm.full[st], phase, P.err, 13)) break;
        if (!mbar_wait(&sm.accempty[buf], aphase ^ 1, P.err, 12)) break;
        tc_fence_after();
        // one UMMA per A slice s and K step over B slices 1 .. S + 1 - s
        // (N = 32 (S + 1 - s)) with D at column 32 (s - 1): product (s, t)
        // lands in level s + t - 2's columns; the first (s = 1, k = 0) spans
        // every level and starts them from zero
        const int base = st * S;
        const uint32_t bs = smem_u32(sm.b[base]);
        const uint64_t b0 = TBK == 64 ? sdesc(bs) : sdesc64(bs);
        for (int s = 1; s <= S; ++s) {
          const uint32_t d = tmem + (uint32_t)buf * buf_cols + (uint32_t)((s - 1) * kThinBN);
          const uint32_t as = smem_u32(sm.a[base + s - 1]);
          const uint64_t a0 = TBK == 64 ? sdesc(as) : sdesc64(as);
          const uint32_t idesc = idesc_bf16_n(kThinBN * (S + 1 - s));
#pragma unroll
          for (int k = 0; k < TBK / 16; ++k)
            umma(d, a0 + (uint64_t)(k * 2), b0 + (uint64_t)(k * 2), idesc, (s == 1 && k == 0) ? 0u : 1u);
        }
        umma_commit(&sm.empty[st]);
        umma_commit(&sm.accfull[buf]);
        if (++st == stages) {
          st = 0;
          phase ^= 1;
        }
        if (++buf == nbuf) {
          buf = 0;
          aphase ^= 1;
        }
      }
      umma_commit(&sm.done);
      mbar_wait(&sm.done, 0, P.err, 16);
    }
  } else {
    // nbuf drain groups of four warps: group g drains this CTA's tiles g,
    // g + nbuf, g + 2 nbuf, ... -- always from accumulator buffer g -- so
    // that nbuf tiles drain at once (a drain, with its exponent loads, TMEM
    // reads and scattered row stores, takes longer than a tile's MMAs); a
    // group without a buffer (S > 5) has no tiles
    const int group = (warp - 2) >> 2;
    const int quarter = warp & 3;
    const uint32_t lane_addr = (uint32_t)(quarter * 32) << 16;
    const int buf = group;
    uint32_t aphase = 0;
    for (int tile = blockIdx.x + group * (int)gridDim.x; group < nbuf && tile < P.total_tiles;
         tile += nbuf * (int)gridDim.x) {
      const TileInfo ti = decode_tile<kThinBN>(P, tile);
      const DevProblem& pr = P.probs[ti.p];
      // only the tile's real columns are read and combined: a drain sized
      // for 8, 16 or 32 columns (the thin problems of a block-sparse
      // contraction often have an occupied block of ~6 as N)
      const int ncol = min(kThinBN, pr.N - ti.n0);
      const int row = ti.m0 + quarter * 32 + lane;
      const int ea = row < pr.M ? pr.eA[row] : 0;
      int eb8[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) eb8[j] = j < ncol ? pr.eB[j] : 0;  // thin tiles start at column 0
      int w_ok = lane == 0 ? (int)mbar_wait(&sm.accfull[buf], aphase, P.err, 14) : 1;
      w_ok = __shfl_sync(0xffffffffu, w_ok, 0);
      if (!w_ok) break;
      __syncwarp();
      tc_fence_after();
      const uint32_t tb = tmem + lane_addr + (uint32_t)buf * buf_cols;
      if (ncol <= 8) thin_drain<8>(tb, L, ncol, pr, row, &sm.accempty[buf], lane, ea, eb8);
      else if (ncol <= 16) thin_drain<16>(tb, L, ncol, pr, row, &sm.accempty[buf], lane, ea, eb8);
      else thin_drain<32>(tb, L, ncol, pr, row, &sm.accempty[buf], lane, ea, eb8);
      aphase ^= 1;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
  }
}

// ---- k-stationary kernel: S <= 4, 64-column output tiles -----------------
//
// The pair-by-pair kernel above streams a k-block's A and B slices once per
// slice pair that uses them (2 S (S + 1) / 2 tile loads per k-block).  Here
// every k-block's S A slices and S B slices are loaded once into a ring of
// (A_s, B_s) slots and all S (S + 1) / 2 products are issued from there into
// per-level TMEM accumulators (level l at columns l * 64 of a buffer, two
// buffers).  A level sums at most S products of 64 K-elements per k-block,
// each below 2^20 in magnitude, so 16 / S k-blocks fit below 2^24 and the
// FP32 sums are exact; the drain warps then combine the levels into an exact
// int64 Y = sum_l X_l 2^(8 (L - l)) per output (|Y| <= K 2^(14 + 8 L) < 2^63
// for L <= 3 and K < 2^24) and scale it to FP64 once per tile.
constexpr int kKsBN = 64;
constexpr int kKsSlots = 8;        // (A slice, B slice) pairs, 24 KB each: two k-blocks of 4 slices
constexpr int kKsDrainWarps = 8;   // 4 TMEM lane quarters x 2 column halves
constexpr int kKsThreads = 64 + 32 * kKsDrainWarps;
constexpr int kKsMaxS = 4;

struct KsSmem {
  alignas(1024) __nv_bfloat16 a[kKsSlots][BM * BK];
  alignas(1024) __nv_bfloat16 b[kKsSlots][kKsBN * BK];
  uint64_t full[kKsSlots], empty[kKsSlots], accfull[2], accempty[2], done;
  uint32_t tmem_base;
};

// S is a template parameter so that the slice-pair loops of the MMA issuer
// (one thread issuing every tcgen05.mma) unroll completely.
template <int S>
__global__ void __launch_bounds__(kKsThreads, 1) split_ks_kernel(const GemmParams P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  KsSmem& sm = *reinterpret_cast<KsSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int L = S - 1;
  constexpr int D = 16 / S;  // k-blocks per exact accumulation group
  constexpr uint32_t kTx = (BM + kKsBN) * BK * 2;
  // a stage is one k-block's S slot pairs behind one full and one empty
  // barrier: one wait and one commit per k-block for the MMA-issuing thread
  constexpr int kStages = kKsSlots / S;
  constexpr uint32_t kCols = 512;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(&sm.full[i], 1);
      mbar_init(&sm.empty[i], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.accfull[b], 1);
      mbar_init(&sm.accempty[b], kKsDrainWarps);
    }
    mbar_init(&sm.done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  const uint32_t buf_cols = (uint32_t)(S * kKsBN);

  if (warp == 0) {
    // ---------------- TMA producer: a k-block's S slice pairs ----------------
    if (lane == 0) {
      int st = 0;
      uint32_t phase = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < P.total_tiles && ok; tile += gridDim.x) {
        const TileInfo ti = decode_tile<kKsBN>(P, tile);
        const CUtensorMap* ma = P.maps + 2 * ti.p;
        const CUtensorMap* mb = P.maps + 2 * ti.p + 1;
        for (int kb = ti.kb0; kb < ti.kb0 + ti.nkb && ok; ++kb) {
          if (!mbar_wait(&sm.empty[st], phase ^ 1, P.err, 21)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&sm.full[st], (uint32_t)S * kTx);
#pragma unroll
          for (int s = 0; s < S; ++s) {
            tma_load_3d(sm.a[st * S + s], ma, &sm.full[st], kb * BK, ti.m0, s);
            tma_load_3d(sm.b[st * S + s], mb, &sm.full[st], kb * BK, ti.n0, s);
          }
          if (++st == kStages) {
            st = 0;
            phase ^= 1;
          }
        }
      }
      for (int i = 0; i < kStages; ++i) {
        if (--st < 0) {
          st = kStages - 1;
          phase ^= 1;
        }
        long long t0 = clock64();
        while (!mbar_try_wait(&sm.full[st], phase) && !mbar_try_wait(&sm.empty[st], phase)) {
          if (clock64() - t0 > kWaitCycles) {
            atomicCAS(P.err, 0, 25);
            break;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int st = 0, buf = 0;
      uint32_t phase = 0, aphase = 0;
      bool ok = true;
      // slot descriptors: slot 0's plus the slot offset in 16-byte units
      // (the address field holds shared-memory address / 16, below 2^14)
      const uint64_t ad0 = sdesc(smem_u32(sm.a[0])), bd0 = sdesc(smem_u32(sm.b[0]));
      constexpr uint64_t kAStep = (uint64_t)(BM * BK * 2) >> 4, kBStep = (uint64_t)(kKsBN * BK * 2) >> 4;
      for (int tile = blockIdx.x; tile < P.total_tiles && ok; tile += gridDim.x) {
        const int nkb = decode_tile<kKsBN>(P, tile).nkb;
        for (int g0 = 0; g0 < nkb && ok; g0 += D) {
          if (!mbar_wait(&sm.accempty[buf], aphase ^ 1, P.err, 22)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const int g1 = min(nkb, g0 + D);
          for (int kb = g0; kb < g1 && ok; ++kb) {
            if (!mbar_wait(&sm.full[st], phase, P.err, 23)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const int base = st * S;
            const uint32_t fresh = kb == g0 ? 0u : 1u;
            // One UMMA per A slice s and K step: B slices 1 .. S + 1 - s sit
            // back to back in the stage (64 rows each), so one instruction of
            // N = 64 (S + 1 - s) forms every product (s, t) with t <= S + 1 - s
            // at once; with D at column 64 (s - 1) of the buffer, product
            // (s, t) lands in columns 64 (s + t - 2), its level's accumulator.
            // The first instruction of a group (s = 1, N = 64 S) spans every
            // level and starts them all from zero.
            const uint64_t b0 = bd0 + (uint64_t)base * kBStep;
#pragma unroll
            for (int s = 1; s <= S; ++s) {
              const uint32_t d = tmem + (uint32_t)buf * buf_cols + (uint32_t)((s - 1) * kKsBN);
              const uint64_t a0 = ad0 + (uint64_t)(base + s - 1) * kAStep;
#pragma unroll
              for (int k = 0; k < BK / 16; ++k)
                umma(d, a0 + (uint64_t)(k * 2), b0 + (uint64_t)(k * 2), idesc_bf16_n(kKsBN * (S + 1 - s)),
                     (s == 1 && k == 0) ? fresh : 1u);
            }
            umma_commit(&sm.empty[st]);
            if (++st == kStages) {
              st = 0;
              phase ^= 1;
            }
          }
          if (!ok) break;
          umma_commit(&sm.accfull[buf]);
          if (++buf == 2) {
            buf = 0;
            aphase ^= 1;
          }
        }
      }
      umma_commit(&sm.done);
      mbar_wait(&sm.done, 0, P.err, 26);
    }
  } else {
    // ---------------- drain: exact int64 level recombination ----------------
    const int quarter = warp & 3;               // TMEM lanes this warp may read
    const int half = (warp - 2) >> 2;           // which 32 of the 64 columns
    const uint32_t lane_addr = (uint32_t)(quarter * 32) << 16;
    int buf = 0;
    uint32_t aphase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < P.total_tiles && ok; tile += gridDim.x) {
      const TileInfo ti = decode_tile<kKsBN>(P, tile);
      const DevProblem& pr = P.probs[ti.p];
      long long Y[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) Y[j] = 0;
      for (int g0 = 0; g0 < ti.nkb; g0 += D) {
        int w_ok = lane == 0 ? (int)mbar_wait(&sm.accfull[buf], aphase, P.err, 24) : 1;
        w_ok = __shfl_sync(0xffffffffu, w_ok, 0);
        if (!w_ok) {
          ok = false;
          break;
        }
        __syncwarp();
        tc_fence_after();
        for (int l = 0; l <= L; ++l) {
          uint32_t r[2][16];
          const uint32_t col = (uint32_t)buf * buf_cols + (uint32_t)(l * kKsBN + half * 32);
          tmem_ld16(tmem + lane_addr + col, r[0]);
          tmem_ld16(tmem + lane_addr + col + 16, r[1]);
          tmem_wait_ld();
          const int sh = 8 * (L - l);
          const long long w = 1ll << sh;
#pragma unroll
          for (int j = 0; j < 32; ++j) Y[j] += (long long)__float2int_rn(__uint_as_float(r[j >> 4][j & 15])) * w;
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.accempty[buf]);
        if (++buf == 2) {
          buf = 0;
          aphase ^= 1;
        }
      }
      if (!ok) break;
      const int row = ti.m0 + quarter * 32 + lane;
      if (row < pr.M) {
        const int ea = pr.eA[row];
        double* crow = pr.ksplit > 1 ? pr.partial + ((int64_t)ti.kc * pr.M + row) * pr.N : pr.C + (int64_t)row * pr.ldc;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = ti.n0 + half * 32 + j;
          if (col < pr.N) {
            int ex = ea + pr.eB[col] - 2 * 1022 - 14 - 8 * L + 1023;
            ex = ex < 1 ? 1 : (ex > 2046 ? 2046 : ex);
            crow[col] = (double)Y[j] * __longlong_as_double((long long)ex << 52);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
  }
}

// Fixed-order sum of the split-K partial contributions into C.
__global__ void __launch_bounds__(256) split_reduce_kernel(const DevProblem* __restrict__ probs,
                                                           const int* __restrict__ red_prob,
                                                           const int64_t* __restrict__ red_first, int nred,
                                                           int64_t total) {
  dev::split_reduce_body<false>(probs, red_prob, red_first, nred, total, blockIdx.x, gridDim.x);
}

// Operand splits (dev::row_exponent_body, dev::digits_body, dev::short_rows_body).
__global__ void __launch_bounds__(256) row_exponent_kernel(const SplitRowSet* __restrict__ sets, int nsets,
                                                           int64_t total_chunks) {
  __shared__ uint32_t red[8];
  dev::row_exponent_body<false>(sets, nsets, total_chunks, blockIdx.x, gridDim.x, red);
}

__global__ void __launch_bounds__(256) digits_kernel(const SplitRowSet* __restrict__ sets, int nsets,
                                                     int64_t total_chunks, int S) {
  dev::digits_body<false>(sets, nsets, total_chunks, S, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(256) split_rows_kernel(const SplitRowSet* __restrict__ sets, int nsets,
                                                         int64_t total_rows, int S) {
  __shared__ uint32_t red[8];
  dev::split_rows_body<false>(sets, nsets, total_rows, S, blockIdx.x, gridDim.x, red);
}

__global__ void __launch_bounds__(256) split_short_rows_kernel(const SplitRowSet* __restrict__ sets, int nsets,
                                                               int64_t total_rows, int S) {
  dev::short_rows_body<false>(sets, nsets, total_rows, S, blockIdx.x, gridDim.x);
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

int encode_slices(CUtensorMap* map, const __nv_bfloat16* base, int64_t S, int64_t rows, int64_t Kp, int box_rows,
                  int box_k = BK) {
  auto enc = get_encode();
  if (!enc) return fail(GBX_ECUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)S};
  cuuint64_t strides[2] = {(cuuint64_t)(Kp * 2), (cuuint64_t)(rows * Kp * 2)};
  cuuint32_t box[3] = {(cuuint32_t)box_k, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, box_k == BK ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(GBX_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return GBX_OK;
}

}  // namespace

// Output tile width per problem: the smallest modelled time over the
// instantiated widths.  A k-block costs the largest of: tensor 2.72 * BN
// cycles (128 x BN x 64 MACs at ~3000 MAC/clk), shared-memory reads
// (16 KB of A + BN * 128 B of B at 128 B/clk) and L2 -> SM traffic (same
// bytes at ~76 B/clk per SM).  The 256 width spills a little and is de-rated.
// gbx_split_set_width() overrides the choice (tuning).
constexpr int kWidths[4] = {32, 64, 128, 256};
static int g_width_override = 0;

int choose_width(int64_t N, int S) {
  if (g_width_override) return g_width_override;
  // up to 4 slices the k-stationary kernel (64 columns) loads every slice
  // once per k-block and keeps its sums in registers
  if (S <= kKsMaxS) return kKsBN;
  int best = 256;
  double best_cost = 1e300;
  for (int bn : kWidths) {
    const double tiles = (double)((N + bn - 1) / bn);
    const double bytes = 16384.0 + 128.0 * bn;
    double per_kb = std::max(std::max(2.72 * bn, 128.0 + bn), bytes / 76.0);
    if (bn == 256) per_kb *= 1.15;
    const double cost = tiles * per_kb;
    if (cost < best_cost * 0.999) {
      best_cost = cost;
      best = bn;
    }
  }
  return best;
}

struct SplitLaunch {  // the problems of one output tile width
  int bn = 0;
  DevProblem* d_probs = nullptr;
  int* d_tile_first = nullptr;
  CUtensorMap* d_maps = nullptr;
  int nprob = 0, total_tiles = 0;
  // host copies (merged launches of the persistent iteration program)
  std::vector<DevProblem> hp;
  std::vector<CUtensorMap> hm;
  std::vector<int> hfirst;
};

struct SplitPlan {
  int S = 0, L = 0;
  std::vector<SplitProblem> host;
  std::vector<int> width;  // per problem
  std::vector<int> thin;  // per problem: 0, or the thin-K kernel with a 64 (1) or 32 (2) element k-block
  unsigned char* d_persist = nullptr;    // slices and exponents of constant plan operands
  unsigned char* d_own_arena = nullptr;  // the per-run region when no arena was given
  SplitRowSet* d_sets_a = nullptr;  // long rows from the plan's packed A
  SplitRowSet* d_sets_b = nullptr;  // long rows from the plan's packed B
  SplitRowSet* d_short_a = nullptr;  // short rows (first_row counts rows)
  SplitRowSet* d_short_b = nullptr;
  SplitRowSet* d_mid_a = nullptr;  // medium rows, one CTA per row (first_row counts rows)
  SplitRowSet* d_mid_b = nullptr;
  int nlong_a = 0, nlong_b = 0, nshort_a = 0, nshort_b = 0, nmid_a = 0, nmid_b = 0;
  int64_t short_rows_a = 0, short_rows_b = 0, mid_rows_a = 0, mid_rows_b = 0;
  int nsets = 0;
  int64_t rows_a = 0, rows_b = 0;  // (row, K chunk) work items per side
  std::vector<std::pair<void*, size_t>> exp_ranges_a, exp_ranges_b;  // exponent words reset before a split
  std::vector<SplitLaunch> launches;
  DevProblem* d_all = nullptr;  // every problem, for the split-K reduction
  int* d_err = nullptr;
  int* d_red_prob = nullptr;
  int64_t* d_red_first = nullptr;
  int nred = 0;
  int64_t red_total = 0;
  double bytes = 0.0;
  ~SplitPlan() {
    dev_free(d_red_prob);
    dev_free(d_red_first);
    dev_free(d_persist);
    dev_free(d_own_arena);
    dev_free(d_sets_a);
    dev_free(d_sets_b);
    dev_free(d_short_a);
    dev_free(d_short_b);
    dev_free(d_mid_a);
    dev_free(d_mid_b);
    dev_free(d_all);
    for (auto& l : launches) {
      dev_free(l.d_probs);
      dev_free(l.d_tile_first);
      dev_free(l.d_maps);
    }
    dev_free(d_err);
  }
};

template <int BN>
int set_smem_attr() {
  const size_t smem = sizeof(Smem<BN>) + 1024;
  GBX_CUDA(cudaFuncSetAttribute(split_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  return GBX_OK;
}

namespace {

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Where every buffer of a split plan lives.  Region 0 persists with the plan
// (slices and exponents of constant plan operands, split once); region 1 is
// rewritten by every run (the other operands' slices and exponents, split-K
// partial sums) and may be an arena shared with other plans.  Offsets are in
// elements of each region's slice, exponent and partial-sum sub-buffers.
struct SplitLayout {
  struct Prob {
    int bn = 0;
    bool thin = false;
    int kb = BK;  // k-block: 64, or 32 for thin problems with K <= 32
    int64_t Mp = 0, Np = 0, Kp = 0;
    int ra = 0, rb = 0;      // region of the GEMM's A and B slices
    int64_t sa = 0, sb = 0;  // slice offsets
    int64_t ea = 0, eb = 0;  // exponent offsets
    int ks = 1, per = 0;     // K split and k-blocks per range
    int64_t part = -1;       // partial-sum offset (region 1), -1 = none
  };
  std::vector<Prob> p;
  int64_t slices[2] = {0, 0}, exps[2] = {0, 0}, part = 0;
  size_t exps_at(int r) const { return align256(2 * (size_t)slices[r]); }
  size_t part_at() const { return exps_at(1) + align256(4 * (size_t)exps[1]); }
  size_t bytes(int r) const {
    size_t b = exps_at(r) + align256(4 * (size_t)exps[r]);
    if (r == 1) b += align256(8 * (size_t)part);
    return (r == 0 && slices[0] == 0 && exps[0] == 0) || (r == 1 && slices[1] == 0 && exps[1] == 0 && part == 0)
               ? 0
               : b;
  }
};

int split_layout(const std::vector<SplitProblem>& probs, int S, bool static_a, bool static_b, SplitLayout& L) {
  L = SplitLayout();
  int64_t out_tiles = 0;
  for (auto& q : probs) {
    if (q.M <= 0 || q.N <= 0 || q.K <= 0) return fail(GBX_EINVAL, "empty split problem");
    if (q.M >= (1ll << 30) || q.N >= (1ll << 30) || q.K >= (1ll << 30)) return fail(GBX_EUNSUPPORTED, "split problem too large");
    SplitLayout::Prob o;
    // thin-K problems (one k-block, at most 32 columns) take the thin kernel
    o.thin = q.K <= BK && q.N <= kThinBN && S <= 7;
    o.bn = o.thin ? kThinBN : (q.width ? q.width : choose_width(q.N, S));
    // the k-stationary kernel's exact int64 sums need K < 2^24
    if (!o.thin && S <= kKsMaxS && o.bn == kKsBN && q.K >= (1 << 24)) o.bn = 128;
    if (!o.thin && o.bn != 32 && o.bn != 64 && o.bn != 128 && o.bn != 256)
      return fail(GBX_EINVAL, "split tile width %d", o.bn);
    o.Mp = (q.M + BM - 1) / BM * BM;
    o.Np = (q.N + o.bn - 1) / o.bn * o.bn;
    o.kb = o.thin && q.K <= 32 ? 32 : BK;
    o.Kp = (q.K + o.kb - 1) / o.kb * o.kb;
    // the GEMM's A rows come from plan operand B when swapped
    const bool a_const = q.a_is_plan_b ? static_b : static_a;
    const bool b_const = q.a_is_plan_b ? static_a : static_b;
    o.ra = a_const ? 0 : 1;
    o.rb = b_const ? 0 : 1;
    o.sa = L.slices[o.ra];
    L.slices[o.ra] += S * q.M * o.Kp;
    o.sb = L.slices[o.rb];
    L.slices[o.rb] += S * q.N * o.Kp;
    o.ea = L.exps[o.ra];
    L.exps[o.ra] += o.Mp;
    o.eb = L.exps[o.rb];
    L.exps[o.rb] += o.Np;
    out_tiles += (o.Mp / BM) * (o.Np / o.bn);
    L.p.push_back(o);
  }
  for (size_t i = 0; i < probs.size(); ++i) {
    SplitLayout::Prob& o = L.p[i];
    const int nkb = (int)(o.Kp / o.kb);
    if (nkb < 1) return fail(GBX_EINVAL, "split problem without a k-block");
    // split K when the output tiles of all problems leave SMs idle; ranges are
    // whole exact-accumulation chunks: 16 k-blocks for the pair-by-pair
    // kernel, 16 / S for the k-stationary one (whose exact groups are that
    // short, so few-tile problems -- matrix-vector shapes, small outputs with
    // long K -- spread over many more CTAs instead of walking K serially)
    const int chunk = (!o.thin && S <= kKsMaxS && o.bn == kKsBN) ? 16 / S : kChunkKb;
    int ks = 1;
    if (!o.thin && out_tiles < kSplitFill && nkb > 2 * chunk) {
      int want = (int)((kSplitFill + out_tiles - 1) / out_tiles);
      ks = std::max(1, std::min(want, nkb / chunk));
    }
    int per = (nkb + ks - 1) / ks;
    per = (per + chunk - 1) / chunk * chunk;
    ks = (nkb + per - 1) / per;
    o.ks = ks;
    o.per = per;
    if (ks > 1) {
      o.part = L.part;
      L.part += (int64_t)ks * probs[i].M * probs[i].N;
    }
  }
  return GBX_OK;
}

}  // namespace

int split_plan_sizes(const std::vector<SplitProblem>& probs, int slices, bool static_a, bool static_b,
                     size_t* persist_bytes, size_t* arena_bytes) {
  SplitLayout L;
  GBX_TRY(split_layout(probs, slices > 0 ? slices : 6, static_a, static_b, L));
  if (persist_bytes) *persist_bytes = L.bytes(0);
  if (arena_bytes) *arena_bytes = L.bytes(1);
  return GBX_OK;
}

int create_split_plan(const std::vector<SplitProblem>& probs, int slices, SplitPlan** out, const SplitMem* mem) {
  *out = nullptr;
  auto sp = std::make_unique<SplitPlan>();
  sp->S = slices > 0 ? slices : 6;
  if (sp->S < 2 || sp->S > 7) return fail(GBX_EINVAL, "split slices must be in [2, 7]");
  sp->L = sp->S - 1;
  sp->host = probs;
  const int S = sp->S;
  const bool static_a = mem && mem->static_a, static_b = mem && mem->static_b;
  SplitLayout lay;
  GBX_TRY(split_layout(probs, S, static_a, static_b, lay));
  for (auto& o : lay.p) {
    sp->width.push_back(o.bn);
    sp->thin.push_back(o.thin ? (o.kb == 32 ? 2 : 1) : 0);
  }
  unsigned char* base[2] = {nullptr, nullptr};
  const size_t b0 = lay.bytes(0), b1 = lay.bytes(1);
  if (b0) {
    // constant operands are split once: their padding must read as zero
    GBX_TRY(dev_alloc((void**)&sp->d_persist, b0));
    GBX_CUDA(cudaMemset(sp->d_persist, 0, b0));
    base[0] = sp->d_persist;
  }
  if (b1) {
    if (mem && mem->arena) {
      base[1] = mem->arena;
    } else {
      GBX_TRY(dev_alloc((void**)&sp->d_own_arena, b1));
      GBX_CUDA(cudaMemset(sp->d_own_arena, 0, b1));
      base[1] = sp->d_own_arena;
    }
  }
  auto slice_ptr = [&](int r, int64_t off) { return (__nv_bfloat16*)base[r] + off; };
  auto exp_ptr = [&](int r, int64_t off) { return (int*)(base[r] + lay.exps_at(r)) + off; };
  double* part_base = b1 ? (double*)(base[1] + lay.part_at()) : nullptr;
  sp->bytes = (double)b0 + (double)b1;
  std::vector<SplitRowSet> sa, sb, ssa, ssb, msa, msb;
  int64_t sra = 0, srb = 0, mra = 0, mrb = 0;
  std::vector<DevProblem> dp;
  std::vector<CUtensorMap> maps;
  int64_t ra = 0, rb = 0;
  std::vector<int> red;
  std::vector<int64_t> red_first;
  int64_t red_total = 0;
  for (size_t i = 0; i < probs.size(); ++i) {
    const SplitProblem& p = probs[i];
    const SplitLayout::Prob& o = lay.p[i];
    const int bn = o.bn;
    // row sets are grouped by the plan operand they come from, so constant
    // plan operands can be split once
    SplitRowSet a{p.A, p.M, p.K, slice_ptr(o.ra, o.sa), p.M * o.Kp, o.Kp, exp_ptr(o.ra, o.ea), 0,
                  p.lda ? p.lda : p.K};
    SplitRowSet b{p.B, p.N, p.K, slice_ptr(o.rb, o.sb), p.N * o.Kp, o.Kp, exp_ptr(o.rb, o.eb), 0,
                  p.ldb ? p.ldb : p.K};
    SplitRowSet& to_a = p.a_is_plan_b ? b : a;  // rows that come from plan A
    SplitRowSet& to_b = p.a_is_plan_b ? a : b;
    if (to_a.K <= kShortRow) {
      to_a.first_row = sra;
      sra += to_a.rows;
      ssa.push_back(to_a);
    } else if (to_a.K <= kMidRow) {
      to_a.first_row = mra;
      mra += to_a.rows;
      msa.push_back(to_a);
    } else {
      to_a.first_row = ra;
      ra += to_a.rows * ((to_a.K + kSplitChunk - 1) / kSplitChunk);
      sa.push_back(to_a);
      sp->exp_ranges_a.push_back({(void*)to_a.exps, sizeof(int) * (size_t)to_a.rows});
    }
    if (to_b.K <= kShortRow) {
      to_b.first_row = srb;
      srb += to_b.rows;
      ssb.push_back(to_b);
    } else if (to_b.K <= kMidRow) {
      to_b.first_row = mrb;
      mrb += to_b.rows;
      msb.push_back(to_b);
    } else {
      to_b.first_row = rb;
      rb += to_b.rows * ((to_b.K + kSplitChunk - 1) / kSplitChunk);
      sb.push_back(to_b);
      sp->exp_ranges_b.push_back({(void*)to_b.exps, sizeof(int) * (size_t)to_b.rows});
    }
    DevProblem d;
    d.M = (int)p.M;
    d.N = (int)p.N;
    d.K = (int)p.K;
    d.nkb = (int)(o.Kp / o.kb);
    d.tiles_m = (int)(o.Mp / BM);
    d.tiles_n = (int)(o.Np / bn);
    d.ksplit = o.ks;
    d.kb_per_split = o.per;
    d.eA = exp_ptr(o.ra, o.ea);
    d.eB = exp_ptr(o.rb, o.eb);
    d.C = p.C;
    d.partial = nullptr;
    if (o.ks > 1) {
      d.partial = part_base + o.part;
      red.push_back((int)i);
      red_first.push_back(red_total);
      red_total += p.M * p.N;
    }
    d.ldc = p.ldc ? p.ldc : p.N;
    dp.push_back(d);
    CUtensorMap ma, mb;
    // slices hold only the real rows: a tile's rows past M (or N) lie outside
    // the tensor and TMA fills them with zeros without reading memory
    GBX_TRY(encode_slices(&ma, slice_ptr(o.ra, o.sa), S, p.M, o.Kp, BM, o.kb));
    GBX_TRY(encode_slices(&mb, slice_ptr(o.rb, o.sb), S, p.N, o.Kp, bn, o.kb));
    maps.push_back(ma);
    maps.push_back(mb);
  }
  if (!red.empty()) {
    GBX_TRY(dev_alloc((void**)&sp->d_red_prob, sizeof(int) * red.size()));
    GBX_TRY(dev_alloc((void**)&sp->d_red_first, sizeof(int64_t) * red.size()));
    GBX_CUDA(cudaMemcpy(sp->d_red_prob, red.data(), sizeof(int) * red.size(), cudaMemcpyHostToDevice));
    GBX_CUDA(cudaMemcpy(sp->d_red_first, red_first.data(), sizeof(int64_t) * red.size(), cudaMemcpyHostToDevice));
    sp->nred = (int)red.size();
    sp->red_total = red_total;
  }
  sp->nsets = (int)probs.size();
  sp->rows_a = ra;
  sp->rows_b = rb;
  sp->short_rows_a = sra;
  sp->short_rows_b = srb;
  sp->nlong_a = (int)sa.size();
  sp->nlong_b = (int)sb.size();
  sp->nshort_a = (int)ssa.size();
  sp->nshort_b = (int)ssb.size();
  sp->mid_rows_a = mra;
  sp->mid_rows_b = mrb;
  sp->nmid_a = (int)msa.size();
  sp->nmid_b = (int)msb.size();
  auto up = [&](const void* h, size_t bytes, void** d) -> int {
    if (bytes == 0) return GBX_OK;
    GBX_TRY(dev_alloc(d, bytes));
    GBX_CUDA(cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice));
    return GBX_OK;
  };
  GBX_TRY(up(sa.data(), sizeof(SplitRowSet) * sa.size(), (void**)&sp->d_sets_a));
  GBX_TRY(up(sb.data(), sizeof(SplitRowSet) * sb.size(), (void**)&sp->d_sets_b));
  GBX_TRY(up(ssa.data(), sizeof(SplitRowSet) * ssa.size(), (void**)&sp->d_short_a));
  GBX_TRY(up(ssb.data(), sizeof(SplitRowSet) * ssb.size(), (void**)&sp->d_short_b));
  GBX_TRY(up(msa.data(), sizeof(SplitRowSet) * msa.size(), (void**)&sp->d_mid_a));
  GBX_TRY(up(msb.data(), sizeof(SplitRowSet) * msb.size(), (void**)&sp->d_mid_b));
  GBX_TRY(up(dp.data(), sizeof(DevProblem) * dp.size(), (void**)&sp->d_all));
  // one launch per output tile width, plus one for the thin-K problems of
  // each k-block (bn 0: 64, bn 1: 32)
  for (int bn : {0, 1, 32, 64, 128, 256}) {
    std::vector<DevProblem> lp;
    std::vector<CUtensorMap> lm;
    std::vector<int> first;
    int tiles = 0;
    for (size_t i = 0; i < probs.size(); ++i) {
      if (bn <= 1 ? sp->thin[i] != bn + 1 : (sp->thin[i] || sp->width[i] != bn)) continue;
      lp.push_back(dp[i]);
      lm.push_back(maps[2 * i]);
      lm.push_back(maps[2 * i + 1]);
      first.push_back(tiles);
      tiles += dp[i].tiles_m * dp[i].tiles_n * dp[i].ksplit;
    }
    if (lp.empty()) continue;
    SplitLaunch L;
    L.bn = bn;
    L.nprob = (int)lp.size();
    L.total_tiles = tiles;
    GBX_TRY(up(lp.data(), sizeof(DevProblem) * lp.size(), (void**)&L.d_probs));
    GBX_TRY(up(first.data(), sizeof(int) * first.size(), (void**)&L.d_tile_first));
    GBX_TRY(up(lm.data(), sizeof(CUtensorMap) * lm.size(), (void**)&L.d_maps));
    L.hp = lp;
    L.hm = lm;
    L.hfirst = first;
    sp->launches.push_back(std::move(L));
  }
  GBX_TRY(dev_alloc((void**)&sp->d_err, sizeof(int)));
  GBX_CUDA(cudaMemset(sp->d_err, 0, sizeof(int)));
  GBX_TRY(set_smem_attr<32>());
  GBX_TRY(set_smem_attr<64>());
  GBX_TRY(set_smem_attr<128>());
  GBX_TRY(set_smem_attr<256>());
  GBX_CUDA(cudaFuncSetAttribute(split_ks_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(KsSmem) + 1024)));
  GBX_CUDA(cudaFuncSetAttribute(split_ks_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(KsSmem) + 1024)));
  GBX_CUDA(cudaFuncSetAttribute(split_ks_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(KsSmem) + 1024)));
  GBX_CUDA(cudaFuncSetAttribute(split_thin_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(ThinSmem<64>) + 1024)));
  GBX_CUDA(cudaFuncSetAttribute(split_thin_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(ThinSmem<32>) + 1024)));
  *out = sp.release();
  return GBX_OK;
}

int split_operands(SplitPlan* sp, bool plan_a, bool plan_b, cudaStream_t st) {
  if (!sp || sp->nsets == 0) return GBX_OK;
  ProgRecorder* rec = prog_recording();
  for (int side = 0; side < 2; ++side) {
    if ((side == 0 && !plan_a) || (side == 1 && !plan_b)) continue;
    const int64_t chunks = side == 0 ? sp->rows_a : sp->rows_b;
    if (chunks > 0) {
      const SplitRowSet* sets = side == 0 ? sp->d_sets_a : sp->d_sets_b;
      const int nsets = side == 0 ? sp->nlong_a : sp->nlong_b;
      for (auto& z : (side == 0 ? sp->exp_ranges_a : sp->exp_ranges_b)) GBX_TRY(zero_async(z.first, z.second, st));
      const int grid = (int)std::min<int64_t>(chunks, 152 * 16);
      if (rec) {
        ProgArgs a;
        a.sets = {sets, chunks, nsets, sp->S};
        GBX_TRY(prog_mem(rec, PK_ROWEXP, (uint32_t)grid, a, {}));
        GBX_TRY(prog_mem(rec, PK_DIGITS, (uint32_t)grid, a, {}));
      } else {
        row_exponent_kernel<<<grid, 256, 0, st>>>(sets, nsets, chunks);
        GBX_CUDA(cudaGetLastError());
        digits_kernel<<<grid, 256, 0, st>>>(sets, nsets, chunks, sp->S);
        GBX_CUDA(cudaGetLastError());
      }
    }
    const int64_t mrows = side == 0 ? sp->mid_rows_a : sp->mid_rows_b;
    if (mrows > 0) {
      const SplitRowSet* sets = side == 0 ? sp->d_mid_a : sp->d_mid_b;
      const int nsets = side == 0 ? sp->nmid_a : sp->nmid_b;
      const int grid = (int)std::min<int64_t>(mrows, 152 * 8);
      if (rec) {
        ProgArgs a;
        a.sets = {sets, mrows, nsets, sp->S};
        GBX_TRY(prog_mem(rec, PK_SPLITROWS, (uint32_t)grid, a, {}));
      } else {
        split_rows_kernel<<<grid, 256, 0, st>>>(sets, nsets, mrows, sp->S);
        GBX_CUDA(cudaGetLastError());
      }
    }
    const int64_t srows = side == 0 ? sp->short_rows_a : sp->short_rows_b;
    if (srows > 0) {
      const SplitRowSet* sets = side == 0 ? sp->d_short_a : sp->d_short_b;
      const int nsets = side == 0 ? sp->nshort_a : sp->nshort_b;
      const int grid = (int)std::min<int64_t>((srows + 7) / 8, 152 * 32);
      if (rec) {
        ProgArgs a;
        a.sets = {sets, srows, nsets, sp->S};
        GBX_TRY(prog_mem(rec, PK_SHORTROWS, (uint32_t)grid, a, {}));
        continue;
      }
      split_short_rows_kernel<<<grid, 256, 0, st>>>(sets, nsets, srows, sp->S);
      GBX_CUDA(cudaGetLastError());
    }
  }
  return GBX_OK;
}

namespace {

template <int BN>
int launch_width(const GemmParams& P, int nsm, cudaStream_t st) {
  const int grid = std::min(P.total_tiles, nsm * SplitCfg<BN>::kCtasPerSm);
  split_gemm_kernel<BN><<<grid, SplitCfg<BN>::kThreads, sizeof(Smem<BN>) + 1024, st>>>(P);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

// The GEMM kernel of one launch class -- bn 0 / 1: thin-K with a 64 / 32
// element k-block; 64 with S <= 4: k-stationary; else the pair-by-pair
// kernel of that output tile width -- over the problems of P.
int launch_split_gemm(int bn, const GemmParams& P, cudaStream_t st) {
  if (P.total_tiles <= 0) return GBX_OK;
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (bn <= 1) {
    if (bn == 0)
      split_thin_kernel<64><<<std::min(P.total_tiles, nsm), kThinThreads, sizeof(ThinSmem<64>) + 1024, st>>>(P);
    else
      split_thin_kernel<32><<<std::min(P.total_tiles, nsm), kThinThreads, sizeof(ThinSmem<32>) + 1024, st>>>(P);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
      cudaFuncAttributes fa;
      std::memset(&fa, 0, sizeof(fa));
      cudaFuncGetAttributes(&fa, bn == 0 ? (const void*)split_thin_kernel<64> : (const void*)split_thin_kernel<32>);
      return fail(GBX_ECUDA, "thin-K launch (k-block %d): %s; dynamic smem %zu (max %d), static %zu, regs %d, max threads %d",
                  bn == 0 ? 64 : 32, cudaGetErrorString(le), (bn == 0 ? sizeof(ThinSmem<64>) : sizeof(ThinSmem<32>)) + 1024,
                  fa.maxDynamicSharedSizeBytes, fa.sharedSizeBytes, fa.numRegs, fa.maxThreadsPerBlock);
    }
    return GBX_OK;
  }
  switch (bn) {
    case 32: return launch_width<32>(P, nsm, st);
    case 64:
      if (P.S <= kKsMaxS) {
        const int g = std::min(P.total_tiles, nsm);
        const size_t sh = sizeof(KsSmem) + 1024;
        if (P.S == 2) split_ks_kernel<2><<<g, kKsThreads, sh, st>>>(P);
        else if (P.S == 3) split_ks_kernel<3><<<g, kKsThreads, sh, st>>>(P);
        else split_ks_kernel<4><<<g, kKsThreads, sh, st>>>(P);
        GBX_CUDA(cudaGetLastError());
        return GBX_OK;
      }
      return launch_width<64>(P, nsm, st);
    case 128: return launch_width<128>(P, nsm, st);
    default: return launch_width<256>(P, nsm, st);
  }
}

GemmParams params_of(const SplitPlan* sp, const SplitLaunch& L) {
  GemmParams P;
  P.probs = L.d_probs;
  P.tile_first = L.d_tile_first;
  P.maps = L.d_maps;
  P.nprob = L.nprob;
  P.total_tiles = L.total_tiles;
  P.S = sp->S;
  P.L = sp->L;
  P.err = sp->d_err;
  return P;
}

}  // namespace

int run_split_plan(SplitPlan* sp, bool plan_a, bool plan_b, cudaStream_t st) {
  if (!sp || sp->nsets == 0) return GBX_OK;
  GBX_TRY(split_operands(sp, plan_a, plan_b, st));
  ProgRecorder* rec = prog_recording();
  for (size_t i = 0; i < sp->launches.size(); ++i) {
    const SplitLaunch& L = sp->launches[i];
    if (L.total_tiles <= 0) continue;
    if (rec) GBX_TRY(prog_split(rec, sp, (int)i));
    else GBX_TRY(launch_split_gemm(L.bn, params_of(sp, L), st));
  }
  if (sp->nred > 0) {
    int rg = (int)std::min<int64_t>((sp->red_total + 255) / 256, 152 * 8);
    if (rec) {
      ProgArgs a;
      a.splitred = {sp->d_all, sp->d_red_prob, sp->d_red_first, sp->red_total, sp->nred};
      return prog_mem(rec, PK_SPLITRED, (uint32_t)rg, a, {});
    }
    split_reduce_kernel<<<rg, 256, 0, st>>>(sp->d_all, sp->d_red_prob, sp->d_red_first, sp->nred, sp->red_total);
    GBX_CUDA(cudaGetLastError());
  }
  return GBX_OK;
}

// ---- merged launches of the persistent iteration program -------------------

int split_launch_class(const SplitPlan* sp, int launch) {
  if (!sp || launch < 0 || launch >= (int)sp->launches.size()) return -1;
  const int bn = sp->launches[launch].bn;
  return bn * 16 + sp->S;  // kernel and slice count
}

struct SplitMerged {
  int bn = 0;
  GemmParams P;
  DevProblem* d_probs = nullptr;
  int* d_first = nullptr;
  CUtensorMap* d_maps = nullptr;
  ~SplitMerged() {
    dev_free(d_probs);
    dev_free(d_first);
    dev_free(d_maps);
  }
};

int split_merge(const std::vector<std::pair<SplitPlan*, int>>& parts, int* err, SplitMerged** out) {
  *out = nullptr;
  if (parts.empty()) return fail(GBX_EINVAL, "split merge: no launches");
  auto m = std::make_unique<SplitMerged>();
  const int cls = split_launch_class(parts[0].first, parts[0].second);
  std::vector<DevProblem> hp;
  std::vector<CUtensorMap> hm;
  std::vector<int> first;
  int64_t tiles = 0;
  for (auto& pr : parts) {
    if (split_launch_class(pr.first, pr.second) != cls) return fail(GBX_EINVAL, "split merge: mixed launch classes");
    const SplitLaunch& L = pr.first->launches[pr.second];
    for (size_t i = 0; i < L.hp.size(); ++i) {
      hp.push_back(L.hp[i]);
      hm.push_back(L.hm[2 * i]);
      hm.push_back(L.hm[2 * i + 1]);
      first.push_back((int)(tiles + L.hfirst[i]));
    }
    tiles += L.total_tiles;
  }
  if (tiles >= (1ll << 31)) return fail(GBX_EUNSUPPORTED, "split merge: too many tiles");
  GBX_TRY(dev_alloc((void**)&m->d_probs, sizeof(DevProblem) * hp.size()));
  GBX_TRY(dev_alloc((void**)&m->d_first, sizeof(int) * first.size()));
  GBX_TRY(dev_alloc((void**)&m->d_maps, sizeof(CUtensorMap) * hm.size()));
  GBX_CUDA(cudaMemcpy(m->d_probs, hp.data(), sizeof(DevProblem) * hp.size(), cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(m->d_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(m->d_maps, hm.data(), sizeof(CUtensorMap) * hm.size(), cudaMemcpyHostToDevice));
  const SplitPlan* sp0 = parts[0].first;
  m->bn = sp0->launches[parts[0].second].bn;
  m->P.probs = m->d_probs;
  m->P.tile_first = m->d_first;
  m->P.maps = m->d_maps;
  m->P.nprob = (int)hp.size();
  m->P.total_tiles = (int)tiles;
  m->P.S = sp0->S;
  m->P.L = sp0->L;
  m->P.err = err;
  *out = m.release();
  return GBX_OK;
}

int split_merged_run(const SplitMerged* m, cudaStream_t st) { return launch_split_gemm(m->bn, m->P, st); }

void split_merged_destroy(SplitMerged* m) { delete m; }

int split_plan_error(SplitPlan* sp) {
  if (!sp) return 0;
  int e = 0;
  if (cudaMemcpy(&e, sp->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return e;
}

double split_plan_tensor_flops(const SplitPlan* sp) {
  if (!sp) return 0.0;
  double f = 0.0;
  const double pairs = sp->S * (sp->S + 1) / 2.0;
  for (size_t i = 0; i < sp->host.size(); ++i) {
    const SplitProblem& p = sp->host[i];
    const int bn = sp->width[i];  // thin-K problems: 32
    double Mp = (double)((p.M + BM - 1) / BM * BM), Np = (double)((p.N + bn - 1) / bn * bn);
    const int kb = sp->thin[i] == 2 ? 32 : BK;
    double Kp = (double)((p.K + kb - 1) / kb * kb);
    f += 2.0 * pairs * Mp * Np * Kp;
  }
  return f;
}

void destroy_split_plan(SplitPlan* sp) { delete sp; }

int split_set_width(int bn) {
  if (bn != 0 && bn != 32 && bn != 64 && bn != 128 && bn != 256) return fail(GBX_EINVAL, "width must be 0, 32, 64, 128 or 256");
  g_width_override = bn;
  return GBX_OK;
}

double split_plan_bytes(const SplitPlan* sp) { return sp ? sp->bytes : 0.0; }

// ---- self-test of the bounded waits ---------------------------------------
// One CTA waits on an mbarrier that nothing arrives on, through the same
// bounded wait as the split kernels' pipeline waits; it gives up after the
// limit, records its stage in the error word and returns.
namespace {
constexpr int kSelftestStage = 31;
__device__ int g_wait_selftest_err;

__global__ void wait_selftest_reset_kernel() { g_wait_selftest_err = 0; }

__global__ void wait_selftest_kernel(long long limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait(&bar, 0, &g_wait_selftest_err, kSelftestStage, limit);
  __syncthreads();
}
}  // namespace

}  // namespace gbx

extern "C" int gbx_wait_selftest(long long limit_cycles, void* stream) {
  using namespace gbx;
  if (limit_cycles < 0 || limit_cycles > kWaitCycles)
    return fail(GBX_EINVAL, "limit_cycles %lld outside [0, %lld]", limit_cycles, (long long)kWaitCycles);
  cudaStream_t st = (cudaStream_t)stream;
  wait_selftest_reset_kernel<<<1, 1, 0, st>>>();
  GBX_CUDA(cudaGetLastError());
  wait_selftest_kernel<<<1, 32, 0, st>>>(limit_cycles);
  GBX_CUDA(cudaGetLastError());
  GBX_CUDA(cudaStreamSynchronize(st));
  int e = 0;
  GBX_CUDA(cudaMemcpyFromSymbol(&e, g_wait_selftest_err, sizeof(int)));
  if (e != 0) return fail(GBX_ETIMEOUT, "a bounded device wait ran out (stage %d)", e);
  return GBX_OK;
}
