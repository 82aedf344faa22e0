// Device bodies of the library's memory-bound and CUDA-core FP64 kernels.
//
// Each body is the whole work of one CTA of its kernel, written against a
// block index `bid` of `nblk` blocks instead of blockIdx / gridDim, so that
// the same code runs as a standalone kernel (tile_move.cu, direct.cu,
// gemm_f64.cu, gemm_split.cu, cc_kernels.cu: bid = blockIdx.x) and as one
// work item of the persistent iteration program (program.cu), which hands
// out (record, block) items from a device-side queue.  All bodies run with
// 256 threads per CTA except the standalone direct kernel (512).
//
// kCoh: the data a body reads may have been written earlier in the same
// persistent launch by another CTA.  The producer's writes are ordered
// before its release-add of the record's block count, and this CTA's thread
// 0 acquires that count before the barrier that starts the body, so the
// writes happen before every load of the body in the PTX memory model --
// for ordinary (weak) loads, ld.global.ca, but not for the non-coherent
// read-only path (ld.global.nc, __ldg) that the standalone kernels use and
// that the compiler may also choose for plain loads through const
// __restrict__ pointers.  Descriptor tables never change while a launch runs
// and keep __ldg.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "cc.h"
#include "common.h"
#include "split_dev.h"

namespace gbx {
namespace dev {

template <bool kCoh, typename T>
__device__ __forceinline__ T ldin(const T* p) {
  if constexpr (kCoh) return __ldca(p);
  else return __ldg(p);
}
// loads that the standalone kernels issue as plain loads (outputs read back
// for accumulation, values another kernel of the same stream wrote)
template <bool kCoh, typename T>
__device__ __forceinline__ T ldrw(const T* p) {
  if constexpr (kCoh) return __ldca(p);
  else return *p;
}

constexpr int kBodyThreads = 256;

// ---- tile moves ---------------------------------------------------------------

constexpr int kMoveThreads = 256;
constexpr int kMoveChunk = 2048;   // elements per work item (general moves)
constexpr int kMove4Chunk = 4096;  // elements per work item (moves of at most four dimensions)

template <bool kCoh>
__device__ __forceinline__ void move_body(const MoveDesc* __restrict__ descs, const uint32_t* __restrict__ first,
                                          int ndesc, uint32_t nchunks, const double* __restrict__ src,
                                          double* __restrict__ dst, double alpha, uint32_t bid, uint32_t nblk) {
  for (uint32_t chunk = bid; chunk < nchunks; chunk += nblk) {
    // binary search: last descriptor whose first chunk <= chunk
    int lo = 0, hi = ndesc - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (__ldg(first + mid) <= chunk) lo = mid; else hi = mid - 1;
    }
    const MoveDesc& md = descs[lo];
    const uint32_t base = (chunk - __ldg(first + lo)) * kMoveChunk;
    const int rank = md.rank;
    const uint32_t n = md.n;
    const int op = md.op;
    // accumulating moves take the run-time factor (a contraction's alpha)
    const double scale = op == 0 ? md.scale : __dmul_rn(md.scale, alpha);
    const double* __restrict__ s = src + md.src;
    double* __restrict__ t = dst + md.dst;
    // all addresses first, then every load, then every store: eight
    // independent loads in flight per thread
    constexpr int kPer = kMoveChunk / kMoveThreads;
    int64_t so[kPer], to[kPer];
    bool in[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      const uint32_t e = base + (uint32_t)(k * kMoveThreads) + threadIdx.x;
      in[k] = e < n;
      so[k] = 0;
      to[k] = 0;
      uint32_t rem = in[k] ? e : 0;
      for (int d = rank - 1; d > 0; --d) {
        const uint32_t q = md.div[d].div(rem);
        const uint32_t i = rem - q * md.ext[d];
        so[k] += (int64_t)i * md.sstr[d];
        to[k] += (int64_t)i * md.dstr[d];
        rem = q;
      }
      so[k] += (int64_t)rem * md.sstr[0];
      to[k] += (int64_t)rem * md.dstr[0];
    }
    double x[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) x[k] = in[k] ? ldin<kCoh>(s + so[k]) : 0.0;
    const unsigned long long sb = (unsigned long long)__double_as_longlong(scale);
    if (op == 0 && (sb & 0x7FFFFFFFFFFFFFFFull) == 0x3FF0000000000000ull) {
      // +-x: a bit copy with the sign bit set on the integer pipe
      const long long flip = (long long)(sb & 0x8000000000000000ull);
#pragma unroll
      for (int k = 0; k < kPer; ++k)
        if (in[k]) t[to[k]] = __longlong_as_double(__double_as_longlong(x[k]) ^ flip);
    } else if (op == 0) {
#pragma unroll
      for (int k = 0; k < kPer; ++k)
        if (in[k]) t[to[k]] = __dmul_rn(scale, x[k]);
    } else {
      double y[kPer];
#pragma unroll
      for (int k = 0; k < kPer; ++k) y[k] = in[k] ? ldrw<kCoh>(t + to[k]) : 0.0;
#pragma unroll
      for (int k = 0; k < kPer; ++k)
        if (in[k]) t[to[k]] = __fma_rn(scale, x[k], y[k]);
    }
  }
}

// Moves of at most four dimensions: the chunk's descriptor comes from a
// table, its fields are read once per chunk into registers and the index
// decode is fully unrolled (three multiply-high divisions per element), so
// the kernel issues a few tens of instructions per element and streams at
// memory speed.  Each thread handles kMove4Chunk / kMoveThreads elements in
// two batches, addresses first, then every load, then every store.  A move
// marked for pairs (contiguous even inner runs at even offsets) goes two
// elements per index decode with 16-byte loads and stores.
template <bool kCoh, int kPer = 8>
__device__ __forceinline__ void move4_body(const MoveDesc4* __restrict__ descs, const uint32_t* __restrict__ chunk_desc,
                                           uint32_t nchunks, const double* __restrict__ src, double* __restrict__ dst,
                                           double alpha, int allow_pairs, uint32_t bid, uint32_t nblk) {
  constexpr int kBatches = kMove4Chunk / (kMoveThreads * kPer);
  constexpr int kPairBatches = kMove4Chunk / (2 * kMoveThreads * kPer);
  static_assert(kPairBatches * 2 * kMoveThreads * kPer == kMove4Chunk, "chunk size");
  for (uint32_t chunk = bid; chunk < nchunks; chunk += nblk) {
    const MoveDesc4* __restrict__ md = descs + __ldg(chunk_desc + chunk);
    const uint32_t n = md->n;
    const uint32_t base = (chunk - md->first) * kMove4Chunk;
    const int op = md->op;
    const double scale = op == 0 ? md->scale : __dmul_rn(md->scale, alpha);
    const FastDiv d1 = md->div[1], d2 = md->div[2], d3 = md->div[3];
    const int64_t s0 = md->sstr[0], s1 = md->sstr[1], s2 = md->sstr[2], s3 = md->sstr[3];
    const int64_t t0 = md->dstr[0], t1 = md->dstr[1], t2 = md->dstr[2], t3 = md->dstr[3];
    const double* __restrict__ s = src + md->src;
    double* __restrict__ t = dst + md->dst;
    // stores of +-x are bit copies with the sign bit set on the integer pipe
    // (a select between x and scale * x would issue the multiply anyway, and
    // FP64 instructions are scarce on this part)
    const unsigned long long sb = (unsigned long long)__double_as_longlong(scale);
    const bool unit = op == 0 && (sb & 0x7FFFFFFFFFFFFFFFull) == 0x3FF0000000000000ull;
    const long long flip = (long long)(sb & 0x8000000000000000ull);
    if (allow_pairs && md->pad == 1) {
      // pairs (2e, 2e + 1): the chunk's kMove4Chunk elements in batches of
      // kPer pairs per thread
#pragma unroll 1
      for (int bt = 0; bt < kPairBatches; ++bt) {
        int64_t so[kPer], to[kPer];
        bool in[kPer];
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
          const uint32_t e = base + 2u * ((uint32_t)((bt * kPer + k) * kMoveThreads) + threadIdx.x);
          in[k] = e < n;
          const uint32_t r = in[k] ? e : 0;
          const uint32_t q3 = d3.div(r), c3 = r - q3 * d3.d;
          const uint32_t q2 = d2.div(q3), c2 = q3 - q2 * d2.d;
          const uint32_t c0 = d1.div(q2), c1 = q2 - c0 * d1.d;
          so[k] = (int64_t)c0 * s0 + (int64_t)c1 * s1 + (int64_t)c2 * s2 + (int64_t)c3 * s3;
          to[k] = (int64_t)c0 * t0 + (int64_t)c1 * t1 + (int64_t)c2 * t2 + (int64_t)c3 * t3;
        }
        double2 x[kPer];
#pragma unroll
        for (int k = 0; k < kPer; ++k)
          x[k] = in[k] ? ldin<kCoh>(reinterpret_cast<const double2*>(s + so[k])) : make_double2(0.0, 0.0);
        if (unit) {
#pragma unroll
          for (int k = 0; k < kPer; ++k)
            if (in[k])
              *reinterpret_cast<double2*>(t + to[k]) =
                  make_double2(__longlong_as_double(__double_as_longlong(x[k].x) ^ flip),
                               __longlong_as_double(__double_as_longlong(x[k].y) ^ flip));
        } else if (op == 0) {
#pragma unroll
          for (int k = 0; k < kPer; ++k)
            if (in[k]) *reinterpret_cast<double2*>(t + to[k]) = make_double2(__dmul_rn(scale, x[k].x), __dmul_rn(scale, x[k].y));
        } else {
          double2 y[kPer];
#pragma unroll
          for (int k = 0; k < kPer; ++k)
            y[k] = in[k] ? ldrw<kCoh>(reinterpret_cast<const double2*>(t + to[k])) : make_double2(0.0, 0.0);
#pragma unroll
          for (int k = 0; k < kPer; ++k)
            if (in[k])
              *reinterpret_cast<double2*>(t + to[k]) =
                  make_double2(__fma_rn(scale, x[k].x, y[k].x), __fma_rn(scale, x[k].y, y[k].y));
        }
      }
      continue;
    }
#pragma unroll 1
    for (int bt = 0; bt < kBatches; ++bt) {
      int64_t so[kPer], to[kPer];
      bool in[kPer];
#pragma unroll
      for (int k = 0; k < kPer; ++k) {
        const uint32_t e = base + (uint32_t)((bt * kPer + k) * kMoveThreads) + threadIdx.x;
        in[k] = e < n;
        const uint32_t r = in[k] ? e : 0;
        const uint32_t q3 = d3.div(r), c3 = r - q3 * d3.d;
        const uint32_t q2 = d2.div(q3), c2 = q3 - q2 * d2.d;
        const uint32_t c0 = d1.div(q2), c1 = q2 - c0 * d1.d;
        so[k] = (int64_t)c0 * s0 + (int64_t)c1 * s1 + (int64_t)c2 * s2 + (int64_t)c3 * s3;
        to[k] = (int64_t)c0 * t0 + (int64_t)c1 * t1 + (int64_t)c2 * t2 + (int64_t)c3 * t3;
      }
      double x[kPer];
#pragma unroll
      for (int k = 0; k < kPer; ++k) x[k] = in[k] ? ldin<kCoh>(s + so[k]) : 0.0;
      if (unit) {
#pragma unroll
        for (int k = 0; k < kPer; ++k)
          if (in[k]) t[to[k]] = __longlong_as_double(__double_as_longlong(x[k]) ^ flip);
      } else if (op == 0) {
#pragma unroll
        for (int k = 0; k < kPer; ++k)
          if (in[k]) t[to[k]] = __dmul_rn(scale, x[k]);
      } else {
        double y[kPer];
#pragma unroll
        for (int k = 0; k < kPer; ++k) y[k] = in[k] ? ldrw<kCoh>(t + to[k]) : 0.0;
#pragma unroll
        for (int k = 0; k < kPer; ++k)
          if (in[k]) t[to[k]] = __fma_rn(scale, x[k], y[k]);
      }
    }
  }
}

// ---- fused permuted sum -------------------------------------------------------

constexpr int kFsThreads = 256;
constexpr int kFsPer = kFsItemElems / kFsThreads;
// transposed slabs of one item, rows padded to an odd length: a whole-slab
// item of n elements needs at most n + n / ea <= 2n doubles
constexpr int kFsStage = 2 * kFsItemElems;
static_assert(kFsPer * kFsThreads == kFsItemElems, "item size");

struct FsSmem {
  double stage[kFsStage];
  const double* base[kFsMaxSlots];  // indexed by the term's slot
  // the item and its terms, read field by field (keeps registers free for
  // the elements in flight)
  FsItem item;
  FsTerm terms[kFsMaxTerms];
};

// One CTA per work item (grid-stride over items).  Threads hold kFsPer
// destination elements each, in destination order, and add the terms one
// after the other: rows of slabs that are contiguous in the source's own
// order are read directly (coalesced); slabs stored transposed are first
// copied into shared memory in source order and read back transposed, so
// both sides stay coalesced; anything else is gathered.  Stores are
// coalesced along the destination.
template <bool kCoh>
__device__ __forceinline__ void fused_sum_body(const FsItem* __restrict__ items, int nitems,
                                               const FsTerm* __restrict__ terms, const FsSrc& src,
                                               const double* __restrict__ scale, double* __restrict__ out,
                                               uint32_t bid, uint32_t nblk, FsSmem& sm) {
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < kFsMaxSlots; ++k) sm.base[k] = src.p[k];
  }
  for (int i = (int)bid; i < nitems; i += (int)nblk) {
    __syncthreads();  // the previous item is finished with the item, its terms and stage
    if (threadIdx.x == 0) sm.item = items[i];
    __syncthreads();
    const FsItem& it = sm.item;
    if (threadIdx.x < it.nterm) sm.terms[threadIdx.x] = terms[it.term0 + threadIdx.x];
    __syncthreads();
    const uint32_t E = it.fE.d, ea = it.fea.d, eb = it.feb.d, O1 = it.fo1.d;
    double acc[kFsPer];
    // element k of this thread: e = tid + k * threads (lanes past the end
    // repeat the last element: valid addresses, no store); the outer indices
    // of its slab, packed as o0 << 16 | o1, and its index q within the slab
    uint32_t oo[kFsPer], qk[kFsPer];
#pragma unroll
    for (int k = 0; k < kFsPer; ++k) {
      acc[k] = 0.0;
      const uint32_t f = it.f0 + min((uint32_t)(threadIdx.x + k * kFsThreads), it.n - 1);
      const uint32_t sg = it.fE.div(f);
      const uint32_t o0 = it.fo1.div(sg);
      qk[k] = f - sg * E;
      oo[k] = (o0 << 16) | (sg - o0 * O1);
    }
#define FS_ELEM(k, o0, o1, q)      \
  const uint32_t o0 = oo[k] >> 16;  \
  const uint32_t o1 = oo[k] & 0xFFFFu; \
  const uint32_t q = qk[k]
    // offsets inside a source tile are 32-bit (a tile holds fewer than 2^31
    // elements): one multiply-add each instead of 64-bit products
    auto gather = [&](const FsTerm& tm, double* x) {
      const double* __restrict__ p = sm.base[tm.slot] + tm.off;
      const uint32_t so0 = (uint32_t)tm.so0, so1 = (uint32_t)tm.so1;
      if (tm.mode == 1 && it.whole) {
        const uint32_t pa = ea | 1u, sp = eb * pa;
        const uint32_t s_first = it.fE.div(it.f0);
        __syncthreads();  // earlier reads of stage are done
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          const uint32_t e = min((uint32_t)(threadIdx.x + k * kFsThreads), it.n - 1);
          const uint32_t sl = it.fE.div(e);
          const uint32_t sg = s_first + sl, o0 = it.fo1.div(sg), o1 = sg - o0 * O1;
          x[k] = ldin<kCoh>(p + (o0 * so0 + o1 * so1 + (e - sl * E)));
        }
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          const uint32_t e = threadIdx.x + k * kFsThreads;
          if (e < it.n) {
            const uint32_t sl = it.fE.div(e);
            const uint32_t qq = e - sl * E;  // source order within the slab: b * ea + a
            const uint32_t b = it.fea.div(qq);
            sm.stage[sl * sp + b * pa + (qq - b * ea)] = x[k];
          }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          const uint32_t e = min((uint32_t)(threadIdx.x + k * kFsThreads), it.n - 1);
          const uint32_t sl = it.fE.div(e), q = qk[k];
          const uint32_t a = it.feb.div(q);
          x[k] = sm.stage[sl * sp + (q - a * eb) * pa + a];
        }
      } else if (tm.mode == 0) {
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          FS_ELEM(k, o0, o1, q);
          x[k] = ldin<kCoh>(p + (o0 * so0 + o1 * so1 + q));
        }
      } else {
        const uint32_t sa = (uint32_t)tm.sa, sb = (uint32_t)tm.sb;
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          FS_ELEM(k, o0, o1, q);
          const uint32_t a = it.feb.div(q);
          x[k] = ldin<kCoh>(p + (o0 * so0 + o1 * so1 + a * sa + (q - a * eb) * sb));
        }
      }
    };
    // FP64 instructions are the scarce resource here (the FP64 pipe issues
    // about 1.6 per clock per SM, fewer than the elements HBM delivers): the
    // first term of a +-1 coefficient is a sign flip on the bits (0 + c x
    // with -0 turned into +0), every other term one fused multiply-add --
    // the separately rounded product and sum whenever c x is exact, as it is
    // for c = +-2^k
    uint32_t t0 = 0;
    if (it.nterm > 0) {
      const unsigned long long cbits = (unsigned long long)__double_as_longlong(sm.terms[0].coef);
      if ((cbits & 0x7FFFFFFFFFFFFFFFull) == 0x3FF0000000000000ull) {
        double x[kFsPer];
        gather(sm.terms[0], x);
        const unsigned long long sign = cbits & 0x8000000000000000ull;
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          const unsigned long long b = (unsigned long long)__double_as_longlong(x[k]) ^ sign;
          acc[k] = __longlong_as_double((long long)(b == 0x8000000000000000ull ? 0ull : b));
        }
        t0 = 1;
      }
    }
    for (uint32_t t = t0; t < it.nterm; ++t) {
      double x[kFsPer];
      gather(sm.terms[t], x);
      const double c = sm.terms[t].coef;
#pragma unroll
      for (int k = 0; k < kFsPer; ++k) acc[k] = __fma_rn(c, x[k], acc[k]);
    }
#undef FS_ELEM
#pragma unroll
    for (int k = 0; k < kFsPer; ++k) {
      const uint32_t e = threadIdx.x + k * kFsThreads;
      if (e < it.n) {
        double v = acc[k];
        if (scale) v = __dmul_rn(v, ldin<kCoh>(scale + it.dst + e));
        out[it.dst + e] = v;
      }
    }
  }
}

// ---- direct FP64 contraction ----------------------------------------------------

constexpr int kDirPer = 4;  // output elements per thread and pass

struct DirSmem {
  DirItem item;
  DirPair pairs[kDirMaxPairs];
};

// One CTA per work item (grid-stride), kThr threads.  Each thread holds
// kDirPer output elements per pass (kDirItemElems / (kThr kDirPer) passes),
// in output order; for every tile pair it forms their operand base offsets,
// then walks the contracted indices with all kDirPer loads of A and of B in
// flight.  Consecutive lanes hold consecutive output elements, so the
// operand that carries the output's last dimension is read coalesced and the
// other one is (mostly) a broadcast.  Every output element is the same
// sequence of fused multiply-adds whatever kThr is.
// kStore: C = alpha * sum (the items cover every element of C, which holds
// no earlier value), else C += alpha * sum -- a template parameter, so that
// the accumulating kernel's C loads are scheduled as without the choice.
template <int kThr, bool kCoh, bool kStore>
__device__ __forceinline__ void direct_body(const DirItem* __restrict__ items, int nitems,
                                            const DirPair* __restrict__ pairs, const double* __restrict__ A,
                                            const double* __restrict__ B, double* __restrict__ C, double alpha,
                                            uint32_t bid, uint32_t nblk, DirSmem& sm) {
  constexpr int kPasses = kDirItemElems / (kThr * kDirPer);
  static_assert(kPasses * kThr * kDirPer == kDirItemElems, "item size");
  for (int i = (int)bid; i < nitems; i += (int)nblk) {
    __syncthreads();  // the previous item is finished with the item and its pairs
    if (threadIdx.x == 0) sm.item = items[i];
    __syncthreads();
    const DirItem& it = sm.item;
    if (threadIdx.x < it.npair) sm.pairs[threadIdx.x] = pairs[it.pair0 + threadIdx.x];
    __syncthreads();
    const uint32_t e1 = it.f1.d, e2 = it.f2.d, e3 = it.f3.d;
#pragma unroll 1
    for (int pass = 0; pass < kPasses; ++pass) {
      const uint32_t e0 = (uint32_t)(pass * kThr * kDirPer) + threadIdx.x;
      double acc[kDirPer];
#pragma unroll
      for (int k = 0; k < kDirPer; ++k) acc[k] = 0.0;
      for (uint32_t p = 0; p < it.npair; ++p) {
        const DirPair& pr = sm.pairs[p];
        // offsets inside the operand tiles (a tile holds fewer than 2^31 elements)
        uint32_t ba[kDirPer], bb[kDirPer];
#pragma unroll
        for (int k = 0; k < kDirPer; ++k) {
          // lanes past the end repeat the last element (valid addresses, no store)
          const uint32_t f = it.f0 + min(e0 + (uint32_t)(k * kThr), it.n - 1);
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
              x[k] = __double_as_longlong(ldin<kCoh>(pa + ba[k]));
              y[k] = ldin<kCoh>(pb + bb[k]);
            }
#pragma unroll
            for (int k = 0; k < kDirPer; ++k) acc[k] = __fma_rn(__longlong_as_double(x[k] ^ flip), y[k], acc[k]);
          }
        }
      }
#pragma unroll
      for (int k = 0; k < kDirPer; ++k) {
        const uint32_t e = e0 + (uint32_t)(k * kThr);
        if (e < it.n) {
          double* c = C + it.coff + e;
          if constexpr (kStore) *c = __dmul_rn(alpha, acc[k]);
          else *c = __fma_rn(alpha, acc[k], ldrw<kCoh>(c));
        }
      }
    }
  }
}

// ---- split-precision operand preparation -------------------------------------

// Splitting runs in two passes over (row, K chunk) work items so that rows
// with very long K spread over the whole GPU.  Pass 1 takes the largest biased
// exponent of each row chunk and folds it into the row with atomicMax (exact,
// order independent); pass 2 writes the digits.
constexpr int kSplitChunk = 2048;
constexpr int64_t kShortRow = 1024;  // rows up to this length: one warp per row, both passes fused

__device__ __forceinline__ void locate_chunk(const SplitRowSet* __restrict__ sets, int nsets, int64_t chunk,
                                             int& set, int64_t& row, int64_t& k0) {
  int lo = 0, hi = nsets - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sets[mid].first_row <= chunk) lo = mid; else hi = mid - 1;
  }
  set = lo;
  const SplitRowSet& rs = sets[lo];
  const int64_t per_row = (rs.K + kSplitChunk - 1) / kSplitChunk;
  const int64_t local = chunk - rs.first_row;
  row = local / per_row;
  k0 = (local - row * per_row) * kSplitChunk;
}

// One element's S slices: X = the element scaled by 2^-(emax - 1022 - F +
// 53) and rounded half up to an integer of F = 7 + 8 (S - 1) bits, cut into
// balanced base-256 digits (the digits of |X|, with X's sign), least
// significant in slice S - 1.  For S <= 4 (F <= 31) |X| <= 2^31 and the
// digits come from 32-bit arithmetic: d = ((U + 128) & 255) - 128 and
// U <- (U + 128) >> 8, since U - d = (U + 128) rounded down to a multiple of
// 256.  Larger S keeps 64-bit arithmetic.
__device__ __forceinline__ void write_digits(long long bits, uint32_t emax, int F, int S, __nv_bfloat16* out,
                                             int64_t stride) {
  const uint32_t e = (uint32_t)((bits >> 52) & 0x7FF);
  const bool neg = bits < 0;
  unsigned long long U = 0;
  if (e != 0 && emax != 0) {
    const unsigned long long mant = ((unsigned long long)bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 53 + (int)(emax - e) - F;  // U = mant * 2^-sh, rounded half up
    if (sh <= 0) U = mant << (-sh);
    else if (sh < 64) U = (mant + (1ull << (sh - 1))) >> sh;
  }
  if (F <= 31) {
    uint32_t u = (uint32_t)U;  // <= 2^31
    for (int s = S - 1; s >= 1; --s) {
      const int d = (int)((u + 128u) & 255u) - 128;
      u = (u + 128u) >> 8;
      out[s * stride] = __int2bfloat16_rn(neg ? -d : d);
    }
    out[0] = __int2bfloat16_rn(neg ? -(int)u : (int)u);
  } else {
    unsigned long long u = U;
    for (int s = S - 1; s >= 1; --s) {
      const int d = (int)((u + 128ull) & 255ull) - 128;
      u = (u + 128ull) >> 8;
      out[s * stride] = __int2bfloat16_rn(neg ? -d : d);
    }
    out[0] = __int2bfloat16_rn(neg ? -(int)u : (int)u);
  }
}

template <bool kCoh>
__device__ __forceinline__ void row_exponent_body(const SplitRowSet* __restrict__ sets, int nsets,
                                                  int64_t total_chunks, uint32_t bid, uint32_t nblk, uint32_t* red) {
  for (int64_t chunk = bid; chunk < total_chunks; chunk += nblk) {
    int set;
    int64_t row, k0;
    locate_chunk(sets, nsets, chunk, set, row, k0);
    const SplitRowSet& rs = sets[set];
    const double* src = rs.src + row * rs.ld;
    const int64_t k1 = min(rs.K, k0 + kSplitChunk);
    uint32_t emax = 0;
    // four loads in flight per thread (the loop is bound by load latency)
    for (int64_t k = k0 + threadIdx.x; k < k1; k += 4 * 256) {
      long long v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = k + u * 256 < k1 ? __double_as_longlong(ldin<kCoh>(src + k + u * 256)) : 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) emax = max(emax, (uint32_t)((v[u] >> 52) & 0x7FF));
    }
    for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = emax;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t m = 0;
      for (int w = 0; w < 8; ++w) m = max(m, red[w]);
      if (m) atomicMax((unsigned int*)(rs.exps + row), m);
    }
    __syncthreads();
  }
}

// exps hold the largest biased exponent of each row (0 for an all-zero row).
template <bool kCoh>
__device__ __forceinline__ void digits_body(const SplitRowSet* __restrict__ sets, int nsets, int64_t total_chunks,
                                            int S, uint32_t bid, uint32_t nblk) {
  const int F = 7 + 8 * (S - 1);
  for (int64_t chunk = bid; chunk < total_chunks; chunk += nblk) {
    int set;
    int64_t row, k0;
    locate_chunk(sets, nsets, chunk, set, row, k0);
    const SplitRowSet& rs = sets[set];
    const double* src = rs.src + row * rs.ld;
    __nv_bfloat16* dst = rs.dst + row * rs.Kp;
    const uint32_t emax = (uint32_t)ldrw<kCoh>(rs.exps + row);
    const int64_t k1 = min(rs.K, k0 + kSplitChunk);
    for (int64_t k = k0 + threadIdx.x; k < k1; k += 4 * 256) {
      long long v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = k + u * 256 < k1 ? __double_as_longlong(ldin<kCoh>(src + k + u * 256)) : 0;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (k + u * 256 < k1) write_digits(v[u], emax, F, S, dst + k + u * 256, rs.slice_stride);
    }
    // the row's last chunk also clears its K padding (the slice buffers may be
    // an arena shared with other plans, so nothing else keeps it zero)
    if (k1 == rs.K)
      for (int64_t k = rs.K + threadIdx.x; k < rs.Kp; k += 256)
        for (int s = 0; s < S; ++s) dst[s * rs.slice_stride + k] = __int2bfloat16_rn(0);
  }
}

// Rows of medium length (kShortRow < K <= kMidRow): one CTA per row takes
// the row's largest exponent (block reduction, written to exps directly)
// and then writes the digits, every thread re-reading the elements it read
// for the maximum -- from L1 or L2 instead of HBM, so the row crosses HBM
// once.  The row sets here carry first_row in rows.
constexpr int64_t kMidRow = 16384;

// A row of at most kPer * 256 elements: every element loaded at once (one
// HBM round trip per row instead of one per 1024 elements and pass), the
// exponent reduced across the CTA, the digits written from the registers.
template <bool kCoh, int kPer>
__device__ __forceinline__ void split_row_in_registers(const SplitRowSet& rs, int64_t row, const double* src, int F,
                                                       int S, uint32_t* red) {
  const int K = (int)rs.K;
  long long v[kPer];
#pragma unroll
  for (int u = 0; u < kPer; ++u) {
    const int k = (int)threadIdx.x + u * 256;
    v[u] = k < K ? __double_as_longlong(ldin<kCoh>(src + k)) : 0;
  }
  uint32_t emax = 0;
#pragma unroll
  for (int u = 0; u < kPer; ++u) emax = max(emax, (uint32_t)((v[u] >> 52) & 0x7FF));
  for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  __syncthreads();  // the previous row is done with red
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = emax;
  __syncthreads();
  uint32_t m = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) m = max(m, red[w]);
  if (threadIdx.x == 0) rs.exps[row] = (int)m;
  __nv_bfloat16* dst = rs.dst + row * rs.Kp;
#pragma unroll
  for (int u = 0; u < kPer; ++u) {
    const int k = (int)threadIdx.x + u * 256;
    if (k < K) write_digits(v[u], m, F, S, dst + k, rs.slice_stride);
  }
  for (int64_t k = K + threadIdx.x; k < rs.Kp; k += 256)
    for (int s = 0; s < S; ++s) dst[s * rs.slice_stride + k] = __int2bfloat16_rn(0);
}

template <bool kCoh>
__device__ __forceinline__ void split_rows_body(const SplitRowSet* __restrict__ sets, int nsets, int64_t total_rows,
                                                int S, uint32_t bid, uint32_t nblk, uint32_t* red) {
  const int F = 7 + 8 * (S - 1);
  for (int64_t rg = bid; rg < total_rows; rg += nblk) {
    int lo = 0, hi = nsets - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (sets[mid].first_row <= rg) lo = mid; else hi = mid - 1;
    }
    const SplitRowSet& rs = sets[lo];
    const int64_t row = rg - rs.first_row;
    const double* src = rs.src + row * rs.ld;
    const int64_t K = rs.K;
    if (K <= 8 * 256) {
      split_row_in_registers<kCoh, 8>(rs, row, src, F, S, red);
      continue;
    }
    if (K <= 16 * 256) {
      split_row_in_registers<kCoh, 16>(rs, row, src, F, S, red);
      continue;
    }
    uint32_t emax = 0;
    for (int64_t k = threadIdx.x; k < K; k += 4 * 256) {
      long long v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = k + u * 256 < K ? __double_as_longlong(ldin<kCoh>(src + k + u * 256)) : 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) emax = max(emax, (uint32_t)((v[u] >> 52) & 0x7FF));
    }
    for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    __syncthreads();  // the previous row is done with red
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = emax;
    __syncthreads();
    uint32_t m = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) m = max(m, red[w]);
    if (threadIdx.x == 0) rs.exps[row] = (int)m;
    __nv_bfloat16* dst = rs.dst + row * rs.Kp;
    for (int64_t k = threadIdx.x; k < K; k += 4 * 256) {
      long long v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = k + u * 256 < K ? __double_as_longlong(ldin<kCoh>(src + k + u * 256)) : 0;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (k + u * 256 < K) write_digits(v[u], m, F, S, dst + k + u * 256, rs.slice_stride);
    }
    for (int64_t k = K + threadIdx.x; k < rs.Kp; k += 256)
      for (int s = 0; s < S; ++s) dst[s * rs.slice_stride + k] = __int2bfloat16_rn(0);
  }
}

// Short rows: one warp handles a whole row (exponent by warp shuffles, then
// the digits); the row sets here carry first_row in rows.
template <bool kCoh>
__device__ __forceinline__ void short_rows_body(const SplitRowSet* __restrict__ sets, int nsets, int64_t total_rows,
                                                int S, uint32_t bid, uint32_t nblk) {
  const int F = 7 + 8 * (S - 1);
  const int lane = threadIdx.x & 31;
  for (int64_t rg = (int64_t)bid * 8 + (threadIdx.x >> 5); rg < total_rows; rg += (int64_t)nblk * 8) {
    int lo = 0, hi = nsets - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (sets[mid].first_row <= rg) lo = mid; else hi = mid - 1;
    }
    const SplitRowSet& rs = sets[lo];
    const int64_t row = rg - rs.first_row;
    const double* src = rs.src + row * rs.ld;
    uint32_t emax = 0;
    for (int64_t k = lane; k < rs.K; k += 32)
      emax = max(emax, (uint32_t)((__double_as_longlong(ldin<kCoh>(src + k)) >> 52) & 0x7FF));
    for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    if (lane == 0) rs.exps[row] = (int)emax;
    __nv_bfloat16* dst = rs.dst + row * rs.Kp;
    for (int64_t k = lane; k < rs.K; k += 32)
      write_digits(__double_as_longlong(ldin<kCoh>(src + k)), emax, F, S, dst + k, rs.slice_stride);
    for (int64_t k = rs.K + lane; k < rs.Kp; k += 32)
      for (int s = 0; s < S; ++s) dst[s * rs.slice_stride + k] = __int2bfloat16_rn(0);
  }
}

// Fixed-order sum of the split GEMM's K-range partial contributions into C.
template <bool kCoh>
__device__ __forceinline__ void split_reduce_body(const DevProblem* __restrict__ probs, const int* __restrict__ red_prob,
                                                  const int64_t* __restrict__ red_first, int nred, int64_t total,
                                                  uint32_t bid, uint32_t nblk) {
  for (int64_t e = (int64_t)bid * 256 + threadIdx.x; e < total; e += (int64_t)nblk * 256) {
    int lo = 0, hi = nred - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (red_first[mid] <= e) lo = mid; else hi = mid - 1;
    }
    const DevProblem& p = probs[red_prob[lo]];
    const int64_t i = e - red_first[lo];
    const int64_t mn = (int64_t)p.M * p.N;
    double acc = 0.0;
    for (int c = 0; c < p.ksplit; ++c) acc += ldrw<kCoh>(p.partial + c * mn + i);
    const int64_t row = i / p.N, col = i - row * p.N;
    p.C[row * p.ldc + col] = acc;
  }
}

// ---- CUDA-core FP64 GEMM shapes ---------------------------------------------------

constexpr int kSmallK = 8;
constexpr int kSmallKElems = 2048;   // output elements per CTA
constexpr int kSmallOutDim = 16;     // small outputs: at most 16 x 16 ...
constexpr int kGemvDim = 2;          // matrix-vector problems: one side at most this
constexpr int kRedThreads = 256;
constexpr int kRedChunk = 2048;

__device__ __forceinline__ int find_problem(const int* __restrict__ first, int nprob, int blk) {
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= blk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Matrix-vector shapes (variant 8): one warp per output of the wide side --
// column j of C when A is the thin operand (m <= 2), row i when B is (n <=
// 2).  The lanes stride K, so the wide operand's row is read once and
// coalesced when its K stride is 1; each lane keeps one partial sum per thin
// row, and the warp adds them in a fixed butterfly order (deterministic).
// Eight warps per CTA: a work item is eight consecutive wide-side outputs
// over one K range; with several ranges (few outputs, long K) each writes
// its raw sums to a partial slab that the split-K reduction adds in order.
template <bool kCoh>
__device__ __forceinline__ void gemv_body(const GemmProblem* __restrict__ probs, int nprob,
                                          const int* __restrict__ block_first, int total_blocks, uint32_t bid,
                                          uint32_t nblk) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int blk = (int)bid; blk < total_blocks; blk += (int)nblk) {
    const int pi = find_problem(block_first, nprob, blk);
    const GemmProblem& p = probs[pi];
    const bool a_thin = p.m <= kGemvDim && p.m <= p.n;
    const int tn = a_thin ? p.m : p.n;
    const int64_t wide = a_thin ? p.n : p.m;
    const int64_t groups = (wide + 7) / 8;
    const int64_t local = blk - block_first[pi];
    const int kc = (int)(local / groups);
    const int64_t w = (local - kc * groups) * 8 + warp;
    if (w >= wide) continue;
    const int64_t k0 = (int64_t)kc * p.kchunk, k1 = min((int64_t)p.k, k0 + p.kchunk);
    const double* W = a_thin ? p.B + w * p.b_rs : p.A + w * p.a_rs;
    const int64_t wcs = a_thin ? p.b_cs : p.a_cs;
    const double* T = a_thin ? p.A : p.B;
    const int64_t trs = a_thin ? p.a_rs : p.b_rs, tcs = a_thin ? p.a_cs : p.b_cs;
    double acc[kGemvDim];
#pragma unroll
    for (int j = 0; j < kGemvDim; ++j) acc[j] = 0.0;
    for (int64_t k = k0 + lane; k < k1; k += 32) {
      const double x = ldin<kCoh>(W + k * wcs);
#pragma unroll
      for (int j = 0; j < kGemvDim; ++j)
        if (j < tn) acc[j] = fma(x, ldin<kCoh>(T + j * trs + k * tcs), acc[j]);
    }
#pragma unroll
    for (int j = 0; j < kGemvDim; ++j) {
      if (j >= tn) break;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
    }
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < kGemvDim; ++j) {
        if (j >= tn) break;
        const int64_t row = a_thin ? j : w, col = a_thin ? w : j;
        if (p.ksplit > 1) {
          p.partial[(int64_t)kc * p.m * p.n + row * p.n + col] = acc[j];
        } else {
          double* c = p.C + row * p.c_rs + col;
          const double v = __dmul_rn(p.alpha, acc[j]);
          *c = p.accumulate ? __dadd_rn(ldrw<kCoh>(c), v) : v;
        }
      }
    }
  }
}

// K <= 8: every output element is its own k-ordered FMA chain (outer
// products and other tiny-K contractions), written coalesced along columns.
template <bool kCoh>
__device__ __forceinline__ void small_k_body(const GemmProblem* __restrict__ probs, int nprob,
                                             const int* __restrict__ block_first, int total_blocks, uint32_t bid,
                                             uint32_t nblk) {
  for (int blk = (int)bid; blk < total_blocks; blk += (int)nblk) {
    const int pi = find_problem(block_first, nprob, blk);
    const GemmProblem& p = probs[pi];
    const int64_t mn = (int64_t)p.m * p.n;
    const int64_t e0 = (int64_t)(blk - block_first[pi]) * kSmallKElems;
    for (int r = 0; r < kSmallKElems / 256; ++r) {
      const int64_t e = e0 + r * 256 + threadIdx.x;
      if (e >= mn) break;
      const int64_t i = e / p.n, j = e - i * p.n;
      double acc = 0.0;
      for (int k = 0; k < p.k; ++k)
        acc = fma(ldin<kCoh>(p.A + i * p.a_rs + (int64_t)k * p.a_cs), ldin<kCoh>(p.B + j * p.b_rs + (int64_t)k * p.b_cs),
                  acc);
      double* c = p.C + i * p.c_rs + j;
      const double v = __dmul_rn(p.alpha, acc);
      *c = p.accumulate ? __dadd_rn(ldrw<kCoh>(c), v) : v;
    }
  }
}

struct SmallOutSmem {
  double As[kSmallOutDim][65];
  double Bs[kSmallOutDim][65];
  double red[256];
};

// Small output, long K (variant 7): work item = one K chunk of one problem;
// the CTA stages 64-wide K slices of all m rows of A and n rows of B in
// shared memory, thread t accumulates output t % (m n) over every
// (256 / (m n))-th k of the slice, and the lanes of an output are summed in
// a fixed order into the chunk's partial (or C when there is one chunk).
template <bool kCoh>
__device__ __forceinline__ void small_out_body(const GemmProblem* __restrict__ probs, int nprob,
                                               const int* __restrict__ item_first, int total, uint32_t bid,
                                               uint32_t nblk, SmallOutSmem& sm) {
  const int tid = threadIdx.x;
  for (int item = (int)bid; item < total; item += (int)nblk) {
    const int pi = find_problem(item_first, nprob, item);
    const GemmProblem& p = probs[pi];
    const int c = item - item_first[pi];
    const int P = p.m * p.n, lanes = 256 / P;
    const int out = tid % P, lane = tid / P;
    const bool active = lane < lanes;
    const int i = out / p.n, j = out - i * p.n;
    const int k0 = c * p.kchunk, k1 = min(p.k, k0 + p.kchunk);
    double acc = 0.0;
    for (int kk = k0; kk < k1; kk += 64) {
      const int kc = min(64, k1 - kk);
      __syncthreads();
      for (int e = tid; e < p.m * 64; e += 256) {
        const int r = e >> 6, q = e & 63;
        sm.As[r][q] = q < kc ? ldin<kCoh>(p.A + (int64_t)r * p.a_rs + (int64_t)(kk + q) * p.a_cs) : 0.0;
      }
      for (int e = tid; e < p.n * 64; e += 256) {
        const int r = e >> 6, q = e & 63;
        sm.Bs[r][q] = q < kc ? ldin<kCoh>(p.B + (int64_t)r * p.b_rs + (int64_t)(kk + q) * p.b_cs) : 0.0;
      }
      __syncthreads();
      if (active)
        for (int q = lane; q < kc; q += lanes) acc = fma(sm.As[i][q], sm.Bs[j][q], acc);
    }
    __syncthreads();
    sm.red[tid] = active ? acc : 0.0;
    __syncthreads();
    if (tid < P) {
      double sum = 0.0;
      for (int l = 0; l < lanes; ++l) sum = __dadd_rn(sum, sm.red[l * P + tid]);
      if (p.ksplit > 1) {
        p.partial[(int64_t)c * P + tid] = sum;
      } else {
        double* cp = p.C + (int64_t)i * p.c_rs + j;
        const double v = __dmul_rn(p.alpha, sum);
        *cp = p.accumulate ? __dadd_rn(ldrw<kCoh>(cp), v) : v;
      }
    }
  }
}

// Fixed-order reduction of split-K partials into C.
template <bool kCoh>
__device__ __forceinline__ void splitk_reduce_body(const GemmProblem* __restrict__ probs,
                                                   const int* __restrict__ red_prob,
                                                   const uint32_t* __restrict__ red_first, int nred, uint32_t nchunks,
                                                   uint32_t bid, uint32_t nblk) {
  for (uint32_t chunk = bid; chunk < nchunks; chunk += nblk) {
    int lo = 0, hi = nred - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (red_first[mid] <= chunk) lo = mid; else hi = mid - 1;
    }
    const GemmProblem& p = probs[red_prob[lo]];
    const int64_t mn = (int64_t)p.m * p.n;
    const int64_t base = (int64_t)(chunk - red_first[lo]) * kRedChunk;
    for (int k = 0; k < kRedChunk / kRedThreads; ++k) {
      int64_t e = base + k * kRedThreads + threadIdx.x;
      if (e >= mn) break;
      double s = 0.0;
      for (int c = 0; c < p.ksplit; ++c) s = __dadd_rn(s, ldrw<kCoh>(p.partial + (int64_t)c * mn + e));
      int64_t row = e / p.n, col = e - row * p.n;
      double* cp = p.C + row * p.c_rs + col;
      double v = __dmul_rn(p.alpha, s);
      *cp = p.accumulate ? __dadd_rn(ldrw<kCoh>(cp), v) : v;
    }
  }
}

// ---- coupled-cluster element-wise work -------------------------------------------

constexpr int kCcThreads = 256;
constexpr int kCcChunk = 2048;

// tau, taut and Q from t2 and t1 (see CCAmpTile in cc.h).
template <bool kCoh>
__device__ __forceinline__ void cc_amp_body(const CCAmpTile* __restrict__ tiles, const CCAmpItem* __restrict__ items,
                                            int nitems, const double* __restrict__ t1, const double* __restrict__ t2,
                                            double* __restrict__ tau, double* __restrict__ taut,
                                            double* __restrict__ Q, uint32_t bid, uint32_t nblk) {
  constexpr int kPer = kCcChunk / kCcThreads;
  for (int i = (int)bid; i < nitems; i += (int)nblk) {
    const CCAmpItem it = items[i];
    const CCAmpTile& tl = tiles[it.tile];
    const uint32_t ej = tl.fj.d, ea = tl.fa.d, eb = tl.fb.d;
    const int64_t o_ia = tl.t1[0], o_jb = tl.t1[1], o_ib = tl.t1[2], o_ja = tl.t1[3];
    const bool h1 = o_ia >= 0 && o_jb >= 0, h2 = o_ib >= 0 && o_ja >= 0;
    double x[kPer], p1[kPer], d[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      const uint32_t e = min((uint32_t)(threadIdx.x + k * kCcThreads), it.n - 1);
      const uint32_t f = it.f0 + e;
      const uint32_t r1 = tl.fb.div(f), b = f - r1 * eb;
      const uint32_t r2 = tl.fa.div(r1), a = r1 - r2 * ea;
      const uint32_t ii = tl.fj.div(r2), j = r2 - ii * ej;
      x[k] = ldin<kCoh>(t2 + tl.off + f);
      p1[k] = h1 ? __dmul_rn(ldin<kCoh>(t1 + o_ia + (int64_t)ii * ea + a), ldin<kCoh>(t1 + o_jb + (int64_t)j * eb + b))
                 : 0.0;
      // d = t1_ia t1_jb - t1_ib t1_ja, the second product inside one fused
      // multiply-add
      d[k] = h2 ? __fma_rn(-ldin<kCoh>(t1 + o_ib + (int64_t)ii * eb + b), ldin<kCoh>(t1 + o_ja + (int64_t)j * ea + a),
                           p1[k])
                : p1[k];
    }
    // five FP64 instructions per element (the FP64 pipe, not HBM, bounds
    // element-wise FP64 work on this part): p1 and d above; tau = t2 + d,
    // taut = t2 + d / 2 and Q = t2 / 2 + p1 (fused multiply-adds by 1/2,
    // which is exact)
    const bool hd = h1 || h2;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      const uint32_t e = threadIdx.x + k * kCcThreads;
      if (e >= it.n) continue;
      const int64_t at = tl.off + it.f0 + e;
      // 0 + t2 (turns -0 into +0) on the bits
      const unsigned long long xb = (unsigned long long)__double_as_longlong(x[k]);
      const double x0 = __longlong_as_double((long long)(xb == 0x8000000000000000ull ? 0ull : xb));
      tau[at] = hd ? __dadd_rn(x0, d[k]) : x0;
      taut[at] = hd ? __fma_rn(0.5, d[k], x0) : x0;
      Q[at] = __fma_rn(0.5, x[k], p1[k]);
    }
  }
}

template <bool kCoh>
__device__ __forceinline__ void mul_body(const double* __restrict__ a, const double* __restrict__ b,
                                         double* __restrict__ out, int64_t n, uint32_t bid, uint32_t nblk) {
  for (int64_t i = (int64_t)bid * kCcThreads + threadIdx.x; i < n; i += (int64_t)nblk * kCcThreads)
    out[i] = __dmul_rn(ldrw<kCoh>(a + i), ldrw<kCoh>(b + i));
}

// Per-CTA partial sums of x*y over n elements, in a fixed order.
template <bool kCoh>
__device__ __forceinline__ void dot_partial_body(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                                                 double* __restrict__ partial, uint32_t bid, uint32_t nblk,
                                                 double* red) {
  double s = 0.0;
  int64_t per = (n + nblk - 1) / nblk;
  int64_t lo = per * bid, hi = min(n, lo + per);
  for (int64_t i = lo + threadIdx.x; i < hi; i += kCcThreads) s = fma(ldrw<kCoh>(x + i), ldrw<kCoh>(y + i), s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kCcThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[bid] = red[0];
}

// The partials are staged through shared memory by all threads, 256 at a
// time, and added by one thread in index order (the same sum as one thread
// reading them one by one, without its chain of dependent global loads).
template <bool kCoh>
__device__ __forceinline__ void energy_final_body(const double* __restrict__ partial, int np, double scale,
                                                  double* __restrict__ hist, int* __restrict__ count, int cap,
                                                  uint32_t bid, double* stage) {
  if (bid != 0) return;
  double s = 0.0;
  for (int i0 = 0; i0 < np; i0 += kCcThreads) {
    __syncthreads();
    if (i0 + (int)threadIdx.x < np) stage[threadIdx.x] = ldrw<kCoh>(partial + i0 + threadIdx.x);
    __syncthreads();
    if (threadIdx.x == 0) {
      const int n = min(kCcThreads, np - i0);
      for (int i = 0; i < n; ++i) s += stage[i];
    }
  }
  if (threadIdx.x == 0) {
    int k = ldrw<kCoh>(count);
    if (k < cap) hist[k] = s * scale;
    *count = k + 1;
  }
}

// ---- zero fill -----------------------------------------------------------------

// bytes a multiple of 4 from a 4-byte aligned p (16-byte words when both allow).
__device__ __forceinline__ void zero_body(void* p, uint64_t bytes, uint32_t bid, uint32_t nblk) {
  if ((((uintptr_t)p | bytes) & 15) == 0) {
    uint4* q = reinterpret_cast<uint4*>(p);
    const uint64_t n = bytes >> 4;
    for (uint64_t i = (uint64_t)bid * kBodyThreads + threadIdx.x; i < n; i += (uint64_t)nblk * kBodyThreads)
      q[i] = make_uint4(0u, 0u, 0u, 0u);
  } else {
    uint32_t* q = reinterpret_cast<uint32_t*>(p);
    const uint64_t n = bytes >> 2;
    for (uint64_t i = (uint64_t)bid * kBodyThreads + threadIdx.x; i < n; i += (uint64_t)nblk * kBodyThreads) q[i] = 0u;
  }
}

}  // namespace dev
}  // namespace gbx
