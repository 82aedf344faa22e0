// Strided tile moves: the single kernel behind every block permute, big-matrix
// pack / unpack and permuted accumulate of the library.
//
// A launch covers a whole set of moves (e.g. every tile of one operand of one
// contraction).  Each CTA takes one 2048-element chunk of one move; threads
// walk the chunk in destination order, so stores are coalesced along the
// destination's fastest dimension and loads go through the read-only cache.
// Pure copies (op 0, scale 1) move bits unchanged, so permutes are bit-exact.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.h"

namespace gbx {

namespace {
constexpr int kMoveThreads = 256;
constexpr int kMoveChunk = 2048;   // elements per CTA (general moves)
constexpr int kMove4Chunk = 4096;  // elements per CTA (moves of at most four dimensions)
}  // namespace

MoveDesc make_move(int rank, const int64_t* ext, const int64_t* sstr, const int64_t* dstr, int64_t src,
                   int64_t dst, int op, double scale) {
  // drop unit extents, then order by destination stride (largest first)
  int idx[kMaxDims];
  int r = 0;
  for (int d = 0; d < rank; ++d)
    if (ext[d] != 1) idx[r++] = d;
  std::stable_sort(idx, idx + r, [&](int a, int b) { return dstr[a] > dstr[b]; });
  int64_t e[kMaxDims], s[kMaxDims], t[kMaxDims];
  int m = 0;
  for (int i = 0; i < r; ++i) {
    int d = idx[i];
    // merge with the previous (outer) dim when contiguous in both buffers
    if (m > 0 && s[m - 1] == sstr[d] * ext[d] && t[m - 1] == dstr[d] * ext[d]) {
      e[m - 1] *= ext[d];
      s[m - 1] = sstr[d];
      t[m - 1] = dstr[d];
    } else {
      e[m] = ext[d];
      s[m] = sstr[d];
      t[m] = dstr[d];
      ++m;
    }
  }
  MoveDesc md;
  std::memset(&md, 0, sizeof(md));
  if (m == 0) {  // a single element
    e[0] = 1;
    s[0] = 0;
    t[0] = 0;
    m = 1;
  }
  md.rank = m;
  int64_t n = 1;
  for (int i = 0; i < m; ++i) {
    md.ext[i] = (uint32_t)e[i];
    md.sstr[i] = s[i];
    md.dstr[i] = t[i];
    md.div[i] = FastDiv::make((uint32_t)e[i]);
    n *= e[i];
  }
  for (int i = 0; i < rank; ++i)
    if (ext[i] == 0) n = 0;
  md.n = (uint32_t)n;
  md.src = src;
  md.dst = dst;
  md.op = op;
  md.scale = scale;
  return md;
}

int MoveSet::upload() {
  release();
  ndesc = (int)host.size();
  if (ndesc == 0) return GBX_OK;
  bool small = true;
  for (const MoveDesc& m : host) {
    uint64_t prod = 1;
    for (int d = 0; d < m.rank; ++d) prod *= m.ext[d];
    if (prod >= (1ull << 31) || (prod != m.n && m.n != 0))
      return fail(GBX_EUNSUPPORTED, "tile move of %llu elements (at most 2^31 - 1)", (unsigned long long)prod);
    small = small && m.rank <= 4;
  }
  if (small) {
    std::vector<MoveDesc4> h4(ndesc);
    std::vector<uint32_t> cd;
    uint64_t c = 0;
    for (int i = 0; i < ndesc; ++i) {
      const MoveDesc& m = host[i];
      MoveDesc4& q = h4[i];
      std::memset(&q, 0, sizeof(q));
      const int pad = 4 - m.rank;
      for (int d = 0; d < 4; ++d) {
        const bool real = d >= pad;
        q.ext[d] = real ? m.ext[d - pad] : 1u;
        q.sstr[d] = real ? m.sstr[d - pad] : 0;
        q.dstr[d] = real ? m.dstr[d - pad] : 0;
        q.div[d] = FastDiv::make(q.ext[d]);
      }
      q.src = m.src;
      q.dst = m.dst;
      q.n = m.n;
      q.op = m.op;
      q.scale = m.scale;
      // moves whose innermost run is contiguous on both sides, of even
      // length, starting at even offsets with even outer strides go two
      // elements at a time (16-byte loads and stores)
      bool pair = q.ext[3] % 2 == 0 && q.sstr[3] == 1 && q.dstr[3] == 1 && m.src % 2 == 0 && m.dst % 2 == 0;
      for (int d = 0; d < 3 && pair; ++d) pair = q.sstr[d] % 2 == 0 && q.dstr[d] % 2 == 0;
      q.pad = pair ? 1 : 0;
      q.first = (uint32_t)c;
      const uint64_t nc = (m.n + kMove4Chunk - 1) / kMove4Chunk;
      c += nc;
      if (c >= (1ull << 31)) return fail(GBX_EUNSUPPORTED, "move set too large (%llu chunks)", (unsigned long long)c);
      for (uint64_t k = 0; k < nc; ++k) cd.push_back((uint32_t)i);
    }
    nchunks = (uint32_t)c;
    GBX_TRY(dev_alloc((void**)&d_desc4, sizeof(MoveDesc4) * ndesc));
    GBX_CUDA(cudaMemcpy(d_desc4, h4.data(), sizeof(MoveDesc4) * ndesc, cudaMemcpyHostToDevice));
    if (nchunks) {
      GBX_TRY(dev_alloc((void**)&d_chunk_desc, sizeof(uint32_t) * nchunks));
      GBX_CUDA(cudaMemcpy(d_chunk_desc, cd.data(), sizeof(uint32_t) * nchunks, cudaMemcpyHostToDevice));
    }
    return GBX_OK;
  }
  std::vector<uint32_t> first(ndesc + 1);
  uint64_t c = 0;
  for (int i = 0; i < ndesc; ++i) {
    first[i] = (uint32_t)c;
    c += (host[i].n + kMoveChunk - 1) / kMoveChunk;
  }
  first[ndesc] = (uint32_t)c;
  if (c >= (1ull << 31)) return fail(GBX_EUNSUPPORTED, "move set too large (%llu chunks)", (unsigned long long)c);
  nchunks = (uint32_t)c;
  GBX_TRY(dev_alloc((void**)&d_desc, sizeof(MoveDesc) * ndesc));
  GBX_TRY(dev_alloc((void**)&d_first, sizeof(uint32_t) * (ndesc + 1)));
  GBX_CUDA(cudaMemcpy(d_desc, host.data(), sizeof(MoveDesc) * ndesc, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(d_first, first.data(), sizeof(uint32_t) * (ndesc + 1), cudaMemcpyHostToDevice));
  return GBX_OK;
}

size_t MoveSet::device_bytes() const {
  if (host.empty()) return 0;
  bool small = true;
  uint64_t c = 0;
  for (const MoveDesc& m : host) {
    small = small && m.rank <= 4;
    c += (m.n + kMove4Chunk - 1) / kMove4Chunk;
  }
  if (small) return host.size() * sizeof(MoveDesc4) + c * sizeof(uint32_t);
  return host.size() * sizeof(MoveDesc) + (host.size() + 1) * sizeof(uint32_t);
}

void MoveSet::release() {
  dev_free(d_desc);
  dev_free(d_first);
  dev_free(d_desc4);
  dev_free(d_chunk_desc);
  d_desc = nullptr;
  d_first = nullptr;
  d_desc4 = nullptr;
  d_chunk_desc = nullptr;
  nchunks = 0;
}

__global__ void __launch_bounds__(kMoveThreads) tile_move_kernel(const MoveDesc* __restrict__ descs,
                                                                 const uint32_t* __restrict__ first, int ndesc,
                                                                 uint32_t nchunks, const double* __restrict__ src,
                                                                 double* __restrict__ dst, double alpha) {
  for (uint32_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
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
    for (int k = 0; k < kPer; ++k) x[k] = in[k] ? __ldg(s + so[k]) : 0.0;
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
      for (int k = 0; k < kPer; ++k) y[k] = in[k] ? t[to[k]] : 0.0;
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
__global__ void __launch_bounds__(kMoveThreads) tile_move4_kernel(const MoveDesc4* __restrict__ descs,
                                                                  const uint32_t* __restrict__ chunk_desc,
                                                                  uint32_t nchunks, const double* __restrict__ src,
                                                                  double* __restrict__ dst, double alpha,
                                                                  int allow_pairs) {
  constexpr int kPer = 8;
  constexpr int kBatches = kMove4Chunk / (kMoveThreads * kPer);
  for (uint32_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
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
      // pairs (2e, 2e + 1): the chunk's kMove4Chunk elements in one batch of
      // kPer pairs per thread
      int64_t so[kPer], to[kPer];
      bool in[kPer];
#pragma unroll
      for (int k = 0; k < kPer; ++k) {
        const uint32_t e = base + 2u * ((uint32_t)(k * kMoveThreads) + threadIdx.x);
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
        x[k] = in[k] ? __ldg(reinterpret_cast<const double2*>(s + so[k])) : make_double2(0.0, 0.0);
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
          y[k] = in[k] ? *reinterpret_cast<const double2*>(t + to[k]) : make_double2(0.0, 0.0);
#pragma unroll
        for (int k = 0; k < kPer; ++k)
          if (in[k])
            *reinterpret_cast<double2*>(t + to[k]) =
                make_double2(__fma_rn(scale, x[k].x, y[k].x), __fma_rn(scale, x[k].y, y[k].y));
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
      for (int k = 0; k < kPer; ++k) x[k] = in[k] ? __ldg(s + so[k]) : 0.0;
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
        for (int k = 0; k < kPer; ++k) y[k] = in[k] ? t[to[k]] : 0.0;
#pragma unroll
        for (int k = 0; k < kPer; ++k)
          if (in[k]) t[to[k]] = __fma_rn(scale, x[k], y[k]);
      }
    }
  }
}

int run_moves_scaled(const MoveSet& ms, const double* src, double* dst, double alpha, cudaStream_t st) {
  if (ms.ndesc == 0 || ms.nchunks == 0) return GBX_OK;
  if (ms.d_desc4) {
    const int grid = (int)std::min<uint32_t>(ms.nchunks, 152u * 8u);
    // pairs need 16-byte aligned buffer bases (descriptor offsets are even)
    const int pairs = (((uintptr_t)src | (uintptr_t)dst) & 15) == 0 ? 1 : 0;
    tile_move4_kernel<<<grid, kMoveThreads, 0, st>>>(ms.d_desc4, ms.d_chunk_desc, ms.nchunks, src, dst, alpha,
                                                     pairs);
    GBX_CUDA(cudaGetLastError());
    return GBX_OK;
  }
  int grid = (int)std::min<uint32_t>(ms.nchunks, 152u * 16u);
  tile_move_kernel<<<grid, kMoveThreads, 0, st>>>(ms.d_desc, ms.d_first, ms.ndesc, ms.nchunks, src, dst, alpha);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

int run_moves(const MoveSet& ms, const double* src, double* dst, cudaStream_t st) {
  return run_moves_scaled(ms, src, dst, 1.0, st);
}

namespace {
constexpr int kFsThreads = 256;
constexpr int kFsPer = kFsItemElems / kFsThreads;
// transposed slabs of one item, rows padded to an odd length: a whole-slab
// item of n elements needs at most n + n / ea <= 2n doubles
constexpr int kFsStage = 2 * kFsItemElems;
static_assert(kFsPer * kFsThreads == kFsItemElems, "item size");
}  // namespace

// One CTA per work item (grid-stride over items).  Threads hold kFsPer
// destination elements each, in destination order, and add the terms one
// after the other: rows of slabs that are contiguous in the source's own
// order are read directly (coalesced); slabs stored transposed are first
// copied into shared memory in source order and read back transposed, so
// both sides stay coalesced; anything else is gathered.  Stores are
// coalesced along the destination.
__global__ void __launch_bounds__(kFsThreads, 3)
    fused_sum_kernel(const FsItem* __restrict__ items, int nitems, const FsTerm* __restrict__ terms, FsSrc src,
                     const double* __restrict__ scale, double* __restrict__ out) {
  __shared__ double stage[kFsStage];
  __shared__ const double* base[kFsMaxSlots];  // indexed by the term's slot
  // the item and its terms, read field by field (keeps registers free for
  // the elements in flight)
  __shared__ FsItem s_item;
  __shared__ FsTerm s_terms[kFsMaxTerms];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < kFsMaxSlots; ++k) base[k] = src.p[k];
  }
  for (int i = blockIdx.x; i < nitems; i += gridDim.x) {
    __syncthreads();  // the previous item is finished with s_item, s_terms and stage
    if (threadIdx.x == 0) s_item = items[i];
    __syncthreads();
    const FsItem& it = s_item;
    if (threadIdx.x < it.nterm) s_terms[threadIdx.x] = terms[it.term0 + threadIdx.x];
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
      const double* __restrict__ p = base[tm.slot] + tm.off;
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
          x[k] = __ldg(p + (o0 * so0 + o1 * so1 + (e - sl * E)));
        }
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          const uint32_t e = threadIdx.x + k * kFsThreads;
          if (e < it.n) {
            const uint32_t sl = it.fE.div(e);
            const uint32_t qq = e - sl * E;  // source order within the slab: b * ea + a
            const uint32_t b = it.fea.div(qq);
            stage[sl * sp + b * pa + (qq - b * ea)] = x[k];
          }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          const uint32_t e = min((uint32_t)(threadIdx.x + k * kFsThreads), it.n - 1);
          const uint32_t sl = it.fE.div(e), q = qk[k];
          const uint32_t a = it.feb.div(q);
          x[k] = stage[sl * sp + (q - a * eb) * pa + a];
        }
      } else if (tm.mode == 0) {
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          FS_ELEM(k, o0, o1, q);
          x[k] = __ldg(p + (o0 * so0 + o1 * so1 + q));
        }
      } else {
        const uint32_t sa = (uint32_t)tm.sa, sb = (uint32_t)tm.sb;
#pragma unroll
        for (int k = 0; k < kFsPer; ++k) {
          FS_ELEM(k, o0, o1, q);
          const uint32_t a = it.feb.div(q);
          x[k] = __ldg(p + (o0 * so0 + o1 * so1 + a * sa + (q - a * eb) * sb));
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
      const unsigned long long cbits = (unsigned long long)__double_as_longlong(s_terms[0].coef);
      if ((cbits & 0x7FFFFFFFFFFFFFFFull) == 0x3FF0000000000000ull) {
        double x[kFsPer];
        gather(s_terms[0], x);
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
      gather(s_terms[t], x);
      const double c = s_terms[t].coef;
#pragma unroll
      for (int k = 0; k < kFsPer; ++k) acc[k] = __fma_rn(c, x[k], acc[k]);
    }
#undef FS_ELEM
#pragma unroll
    for (int k = 0; k < kFsPer; ++k) {
      const uint32_t e = threadIdx.x + k * kFsThreads;
      if (e < it.n) {
        double v = acc[k];
        if (scale) v = __dmul_rn(v, __ldg(scale + it.dst + e));
        out[it.dst + e] = v;
      }
    }
  }
}

int run_fused_sum(const FsItem* items, int nitems, const FsTerm* terms, const FsSrc& src, const double* scale,
                  double* out, cudaStream_t st) {
  if (nitems == 0) return GBX_OK;
  const int grid = std::min(nitems, 152 * 6);
  fused_sum_kernel<<<grid, kFsThreads, 0, st>>>(items, nitems, terms, src, scale, out);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

}  // namespace gbx
