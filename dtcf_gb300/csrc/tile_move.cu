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

#include "bodies.cuh"
#include "common.h"
#include "program.h"

namespace gbx {

namespace {
using dev::kMove4Chunk;
using dev::kMoveChunk;
using dev::kMoveThreads;
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
  dev::move_body<false>(descs, first, ndesc, nchunks, src, dst, alpha, blockIdx.x, gridDim.x);
}

// Moves of at most four dimensions (dev::move4_body).
__global__ void __launch_bounds__(kMoveThreads) tile_move4_kernel(const MoveDesc4* __restrict__ descs,
                                                                  const uint32_t* __restrict__ chunk_desc,
                                                                  uint32_t nchunks, const double* __restrict__ src,
                                                                  double* __restrict__ dst, double alpha,
                                                                  int allow_pairs) {
  dev::move4_body<false>(descs, chunk_desc, nchunks, src, dst, alpha, allow_pairs, blockIdx.x, gridDim.x);
}

int run_moves_scaled(const MoveSet& ms, const double* src, double* dst, double alpha, cudaStream_t st) {
  if (ms.ndesc == 0 || ms.nchunks == 0) return GBX_OK;
  ProgRecorder* rec = prog_recording();
  if (ms.d_desc4) {
    const int grid = (int)std::min<uint32_t>(ms.nchunks, 152u * 8u);
    // pairs need 16-byte aligned buffer bases (descriptor offsets are even)
    const int pairs = (((uintptr_t)src | (uintptr_t)dst) & 15) == 0 ? 1 : 0;
    if (rec) {
      ProgArgs a;
      a.move4 = {ms.d_desc4, ms.d_chunk_desc, ms.nchunks, pairs, src, dst, alpha};
      return prog_mem(rec, PK_MOVE4, (uint32_t)grid, a, {{src, false}, {dst, true}});
    }
    tile_move4_kernel<<<grid, kMoveThreads, 0, st>>>(ms.d_desc4, ms.d_chunk_desc, ms.nchunks, src, dst, alpha,
                                                     pairs);
    GBX_CUDA(cudaGetLastError());
    return GBX_OK;
  }
  int grid = (int)std::min<uint32_t>(ms.nchunks, 152u * 16u);
  if (rec) {
    ProgArgs a;
    a.move = {ms.d_desc, ms.d_first, ms.ndesc, ms.nchunks, src, dst, alpha};
    return prog_mem(rec, PK_MOVE, (uint32_t)grid, a, {{src, false}, {dst, true}});
  }
  tile_move_kernel<<<grid, kMoveThreads, 0, st>>>(ms.d_desc, ms.d_first, ms.ndesc, ms.nchunks, src, dst, alpha);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

int run_moves(const MoveSet& ms, const double* src, double* dst, cudaStream_t st) {
  return run_moves_scaled(ms, src, dst, 1.0, st);
}

// One CTA per work item of the fused sum (dev::fused_sum_body).
__global__ void __launch_bounds__(dev::kFsThreads, 3)
    fused_sum_kernel(const FsItem* __restrict__ items, int nitems, const FsTerm* __restrict__ terms, FsSrc src,
                     const double* __restrict__ scale, double* __restrict__ out) {
  __shared__ dev::FsSmem sm;
  dev::fused_sum_body<false>(items, nitems, terms, src, scale, out, blockIdx.x, gridDim.x, sm);
}

int run_fused_sum(const FsItem* items, int nitems, const FsTerm* terms, const FsSrc& src, const double* scale,
                  double* out, cudaStream_t st) {
  if (nitems == 0) return GBX_OK;
  const int grid = std::min(nitems, 152 * 6);
  if (ProgRecorder* rec = prog_recording()) {
    ProgArgs a;
    a.fused.items = items;
    a.fused.terms = terms;
    a.fused.scale = scale;
    a.fused.out = out;
    a.fused.nitems = nitems;
    a.fused.src = src;
    std::vector<ProgTouch> t = {{scale, false}, {out, true}};
    for (int k = 0; k < kFsMaxSlots; ++k) t.push_back({src.p[k], false});
    return prog_mem(rec, PK_FUSED, (uint32_t)grid, a, t);
  }
  fused_sum_kernel<<<grid, dev::kFsThreads, 0, st>>>(items, nitems, terms, src, scale, out);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

}  // namespace gbx
