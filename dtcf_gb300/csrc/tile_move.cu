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
constexpr int kMoveChunk = 2048;  // elements per CTA
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

void MoveSet::release() {
  dev_free(d_desc);
  dev_free(d_first);
  d_desc = nullptr;
  d_first = nullptr;
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
    if (op == 0) {
#pragma unroll
      for (int k = 0; k < kPer; ++k)
        if (in[k]) t[to[k]] = (scale == 1.0) ? x[k] : __dmul_rn(scale, x[k]);
    } else {
      double y[kPer];
#pragma unroll
      for (int k = 0; k < kPer; ++k) y[k] = in[k] ? t[to[k]] : 0.0;
#pragma unroll
      for (int k = 0; k < kPer; ++k)
        if (in[k]) t[to[k]] = __dadd_rn(y[k], __dmul_rn(scale, x[k]));
    }
  }
}

int run_moves_scaled(const MoveSet& ms, const double* src, double* dst, double alpha, cudaStream_t st) {
  if (ms.ndesc == 0 || ms.nchunks == 0) return GBX_OK;
  int grid = (int)std::min<uint32_t>(ms.nchunks, 152u * 16u);
  tile_move_kernel<<<grid, kMoveThreads, 0, st>>>(ms.d_desc, ms.d_first, ms.ndesc, ms.nchunks, src, dst, alpha);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

int run_moves(const MoveSet& ms, const double* src, double* dst, cudaStream_t st) {
  return run_moves_scaled(ms, src, dst, 1.0, st);
}

}  // namespace gbx
