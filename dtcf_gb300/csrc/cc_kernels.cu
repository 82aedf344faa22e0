// Element-wise kernels of the coupled-cluster driver: synthetic integral
// generation, orbital-energy denominators (MP2 guess, Jacobi update), the
// amplitude combinations tau / taut / Q and the deterministic FP64 dot
// product behind the correlation energy.
//
// All of them walk a list of tiles; a tile carries its element offset, rank,
// extents and the global orbital index of the first orbital of each block.
#include <algorithm>

#include "bodies.cuh"
#include "cc.h"
#include "program.h"

namespace gbx {

namespace {
constexpr int kThreads = dev::kCcThreads;
constexpr int kChunk = dev::kCcChunk;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return z;
}

// <pq||rs> of the synthetic Hamiltonian (see cc.h for the definition).
__device__ __forceinline__ double integral(int p, int q, int r, int s, const CCDeviceTables& t) {
  if (p == q || r == s) return 0.0;
  if ((t.irrep[p] ^ t.irrep[q] ^ t.irrep[r] ^ t.irrep[s]) != 0) return 0.0;
  double sg = 1.0;
  if (p > q) {
    int x = p; p = q; q = x;
    sg = -sg;
  }
  if (r > s) {
    int x = r; r = s; s = x;
    sg = -sg;
  }
  uint64_t P = (uint64_t)p * (uint64_t)t.norb + (uint64_t)q;
  uint64_t R = (uint64_t)r * (uint64_t)t.norb + (uint64_t)s;
  if (P > R) {
    uint64_t x = P; P = R; R = x;
  }
  uint64_t h = mix64(t.seed_int ^ (P * 0x9E3779B97F4A7C15ull + R * 0xC2B2AE3D27D4EB4Full));
  double v = t.mag[(q - p) + (s - r)];
  return ((h >> 63) ? -v : v) * sg;
}
}  // namespace

__global__ void __launch_bounds__(kThreads) cc_tile_kernel(const CCTile* __restrict__ tiles,
                                                           const uint32_t* __restrict__ first, int ntiles,
                                                           uint32_t nchunks, int op, CCDeviceTables tab,
                                                           const double* __restrict__ in, double* __restrict__ out) {
  for (uint32_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
    int lo = 0, hi = ntiles - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (__ldg(first + mid) <= chunk) lo = mid; else hi = mid - 1;
    }
    const CCTile& t = tiles[lo];
    const uint32_t base = (chunk - __ldg(first + lo)) * kChunk;
    for (int k = 0; k < kChunk / kThreads; ++k) {
      uint32_t e = base + (uint32_t)(k * kThreads) + threadIdx.x;
      if (e >= t.n) break;
      int g[4];
      uint32_t rem = e;
      for (int d = t.rank - 1; d >= 0; --d) {
        uint32_t q = rem / t.ext[d];
        g[d] = t.gstart[d] + (int)(rem - q * t.ext[d]);
        rem = q;
      }
      const int64_t o = t.off + e;
      if (op == CC_OP_INTEGRAL) {
        out[o] = integral(g[0], g[1], g[2], g[3], tab);
      } else {
        // denominator: sum over occupied indices of eps minus over virtual ones
        double dnm = 0.0;
        for (int d = 0; d < t.rank; ++d) {
          double ev = tab.eps[g[d]];
          dnm = (g[d] < tab.nocc) ? __dadd_rn(dnm, ev) : __dsub_rn(dnm, ev);
        }
        out[o] = op == CC_OP_DENOM ? __ddiv_rn(in[o], dnm) : __ddiv_rn(1.0, dnm);
      }
    }
  }
}

__global__ void __launch_bounds__(kThreads) mul_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                       double* __restrict__ out, int64_t n) {
  dev::mul_body<false>(a, b, out, n, blockIdx.x, gridDim.x);
}

// Per-CTA partial sums of x*y over n elements, in a fixed order.
__global__ void __launch_bounds__(kThreads) dot_partial_kernel(const double* __restrict__ x,
                                                               const double* __restrict__ y, int64_t n,
                                                               double* __restrict__ partial) {
  __shared__ double red[kThreads];
  dev::dot_partial_body<false>(x, y, n, partial, blockIdx.x, gridDim.x, red);
}

__global__ void dot_final_kernel(const double* __restrict__ partial, int np, double scale, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < np; ++i) s += partial[i];
    *out = s * scale;
  }
}

__global__ void __launch_bounds__(kThreads) energy_final_kernel(const double* __restrict__ partial, int np,
                                                                double scale, double* __restrict__ hist,
                                                                int* __restrict__ count, int cap) {
  __shared__ double stage[kThreads];
  dev::energy_final_body<false>(partial, np, scale, hist, count, cap, blockIdx.x, stage);
}

int run_energy(const double* V, const double* tau, int64_t n, double* partial, int npartial, double* hist, int* count,
               int cap, cudaStream_t st) {
  if (ProgRecorder* rec = prog_recording()) {
    ProgArgs a;
    a.dot = {V, tau, partial, n};
    GBX_TRY(prog_mem(rec, PK_DOTPART, (uint32_t)npartial, a, {{V, false}, {tau, false}, {partial, true}}));
    a.efin = {partial, hist, count, 0.25, npartial, cap};
    return prog_mem(rec, PK_ENERGYFIN, 1, a, {{partial, false}, {hist, true}, {count, true}});
  }
  dot_partial_kernel<<<npartial, kThreads, 0, st>>>(V, tau, n, partial);
  GBX_CUDA(cudaGetLastError());
  energy_final_kernel<<<1, kThreads, 0, st>>>(partial, npartial, 0.25, hist, count, cap);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

int CCTileSet::upload(const std::vector<CCTile>& h) {
  release();
  ntiles = (int)h.size();
  if (!ntiles) return GBX_OK;
  std::vector<uint32_t> f(ntiles + 1);
  uint64_t c = 0;
  for (int i = 0; i < ntiles; ++i) {
    f[i] = (uint32_t)c;
    c += (h[i].n + kChunk - 1) / kChunk;
  }
  f[ntiles] = (uint32_t)c;
  nchunks = (uint32_t)c;
  GBX_TRY(dev_alloc((void**)&d_tiles, sizeof(CCTile) * ntiles));
  GBX_TRY(dev_alloc((void**)&d_first, sizeof(uint32_t) * (ntiles + 1)));
  GBX_CUDA(cudaMemcpy(d_tiles, h.data(), sizeof(CCTile) * ntiles, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(d_first, f.data(), sizeof(uint32_t) * (ntiles + 1), cudaMemcpyHostToDevice));
  return GBX_OK;
}

void CCTileSet::release() {
  dev_free(d_tiles);
  dev_free(d_first);
  d_tiles = nullptr;
  d_first = nullptr;
  ntiles = 0;
  nchunks = 0;
}

__global__ void __launch_bounds__(kThreads) cc_amp_kernel(const CCAmpTile* __restrict__ tiles,
                                                         const CCAmpItem* __restrict__ items, int nitems,
                                                         const double* __restrict__ t1,
                                                         const double* __restrict__ t2, double* __restrict__ tau,
                                                         double* __restrict__ taut, double* __restrict__ Q) {
  dev::cc_amp_body<false>(tiles, items, nitems, t1, t2, tau, taut, Q, blockIdx.x, gridDim.x);
}

int CCAmpSet::upload(const std::vector<CCAmpTile>& tiles, const std::vector<CCAmpItem>& items) {
  release();
  nitems = (int)items.size();
  if (!nitems) return GBX_OK;
  GBX_TRY(dev_alloc((void**)&d_tiles, sizeof(CCAmpTile) * tiles.size()));
  GBX_TRY(dev_alloc((void**)&d_items, sizeof(CCAmpItem) * items.size()));
  GBX_CUDA(cudaMemcpy(d_tiles, tiles.data(), sizeof(CCAmpTile) * tiles.size(), cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(d_items, items.data(), sizeof(CCAmpItem) * items.size(), cudaMemcpyHostToDevice));
  bytes = sizeof(CCAmpTile) * tiles.size() + sizeof(CCAmpItem) * items.size();
  return GBX_OK;
}

void CCAmpSet::release() {
  dev_free(d_tiles);
  dev_free(d_items);
  d_tiles = nullptr;
  d_items = nullptr;
  nitems = 0;
}

int run_cc_amp(const CCAmpSet& s, const double* t1, const double* t2, double* tau, double* taut, double* Q,
               cudaStream_t st) {
  if (s.nitems == 0) return GBX_OK;
  const int grid = std::min(s.nitems, 152 * 8);
  if (ProgRecorder* rec = prog_recording()) {
    ProgArgs a;
    a.amp = {s.d_tiles, s.d_items, t1, t2, tau, taut, Q, s.nitems};
    return prog_mem(rec, PK_AMP, (uint32_t)grid, a,
                    {{t1, false}, {t2, false}, {tau, true}, {taut, true}, {Q, true}});
  }
  cc_amp_kernel<<<grid, kThreads, 0, st>>>(s.d_tiles, s.d_items, s.nitems, t1, t2, tau, taut, Q);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

int run_mul(const double* a, const double* b, double* out, int64_t n, cudaStream_t st) {
  if (n <= 0) return GBX_OK;
  const int grid = (int)std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 16);
  if (ProgRecorder* rec = prog_recording()) {
    ProgArgs pa;
    pa.mul = {a, b, out, n};
    return prog_mem(rec, PK_MUL, (uint32_t)grid, pa, {{a, false}, {b, false}, {out, true}});
  }
  mul_kernel<<<grid, kThreads, 0, st>>>(a, b, out, n);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

int run_cc_tiles(const CCTileSet& ts, int op, const CCDeviceTables& tab, const double* in, double* out,
                 cudaStream_t st) {
  if (ts.ntiles == 0 || ts.nchunks == 0) return GBX_OK;
  int grid = (int)std::min<uint32_t>(ts.nchunks, 152u * 16u);
  cc_tile_kernel<<<grid, kThreads, 0, st>>>(ts.d_tiles, ts.d_first, ts.ntiles, ts.nchunks, op, tab, in, out);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

int run_dot(const double* x, const double* y, int64_t n, double scale, double* partial, int npartial, double* out,
            cudaStream_t st) {
  dot_partial_kernel<<<npartial, kThreads, 0, st>>>(x, y, n, partial);
  GBX_CUDA(cudaGetLastError());
  dot_final_kernel<<<1, 32, 0, st>>>(partial, npartial, scale, out);
  GBX_CUDA(cudaGetLastError());
  return GBX_OK;
}

}  // namespace gbx
