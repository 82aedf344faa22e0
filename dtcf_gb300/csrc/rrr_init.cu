// RRR tensor initialization on the device: Tensor::initialize on one process
// (tensor.cc:315-335).
//
// Unique tiles.  generate_data (tensor.cc:652-694) walks the block grid in
// lexicographic order (dimension 0 slowest) and keeps an address when
// isValid holds (tensor.cc:605-640): inside every symmetry group ('a'/'A' and
// 'b'/'B' in the symmetry string) the coordinates do not increase from left
// to right.  Here the grid's points are split into chunks, one CTA each:
// pass 1 counts the valid points of every chunk, pass 2 (one CTA) turns the
// counts into chunk offsets, pass 3 writes every valid address at its
// position -- within a chunk in rounds of one point per thread, each round
// compacted by a CTA-wide prefix sum -- so the output order is the
// generation order.
//
// Values.  get_value (tensor.cc:744-758) gives every element of a block the
// same constant: value = 0, then value += sin(address_d) for d from the last
// dimension down to the first.  The sines of the grid coordinates 0 .. max
// vgrid - 1 are taken on the host (the reference's own libm sin) and the
// device adds them in the reference's order, so the values are bit-exact.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"

namespace gbx {

namespace {

constexpr int kRrrThreads = 256;
constexpr int kRrrRounds = 16;
constexpr int kRrrChunk = kRrrThreads * kRrrRounds;  // grid points per CTA

struct RrrShape {
  int dims;
  int vgrid[kMaxDims];
  int group[kMaxDims];  // symmetry group per dimension, -1 = none
};

__device__ __forceinline__ bool rrr_point(const RrrShape& s, uint64_t lin, int* a) {
  for (int d = s.dims - 1; d >= 0; --d) {
    const uint64_t v = (uint64_t)s.vgrid[d];
    a[d] = (int)(lin % v);
    lin /= v;
  }
  for (int i = 0; i < s.dims; ++i)
    for (int j = i + 1; j < s.dims; ++j)
      if (s.group[i] >= 0 && s.group[i] == s.group[j] && a[i] < a[j]) return false;
  return true;
}

__global__ void __launch_bounds__(kRrrThreads) rrr_count_kernel(const RrrShape s, uint64_t npts,
                                                                uint32_t* __restrict__ counts) {
  __shared__ uint32_t warp_sum[kRrrThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kRrrChunk;
  uint32_t c = 0;
  for (int r = 0; r < kRrrRounds; ++r) {
    const uint64_t p = base + (uint64_t)r * kRrrThreads + threadIdx.x;
    int a[kMaxDims];
    if (p < npts && rrr_point(s, p, a)) ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kRrrThreads / 32; ++w) t += warp_sum[w];
    counts[blockIdx.x] = t;
  }
}

// counts -> exclusive offsets in place; offsets[n] = total (one CTA).
__global__ void __launch_bounds__(kRrrThreads) rrr_scan_kernel(uint32_t* __restrict__ counts, uint32_t n) {
  __shared__ uint32_t part[kRrrThreads];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t b = 0; b < n; b += kRrrThreads) {
    const uint32_t i = b + threadIdx.x;
    const uint32_t v = i < n ? counts[i] : 0u;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kRrrThreads; o <<= 1) {  // inclusive Hillis-Steele scan
      const uint32_t add = (int)threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
      __syncthreads();
      part[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < n) counts[i] = carry + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == kRrrThreads - 1) carry += part[kRrrThreads - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[n] = carry;
}

__global__ void __launch_bounds__(kRrrThreads) rrr_write_kernel(const RrrShape s, uint64_t npts,
                                                                const uint32_t* __restrict__ offsets,
                                                                int* __restrict__ out, uint32_t capacity) {
  __shared__ uint32_t warp_sum[kRrrThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kRrrChunk;
  uint32_t pos = offsets[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int r = 0; r < kRrrRounds; ++r) {
    const uint64_t p = base + (uint64_t)r * kRrrThreads + threadIdx.x;
    int a[kMaxDims];
    const bool ok = p < npts && rrr_point(s, p, a);
    const uint32_t ballot = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) warp_sum[warp] = __popc(ballot);
    __syncthreads();
    uint32_t before = 0, round = 0;
    for (int w = 0; w < kRrrThreads / 32; ++w) {
      if (w < warp) before += warp_sum[w];
      round += warp_sum[w];
    }
    before += __popc(ballot & ((1u << lane) - 1u));
    if (ok && pos + before < capacity)
      for (int d = 0; d < s.dims; ++d) out[(uint64_t)(pos + before) * s.dims + d] = a[d];
    pos += round;
    __syncthreads();
  }
}

// Every element of tile t = value of its address (sines from the table).
// A coordinate outside the grid (not a tile address of this grid) gives NaN.
__global__ void __launch_bounds__(kRrrThreads) rrr_fill_kernel(int dims, const int* __restrict__ addr, int ntiles,
                                                               int64_t bs, const double* __restrict__ sinv, int vmax,
                                                               double* __restrict__ tiles) {
  const int64_t total = (int64_t)ntiles * bs;
  for (int64_t e = (int64_t)blockIdx.x * kRrrThreads + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * kRrrThreads) {
    const int64_t t = e / bs;
    double v = 0.0;
    for (int d = dims - 1; d >= 0; --d) {
      const int a = addr[t * dims + d];
      v += (a >= 0 && a < vmax) ? sinv[a] : __longlong_as_double(0x7FF8000000000000ll);
    }
    tiles[e] = v;
  }
}

int shape_of(int dims, const char* sym, const int* vgrid, RrrShape& s, uint64_t& npts) {
  if (dims < 1 || dims > kMaxDims || !sym || !vgrid || (int)std::strlen(sym) != dims)
    return fail(GBX_EINVAL, "bad RRR tensor shape");
  std::memset(&s, 0, sizeof(s));
  s.dims = dims;
  npts = 1;
  for (int d = 0; d < dims; ++d) {
    if (vgrid[d] < 1) return fail(GBX_EINVAL, "vgrid[%d] = %d", d, vgrid[d]);
    s.vgrid[d] = vgrid[d];
    const char c = sym[d];
    s.group[d] = (c == 'a' || c == 'A') ? 0 : (c == 'b' || c == 'B') ? 1 : -1;
    npts *= (uint64_t)vgrid[d];
  }
  if (npts / kRrrChunk >= (1ull << 31)) return fail(GBX_EUNSUPPORTED, "block grid too large");
  return GBX_OK;
}

}  // namespace
}  // namespace gbx

using namespace gbx;

extern "C" {

int gbx_rrr_unique_tiles(int dims, const char* sym, const int* vgrid, int* d_tile_address, int capacity,
                         int* num_tiles, void* stream) {
  if (!num_tiles || capacity < 0 || (capacity > 0 && !d_tile_address)) return fail(GBX_EINVAL, "bad arguments");
  RrrShape s;
  uint64_t npts = 0;
  GBX_TRY(shape_of(dims, sym, vgrid, s, npts));
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t nchunks = (uint32_t)((npts + kRrrChunk - 1) / kRrrChunk);
  uint32_t* d_counts = nullptr;
  GBX_CUDA(cudaMallocAsync((void**)&d_counts, sizeof(uint32_t) * (nchunks + 1), st));
  rrr_count_kernel<<<nchunks, kRrrThreads, 0, st>>>(s, npts, d_counts);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    rrr_scan_kernel<<<1, kRrrThreads, 0, st>>>(d_counts, nchunks);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && capacity > 0) {
    rrr_write_kernel<<<nchunks, kRrrThreads, 0, st>>>(s, npts, d_counts, d_tile_address, (uint32_t)capacity);
    e = cudaGetLastError();
  }
  uint32_t total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, d_counts + nchunks, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d_counts, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "RRR unique tiles", __FILE__, __LINE__);
  *num_tiles = (int)total;
  if (capacity > 0 && (int)total > capacity)
    return fail(GBX_EINVAL, "%u unique tiles, room for %d", total, capacity);
  return GBX_OK;
}

int gbx_rrr_initialize(int dims, const int* vgrid, const int* d_tile_address, int num_tiles, int64_t block_size,
                       double* d_tiles, void* stream) {
  if (dims < 1 || dims > kMaxDims || !vgrid || num_tiles < 0 || block_size < 0 ||
      (num_tiles > 0 && block_size > 0 && (!d_tile_address || !d_tiles)))
    return fail(GBX_EINVAL, "bad arguments");
  if (num_tiles == 0 || block_size == 0) return GBX_OK;
  int vmax = 0;
  for (int d = 0; d < dims; ++d) {
    if (vgrid[d] < 1) return fail(GBX_EINVAL, "vgrid[%d] = %d", d, vgrid[d]);
    vmax = std::max(vmax, vgrid[d]);
  }
  // the reference's get_value: sin of the (virtual) block coordinate
  std::vector<double> sinv(vmax);
  for (int v = 0; v < vmax; ++v) sinv[v] = std::sin((double)v);
  cudaStream_t st = (cudaStream_t)stream;
  double* d_sin = nullptr;
  GBX_CUDA(cudaMallocAsync((void**)&d_sin, sizeof(double) * vmax, st));
  cudaError_t e = cudaMemcpyAsync(d_sin, sinv.data(), sizeof(double) * vmax, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const int64_t total = (int64_t)num_tiles * block_size;
    const int grid = (int)std::min<int64_t>((total + kRrrThreads - 1) / kRrrThreads, 152 * 16);
    rrr_fill_kernel<<<grid, kRrrThreads, 0, st>>>(dims, d_tile_address, num_tiles, block_size, d_sin, vmax,
                                                  d_tiles);
    e = cudaGetLastError();
  }
  // the host table must outlive the copy
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(d_sin, st);
  if (e != cudaSuccess) return cuda_fail(e, "RRR initialize", __FILE__, __LINE__);
  return GBX_OK;
}

}  // extern "C"
