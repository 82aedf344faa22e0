// Shared definitions of the gbx library: error state, CUDA checks, the
// tile-move descriptor used by every permute / pack / unpack, and the GEMM
// problem descriptors.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gbx.h"

namespace gbx {

void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define GBX_CUDA(call)                                                         \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess) return ::gbx::cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define GBX_TRY(call)            \
  do {                           \
    int _rc = (call);            \
    if (_rc != GBX_OK) return _rc; \
  } while (0)

constexpr int kMaxDims = 8;

// Unsigned division by a run-time invariant divisor d (1 <= d < 2^31) as a
// multiply-high and shift (Granlund & Montgomery, "Division by invariant
// integers using multiplication", 1994): q = (mulhi(n, m) + n) >> s with
// s = ceil(log2 d) and m = floor(2^32 (2^s - d) / d) + 1, exact for n < 2^31.
struct FastDiv {
  uint32_t d, m, s;
  static FastDiv make(uint32_t d_) {
    FastDiv f;
    f.d = d_;
    uint32_t s = 0;
    while ((1ull << s) < d_) ++s;
    f.s = s;
    f.m = (uint32_t)(((1ull << 32) * ((1ull << s) - d_)) / d_ + 1);
    return f;
  }
#ifdef __CUDACC__
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    return (uint32_t)(((uint64_t)__umulhi(n, m) + n) >> s);
  }
#endif
};

// One strided tile move: for every index tuple idx over ext[0..rank-1],
//   dst[dst + sum idx_d * dstr_d]  (op)=  scale * src[src + sum idx_d * sstr_d]
// op 0 stores (a plain copy when scale == 1, bit-exact), op 1 accumulates
// dst + scale * x with one fused multiply-add: the separately rounded product
// and sum whenever scale * x is exact (scale = +-2^k), one FP64 instruction
// instead of two (the FP64 pipe, not HBM, bounds element-wise FP64 work on
// this part).  The host orders the dimensions so that the last one has the
// smallest destination stride.
struct MoveDesc {
  int64_t src, dst;
  int64_t sstr[kMaxDims];
  int64_t dstr[kMaxDims];
  FastDiv div[kMaxDims];
  uint32_t ext[kMaxDims];
  uint32_t n;  // elements (product of ext), < 2^31
  int32_t rank;
  int32_t op;
  int32_t pad;
  double scale;
};

// Host-side builder: fills a MoveDesc from extents and strides, merging
// dimensions that are contiguous in both source and destination and ordering
// the rest by destination stride.
MoveDesc make_move(int rank, const int64_t* ext, const int64_t* sstr, const int64_t* dstr, int64_t src,
                   int64_t dst, int op, double scale);

// Compact form of a move of at most four dimensions (padded in front with
// unit extents), with the first chunk of its launch schedule.
struct MoveDesc4 {
  int64_t src, dst;
  int64_t sstr[4], dstr[4];
  FastDiv div[4];
  uint32_t ext[4];
  uint32_t n, first;
  int32_t op, pad;
  double scale;
};

// A set of moves uploaded to the device with its launch schedule.  When every
// move has at most four dimensions the compact descriptors and a chunk ->
// descriptor table are uploaded instead of the general ones.
struct MoveSet {
  std::vector<MoveDesc> host;
  MoveDesc* d_desc = nullptr;
  uint32_t* d_first = nullptr;  // first chunk of each descriptor (prefix sum)
  MoveDesc4* d_desc4 = nullptr;
  uint32_t* d_chunk_desc = nullptr;  // descriptor of each chunk
  uint32_t nchunks = 0;
  int ndesc = 0;
  int upload();   // copies host -> device (allocates)
  void release();
  size_t device_bytes() const;  // what upload() allocates
  ~MoveSet() { release(); }
};

// Runs every move of the set on (src, dst) buffers; accumulating moves use
// scale * alpha.
int run_moves(const MoveSet& ms, const double* src, double* dst, cudaStream_t st);
int run_moves_scaled(const MoveSet& ms, const double* src, double* dst, double alpha, cudaStream_t st);

// Fused permuted sum over one destination layout of rank 2..4: every
// destination element is formed in one pass as
//   out = (0 + coef_0 * x_0 + coef_1 * x_1 + ...) [* scale]
// in term order, each term added with one fused multiply-add (the separately
// rounded product and sum whenever coef * x is exact, as for coef = +-2^k),
// x_t the element of source term t under that term's permutation.  A
// destination tile is a sequence of slabs: a slab is its last two dimensions
// (extents ea x eb, contiguous), slab s sits at outer indices (o0, o1) =
// (s / O1, s % O1) of its first two dimensions (padded with unit extents).
constexpr int kFsMaxSlots = 8;     // distinct source buffers of one plan
constexpr int kFsMaxTerms = 16;    // terms of one plan
constexpr int kFsItemElems = 2048; // destination elements per work item

// One (destination tile, term) pair.
struct FsTerm {
  int64_t off;       // source offset of the destination tile's first element
  int64_t so0, so1;  // source strides of the destination's two outer dimensions
  int64_t sa, sb;    // source strides of the slab dimensions
  double coef;       // coefficient with the layout's sign factor
  int32_t slot;      // source buffer
  int32_t mode;      // 0 slabs contiguous in order, 1 slabs contiguous transposed, 2 gather
};

// A run of destination elements inside one tile.
struct FsItem {
  int64_t dst;               // destination (and scale) offset of the first element
  FastDiv fE, fea, feb, fo1; // slab size ea * eb, the slab extents, O1
  uint32_t f0;               // index of the first element within the tile
  uint32_t n;                // elements (<= kFsItemElems)
  uint32_t term0, nterm;
  uint32_t whole;            // whole slabs only (transposed slabs staged in shared memory)
};

struct FsSrc {
  const double* p[kFsMaxSlots];
};

int run_fused_sum(const FsItem* items, int nitems, const FsTerm* terms, const FsSrc& src, const double* scale,
                  double* out, cudaStream_t st);

// Direct FP64 contraction (no packing): for a contraction whose contracted
// extent per output element is small, every output element is formed in
// place from the stored operand tiles,
//   C[c] = alpha * acc + C[c],  acc = sum over tile pairs p and contracted
//   indices k of (+-) A[offA_p + c . sA_p + k . sAk_p] * B[offB_p + ...]
// with one fused multiply-add per product (FP64 instructions are the bound
// on this part, so no separate pack, GEMM and unpack passes).
constexpr int kDirMaxPairs = 32;     // operand tile pairs of one output tile
constexpr int kDirItemElems = 2048;  // output elements per work item

struct DirPair {
  int64_t offA, offB;      // stored operand tiles
  int64_t sA[4], sB[4];    // strides of the output tile's dims (rank padded to 4 in front; 0 = not in operand)
  int64_t sAk[2], sBk[2];  // strides of the contracted dims
  uint32_t ek[2];          // contracted extents (1 when unused)
  int32_t neg;             // sign factor of the pair is -1
  int32_t pad;
};

struct DirItem {
  int64_t coff;           // C offset of the item's first element
  FastDiv f1, f2, f3;     // extents of output dims 1..3
  uint32_t f0, n;         // first element within the tile, count
  uint32_t pair0, npair;
};

// overwrite: C = alpha A B (the items cover all of C), else C += alpha A B
int run_direct(const DirItem* items, int nitems, const DirPair* pairs, const double* A, const double* B, double* C,
               double alpha, bool overwrite, cudaStream_t st);

// One FP64 GEMM problem of a grouped launch (element strides).
struct GemmProblem {
  const double* A;
  const double* B;
  double* C;
  int64_t a_rs, a_cs, b_rs, b_cs, c_rs;
  int m, n, k;
  double alpha;
  int accumulate;
  // split-K and tile shape (filled by F64Gemm::build)
  int ksplit, kchunk, pad_;
  double* partial;
};

// Grouped FP64 GEMM: C_p (+)= alpha_p * A_p * B_p^T for all problems in one
// persistent launch (plus a fixed-order split-K reduction when needed).
struct F64Gemm {
  struct Sub {  // one launch: the problems of one tile shape
    GemmProblem* d_probs = nullptr;
    int* d_first = nullptr;
    int* d_ticket = nullptr;
    int nprob = 0, total_tiles = 0, variant = 0;
    std::vector<int> first;  // host copy of d_first (per-problem launches)
  };
  std::vector<Sub> subs;
  GemmProblem* d_all = nullptr;  // every problem (for the split-K reduction)
  double* d_partial = nullptr;
  int* d_red_prob = nullptr;
  uint32_t* d_red_first = nullptr;
  int nprob = 0, nred = 0;
  uint32_t red_chunks = 0;
  double workspace_bytes = 0.0;
  bool async_stream_set = false;
  cudaStream_t async_stream = nullptr;
  // async: allocate / upload stream-ordered on st (for one-shot leaf calls).
  // variants: tile shape per problem (f64_variant numbering; -1 = model).
  int build(const std::vector<GemmProblem>& probs, bool async = false, cudaStream_t st = nullptr,
            const std::vector<int>* variants = nullptr);
  int run(cudaStream_t st) const;
  // One shape's launch (its work-queue ticket reset first).
  static int run_sub(const Sub& sb, cudaStream_t st);
  // One launch per problem (static schedule), then the split-K reduction:
  // the per-launch baseline against the single persistent launch of run().
  int run_each(cudaStream_t st) const;
  void release();
  ~F64Gemm() { release(); }
};
// Split-K partial-sum elements F64Gemm::build allocates for these problems
// (model tile shapes).
int64_t f64_partial_elems(const std::vector<GemmProblem>& probs);
// Tile shapes shared by the host planner and the kernels.
int f64_variant(int m, int n);
int f64_variant(int m, int n, int k);
// As f64_variant, plus variant 7 (at most 16 x 16 outputs, long K) for planned launches.
int f64_variant_planned(int m, int n, int k);
int f64_tile_m(int variant);
int f64_tile_n(int variant);
int f64_tiles(int m, int n);

// Device scratch allocation helpers (the library's own allocations go
// through these so that OOM surfaces as GBX_ENOMEM).
int dev_alloc(void** p, size_t bytes);
void dev_free(void* p);
// While alive, library allocations made on this thread are counted in *acc
// (and subtracted again when freed, on any thread).
struct AllocAccount {
  explicit AllocAccount(std::atomic<int64_t>* acc);
  ~AllocAccount();
  std::atomic<int64_t>* prev;
};
// While alive, library allocations made on this thread come from the
// stream-ordered allocator on `st` and are later freed on it (cudaFreeAsync),
// so releasing them does not wait for the whole device as cudaFree does.  The
// caller must ensure no work still uses memory it frees.
struct StreamOrderedAlloc {
  explicit StreamOrderedAlloc(cudaStream_t st);
  ~StreamOrderedAlloc();
  bool prev_on;
  cudaStream_t prev;
};

}  // namespace gbx
