// Block-sparse tensor layouts and contraction plans.
//
// A tensor is a set of stored tiles; each tile is a dense row-major block over
// one block of every dimension.  A dimension is a list of blocks, each with an
// extent and an irrep (spatial-symmetry label, 0 when unused).  Dimensions may
// form permutational symmetry groups; a layout that stores only canonical
// tiles (block coordinates non-increasing within each group, as RRR stores
// them, tensor.cc:617-640) recovers the others by permuting the stored tile
// and multiplying by sign^(number of transpositions).
//
// A contraction C[c] += alpha * sum A[a] B[b] is planned once:
//   - A is packed, per irrep h of its external block tuple, into a row-major
//     matrix A_h (rows: external tuples of A that C needs, columns: contracted
//     tuples), B into B_h likewise, both with the contracted tuples in the
//     same order -- the row/column placement of create_big_matrix
//     (transpose_helper.cc:20-171) with lexicographic block order;
//   - C_h = A_h * B_h^T runs as one grouped GEMM over all h;
//   - C's stored tiles are unpacked from C_h and accumulated with alpha.
// Packs and unpacks are tile moves (permute + place) run as one launch each.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.h"
#include "split.h"

namespace gbx {

struct BlockDim {
  std::vector<int> ext;
  std::vector<int> irrep;
  std::vector<int64_t> start;  // first element of each block along the dimension
  int64_t total = 0;
  static std::shared_ptr<BlockDim> uniform(int nblocks, int extent);
  static std::shared_ptr<BlockDim> make(const std::vector<int>& ext, const std::vector<int>& irrep);
  bool same_as(const BlockDim& o) const { return ext == o.ext && irrep == o.irrep; }
};

using Coords = std::vector<int>;

inline uint64_t coord_key(const int* c, int rank) {
  uint64_t k = 0;
  for (int d = 0; d < rank; ++d) k = k * 65536u + (uint64_t)c[d];
  return k;
}

struct TensorLayout {
  int rank = 0;
  std::vector<std::shared_ptr<BlockDim>> dims;
  std::vector<int> group;  // symmetry group per dim, -1 = none
  int sign = 1;            // +1 symmetric, -1 antisymmetric groups
  std::vector<Coords> tiles;
  std::vector<int64_t> off;
  std::unordered_map<uint64_t, int> index;
  int64_t nelem = 0;

  // Appends a stored tile (offsets assigned in order).
  void add_tile(const Coords& c);
  int find(const int* c) const {
    auto it = index.find(coord_key(c, rank));
    return it == index.end() ? -1 : it->second;
  }
  int64_t tile_size(const int* c) const {
    int64_t n = 1;
    for (int d = 0; d < rank; ++d) n *= dims[d]->ext[c[d]];
    return n;
  }
  int irrep_of(const int* c) const {
    int h = 0;
    for (int d = 0; d < rank; ++d) h ^= dims[d]->irrep[c[d]];
    return h;
  }
  // Resolves virtual tile coords v to a stored tile: returns its id (or -1
  // when the tile is not stored), sets src_dim[d] = the stored tile's
  // dimension that becomes virtual dimension d, and the sign factor.
  int resolve(const int* v, int* src_dim, double* factor) const;
  // All tiles with irrep XOR zero, optionally canonical only.
  static TensorLayout full(const std::vector<std::shared_ptr<BlockDim>>& dims, const std::vector<int>& group,
                           int sign, bool canonical_only);
};

// Parsed index labels of a contraction.
struct ContractionSpec {
  std::vector<int> extA;          // dims of A kept in C (A order)
  std::vector<int> extB;          // dims of B kept in C (B order)
  std::vector<int> contrA;        // contracted dims of A (A order)
  std::vector<int> contrB;        // matching dims of B
  std::vector<int> c_from;        // per C dim: index into extA (>=0) or -(1 + index into extB)
};

int parse_contraction(const std::vector<std::string>& la, const std::vector<std::string>& lb,
                      const std::vector<std::string>& lc, ContractionSpec& out);
std::vector<std::string> split_labels(const char* s);

struct GroupBlock {   // one irrep block of the packed operands
  int h;
  int64_t M, N, K;
  int64_t a_off, b_off, c_off;  // element offsets in the packed buffers
  int engine = 0;               // 0 FP64 (DMMA), 1 split (tcgen05)
  bool swap = false;            // split engine computes C^T = B A^T (C block stored N x M)
};

// Engine and orientation of one packed GEMM from a throughput model of this
// GPU: FP64 DMMA near 0.95 TFLOP/s on 64x64 tiles, the split engine near
// 1 PFLOP/s of bf16 slice products on 128x64 tiles (S(S+1)/2 products).
void choose_engine(GroupBlock& g, bool split_engine, bool split_all, int slices);

enum class Engine { F64 = 0, Split = 1 };



struct ContractionPlan {
  TensorLayout A, B, C;
  ContractionSpec spec;
  std::vector<GroupBlock> groups;
  int64_t a_elems = 0, b_elems = 0, c_elems = 0;
  bool a_needs_zero = false, b_needs_zero = false;
  MoveSet packA, packB, unpackC;
  // F64 engine
  F64Gemm f64;
  // Packed operands.  A constant operand read by FP64 groups keeps its own
  // buffer; every other packed buffer, the split engine's per-run slices and
  // partial sums live in the workspace arena (the plan's own, or one shared
  // by plans that never run at the same time).  A constant operand that is
  // kept only as split slices is packed into scratch that prepare_static
  // alone reads.
  double *d_Abig = nullptr, *d_Bbig = nullptr, *d_Cbig = nullptr;
  double *d_keepA = nullptr, *d_keepB = nullptr;
  unsigned char* d_own_arena = nullptr;
  Engine engine = Engine::F64;
  int slices = 0;
  SplitPlan* split = nullptr;
  double flops = 0.0;        // algorithmic: 2 * sum over nonzero triples m*n*k
  double gemm_flops = 0.0;   // what the packed GEMMs execute
  // Operands whose values never change (integrals) are packed and split once
  // by prepare_static and skipped by execute.  Set before build().
  bool a_static = false, b_static = false;
  bool static_ready = false;
  int n_split_groups = 0, n_f64_groups = 0;
  bool split_all = false;
  int split_width = 0;  // output tile width of every split problem (0 = the model's choice)
  unsigned char* split_arena = nullptr;  // the split plan's per-run region and its capacity
  size_t split_arena_cap = 0;
  // Direct engine (no packing): chosen when the contracted extent per output
  // element is small.  The packed GEMM shapes (groups) are still planned and
  // reported; nothing is packed, split or allocated for them.
  bool direct = false;
  std::vector<DirItem> dir_items;
  std::vector<DirPair> dir_pairs;
  DirItem* d_dir_items = nullptr;
  DirPair* d_dir_pairs = nullptr;
  bool dir_overwrite = false;  // C = alpha A B instead of C += (the items cover all of C)
  // Nonzero: the unpack stores store_scale * A B into C, whatever factor
  // execute is given (set_overwrite on a packed plan).
  double store_scale = 0.0;
  // Makes the plan write C = alpha A B instead of accumulating, when it writes
  // every element of C (the direct items, or the unpack moves: one per C
  // tile); call before build.  false: nothing changed.
  bool set_overwrite(double alpha, int64_t c_elems);

  ~ContractionPlan();
  // Device bytes the plan keeps for itself, the arena bytes one execute
  // needs and the scratch bytes prepare_static needs (host arithmetic only;
  // valid once planned, before build).
  int sizes(size_t* persist, size_t* arena, size_t* static_scratch = nullptr) const;
  // FP64 split-K workspace the FP64 groups will allocate (bytes).
  double f64_workspace_estimate() const;
  // Allocates the persistent buffers, binds the arena (nullptr: the plan's
  // own) and the static scratch (nullptr: after the arena), uploads the
  // launch descriptors.
  int build(unsigned char* arena = nullptr, unsigned char* static_scratch = nullptr);
  int prepare_static(const double* dA, const double* dB, cudaStream_t st);
  // Packs and splits the changing operands without running the GEMM (so a
  // GEMM can be timed alone on current data).
  int stage(const double* dA, const double* dB, cudaStream_t st);
  // C += alpha * A * B.
  int execute(const double* dA, const double* dB, double* dC, double alpha, cudaStream_t st);
  // Autotuner: times the split GEMMs (with their per-run splits) at output
  // tile widths 64, 128 and 256 against the current choice and keeps the
  // fastest.  Call right after prepare_static, while the static scratch
  // still holds this plan's constant operands; timing runs on st.
  int tune_split(cudaStream_t st, int reps = 3);

 private:
  void split_problems(std::vector<SplitProblem>& sp) const;
  bool keeps_a() const { return a_static && n_f64_groups > 0; }
  bool keeps_b() const { return b_static && n_f64_groups > 0; }
};

// Largest average number of products per output element (flops / (2 * C
// elements)) for which a contraction runs on the direct engine.
constexpr double kDirectMaxK = 16.0;

// split_all: every packed GEMM of a split plan uses the split engine (tests),
// and no contraction takes the direct engine.
// defer: plan only (host); the caller sets the static flags and calls build().
// Two contracted indices in which A and B are both antisymmetric (or both
// symmetric): sum_{x,y} A_..xy B_..xy = 2 sum_{X>Y blocks} + sum_{X=Y blocks},
// so the packed GEMMs run over block pairs X >= Y only, the off-diagonal ones
// weighted 2 in one operand's pack (scale_b: B's, else A's) -- close to half
// the contracted extent.  Both indices must have the same blocking.
struct ContractionPair {
  std::string x, y;
  bool scale_b = true;
};

int plan_contraction(const TensorLayout& A, const TensorLayout& B, const TensorLayout& C,
                     const std::vector<std::string>& la, const std::vector<std::string>& lb,
                     const std::vector<std::string>& lc, Engine e, int nslices,
                     std::unique_ptr<ContractionPlan>& out, bool split_all = false, bool defer = false,
                     const ContractionPair* pair = nullptr);

// Tile moves accumulating alpha * permuted A into C: C[c] += alpha * A[a],
// the DLTC Summation (DLTC/task.cc:51-81) over block-sparse layouts.
struct SumPlan {
  TensorLayout A, C;
  MoveSet moves;
  int execute(const double* dA, double* dC, double alpha, cudaStream_t st);
};
int check_moves(const MoveSet& ms, int64_t src_elems, int64_t dst_elems, const char* what);

// Several Summations (DLTC/task.cc:51-81) into one destination, fused:
//   out[c] = (sum_t coef_t * A_t[perm_t(c)]) [* scale[c]]
// in one pass over the destination, each element formed as 0 + c_0 x_0 +
// c_1 x_1 + ... in term order, one fused multiply-add per term -- for
// coefficients +-2^k the result of zeroing C, running the terms as separate
// sums in that order and multiplying by scale.  A term may read a layout that stores canonical
// tiles only (sign factors applied).  out must not alias a source.
struct FusedTermSpec {
  const TensorLayout* A;
  std::vector<std::string> la;
  double coef;
  int slot;  // index of the term's source buffer in execute's src
};

struct FusedSumPlan {
  TensorLayout C;
  int nslots = 0;
  std::vector<FsItem> items;
  std::vector<FsTerm> terms;
  FsItem* d_items = nullptr;
  FsTerm* d_terms = nullptr;
  int upload();
  void release();
  ~FusedSumPlan() { release(); }
  size_t device_bytes() const { return items.size() * sizeof(FsItem) + terms.size() * sizeof(FsTerm); }
  int execute(const double* const* src, const double* scale, double* out, cudaStream_t st) const;
};
// lc: labels of C; each term's la names the same labels in its own order.
// Destination tiles that differ by a swap of their first two or last two
// block coordinates are scheduled together, so that the permuted reads of
// one source tile by its partner tiles hit L2.
int plan_fused_sum(const TensorLayout& C, const std::vector<std::string>& lc, const std::vector<FusedTermSpec>& terms,
                   std::unique_ptr<FusedSumPlan>& out);
int plan_sum(const TensorLayout& A, const TensorLayout& C, const std::vector<std::string>& la,
             const std::vector<std::string>& lc, double coef, std::unique_ptr<SumPlan>& out, bool defer = false);

}  // namespace gbx
