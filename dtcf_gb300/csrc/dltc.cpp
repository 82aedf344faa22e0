// DLTC executor: the Multiplication / Summation expressions of DLTC's
// residual tables over tensors held as Global Arrays hold them -- dense,
// row-major over the tensor's index order, each index of extent O (hole
// name) or V (particle name) and cut into tiles of wbO / wbV
// (DLTC/dltc_tensor.cc:14-40, 169-267).
//
// task_mul (DLTC/task.cc:83-137) loops over C's tiles and, for each, over
// the contracted tiles: every A tile is transposed into at order (external
// names from A, then contracted names), every B tile into bt order
// (contracted, then external names from B), multiplied into a ct-ordered
// tile (externals of A, then of B), which is transposed back into C's order
// and accumulated with the expression's coefficient.  The orders follow the
// Multiplication constructor (DLTC/expr.cc:13-67): names sorted by their
// IndexName value.  On the GPU the same tile loop over a whole range of
// tiles is one permute of A's range into at order, one of B's into bt order,
// one GEMM over the range, and one permute-accumulate of the product into
// C's range: the sums over the contracted tiles become the GEMM's K loop, so
// results equal the tile loop's up to the order of FP64 additions.  A
// permute whose order is already the tensor's (and covers it whole) reads
// the tensor in place; a product already in C's order accumulates into C
// directly.  task_sum (DLTC/task.cc:51-81) is one permute-accumulate.
#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gbx_dltc.h"
#include "common.h"
#include "plan.h"
#include "split.h"

namespace gbx {
namespace {

struct Dims {
  int O, V, wbO, wbV, nocc;
  bool hole(int name) const { return name < nocc; }
  int ext(int name) const { return hole(name) ? O : V; }
  int wb(int name) const { return hole(name) ? wbO : wbV; }
};

int check_dims(const gbx_dltc_dims* d) {
  if (!d) return fail(GBX_EINVAL, "dims is NULL");
  if (d->O < 1 || d->V < 1 || d->wbO < 1 || d->wbV < 1 || d->nocc_names < 0)
    return fail(GBX_EINVAL, "bad DLTC dims (O %d, V %d, wbO %d, wbV %d)", d->O, d->V, d->wbO, d->wbV);
  if (d->O % d->wbO || d->V % d->wbV)
    return fail(GBX_EINVAL, "O (%d) and V (%d) must be multiples of the tile widths (%d, %d)", d->O, d->V, d->wbO,
                d->wbV);
  return GBX_OK;
}

int check_ids(int r, const int* ids, const char* what) {
  if (r < 1 || r > kMaxDims) return fail(GBX_EINVAL, "%s: rank %d outside [1, %d]", what, r, kMaxDims);
  for (int i = 0; i < r; ++i) {
    if (ids[i] < 0 || ids[i] >= GBX_DLTC_MAX_NAMES) return fail(GBX_EINVAL, "%s: index name %d out of range", what, ids[i]);
    for (int j = 0; j < i; ++j)
      if (ids[j] == ids[i]) return fail(GBX_EINVAL, "%s: index name %d repeated", what, ids[i]);
  }
  return GBX_OK;
}

// The orders of a Multiplication (DLTC/expr.cc:13-67): names in A only (m),
// in B only (n), in both (k), each list sorted by name.
struct Orders {
  std::vector<int> m, n, k;
};
Orders derive(int rA, const int* idA, int rB, const int* idB) {
  int tab[GBX_DLTC_MAX_NAMES] = {0};
  for (int i = 0; i < rA; ++i) tab[idA[i]] += 1;
  for (int i = 0; i < rB; ++i) tab[idB[i]] += 2;
  Orders o;
  for (int x = 0; x < GBX_DLTC_MAX_NAMES; ++x) {
    if (tab[x] == 1) o.m.push_back(x);
    if (tab[x] == 2) o.n.push_back(x);
    if (tab[x] == 3) o.k.push_back(x);
  }
  return o;
}

// Element range [lo, hi) of each name (tile ranges * tile width; whole
// extents when lo / hi are NULL).
struct Ranges {
  int64_t lo[GBX_DLTC_MAX_NAMES], len[GBX_DLTC_MAX_NAMES];
};
int make_ranges(const Dims& D, const int* lo, const int* hi, Ranges& R) {
  for (int x = 0; x < GBX_DLTC_MAX_NAMES; ++x) {
    const int ntile = D.ext(x) / D.wb(x);
    int a = lo ? lo[x] : 0, b = hi ? hi[x] : ntile;
    if (a < 0 || b > ntile) return fail(GBX_EINVAL, "tile range [%d, %d) of name %d outside [0, %d)", a, b, x, ntile);
    if (b < a) b = a;
    R.lo[x] = (int64_t)a * D.wb(x);
    R.len[x] = (int64_t)(b - a) * D.wb(x);
  }
  return GBX_OK;
}

// Row-major strides of a dense tensor over its index order.
void dense_strides(const Dims& D, int r, const int* ids, int64_t* str) {
  int64_t s = 1;
  for (int d = r - 1; d >= 0; --d) {
    str[d] = s;
    s *= D.ext(ids[d]);
  }
}

int64_t dense_elems(const Dims& D, int r, const int* ids) {
  int64_t n = 1;
  for (int d = 0; d < r; ++d) n *= D.ext(ids[d]);
  return n;
}

// Host-side bounds check of a move list against its buffers.
int check_list(const std::vector<MoveDesc>& v, int64_t src_elems, int64_t dst_elems, const char* what) {
  MoveSet ms;
  ms.host = v;
  return check_moves(ms, src_elems, dst_elems, what);
}

// Strides of a packed buffer laid out over the names `order` (range lengths).
void packed_strides(const Ranges& R, const std::vector<int>& order, std::map<int, int64_t>& str) {
  int64_t s = 1;
  for (int i = (int)order.size() - 1; i >= 0; --i) {
    str[order[i]] = s;
    s *= R.len[order[i]];
  }
}
int64_t range_elems(const Ranges& R, const std::vector<int>& names) {
  int64_t n = 1;
  for (int x : names) n *= R.len[x];
  return n;
}

bool whole(const Dims& D, const Ranges& R, int r, const int* ids) {
  for (int d = 0; d < r; ++d)
    if (R.lo[ids[d]] != 0 || R.len[ids[d]] != D.ext(ids[d])) return false;
  return true;
}
bool same_order(int r, const int* ids, const std::vector<int>& order) {
  if ((int)order.size() != r) return false;
  for (int d = 0; d < r; ++d)
    if (ids[d] != order[d]) return false;
  return true;
}

// Move between a dense tensor's range (its own index order) and a packed
// buffer over `order`: to_packed = gather into the buffer, else scatter
// (op 1 accumulates scale * packed).
MoveDesc tensor_move(const Dims& D, const Ranges& R, int r, const int* ids, const std::vector<int>& order,
                     bool to_packed, int op, double scale) {
  int64_t ext[kMaxDims], ts[kMaxDims], ps[kMaxDims];
  int64_t dstr[kMaxDims];
  dense_strides(D, r, ids, dstr);
  std::map<int, int64_t> pstr;
  packed_strides(R, order, pstr);
  int64_t off = 0;
  for (int d = 0; d < r; ++d) {
    ext[d] = R.len[ids[d]];
    ts[d] = dstr[d];
    ps[d] = pstr.at(ids[d]);
    off += R.lo[ids[d]] * dstr[d];
  }
  return to_packed ? make_move(r, ext, ts, ps, off, 0, op, scale) : make_move(r, ext, ps, ts, 0, off, op, scale);
}

// Names of C that are not names of the product (a Multiplication whose C
// carries other names is not a valid DLTC expression).
int check_c(int rC, const int* idC, const Orders& o) {
  if (rC != (int)(o.m.size() + o.n.size()))
    return fail(GBX_EINVAL, "C has %d indices, the product %zu", rC, o.m.size() + o.n.size());
  for (int d = 0; d < rC; ++d) {
    bool found = std::find(o.m.begin(), o.m.end(), idC[d]) != o.m.end() ||
                 std::find(o.n.begin(), o.n.end(), idC[d]) != o.n.end();
    if (!found) return fail(GBX_EINVAL, "index name %d of C is not an external index of A or B", idC[d]);
  }
  return GBX_OK;
}

// One prepared expression: its moves, GEMM and workspace needs.
struct Op {
  int kind = GBX_DLTC_MUL;
  double coef = 1.0;
  int c = -1, a = -1, b = -1;  // tensor numbers (programs)
  // Multiplication
  bool pack_a = false, pack_b = false, unpack_c = false;
  std::vector<MoveDesc> mv_a, mv_b, mv_c;  // gathers of A, B; scatter of the product
  int64_t M = 0, N = 0, K = 0;
  int64_t ws_a = 0, ws_b = 0, ws_c = 0;     // workspace elements
  bool b_nk = false;                        // B packed as N x K (split engine), else K x N
  // Summation
  std::vector<MoveDesc> mv_sum;
  double flops = 0.0;
};

int prepare_mul(const Dims& D, const Ranges& R, double coef, int rC, const int* idC, int rA, const int* idA, int rB,
                const int* idB, int mode, Op& op) {
  GBX_TRY(check_ids(rC, idC, "C"));
  GBX_TRY(check_ids(rA, idA, "A"));
  GBX_TRY(check_ids(rB, idB, "B"));
  Orders o = derive(rA, idA, rB, idB);
  GBX_TRY(check_c(rC, idC, o));
  op.kind = GBX_DLTC_MUL;
  op.coef = coef;
  std::vector<int> at = o.m, bt = o.k, ct = o.m;
  at.insert(at.end(), o.k.begin(), o.k.end());
  bt.insert(bt.end(), o.n.begin(), o.n.end());
  ct.insert(ct.end(), o.n.begin(), o.n.end());
  op.b_nk = mode == GBX_MODE_SPLIT;
  if (op.b_nk) {  // the split engine takes B as N x K
    bt = o.n;
    bt.insert(bt.end(), o.k.begin(), o.k.end());
  }
  op.M = range_elems(R, o.m);
  op.N = range_elems(R, o.n);
  op.K = range_elems(R, o.k);
  const int64_t lim = (int64_t)1 << 31;
  if (dense_elems(D, rA, idA) >= lim || dense_elems(D, rB, idB) >= lim || dense_elems(D, rC, idC) >= lim ||
      op.M * op.K >= lim || op.N * op.K >= lim || op.M * op.N >= lim)
    return fail(GBX_EUNSUPPORTED, "DLTC tensor or product of 2^31 elements or more");
  op.flops = 2.0 * (double)op.M * (double)op.N * (double)op.K;
  // A: read in place when at order is A's order over the whole tensor
  op.pack_a = !(same_order(rA, idA, at) && whole(D, R, rA, idA));
  if (op.pack_a) {
    op.mv_a.push_back(tensor_move(D, R, rA, idA, at, true, 0, 1.0));
    op.ws_a = op.M * op.K;
  }
  op.pack_b = !(same_order(rB, idB, bt) && whole(D, R, rB, idB));
  if (op.pack_b) {
    op.mv_b.push_back(tensor_move(D, R, rB, idB, bt, true, 0, 1.0));
    op.ws_b = op.N * op.K;
  }
  // the split engine overwrites its output: its product always goes through ct
  op.unpack_c = mode == GBX_MODE_SPLIT || !(same_order(rC, idC, ct) && whole(D, R, rC, idC));
  if (op.unpack_c) {
    op.mv_c.push_back(tensor_move(D, R, rC, idC, ct, false, 1, coef));
    op.ws_c = op.M * op.N;
  }
  GBX_TRY(check_list(op.mv_a, dense_elems(D, rA, idA), op.ws_a, "DLTC pack of A"));
  GBX_TRY(check_list(op.mv_b, dense_elems(D, rB, idB), op.ws_b, "DLTC pack of B"));
  GBX_TRY(check_list(op.mv_c, op.ws_c, dense_elems(D, rC, idC), "DLTC unpack of C"));
  return GBX_OK;
}

int prepare_sum(const Dims& D, const Ranges& R, double coef, int rC, const int* idC, int rA, const int* idA, Op& op) {
  GBX_TRY(check_ids(rC, idC, "C"));
  GBX_TRY(check_ids(rA, idA, "A"));
  if (rC != rA) return fail(GBX_EINVAL, "Summation: ranks of C (%d) and A (%d) differ", rC, rA);
  for (int d = 0; d < rC; ++d)
    if (std::find(idA, idA + rA, idC[d]) == idA + rA) return fail(GBX_EINVAL, "Summation: name %d of C not in A", idC[d]);
  op.kind = GBX_DLTC_SUM;
  op.coef = coef;
  if (dense_elems(D, rA, idA) >= ((int64_t)1 << 31))
    return fail(GBX_EUNSUPPORTED, "DLTC tensor of 2^31 elements or more");
  // C's range += coef * A's range, through A's order: one move from A to C
  int64_t ext[kMaxDims], sa[kMaxDims], sc[kMaxDims], dA[kMaxDims], dC[kMaxDims];
  dense_strides(D, rA, idA, dA);
  dense_strides(D, rC, idC, dC);
  int64_t offA = 0, offC = 0;
  for (int d = 0; d < rA; ++d) {
    const int x = idA[d];
    ext[d] = R.len[x];
    sa[d] = dA[d];
    const int dc = (int)(std::find(idC, idC + rC, x) - idC);
    sc[d] = dC[dc];
    offA += R.lo[x] * dA[d];
    offC += R.lo[x] * dC[dc];
  }
  op.mv_sum.push_back(make_move(rA, ext, sa, sc, offA, offC, 1, coef));
  op.flops = 0.0;
  return check_list(op.mv_sum, dense_elems(D, rA, idA), dense_elems(D, rC, idC), "DLTC sum");
}

}  // namespace
}  // namespace gbx

using namespace gbx;

// ---- one-shot task calls -------------------------------------------------

namespace {
// Stream-ordered run of a small move list (descriptors uploaded, freed on
// the stream).
int run_moves_once(const std::vector<MoveDesc>& v, const double* src, double* dst, cudaStream_t st) {
  if (v.empty() || v[0].n == 0) return GBX_OK;
  MoveSet ms;
  ms.host = v;
  uint32_t first[2] = {0, (uint32_t)((v[0].n + 2047) / 2048)};
  void *dd = nullptr, *df = nullptr;
  GBX_CUDA(cudaMallocAsync(&dd, sizeof(MoveDesc), st));
  GBX_CUDA(cudaMemcpyAsync(dd, v.data(), sizeof(MoveDesc), cudaMemcpyHostToDevice, st));
  GBX_CUDA(cudaMallocAsync(&df, sizeof(first), st));
  GBX_CUDA(cudaMemcpyAsync(df, first, sizeof(first), cudaMemcpyHostToDevice, st));
  ms.d_desc = (MoveDesc*)dd;
  ms.d_first = (uint32_t*)df;
  ms.ndesc = 1;
  ms.nchunks = first[1];
  int rc = run_moves(ms, src, dst, st);
  cudaFreeAsync(dd, st);
  cudaFreeAsync(df, st);
  ms.d_desc = nullptr;
  ms.d_first = nullptr;
  return rc;
}

// Runs one prepared Multiplication with workspace at ws (at least
// ws_a + ws_b + ws_c elements); gemm (FP64) or split built by the caller.
int run_mul_op(const Op& op, const double* A, const double* B, double* C, double* ws, const MoveSet* ma,
               const MoveSet* mb, const MoveSet* mc, F64Gemm* g, SplitPlan* sp, cudaStream_t st) {
  if (op.M == 0 || op.N == 0) return GBX_OK;
  double* wa = ws;
  double* wb = ws + op.ws_a;
  double* wc = ws + op.ws_a + op.ws_b;
  if (op.pack_a) GBX_TRY(ma ? run_moves(*ma, A, wa, st) : run_moves_once(op.mv_a, A, wa, st));
  if (op.pack_b) GBX_TRY(mb ? run_moves(*mb, B, wb, st) : run_moves_once(op.mv_b, B, wb, st));
  if (sp) GBX_TRY(run_split_plan(sp, true, true, st));
  else GBX_TRY(g->run(st));
  if (op.unpack_c) GBX_TRY(mc ? run_moves(*mc, wc, C, st) : run_moves_once(op.mv_c, wc, C, st));
  return GBX_OK;
}

// GEMM problem of a prepared Multiplication: ct[M x N] (or C itself) =
// at[M x K] * bt[K x N] (bt stored K x N; N x K for the split engine).
GemmProblem gemm_problem(const Op& op, const double* A, const double* B, double* C, double* ws) {
  GemmProblem p;
  std::memset(&p, 0, sizeof(p));
  p.A = op.pack_a ? ws : A;
  p.B = op.pack_b ? ws + op.ws_a : B;
  p.C = op.unpack_c ? ws + op.ws_a + op.ws_b : C;
  p.a_rs = op.K;
  p.a_cs = 1;
  if (op.b_nk) {
    p.b_rs = op.K;
    p.b_cs = 1;
  } else {
    p.b_rs = 1;
    p.b_cs = op.N;
  }
  p.c_rs = op.N;
  p.m = (int)op.M;
  p.n = (int)op.N;
  p.k = (int)op.K;
  p.alpha = op.unpack_c ? 1.0 : op.coef;
  p.accumulate = op.unpack_c ? 0 : 1;
  return p;
}

int make_split(const Op& op, const GemmProblem& p, SplitPlan** out) {
  // C = A * B^T (overwrites): the product goes to the packed ct buffer,
  // which the scatter then accumulates with the coefficient
  if (!op.unpack_c) return fail(GBX_EINVAL, "split DLTC product must go through the ct buffer");
  SplitProblem s;
  s.A = p.A;
  s.B = p.B;
  s.C = p.C;
  s.M = op.M;
  s.N = op.N;
  s.K = op.K;
  return create_split_plan({s}, 0, out);
}
}  // namespace

extern "C" {

int gbx_dltc_mul_orders(int rA, const int* idA, int rB, const int* idB, int* m_ids, int* nm, int* n_ids, int* nn,
                        int* k_ids, int* nk) {
  GBX_TRY(check_ids(rA, idA, "A"));
  GBX_TRY(check_ids(rB, idB, "B"));
  Orders o = derive(rA, idA, rB, idB);
  if (nm) *nm = (int)o.m.size();
  if (nn) *nn = (int)o.n.size();
  if (nk) *nk = (int)o.k.size();
  if (m_ids) std::copy(o.m.begin(), o.m.end(), m_ids);
  if (n_ids) std::copy(o.n.begin(), o.n.end(), n_ids);
  if (k_ids) std::copy(o.k.begin(), o.k.end(), k_ids);
  return GBX_OK;
}

int gbx_dltc_task_mul(double coef, int rC, const int* idC, double* d_C, int rA, const int* idA, const double* d_A,
                      int rB, const int* idB, const double* d_B, const gbx_dltc_dims* dims, const int* lo,
                      const int* hi, int mode, void* stream) {
  GBX_TRY(check_dims(dims));
  if (mode != GBX_MODE_FP64 && mode != GBX_MODE_SPLIT) return fail(GBX_EINVAL, "mode must be FP64 or SPLIT");
  Dims D{dims->O, dims->V, dims->wbO, dims->wbV, dims->nocc_names};
  Ranges R;
  GBX_TRY(make_ranges(D, lo, hi, R));
  Op op;
  GBX_TRY(prepare_mul(D, R, coef, rC, idC, rA, idA, rB, idB, mode, op));
  if (op.M == 0 || op.N == 0) return GBX_OK;
  if (op.M >= (1ll << 31) || op.N >= (1ll << 31) || op.K >= (1ll << 31))
    return fail(GBX_EUNSUPPORTED, "DLTC product too large");
  cudaStream_t st = (cudaStream_t)stream;
  double* ws = nullptr;
  const int64_t wse = op.ws_a + op.ws_b + op.ws_c;
  if (wse) GBX_CUDA(cudaMallocAsync((void**)&ws, sizeof(double) * wse, st));
  GemmProblem p = gemm_problem(op, d_A, d_B, d_C, ws);
  int rc = GBX_OK;
  if (mode == GBX_MODE_SPLIT) {
    SplitPlan* sp = nullptr;
    rc = make_split(op, p, &sp);
    if (rc == GBX_OK) rc = run_mul_op(op, d_A, d_B, d_C, ws, nullptr, nullptr, nullptr, nullptr, sp, st);
    if (sp) {
      // the plan's buffers are freed only after its work has finished
      cudaError_t e = cudaStreamSynchronize(st);
      if (rc == GBX_OK && e != cudaSuccess) rc = cuda_fail(e, "split DLTC product", __FILE__, __LINE__);
      if (rc == GBX_OK) {
        const int err = split_plan_error(sp);
        if (err != 0) rc = fail(GBX_ETIMEOUT, "split GEMM: a bounded device wait ran out (stage %d)", err);
      }
      destroy_split_plan(sp);
    }
  } else {
    F64Gemm g;
    rc = g.build({p}, true, st);
    if (rc == GBX_OK) rc = run_mul_op(op, d_A, d_B, d_C, ws, nullptr, nullptr, nullptr, &g, nullptr, st);
  }
  if (ws) cudaFreeAsync(ws, st);
  return rc;
}

int gbx_dltc_task_sum(double coef, int rC, const int* idC, double* d_C, int rA, const int* idA, const double* d_A,
                      const gbx_dltc_dims* dims, const int* lo, const int* hi, void* stream) {
  GBX_TRY(check_dims(dims));
  Dims D{dims->O, dims->V, dims->wbO, dims->wbV, dims->nocc_names};
  Ranges R;
  GBX_TRY(make_ranges(D, lo, hi, R));
  Op op;
  GBX_TRY(prepare_sum(D, R, coef, rC, idC, rA, idA, op));
  return run_moves_once(op.mv_sum, d_A, d_C, (cudaStream_t)stream);
}

}  // extern "C"

// ---- residual tables and programs ------------------------------------------

namespace {

struct TableTensor {
  std::string name;
  std::vector<int> types;  // 0 HOL, 1 PAR per index
};
struct TableExpr {
  int kind, index, layer;
  int c, a, b;
  std::vector<int> idC, idA, idB;
  double coef;
};
struct Table {
  std::vector<TableTensor> tensors;
  std::vector<TableExpr> exprs;  // execution order: layer by layer
  int nlayers = 0;
};

// The residual tables of DLTC/ccd-t2.cc:45-95 (layers 97-134),
// DLTC/ccsd-t1.cc:40-109 (layers 111-165) and DLTC/ccsd-t2.cc:55-216 (layers
// 218-310), restated line by line in a compact text form:
//   "T name HP.."            a tensor (H hole, P particle per index)
//   "m i C[..] A[..] B[..] coef"   Multiplication m[i]: C += coef * A * B
//   "s i C[..] A[..] coef"         Summation s[i]: C += coef * A
//   "L m0 s1 ..."           one dependency layer, in the reference's exec order
// Index names are h1..h12, p1..p12 (IndexName values 0..23).
const char* const kCcdT2 = R"(
T R_VVOO PPHH
T F_OO HH
T F_VV PP
T T_VVOO PPHH
T V_OOOO HHHH
T V_VVOO PPHH
T V_OOVV HHPP
T V_OVOV HPHP
T V_VVVV PPPP
T I_OO HH
T I_VV PP
T I_OOOO HHHH
T I_OVOV HPHP
s 0 R_VVOO[p3,p4,h1,h2] V_VVOO[p3,p4,h1,h2] 1
s 1 I_OO[h5,h1] F_OO[h5,h1] 1
m 0 I_OO[h5,h1] T_VVOO[p6,p7,h1,h8] V_OOVV[h5,h8,p6,p7] 1
m 1 R_VVOO[p3,p4,h1,h2] T_VVOO[p3,p4,h1,h5] I_OO[h5,h2] 1
s 2 I_VV[p3,p5] F_VV[p3,p5] 1
m 2 I_VV[p3,p5] T_VVOO[p3,p6,h7,h8] V_OOVV[h7,h8,p5,p6] 1
m 3 R_VVOO[p3,p4,h1,h2] T_VVOO[p3,p5,h1,h2] I_VV[p4,p5] 1
s 3 I_OOOO[h7,h9,h1,h2] V_OOOO[h7,h9,h1,h2] 1
m 4 I_OOOO[h7,h9,h1,h2] T_VVOO[p5,p6,h1,h2] V_OOVV[h7,h9,p5,p6] 1
m 5 R_VVOO[p3,p4,h1,h2] T_VVOO[p3,p4,h7,h9] I_OOOO[h7,h9,h1,h2] 1
s 4 I_OVOV[h6,p3,h1,p5] V_OVOV[h6,p3,h1,p5] 1
m 6 I_OVOV[h6,p3,h1,p5] T_VVOO[p3,p7,h1,h8] V_OOVV[h6,h8,p5,p7] 1
m 7 R_VVOO[p3,p4,h1,h2] T_VVOO[p3,p5,h1,h6] I_OVOV[h6,p4,h2,p5] 1
m 8 R_VVOO[p3,p4,h1,h2] T_VVOO[p5,p6,h1,h2] V_VVVV[p3,p4,p5,p6] 1
L s0 s1 m0 s2 m2 s3 m4 s4 m6 m8
L m1 m3 m5 m7
)";

const char* const kCcsdT1 = R"(
T F_OO HH
T F_OV HP
T F_VO PH
T F_VV PP
T I_1 HH
T I_2 HP
T I_3 PP
T I_4 HP
T I_5 HHHP
T R PH
T T_VO PH
T T_VVOO PPHH
T V_OOOV HHHP
T V_OOVV HHPP
T V_OVOV HPHP
T V_OVVV HPPP
s 0 R[p2,h1] F_VO[p2,h1] 1
m 0 R[p2,h1] T_VO[p3,h4] V_OVOV[h4,p2,h1,p3] -1
m 1 R[p2,h1] T_VVOO[p3,p4,h1,h5] V_OVVV[h5,p2,p3,p4] -0.5
s 1 I_1[h7,h1] F_OO[h7,h1] 1
m 2 I_1[h7,h1] T_VO[p4,h5] V_OOOV[h5,h7,h1,p4] -1
m 3 I_1[h7,h1] T_VVOO[p3,p4,h1,h5] V_OOVV[h5,h7,p3,p4] -0.5
s 2 I_2[h7,p3] F_OV[h7,p3] 1
m 4 I_2[h7,p3] T_VO[p5,h6] V_OOVV[h6,h7,p3,p5] -1
m 5 I_1[h7,h1] T_VO[p3,h1] I_2[h7,p3] 1
m 6 R[p2,h1] T_VO[p2,h7] I_1[h7,h1] -1
s 3 I_3[p2,p3] F_VV[p2,p3] 1
m 7 I_3[p2,p3] T_VO[p4,h5] V_OVVV[h5,p2,p3,p4] -1
m 8 R[p2,h1] T_VO[p3,h1] I_3[p2,p3] 1
s 4 I_4[h8,p7] F_OV[h8,p7] 1
m 9 I_4[h8,p7] T_VO[p5,h6] V_OOVV[h6,h8,p5,p7] 1
m 10 R[p2,h1] T_VVOO[p2,p7,h1,h8] I_4[h8,p7] 1
s 5 I_5[h4,h5,h1,p3] V_OOOV[h4,h5,h1,p3] 1
m 11 I_5[h4,h5,h1,p3] T_VO[p6,h1] V_OOVV[h4,h5,p3,p6] -1
m 12 R[p2,h1] T_VVOO[p2,p3,h4,h5] I_5[h4,h5,h1,p3] -0.5
L s0 m0 m1 s1 m2 m3 s2 m4 s3 m7 s4 m9 s5 m11
L m5 m8 m10 m12
L m6
)";

const char* const kCcsdT2 = R"(
T R PPHH
T F_OO HH
T F_OV HP
T F_VV PP
T T_VO PH
T T_VVOO PPHH
T V_OOOO HHHH
T V_OOOV HHHP
T V_OOVV HHPP
T V_OVOO HPHH
T V_OVOV HPHP
T V_OVVV HPPP
T V_VVOO PPHH
T V_VVOV PPHP
T V_VVVV PPPP
T I_1 HPHH
T I_2 HHHH
T I_3 HHHP
T I_4 HPHP
T I_5 HP
T I_6 HHHP
T I_7 PPHP
T I_8 HH
T I_9 HP
T I_10 PP
T I_11 HHHH
T I_12 HHHP
T I_13 HPHP
s 0 R[p3,p4,h1,h2] V_VVOO[p3,p4,h1,h2] 1
m 0 R[p3,p4,h1,h2] T_VVOO[p5,p6,h1,h2] V_VVVV[p3,p4,p5,p6] 0.5
s 1 I_1[h10,p3,h1,h2] V_OVOO[h10,p3,h1,h2] 1
m 1 I_1[h10,p3,h1,h2] T_VVOO[p5,p6,h1,h2] V_OVVV[h10,p3,p5,p6] 0.5
s 2 I_2[h10,h11,h1,h2] V_OOOO[h10,h11,h1,h2] -1
m 2 I_2[h10,h11,h1,h2] T_VVOO[p7,p8,h1,h2] V_OOVV[h10,h11,p7,p8] -0.5
s 3 I_3[h10,h11,h1,p5] V_OOOV[h10,h11,h1,p5] 1
m 3 I_3[h10,h11,h1,p5] T_VO[p6,h1] V_OOVV[h10,h11,p5,p6] -0.5
m 4 I_2[h10,h11,h1,h2] T_VO[p5,h1] I_3[h10,h11,h2,p5] 1
m 5 I_1[h10,p3,h1,h2] T_VO[p3,h11] I_2[h10,h11,h1,h2] 0.5
s 4 I_4[h10,p3,h1,p5] V_OVOV[h10,p3,h1,p5] 1
m 6 I_4[h10,p3,h1,p5] T_VO[p6,h1] V_OVVV[h10,p3,p5,p6] -0.5
m 7 I_1[h10,p3,h1,h2] T_VO[p5,h1] I_4[h10,p3,h2,p5] -1
s 5 I_5[h10,p5] F_OV[h10,p5] 1
m 8 I_5[h10,p5] T_VO[p6,h7] V_OOVV[h7,h10,p5,p6] -1
m 9 I_1[h10,p3,h1,h2] T_VVOO[p3,p5,h1,h2] I_5[h10,p5] -1
s 6 I_6[h7,h10,h1,p9] V_OOOV[h7,h10,h1,p9] 1
m 10 I_6[h7,h10,h1,p9] T_VO[p5,h1] V_OOVV[h7,h10,p5,p9] 1
m 11 I_1[h10,p3,h1,h2] T_VVOO[p3,p9,h1,h7] I_6[h7,h10,h2,p9] 1
m 12 R[p3,p4,h1,h2] T_VO[p3,h10] I_1[h10,p4,h1,h2] -1
s 7 I_7[p3,p4,h1,p5] V_VVOV[p3,p4,h1,p5] 1
m 13 I_7[p3,p4,h1,p5] T_VO[p6,h1] V_VVVV[p3,p4,p5,p6] -0.5
m 14 R[p3,p4,h1,h2] T_VO[p5,h1] I_7[p3,p4,h2,p5] -1
s 8 I_8[h9,h1] F_OO[h9,h1] 1
m 15 I_8[h9,h1] T_VO[p6,h7] V_OOOV[h7,h9,h1,p6] -1
m 16 I_8[h9,h1] T_VVOO[p6,p7,h1,h8] V_OOVV[h8,h9,p6,p7] -0.5
s 9 I_9[h9,p8] F_OV[h9,p8] 1
m 17 I_9[h9,p8] T_VO[p6,h7] V_OOVV[h7,h9,p6,p8] 1
m 18 I_8[h9,h1] T_VO[p8,h1] I_9[h9,p8] 1
m 19 R[p3,p4,h1,h2] T_VVOO[p3,p4,h1,h9] I_8[h9,h2] -1
s 10 I_10[p3,p5] F_VV[p3,p5] 1
m 20 I_10[p3,p5] T_VO[p6,h7] V_OVVV[h7,p3,p5,p6] -1
m 21 I_10[p3,p5] T_VVOO[p3,p6,h7,h8] V_OOVV[h7,h8,p5,p6] -0.5
m 22 R[p3,p4,h1,h2] T_VVOO[p3,p5,h1,h2] I_10[p4,p5] 1
s 11 I_11[h9,h11,h1,h2] V_OOOO[h9,h11,h1,h2] -1
m 23 I_11[h9,h11,h1,h2] T_VVOO[p5,p6,h1,h2] V_OOVV[h9,h11,p5,p6] -0.5
s 12 I_12[h9,h11,h1,p8] V_OOOV[h9,h11,h1,p8] 1
m 24 I_12[h9,h11,h1,p8] T_VO[p6,h1] V_OOVV[h9,h11,p6,p8] 0.5
m 25 I_11[h9,h11,h1,h2] T_VO[p8,h1] I_12[h9,h11,h2,p8] 1
m 26 R[p3,p4,h1,h2] T_VVOO[p3,p4,h9,h11] I_11[h9,h11,h1,h2] -0.5
s 13 I_13[h6,p3,h1,p5] V_OVOV[h6,p3,h1,p5] 1
m 27 I_13[h6,p3,h1,p5] T_VO[p7,h1] V_OVVV[h6,p3,p5,p7] -1
m 28 I_13[h6,p3,h1,p5] T_VVOO[p3,p7,h1,h8] V_OOVV[h6,h8,p5,p7] -0.5
m 29 R[p3,p4,h1,h2] T_VVOO[p3,p5,h1,h6] I_13[h6,p4,h2,p5] -1
L s0 m0 s1 m1 s2 m2 s3 m3 s4 m6 s5 m8 s6 m10 s7 m13 s8 m15 m16 s9 m17 s10 m20 m21 s11 m23 s12 m24 s13 m27 m28
L m4 m7 m9 m11 m14 m18 m22 m25 m29
L m5 m19 m26
L m12
)";

}  // namespace

namespace {

int parse_names(const std::string& s, std::vector<int>& ids) {
  // "h1,p3,..." -> IndexName values (h1..h12 = 0..11, p1..p12 = 12..23)
  ids.clear();
  std::stringstream ss(s);
  std::string tok;
  while (std::getline(ss, tok, ',')) {
    if (tok.size() < 2 || (tok[0] != 'h' && tok[0] != 'p')) return -1;
    const int k = std::atoi(tok.c_str() + 1);
    if (k < 1 || k > 12) return -1;
    ids.push_back((tok[0] == 'h' ? 0 : 12) + k - 1);
  }
  return 0;
}

// "Name[h1,p2]" -> tensor number, index names
int parse_ref(const Table& t, const std::string& tok, int* tensor, std::vector<int>& ids) {
  const size_t b = tok.find('['), e = tok.find(']');
  if (b == std::string::npos || e == std::string::npos) return -1;
  const std::string name = tok.substr(0, b);
  *tensor = -1;
  for (size_t i = 0; i < t.tensors.size(); ++i)
    if (t.tensors[i].name == name) *tensor = (int)i;
  if (*tensor < 0) return -1;
  if (parse_names(tok.substr(b + 1, e - b - 1), ids) != 0) return -1;
  return ids.size() == t.tensors[*tensor].types.size() ? 0 : -1;
}

int parse_table(const char* text, Table& t) {
  std::stringstream in(text);
  std::string line;
  std::vector<TableExpr> defs;
  std::vector<std::vector<std::string>> layers;
  while (std::getline(in, line)) {
    std::stringstream ls(line);
    std::string kw;
    if (!(ls >> kw)) continue;
    if (kw == "T") {
      TableTensor tt;
      std::string ty;
      ls >> tt.name >> ty;
      for (char c : ty) tt.types.push_back(c == 'H' ? 0 : 1);
      t.tensors.push_back(tt);
    } else if (kw == "m" || kw == "s") {
      TableExpr x;
      x.kind = kw == "m" ? GBX_DLTC_MUL : GBX_DLTC_SUM;
      std::string c, a, b;
      ls >> x.index >> c >> a;
      if (x.kind == GBX_DLTC_MUL) ls >> b;
      ls >> x.coef;
      if (parse_ref(t, c, &x.c, x.idC) || parse_ref(t, a, &x.a, x.idA)) return -1;
      x.b = -1;
      if (x.kind == GBX_DLTC_MUL && parse_ref(t, b, &x.b, x.idB)) return -1;
      defs.push_back(x);
    } else if (kw == "L") {
      std::vector<std::string> l;
      std::string e;
      while (ls >> e) l.push_back(e);
      layers.push_back(l);
    } else {
      return -1;
    }
  }
  for (size_t li = 0; li < layers.size(); ++li)
    for (const std::string& e : layers[li]) {
      const int kind = e[0] == 'm' ? GBX_DLTC_MUL : GBX_DLTC_SUM;
      const int idx = std::atoi(e.c_str() + 1);
      bool found = false;
      for (const TableExpr& d : defs)
        if (d.kind == kind && d.index == idx) {
          TableExpr x = d;
          x.layer = (int)li;
          t.exprs.push_back(x);
          found = true;
        }
      if (!found) return -1;
    }
  t.nlayers = (int)layers.size();
  return t.exprs.size() == defs.size() ? 0 : -1;
}

int get_table(int which, Table& t) {
  const char* text = which == GBX_DLTC_CCD_T2 ? kCcdT2 : which == GBX_DLTC_CCSD_T1 ? kCcsdT1
                     : which == GBX_DLTC_CCSD_T2 ? kCcsdT2 : nullptr;
  if (!text) return fail(GBX_EINVAL, "unknown DLTC table %d", which);
  if (parse_table(text, t) != 0) return fail(GBX_EINVAL, "DLTC table %d does not parse", which);
  return GBX_OK;
}

}  // namespace

struct gbx_dltc_program {
  Table table;
  Dims D;
  int mode = GBX_MODE_FP64;
  std::vector<double*> data;
  std::vector<int64_t> elems;
  std::vector<Op> ops;
  std::vector<std::unique_ptr<MoveSet>> ma, mb, mc, msum;
  std::vector<std::unique_ptr<F64Gemm>> gemm;
  std::vector<SplitPlan*> split;
  double* ws = nullptr;
  double flops = 0.0;
  ~gbx_dltc_program() {
    for (SplitPlan* p : split) destroy_split_plan(p);
    gemm.clear();
    dev_free(ws);
    for (double* d : data) dev_free(d);
  }
};

namespace {
int upload_moves(const std::vector<MoveDesc>& v, std::unique_ptr<MoveSet>& out) {
  out.reset(new MoveSet());
  out->host = v;
  return out->upload();
}
}  // namespace

extern "C" {

int gbx_dltc_table(int which, gbx_dltc_expr* exprs, int* nexpr, int* types, int* ntensors, char* names,
                   int name_len) {
  Table t;
  GBX_TRY(get_table(which, t));
  if (nexpr) {
    const int cap = *nexpr;
    *nexpr = (int)t.exprs.size();
    if (exprs) {
      if (cap < (int)t.exprs.size()) return fail(GBX_EINVAL, "expression capacity %d < %zu", cap, t.exprs.size());
      for (size_t i = 0; i < t.exprs.size(); ++i) {
        const TableExpr& x = t.exprs[i];
        gbx_dltc_expr& e = exprs[i];
        std::memset(&e, 0, sizeof(e));
        e.kind = x.kind;
        e.index = x.index;
        e.layer = x.layer;
        e.c = x.c;
        e.a = x.a;
        e.b = x.b;
        e.rc = (int)x.idC.size();
        e.ra = (int)x.idA.size();
        e.rb = (int)x.idB.size();
        std::copy(x.idC.begin(), x.idC.end(), e.idc);
        std::copy(x.idA.begin(), x.idA.end(), e.ida);
        std::copy(x.idB.begin(), x.idB.end(), e.idb);
        e.coef = x.coef;
      }
    }
  }
  if (ntensors) {
    const int cap = *ntensors;
    *ntensors = (int)t.tensors.size();
    if ((types || names) && cap < (int)t.tensors.size())
      return fail(GBX_EINVAL, "tensor capacity %d < %zu", cap, t.tensors.size());
    for (size_t i = 0; i < t.tensors.size() && (types || names); ++i) {
      if (types) {
        types[5 * i] = (int)t.tensors[i].types.size();
        for (int d = 0; d < 4; ++d)
          types[5 * i + 1 + d] = d < (int)t.tensors[i].types.size() ? t.tensors[i].types[d] : -1;
      }
      if (names && name_len > 0) {
        std::strncpy(names + i * name_len, t.tensors[i].name.c_str(), name_len - 1);
        names[i * name_len + name_len - 1] = 0;
      }
    }
  }
  return GBX_OK;
}

int gbx_dltc_program_create(int which, const gbx_dltc_dims* dims, int mode, gbx_dltc_program** out) {
  if (!out) return fail(GBX_EINVAL, "out is NULL");
  *out = nullptr;
  GBX_TRY(check_dims(dims));
  if (mode != GBX_MODE_FP64 && mode != GBX_MODE_SPLIT) return fail(GBX_EINVAL, "mode must be FP64 or SPLIT");
  std::unique_ptr<gbx_dltc_program> p(new gbx_dltc_program());
  GBX_TRY(get_table(which, p->table));
  p->D = Dims{dims->O, dims->V, dims->wbO, dims->wbV, dims->nocc_names};
  p->mode = mode;
  const Dims& D = p->D;
  // tensors: dense over their index order, zeroed as GA_Zero leaves them
  for (const TableTensor& t : p->table.tensors) {
    int64_t n = 1;
    for (int ty : t.types) n *= ty == 0 ? D.O : D.V;
    double* d = nullptr;
    GBX_TRY(dev_alloc((void**)&d, sizeof(double) * std::max<int64_t>(n, 1)));
    p->data.push_back(d);
    p->elems.push_back(n);
    GBX_CUDA(cudaMemset(d, 0, sizeof(double) * std::max<int64_t>(n, 1)));
  }
  Ranges R;
  GBX_TRY(make_ranges(D, nullptr, nullptr, R));
  int64_t ws = 0;
  for (const TableExpr& x : p->table.exprs) {
    // index names must fit the tensors' index types
    auto fits = [&](int t, const std::vector<int>& ids) {
      for (size_t d = 0; d < ids.size(); ++d)
        if ((D.hole(ids[d]) ? 0 : 1) != p->table.tensors[t].types[d]) return false;
      return true;
    };
    if (!fits(x.c, x.idC) || !fits(x.a, x.idA) || (x.b >= 0 && !fits(x.b, x.idB)))
      return fail(GBX_EINVAL, "expression %c%d: index names do not fit the tensors (nocc_names %d)",
                  x.kind == GBX_DLTC_MUL ? 'm' : 's', x.index, D.nocc);
    Op op;
    if (x.kind == GBX_DLTC_MUL)
      GBX_TRY(prepare_mul(D, R, x.coef, (int)x.idC.size(), x.idC.data(), (int)x.idA.size(), x.idA.data(),
                          (int)x.idB.size(), x.idB.data(), mode, op));
    else
      GBX_TRY(prepare_sum(D, R, x.coef, (int)x.idC.size(), x.idC.data(), (int)x.idA.size(), x.idA.data(), op));
    op.c = x.c;
    op.a = x.a;
    op.b = x.b;
    ws = std::max(ws, op.ws_a + op.ws_b + op.ws_c);
    p->flops += op.flops;
    p->ops.push_back(op);
  }
  GBX_TRY(dev_alloc((void**)&p->ws, sizeof(double) * std::max<int64_t>(ws, 1)));
  for (Op& op : p->ops) {
    p->ma.emplace_back();
    p->mb.emplace_back();
    p->mc.emplace_back();
    p->msum.emplace_back();
    p->gemm.emplace_back();
    p->split.push_back(nullptr);
    if (op.kind == GBX_DLTC_SUM) {
      GBX_TRY(upload_moves(op.mv_sum, p->msum.back()));
      continue;
    }
    if (op.M == 0 || op.N == 0) continue;
    if (op.pack_a) GBX_TRY(upload_moves(op.mv_a, p->ma.back()));
    if (op.pack_b) GBX_TRY(upload_moves(op.mv_b, p->mb.back()));
    if (op.unpack_c) GBX_TRY(upload_moves(op.mv_c, p->mc.back()));
    GemmProblem g = gemm_problem(op, p->data[op.a], p->data[op.b], p->data[op.c], p->ws);
    if (mode == GBX_MODE_SPLIT) {
      GBX_TRY(make_split(op, g, &p->split.back()));
    } else {
      p->gemm.back().reset(new F64Gemm());
      GBX_TRY(p->gemm.back()->build({g}));
    }
  }
  *out = p.release();
  return GBX_OK;
}

int gbx_dltc_program_tensor(gbx_dltc_program* p, int tensor, double** d_data, int64_t* elems) {
  if (!p || tensor < 0 || tensor >= (int)p->data.size()) return fail(GBX_EINVAL, "bad tensor %d", tensor);
  if (d_data) *d_data = p->data[tensor];
  if (elems) *elems = p->elems[tensor];
  return GBX_OK;
}

int gbx_dltc_program_run(gbx_dltc_program* p, int first, int count, void* stream) {
  if (!p) return fail(GBX_EINVAL, "program is NULL");
  const int n = (int)p->ops.size();
  if (count < 0) count = n - first;
  if (first < 0 || first + count > n) return fail(GBX_EINVAL, "expressions [%d, %d) outside [0, %d)", first,
                                                  first + count, n);
  cudaStream_t st = (cudaStream_t)stream;
  for (int i = first; i < first + count; ++i) {
    const Op& op = p->ops[i];
    if (op.kind == GBX_DLTC_SUM) {
      GBX_TRY(run_moves(*p->msum[i], p->data[op.a], p->data[op.c], st));
      continue;
    }
    GBX_TRY(run_mul_op(op, p->data[op.a], p->data[op.b], p->data[op.c], p->ws, p->ma[i].get(), p->mb[i].get(),
                       p->mc[i].get(), p->gemm[i].get(), p->split[i], st));
  }
  return GBX_OK;
}

int gbx_dltc_program_check(gbx_dltc_program* p) {
  if (!p) return fail(GBX_EINVAL, "program is NULL");
  for (SplitPlan* sp : p->split) {
    const int err = split_plan_error(sp);
    if (err != 0) return fail(GBX_ETIMEOUT, "split GEMM: a bounded device wait ran out (stage %d)", err);
  }
  return GBX_OK;
}

double gbx_dltc_program_flops(const gbx_dltc_program* p) { return p ? p->flops : 0.0; }

int gbx_dltc_program_destroy(gbx_dltc_program* p) {
  delete p;
  return GBX_OK;
}

}  // extern "C"
