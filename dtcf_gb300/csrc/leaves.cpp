// Error state, device allocation helpers, and the leaf entry points of the C
// ABI: block permutes (RRR and DLTC), big-matrix pack / unpack, and the FP64
// local contraction.  Each leaf builds its tile moves or GEMM problem on the
// host and runs them with stream-ordered temporaries, so a call never
// synchronises the host with the device.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <unordered_map>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "common.h"

namespace gbx {

static thread_local std::string t_err;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_err = buf;
}

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  set_error("CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what, file, line);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return GBX_ENOMEM;
  }
  return GBX_ECUDA;
}

// Every library allocation is recorded with its size and the account that
// was current on the allocating thread, so a job can report the device bytes
// it holds.
namespace {
struct AllocRec {
  size_t bytes;
  std::atomic<int64_t>* account;
  cudaStream_t stream;  // stream-ordered allocation: freed on this stream
  bool ordered;
};
std::mutex g_alloc_mu;
std::unordered_map<void*, AllocRec> g_allocs;
thread_local std::atomic<int64_t>* g_account = nullptr;
thread_local bool g_ordered = false;
thread_local cudaStream_t g_order_stream = nullptr;
}  // namespace

AllocAccount::AllocAccount(std::atomic<int64_t>* acc) : prev(g_account) { g_account = acc; }
AllocAccount::~AllocAccount() { g_account = prev; }

StreamOrderedAlloc::StreamOrderedAlloc(cudaStream_t st) : prev_on(g_ordered), prev(g_order_stream) {
  g_ordered = true;
  g_order_stream = st;
}
StreamOrderedAlloc::~StreamOrderedAlloc() {
  g_ordered = prev_on;
  g_order_stream = prev;
}

int dev_alloc(void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) return GBX_OK;
  cudaError_t e;
  if (g_ordered) {
    // the allocation completes before the memory is handed out, so any
    // stream (and host-synchronous copies) may use it at once
    e = cudaMallocAsync(p, bytes, g_order_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g_order_stream);
  } else {
    e = cudaMalloc(p, bytes);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(e == cudaErrorMemoryAllocation ? GBX_ENOMEM : GBX_ECUDA, "device allocation of %zu bytes failed: %s",
                bytes, cudaGetErrorString(e));
  }
  std::lock_guard<std::mutex> lk(g_alloc_mu);
  g_allocs[*p] = AllocRec{bytes, g_account, g_order_stream, g_ordered};
  if (g_account) g_account->fetch_add((int64_t)bytes);
  return GBX_OK;
}

void dev_free(void* p) {
  if (!p) return;
  bool ordered = false;
  cudaStream_t st = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_alloc_mu);
    auto it = g_allocs.find(p);
    if (it != g_allocs.end()) {
      if (it->second.account) it->second.account->fetch_sub((int64_t)it->second.bytes);
      ordered = it->second.ordered;
      st = it->second.stream;
      g_allocs.erase(it);
    }
  }
  if (ordered) cudaFreeAsync(p, st);
  else cudaFree(p);
}

// Stream-ordered temporary upload of host data (freed on the same stream).
static int upload_async(const void* host, size_t bytes, cudaStream_t st, void** dptr) {
  GBX_CUDA(cudaMallocAsync(dptr, bytes, st));
  GBX_CUDA(cudaMemcpyAsync(*dptr, host, bytes, cudaMemcpyHostToDevice, st));
  return GBX_OK;
}

// Run a small set of moves with stream-ordered descriptor storage.
static int run_moves_async(const std::vector<MoveDesc>& moves, const double* src, double* dst, cudaStream_t st) {
  if (moves.empty()) return GBX_OK;
  MoveSet ms;
  ms.host = moves;
  // build the chunk schedule like MoveSet::upload, but stream-ordered
  std::vector<uint32_t> first(moves.size() + 1);
  uint64_t c = 0;
  for (size_t i = 0; i < moves.size(); ++i) {
    first[i] = (uint32_t)c;
    c += (moves[i].n + 2047) / 2048;
  }
  first[moves.size()] = (uint32_t)c;
  if (c == 0) return GBX_OK;
  void *dd = nullptr, *df = nullptr;
  GBX_TRY(upload_async(moves.data(), sizeof(MoveDesc) * moves.size(), st, &dd));
  GBX_TRY(upload_async(first.data(), sizeof(uint32_t) * first.size(), st, &df));
  ms.d_desc = (MoveDesc*)dd;
  ms.d_first = (uint32_t*)df;
  ms.ndesc = (int)moves.size();
  ms.nchunks = (uint32_t)c;
  int rc = run_moves(ms, src, dst, st);
  cudaFreeAsync(dd, st);
  cudaFreeAsync(df, st);
  ms.d_desc = nullptr;
  ms.d_first = nullptr;
  return rc;
}

// Move describing "source dim i lands at output position perm[i]" for one
// dense row-major block.
static MoveDesc permute_move(int dims, const int* perm, const int* widths, int64_t src, int64_t dst) {
  int64_t ext[kMaxDims], is[kMaxDims], os[kMaxDims], ow[kMaxDims], sstr[kMaxDims], dstr[kMaxDims];
  for (int i = 0; i < dims; ++i) {
    ext[i] = widths[i];
    ow[perm[i]] = widths[i];
  }
  is[dims - 1] = 1;
  os[dims - 1] = 1;
  for (int d = dims - 2; d >= 0; --d) {
    is[d] = is[d + 1] * ext[d + 1];
    os[d] = os[d + 1] * ow[d + 1];
  }
  for (int i = 0; i < dims; ++i) {
    sstr[i] = is[i];
    dstr[i] = os[perm[i]];
  }
  return make_move(dims, ext, sstr, dstr, src, dst, 0, 1.0);
}

static int check_perm(int dims, const int* perm) {
  if (dims < 1 || dims > kMaxDims) return fail(GBX_EINVAL, "dims %d outside [1, %d]", dims, kMaxDims);
  bool seen[kMaxDims] = {false};
  for (int i = 0; i < dims; ++i) {
    if (perm[i] < 0 || perm[i] >= dims || seen[perm[i]]) return fail(GBX_EINVAL, "perm is not a permutation");
    seen[perm[i]] = true;
  }
  return GBX_OK;
}

static int check_widths(int dims, const int* widths) {
  int64_t n = 1;
  for (int i = 0; i < dims; ++i) {
    if (widths[i] < 0) return fail(GBX_EINVAL, "negative width");
    n *= widths[i];
  }
  if (n >= (1ll << 31)) return fail(GBX_EUNSUPPORTED, "block of %lld elements exceeds 2^31", (long long)n);
  return GBX_OK;
}

// Placement of tiles in a big matrix, as create_big_matrix's
// std::map<row rank, std::map<col rank, tile>> orders them
// (transpose_helper.cc:40-111); first insertion wins on duplicates.
static int big_matrix_order(int dims, const int* vgrid, const int* p_map, int num_tiles, const int* paddr,
                            int num_row_dim, std::vector<int>& order, int& nrows, int& ncols) {
  int grid_T[kMaxDims];
  for (int d = 0; d < dims; ++d) grid_T[p_map[d]] = vgrid[d];
  auto rank_of = [&](const int* a, int lo, int hi) {
    int64_t x = 1, r = 0;
    for (int i = dims - 1; i >= 0; --i) {
      if (i >= lo && i < hi) r += (int64_t)a[i] * x;
      x *= grid_T[i];
    }
    return r;
  };
  std::vector<std::tuple<int64_t, int64_t, int>> pl(num_tiles);
  for (int t = 0; t < num_tiles; ++t) {
    const int* a = paddr + (int64_t)t * dims;
    pl[t] = std::make_tuple(rank_of(a, 0, num_row_dim), rank_of(a, num_row_dim, dims), t);
  }
  std::sort(pl.begin(), pl.end());
  order.clear();
  nrows = 0;
  ncols = -1;
  int cur = 0;
  for (int i = 0; i < num_tiles; ++i) {
    if (i > 0 && std::get<0>(pl[i]) == std::get<0>(pl[i - 1]) && std::get<1>(pl[i]) == std::get<1>(pl[i - 1]))
      continue;
    order.push_back(i);
  }
  // count rows / columns over the deduplicated placement
  std::vector<int> tiles;
  tiles.reserve(order.size());
  int64_t prev_row = -1;
  for (size_t j = 0; j < order.size(); ++j) {
    const auto& p = pl[order[j]];
    if (j > 0 && std::get<0>(p) != prev_row) {
      if (ncols >= 0 && cur != ncols) return fail(GBX_EINVAL, "tile pattern is not rectangular");
      ncols = cur;
      cur = 0;
      ++nrows;
    }
    prev_row = std::get<0>(p);
    tiles.push_back(std::get<2>(p));
    ++cur;
  }
  if (!order.empty()) {
    if (ncols >= 0 && cur != ncols) return fail(GBX_EINVAL, "tile pattern is not rectangular");
    ncols = cur;
    ++nrows;
  } else {
    ncols = 0;
  }
  order.swap(tiles);
  return GBX_OK;
}

// loc (optional): the tile data of placement entry t sits at tile slot
// loc[t] instead of t (create_big_matrix_nl's address_to_location).
static int big_matrix_moves(int dims, const int* vgrid, const int* p_map, int num_tiles, const int* paddr,
                            int rpb, int cpb, int nrd, bool to_big, std::vector<MoveDesc>& moves, int* nrows_out,
                            int* ncols_out, const std::vector<int>* loc = nullptr) {
  if (dims < 1 || dims > kMaxDims || num_tiles < 0 || rpb < 0 || cpb < 0 || nrd < 0 || nrd > dims)
    return fail(GBX_EINVAL, "bad big-matrix arguments");
  GBX_TRY(check_perm(dims, p_map));
  std::vector<int> order;
  int nrows = 0, ncols = 0;
  GBX_TRY(big_matrix_order(dims, vgrid, p_map, num_tiles, paddr, nrd, order, nrows, ncols));
  const int64_t bs = (int64_t)rpb * cpb;
  const int64_t total_col = (int64_t)ncols * cpb;
  for (int r = 0; r < nrows; ++r)
    for (int c = 0; c < ncols; ++c) {
      int t = order[(size_t)r * ncols + c];
      int64_t tile_off = (int64_t)(loc ? (*loc)[t] : t) * bs;
      int64_t big_off = (int64_t)r * rpb * total_col + (int64_t)c * cpb;
      int64_t ext[2] = {rpb, cpb};
      int64_t ts[2] = {cpb, 1}, bstr[2] = {total_col, 1};
      if (to_big)
        moves.push_back(make_move(2, ext, ts, bstr, tile_off, big_off, 0, 1.0));
      else
        moves.push_back(make_move(2, ext, bstr, ts, big_off, tile_off, 0, 1.0));
    }
  if (nrows_out) *nrows_out = nrows;
  if (ncols_out) *ncols_out = ncols;
  return GBX_OK;
}

}  // namespace gbx

using namespace gbx;

extern "C" {

const char* gbx_last_error(void) { return t_err.c_str(); }

const char* gbx_version(void) { return "dtcf_gb300 0.1 (sm_103a)"; }

int gbx_transpose(const double* d_in, double* d_out, const int* perm, int dims, const int* widths, void* stream) {
  GBX_TRY(check_perm(dims, perm));
  GBX_TRY(check_widths(dims, widths));
  std::vector<MoveDesc> mv{permute_move(dims, perm, widths, 0, 0)};
  return run_moves_async(mv, d_in, d_out, (cudaStream_t)stream);
}

int gbx_transpose_blocks(const double* d_in, double* d_out, int num_blocks, const int* perms, int dims,
                         const int* widths, void* stream) {
  if (num_blocks < 0) return fail(GBX_EINVAL, "num_blocks < 0");
  GBX_TRY(check_widths(dims, widths));
  int64_t bs = 1;
  for (int i = 0; i < dims; ++i) bs *= widths[i];
  std::vector<MoveDesc> mv;
  mv.reserve(num_blocks);
  for (int b = 0; b < num_blocks; ++b) {
    GBX_TRY(check_perm(dims, perms + (int64_t)b * dims));
    mv.push_back(permute_move(dims, perms + (int64_t)b * dims, widths, b * bs, b * bs));
  }
  return run_moves_async(mv, d_in, d_out, (cudaStream_t)stream);
}

int gbx_dltc_transpose(const double* d_x, const int* ids_x, double* d_y, const int* ids_y, int dim,
                       const int* wb_x, void* stream) {
  if (dim < 1 || dim > kMaxDims) return fail(GBX_EINVAL, "dim %d outside [1, %d]", dim, kMaxDims);
  int perm[kMaxDims];
  for (int j = 0; j < dim; ++j) {
    perm[j] = -1;
    for (int i = 0; i < dim; ++i)
      if (ids_y[i] == ids_x[j]) perm[j] = i;
    if (perm[j] < 0) return fail(GBX_EINVAL, "index name %d of x missing from y", ids_x[j]);
  }
  return gbx_transpose(d_x, d_y, perm, dim, wb_x, stream);
}

int gbx_local_contraction(int n_a, int n_b, int n_k, const double* d_A, const double* d_B, double* d_C, int at,
                          int bt, double alpha, void* stream) {
  if (n_a < 0 || n_b < 0 || n_k < 0) return fail(GBX_EINVAL, "negative extent");
  if (n_a == 0 || n_b == 0) return GBX_OK;
  GemmProblem p;
  std::memset(&p, 0, sizeof(p));
  p.A = d_A;
  p.B = d_B;
  p.C = d_C;
  p.a_rs = at ? 1 : n_k;
  p.a_cs = at ? n_a : 1;
  p.b_rs = bt ? n_k : 1;
  p.b_cs = bt ? 1 : n_b;
  p.c_rs = n_b;
  p.m = n_a;
  p.n = n_b;
  p.k = n_k;
  p.alpha = alpha;
  p.accumulate = 1;
  cudaStream_t st = (cudaStream_t)stream;
  F64Gemm g;
  GBX_TRY(g.build({p}, true, st));
  return g.run(st);
}

int gbx_dltc_compute(double* d_c, const double* d_a, const double* d_b, int m, int n, int k, void* stream) {
  return gbx_local_contraction(m, n, k, d_a, d_b, d_c, 0, 0, 1.0, stream);
}

int gbx_create_big_matrix(int dims, const int* vgrid, const int* p_map, int num_tiles, const double* d_tiles,
                          const int* permuted_address, int row_per_block, int col_per_block, int num_row_dim,
                          double* d_big, int* nrows, int* ncols, void* stream) {
  std::vector<MoveDesc> mv;
  GBX_TRY(big_matrix_moves(dims, vgrid, p_map, num_tiles, permuted_address, row_per_block, col_per_block,
                           num_row_dim, true, mv, nrows, ncols));
  return run_moves_async(mv, d_tiles, d_big, (cudaStream_t)stream);
}

int gbx_create_big_matrix_nl(int dims, const int* vgrid, const int* p_map, int num_tiles, const double* d_tiles,
                             int num_slots, const int* permuted_address, int row_per_block, int col_per_block,
                             int num_row_dim,
                             const int* loc_ranks, const int* loc_slots, int num_locations, double* d_big,
                             int* nrows, int* ncols, void* stream) {
  if (dims < 1 || dims > kMaxDims || num_tiles < 0 || num_locations < 0 || (num_locations && (!loc_ranks || !loc_slots)))
    return fail(GBX_EINVAL, "bad big-matrix arguments");
  GBX_TRY(check_perm(dims, p_map));
  // address_to_location: rank of a tile's permuted address in the permuted
  // grid -> its slot in d_tiles (every placed tile must have one; the
  // reference asserts, transpose_helper.cc:250-251)
  int grid_T[kMaxDims];
  for (int d = 0; d < dims; ++d) grid_T[p_map[d]] = vgrid[d];
  std::map<int64_t, int> where;
  for (int i = 0; i < num_locations; ++i) where.emplace(loc_ranks[i], loc_slots[i]);
  std::vector<int> loc(num_tiles);
  for (int t = 0; t < num_tiles; ++t) {
    const int* a = permuted_address + (int64_t)t * dims;
    int64_t x = 1, r = 0;
    for (int i = dims - 1; i >= 0; --i) {
      r += (int64_t)a[i] * x;
      x *= grid_T[i];
    }
    auto it = where.find(r);
    if (it == where.end()) return fail(GBX_EINVAL, "tile %d (rank %lld) has no location", t, (long long)r);
    if (it->second < 0 || it->second >= num_slots)
      return fail(GBX_EINVAL, "location %d of tile %d outside [0, %d)", it->second, t, num_slots);
    loc[t] = it->second;
  }
  std::vector<MoveDesc> mv;
  GBX_TRY(big_matrix_moves(dims, vgrid, p_map, num_tiles, permuted_address, row_per_block, col_per_block,
                           num_row_dim, true, mv, nrows, ncols, &loc));
  return run_moves_async(mv, d_tiles, d_big, (cudaStream_t)stream);
}

int gbx_revert_big_matrix(int dims, const int* vgrid, const int* p_map, int num_tiles, const int* permuted_address,
                          int row_per_block, int col_per_block, int num_row_dim, const double* d_big, double* d_tiles,
                          void* stream) {
  std::vector<MoveDesc> mv;
  GBX_TRY(big_matrix_moves(dims, vgrid, p_map, num_tiles, permuted_address, row_per_block, col_per_block,
                           num_row_dim, false, mv, nullptr, nullptr));
  return run_moves_async(mv, d_big, d_tiles, (cudaStream_t)stream);
}

int gbx_grouped_gemm_f64(const gbx_triple* triples, int num_triples, void* stream) {
  if (num_triples < 0) return fail(GBX_EINVAL, "num_triples < 0");
  if (num_triples == 0) return GBX_OK;
  std::vector<GemmProblem> probs(num_triples);
  for (int i = 0; i < num_triples; ++i) {
    const gbx_triple& t = triples[i];
    if (t.m < 0 || t.n < 0 || t.k < 0) return fail(GBX_EINVAL, "negative extent");
    GemmProblem& p = probs[i];
    std::memset(&p, 0, sizeof(p));
    p.A = t.A;
    p.B = t.B;
    p.C = t.C;
    p.a_rs = t.a_rs;
    p.a_cs = t.a_cs;
    p.b_rs = t.b_rs;
    p.b_cs = t.b_cs;
    p.c_rs = t.c_rs;
    p.m = t.m;
    p.n = t.n;
    p.k = t.k;
    p.alpha = t.alpha;
    p.accumulate = t.accumulate;
  }
  cudaStream_t st = (cudaStream_t)stream;
  F64Gemm g;
  GBX_TRY(g.build(probs, true, st));
  return g.run(st);
}

}  // extern "C"
