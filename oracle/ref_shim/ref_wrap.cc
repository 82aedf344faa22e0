/* extern "C" entry points over the DTCF reference leaves compiled in place
 * (helper.cc, transpose_helper.cc, block_grid.cc, localcontract.cc, tensor.cc,
 * grid.cc, DLTC/transp-kernel-omp.cc).  Loaded by tests/ to pin the oracle's
 * restatement to the reference itself.  Test infrastructure only. */
#include <cstring>
#include <map>
#include <string>
#include "tensor.h"
#include "transpose_helper.h"
#include "block_grid.h"
#include "localcontract.h"
#include "DLTC/transp-kernel.h"

extern "C" {

void ref_transpose(double* in, double* out, int* perm, int dims, int* widths) {
  transpose(in, out, perm, dims, widths);
}

void ref_local_contraction(int n_a, int n_b, int n_k, double* A, double* B, double* C, int at, int bt,
                           double alpha) {
  local_contraction(n_a, n_b, n_k, A, B, C, at, bt, alpha);
}

long ref_block_rank(int* addr, int dims, int* grid) {
  RRR::Block_Grid g(dims, grid);
  return g.get_block_rank(addr);
}

void ref_block_addr(long rank, int dims, int* grid, int* addr) {
  RRR::Block_Grid g(dims, grid);
  int* a = nullptr;
  g.get_block_addr((int)rank, a);
  std::memcpy(addr, a, sizeof(int) * dims);
  delete[] a;
}

typedef void (*dltc_kernel)(const double*, double*, int, int, int, int);
static const char* kNames[24] = {"ijkl", "ijlk", "ikjl", "iklj", "iljk", "ilkj", "jikl", "jilk",
                                 "jkil", "jkli", "jlik", "jlki", "kijl", "kilj", "kjil", "kjli",
                                 "klij", "klji", "lijk", "likj", "ljik", "ljki", "lkij", "lkji"};
static dltc_kernel kKernels[24] = {
    transpose_ijkl, transpose_ijlk, transpose_ikjl, transpose_iklj, transpose_iljk, transpose_ilkj,
    transpose_jikl, transpose_jilk, transpose_jkil, transpose_jkli, transpose_jlik, transpose_jlki,
    transpose_kijl, transpose_kilj, transpose_kjil, transpose_kjli, transpose_klij, transpose_klji,
    transpose_lijk, transpose_likj, transpose_ljik, transpose_ljki, transpose_lkij, transpose_lkji};

/* name: 4 letters spelling the output order, e.g. "klij". Returns -1 if unknown. */
int ref_dltc_transpose4(const char* name, const double* in, double* out, int di, int dj, int dk, int dl) {
  for (int i = 0; i < 24; ++i)
    if (std::strncmp(name, kNames[i], 4) == 0) { kKernels[i](in, out, di, dj, dk, dl); return 0; }
  return -1;
}

void ref_dltc_transpose2(const double* in, double* out, int di, int dj, int swap) {
  if (swap) transpose_ji(in, out, di, dj); else transpose_ij(in, out, di, dj);
}

static RRR::Tensor* make_tensor(const char* sym, int* sizes, int* vgrid) {
  int dims = (int)std::strlen(sym);
  int* pg = new int[dims];
  int* idmap = new int[dims];
  int* sz = new int[dims];
  int* vg = new int[dims];
  for (int i = 0; i < dims; ++i) { pg[i] = 1; idmap[i] = i; sz[i] = sizes[i]; vg[i] = vgrid[i]; }
  RRR::Grid* g = new RRR::Grid(dims, pg);
  return new RRR::Tensor(std::string(sym), idmap, sz, vg, g);
}

/* Tensor::initialize on one process: tiles and addresses as generated. */
long ref_tensor_tiles(const char* sym, int* sizes, int* vgrid, double* tiles, int* addr, long cap_tiles) {
  RRR::Tensor* t = make_tensor(sym, sizes, vgrid);
  t->initialize();
  long n = t->get_num_actual_tiles();
  if (n > cap_tiles) return -n;
  std::memcpy(tiles, t->get_tensor_tiles(), sizeof(double) * n * t->get_block_size());
  std::memcpy(addr, t->get_tile_addresses(), sizeof(int) * n * t->get_dims());
  return n;
}

long ref_create_big_matrix(const char* sym, int* sizes, int* vgrid, double* tiles, int* perm_addr,
                           int* p_map, int num_tiles, int row_per_block, int col_per_block, int num_row_dim,
                           double* big_out) {
  RRR::Tensor* t = make_tensor(sym, sizes, vgrid);
  std::map<int, std::map<int, int> >* bm = nullptr;
  double* big = nullptr;
  RRR::create_big_matrix(t, tiles, perm_addr, p_map, num_tiles, row_per_block, col_per_block, num_row_dim, bm,
                         big);
  std::memcpy(big_out, big, sizeof(double) * (size_t)num_tiles * t->get_block_size());
  delete[] big;
  delete bm;
  return num_tiles;
}

long ref_create_big_matrix_nl(const char* sym, int* sizes, int* vgrid, double* tiles, int* perm_addr, int* p_map,
                              int num_tiles, int row_per_block, int col_per_block, int num_row_dim, int* loc_ranks,
                              int* loc_slots, int nloc, double* big_out) {
  RRR::Tensor* t = make_tensor(sym, sizes, vgrid);
  std::map<int, std::map<int, int> >* bm = nullptr;
  double* big = nullptr;
  std::map<int, int>* where = new std::map<int, int>();
  for (int i = 0; i < nloc; ++i) (*where)[loc_ranks[i]] = loc_slots[i];
  RRR::create_big_matrix_nl(t, tiles, perm_addr, p_map, num_tiles, row_per_block, col_per_block, num_row_dim, bm,
                            big, where);
  std::memcpy(big_out, big, sizeof(double) * (size_t)num_tiles * t->get_block_size());
  delete[] big;
  delete bm;
  delete where;
  return num_tiles;
}

long ref_revert_big_matrix(const char* sym, int* sizes, int* vgrid, double* tiles_in, int* perm_addr,
                           int* p_map, int num_tiles, int row_per_block, int col_per_block, int num_row_dim,
                           double* big_in, double* tiles_out) {
  RRR::Tensor* t = make_tensor(sym, sizes, vgrid);
  std::map<int, std::map<int, int> >* bm = nullptr;
  double* big = nullptr;
  RRR::create_big_matrix(t, tiles_in, perm_addr, p_map, num_tiles, row_per_block, col_per_block, num_row_dim, bm,
                         big);
  RRR::revert_big_matrix(t, bm, big_in, row_per_block, col_per_block, p_map, tiles_out);
  delete[] big;
  delete bm;
  return num_tiles;
}

}  // extern "C"
