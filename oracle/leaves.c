/*
 * ORACLE -- CPU restatement of DTCF's node-local contraction leaves.
 *
 * This file is test infrastructure.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU arm may load it, and only as the checker or as the timed CPU
 * baseline -- never as part of the product path.
 *
 * Every function restates one reference function (paths are relative to the
 * DTCF source tree) in plain loops, with two documented corrections:
 *   - local_contraction (localcontract.cc:3-20) passes n_b as the leading
 *     dimension of a transposed B; the restatement uses the leading dimension
 *     of the stored matrix (n_k for bt=1, n_a for at=1), so it is correct for
 *     every shape, not only n_b == n_k.
 *   - DLTC transpose (DLTC/transp.cc:16,24) leaves the output unwritten for an
 *     identity permutation; the restatement copies.
 * Parity is pinned by tests/test_oracle_pin.py against the reference sources
 * compiled from the read-only tree (oracle/_ref, built by oracle/Makefile) and
 * against the committed fixtures in tests/golden/.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXD 8

/* Block_Grid::get_block_rank, block_grid.cc:22-36 (row-major rank). */
long orc_block_rank(const int* addr, int dims, const int* grid) {
    long x = 1, r = 0;
    for (int i = dims - 1; i >= 0; --i) { r += (long)addr[i] * x; x *= grid[i]; }
    return r;
}

/* Block_Grid::get_block_addr, block_grid.cc:51-67 (inverse of the rank). */
void orc_block_addr(long rank, int dims, const int* grid, int* addr) {
    long x = 1;
    for (int i = 0; i < dims; ++i) x *= grid[i];
    for (int i = 0; i < dims; ++i) { x /= grid[i]; addr[i] = (int)(rank / x); rank -= (long)addr[i] * x; }
}

/* transpose, helper.cc:275-522.  Source dimension i of a dense row-major block
 * with extents widths[] lands at output position perm[i].  All three branches
 * of the reference (whole memcpy, trailing-run memcpy, element-wise) produce
 * this same mapping; the restatement is the plain element loop. */
void orc_transpose(const double* in, double* out, const int* perm, int dims, const int* widths) {
    int ow[ORC_MAXD], os[ORC_MAXD], idx[ORC_MAXD];
    long n = 1;
    for (int i = 0; i < dims; ++i) { ow[perm[i]] = widths[i]; n *= widths[i]; idx[i] = 0; }
    os[dims - 1] = 1;
    for (int d = dims - 2; d >= 0; --d) os[d] = os[d + 1] * ow[d + 1];
    for (long e = 0; e < n; ++e) {
        long o = 0;
        for (int i = 0; i < dims; ++i) o += (long)idx[i] * os[perm[i]];
        out[o] = in[e];
        for (int i = dims - 1; i >= 0; --i) { if (++idx[i] < widths[i]) break; idx[i] = 0; }
    }
}

/* DLTC position(), DLTC/transp.h:8-17: pos[i] = position in y of x[i]. */
static void orc_position(const int* x, const int* y, int dim, int* pos) {
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j)
            if (y[j] == x[i]) pos[i] = j;
}

/* DLTC transpose dispatcher, DLTC/transp.cc:3-59, with the 26 fixed kernels
 * of DLTC/transp-kernel-omp.cc: output index order is ids_y, block widths are
 * those of x.  The kernel named transpose_<y order> writes
 * out[row-major over y] = in[row-major over x].  Identity copies (see header). */
void orc_dltc_transpose(const double* x, const int* ids_x, double* y, const int* ids_y,
                        int dim, const int* wb_x) {
    int s[ORC_MAXD], perm[ORC_MAXD];
    orc_position(ids_y, ids_x, dim, s);       /* s[i]: input dim that is output dim i */
    for (int i = 0; i < dim; ++i) perm[s[i]] = i;
    orc_transpose(x, y, perm, dim, wb_x);
}

/* Contraction::get_symm_permutation, contraction.cc:132-160.  sg[] is
 * SG_index_map_permanent (0/1 = symmetry group, 3 = none). */
void orc_symm_permutation(const int* tile_addr, const int* sg, int dims, int* sym_perm) {
    for (int i = 0; i < dims; ++i) sym_perm[i] = i;
    for (int i = 0; i < dims; ++i)
        for (int j = i + 1; j < dims; ++j)
            if (tile_addr[i] < tile_addr[j] && sg[i] == sg[j] && sg[i] <= 1) {
                sym_perm[i] = j; sym_perm[j] = i; break;
            }
}

/* Contraction::compose_p_maps, contraction.cc:121-128. */
void orc_compose_p_maps(const int* map1, const int* map2, int dims, int* out) {
    for (int i = 0; i < dims; ++i) out[i] = map2[map1[i]];
}

/* Contraction::generate_permutation_map, contraction.cc:164-282.
 * cntr_A[i] != 0 marks a contracted index of A; a2c / b2c map external
 * indices of A / B to their position in C; contr[2*c], contr[2*c+1] are the
 * (A index, B index) of the c-th contracted pair in contraction-list order.
 * Returns 0, or -1 when the contracted extents of A and B differ (the
 * reference asserts). */
int orc_generate_permutation_map(int dims_A, const int* cntr_A, const int* a2c, const int* range_A,
                                 int dims_B, const int* cntr_B, const int* b2c, const int* range_B,
                                 const int* range_C, int ncontr, const int* contr,
                                 int* p_map_A, int* p_map_B, int* p_map_C, int* inv_p_map_C,
                                 int* inv_range_C, long* n_a, long* n_b, long* n_k) {
    int ea = 0, eb = 0;
    long na = 1, nb = 1, ka = 1, kb = 1;
    for (int i = 0; i < dims_A; ++i) {
        if (cntr_A[i] == 0) {
            na *= range_A[i];
            p_map_A[i] = ea;
            p_map_C[a2c[i]] = ea;
            inv_range_C[ea] = range_C[a2c[i]];
            inv_p_map_C[ea] = a2c[i];
            ++ea;
        } else {
            ka *= range_A[i];
        }
    }
    for (int i = 0; i < dims_B; ++i) {
        if (cntr_B[i] == 0) {
            nb *= range_B[i];
            p_map_B[i] = eb;
            p_map_C[b2c[i]] = ea + eb;
            inv_range_C[ea + eb] = range_C[b2c[i]];
            inv_p_map_C[ea + eb] = b2c[i];
            ++eb;
        } else {
            kb *= range_B[i];
        }
    }
    if (ka != kb) return -1;
    for (int c = 0; c < ncontr; ++c) {
        p_map_A[contr[2 * c]] = ea + c;
        p_map_B[contr[2 * c + 1]] = eb + c;
    }
    *n_a = na; *n_b = nb; *n_k = ka;
    return 0;
}

/* Row / column ranks of create_big_matrix, transpose_helper.cc:40-111: the
 * block grid is permuted (grid_T[p_map[d]] = vgrid[d]); a tile's row rank is
 * the rank of its permuted address with the column coordinates zeroed, its
 * column rank the rank with the row coordinates zeroed. */
typedef struct { long row, col; int tile; } orc_place;

static int orc_place_cmp(const void* a, const void* b) {
    const orc_place* x = (const orc_place*)a;
    const orc_place* y = (const orc_place*)b;
    if (x->row != y->row) return x->row < y->row ? -1 : 1;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return x->tile - y->tile;
}

/* Builds the std::map<row, map<col, tile>> placement of the reference as a
 * sorted list.  On return order[r * ncols + c] is the tile placed at block
 * (r, c).  Returns the number of tiles placed, or -1 when the rows do not all
 * hold the same number of column blocks (the reference asserts,
 * transpose_helper.cc:126). */
static long orc_big_matrix_order(int dims, const int* vgrid, const int* p_map, int num_tiles,
                                 const int* permuted_address, int num_row_dim,
                                 int* order, int* nrows_out, int* ncols_out) {
    int grid_T[ORC_MAXD], tmp[ORC_MAXD];
    for (int d = 0; d < dims; ++d) grid_T[p_map[d]] = vgrid[d];
    orc_place* pl = (orc_place*)malloc(sizeof(orc_place) * (size_t)(num_tiles > 0 ? num_tiles : 1));
    for (int i = 0; i < num_tiles; ++i) {
        const int* a = permuted_address + (long)i * dims;
        memset(tmp, 0, sizeof(tmp));
        for (int j = 0; j < num_row_dim; ++j) tmp[j] = a[j];
        pl[i].row = orc_block_rank(tmp, dims, grid_T);
        memset(tmp, 0, sizeof(tmp));
        for (int j = num_row_dim; j < dims; ++j) tmp[j] = a[j];
        pl[i].col = orc_block_rank(tmp, dims, grid_T);
        pl[i].tile = i;
    }
    qsort(pl, (size_t)num_tiles, sizeof(orc_place), orc_place_cmp);
    /* a (row, col) pair seen twice keeps its first tile, like std::map insert */
    int n = 0, nrows = 0, ncols = -1, cur = 0;
    for (int i = 0; i < num_tiles; ++i) {
        if (i > 0 && pl[i].row == pl[i - 1].row && pl[i].col == pl[i - 1].col) continue;
        if (i > 0 && pl[i].row != pl[n - 1].row) {
            if (ncols >= 0 && cur != ncols) { free(pl); return -1; }
            ncols = cur; cur = 0; ++nrows;
        }
        pl[n++] = pl[i];
        ++cur;
    }
    if (num_tiles > 0) {
        if (ncols >= 0 && cur != ncols) { free(pl); return -1; }
        ncols = cur; ++nrows;
    } else {
        ncols = 0;
    }
    for (int i = 0; i < n; ++i) order[i] = pl[i].tile;
    *nrows_out = nrows; *ncols_out = ncols;
    free(pl);
    return n;
}

/* create_big_matrix, transpose_helper.cc:20-171: tiles (already permuted,
 * each row_per_block x col_per_block) are placed into one row-major matrix of
 * nrows*row_per_block rows and ncols*col_per_block columns. */
long orc_create_big_matrix(int dims, const int* vgrid, const int* p_map, int num_tiles,
                           const double* tiles, const int* permuted_address,
                           int row_per_block, int col_per_block, int num_row_dim,
                           double* big, int* nrows_out, int* ncols_out) {
    int* order = (int*)malloc(sizeof(int) * (size_t)(num_tiles > 0 ? num_tiles : 1));
    long n = orc_big_matrix_order(dims, vgrid, p_map, num_tiles, permuted_address, num_row_dim,
                                  order, nrows_out, ncols_out);
    if (n < 0) { free(order); return n; }
    long bs = (long)row_per_block * col_per_block;
    long total_col = (long)(*ncols_out) * col_per_block;
    for (int r = 0; r < *nrows_out; ++r)
        for (int c = 0; c < *ncols_out; ++c) {
            const double* t = tiles + (long)order[r * (*ncols_out) + c] * bs;
            for (int i = 0; i < row_per_block; ++i)
                memcpy(big + ((long)r * row_per_block + i) * total_col + (long)c * col_per_block,
                       t + (long)i * col_per_block, sizeof(double) * (size_t)col_per_block);
        }
    free(order);
    return n;
}

/* create_big_matrix_nl, transpose_helper.cc:184-328: the placement of
 * create_big_matrix, with the data of entry i taken from tile slot
 * location(rank_i) of tiles, rank_i the block rank of permuted_address[i] in
 * the permuted grid (transpose_helper.cc:237-255); the address_to_location map
 * comes as nloc (ranks[k] -> slots[k]) pairs.  Returns -2 when a placed
 * tile has no location. */
long orc_create_big_matrix_nl(int dims, const int* vgrid, const int* p_map, int num_tiles,
                              const double* tiles, const int* permuted_address,
                              int row_per_block, int col_per_block, int num_row_dim,
                              const int* ranks, const int* slots, int nloc,
                              double* big, int* nrows_out, int* ncols_out) {
    int grid_T[ORC_MAXD];
    for (int d = 0; d < dims; ++d) grid_T[p_map[d]] = vgrid[d];
    int* loc = (int*)malloc(sizeof(int) * (size_t)(num_tiles > 0 ? num_tiles : 1));
    for (int i = 0; i < num_tiles; ++i) {
        long r = orc_block_rank(permuted_address + (long)i * dims, dims, grid_T);
        int k = 0;
        while (k < nloc && ranks[k] != r) ++k;
        if (k == nloc) { free(loc); return -2; }
        loc[i] = slots[k];
    }
    int* order = (int*)malloc(sizeof(int) * (size_t)(num_tiles > 0 ? num_tiles : 1));
    long n = orc_big_matrix_order(dims, vgrid, p_map, num_tiles, permuted_address, num_row_dim,
                                  order, nrows_out, ncols_out);
    if (n < 0) { free(order); free(loc); return n; }
    long bs = (long)row_per_block * col_per_block;
    long total_col = (long)(*ncols_out) * col_per_block;
    for (int r = 0; r < *nrows_out; ++r)
        for (int c = 0; c < *ncols_out; ++c) {
            const double* t = tiles + (long)loc[order[r * (*ncols_out) + c]] * bs;
            for (int i = 0; i < row_per_block; ++i)
                memcpy(big + ((long)r * row_per_block + i) * total_col + (long)c * col_per_block,
                       t + (long)i * col_per_block, sizeof(double) * (size_t)col_per_block);
        }
    free(order);
    free(loc);
    return n;
}

/* revert_big_matrix, transpose_helper.cc:331-409: the inverse placement. */
long orc_revert_big_matrix(int dims, const int* vgrid, const int* p_map, int num_tiles,
                           const int* permuted_address, int row_per_block, int col_per_block,
                           int num_row_dim, const double* big, double* tiles) {
    int nrows, ncols;
    int* order = (int*)malloc(sizeof(int) * (size_t)(num_tiles > 0 ? num_tiles : 1));
    long n = orc_big_matrix_order(dims, vgrid, p_map, num_tiles, permuted_address, num_row_dim,
                                  order, &nrows, &ncols);
    if (n < 0) { free(order); return n; }
    long bs = (long)row_per_block * col_per_block;
    long total_col = (long)ncols * col_per_block;
    for (int r = 0; r < nrows; ++r)
        for (int c = 0; c < ncols; ++c) {
            double* t = tiles + (long)order[r * ncols + c] * bs;
            for (int i = 0; i < row_per_block; ++i)
                memcpy(t + (long)i * col_per_block,
                       big + ((long)r * row_per_block + i) * total_col + (long)c * col_per_block,
                       sizeof(double) * (size_t)col_per_block);
        }
    free(order);
    return n;
}

/* local_contraction, localcontract.cc:3-20, corrected leading dimensions:
 * C[n_a x n_b] += alpha * op(A) * op(B), all row-major, beta = 1.
 * at = 0: A is n_a x n_k; at = 1: A is n_k x n_a.
 * bt = 0: B is n_k x n_b; bt = 1: B is n_b x n_k.
 * The k sum runs in increasing k. */
void orc_local_contraction(long n_a, long n_b, long n_k, const double* A, const double* B,
                           double* C, int at, int bt, double alpha) {
    for (long i = 0; i < n_a; ++i)
        for (long j = 0; j < n_b; ++j) {
            double s = 0.0;
            for (long k = 0; k < n_k; ++k) {
                double a = at ? A[k * n_a + i] : A[i * n_k + k];
                double b = bt ? B[j * n_k + k] : B[k * n_b + j];
                s += a * b;
            }
            C[i * n_b + j] += alpha * s;
        }
}

/* DLTC compute, DLTC/compute.cc:3-36: c[m x n] += a[m x k] * b[k x n]. */
void orc_dltc_compute(long m, long n, long k, const double* a, const double* b, double* c) {
    orc_local_contraction(m, n, k, a, b, c, 0, 0, 1.0);
}

/* ---- DLTC tile loop (task_mul / task_sum) over dense tensors ------------- */

/* A DLTC tensor as GA holds it: dense, row-major over its index order, each
 * index of extent O (hole name, id < nocc) or V (particle name).  Tiles are
 * wbO / wbV wide (DLTC/dltc_tensor.cc:169-267). */
typedef struct {
    int rank; const int* ids; int O, V, wbO, wbV, nocc;
} orc_dltc;

static int orc_ext(const orc_dltc* t, int name) { return name < t->nocc ? t->O : t->V; }
static int orc_wb(const orc_dltc* t, int name) { return name < t->nocc ? t->wbO : t->wbV; }

/* getTile: copies the tile whose tile coordinates (per index name) are in
 * tc[name] into buf (row-major over the tensor's index order). */
static void orc_get_tile(const orc_dltc* t, const double* full, const int* tc, double* buf) {
    int idx[ORC_MAXD], ext[ORC_MAXD], wb[ORC_MAXD], lo[ORC_MAXD];
    long n = 1;
    for (int d = 0; d < t->rank; ++d) {
        ext[d] = orc_ext(t, t->ids[d]); wb[d] = orc_wb(t, t->ids[d]);
        lo[d] = tc[t->ids[d]] * wb[d]; idx[d] = 0; n *= wb[d];
    }
    for (long e = 0; e < n; ++e) {
        long off = 0;
        for (int d = 0; d < t->rank; ++d) off = off * ext[d] + lo[d] + idx[d];
        buf[e] = full[off];
        for (int d = t->rank - 1; d >= 0; --d) { if (++idx[d] < wb[d]) break; idx[d] = 0; }
    }
}

/* accTile (NGA_Acc): full[tile] += coef * buf. */
static void orc_acc_tile(const orc_dltc* t, double* full, const int* tc, const double* buf, double coef) {
    int idx[ORC_MAXD], ext[ORC_MAXD], wb[ORC_MAXD], lo[ORC_MAXD];
    long n = 1;
    for (int d = 0; d < t->rank; ++d) {
        ext[d] = orc_ext(t, t->ids[d]); wb[d] = orc_wb(t, t->ids[d]);
        lo[d] = tc[t->ids[d]] * wb[d]; idx[d] = 0; n *= wb[d];
    }
    for (long e = 0; e < n; ++e) {
        long off = 0;
        for (int d = 0; d < t->rank; ++d) off = off * ext[d] + lo[d] + idx[d];
        full[off] += coef * buf[e];
        for (int d = t->rank - 1; d >= 0; --d) { if (++idx[d] < wb[d]) break; idx[d] = 0; }
    }
}

static void orc_widths(const orc_dltc* t, const int* ids, int n, int* wb) {
    for (int i = 0; i < n; ++i) wb[i] = orc_wb(t, ids[i]);
}

/* Multiplication::Multiplication, DLTC/expr.cc:13-67: m = names only in A,
 * n = names only in B, k = names in both, each in name order;
 * at = m+k, bt = k+n, ct = m+n.  task_mul, DLTC/task.cc:83-137: for every C
 * tile (C's index order, last index fastest), sum over the contracted tiles
 * of transpose(A)->at, transpose(B)->bt, compute; then transpose ct -> C and
 * accumulate with coef.  nnames bounds the name ids. */
int orc_task_mul(double coef,
                 int rC, const int* idC, double* C,
                 int rA, const int* idA, const double* A,
                 int rB, const int* idB, const double* B,
                 int O, int V, int wbO, int wbV, int nocc, int nnames) {
    int tab[64] = {0};
    int m_ids[ORC_MAXD], n_ids[ORC_MAXD], k_ids[ORC_MAXD];
    int nm = 0, nn = 0, nk = 0;
    if (nnames > 64 || rC > ORC_MAXD || rA > ORC_MAXD || rB > ORC_MAXD) return -1;
    for (int i = 0; i < rA; ++i) tab[idA[i]] = 1;
    for (int i = 0; i < rB; ++i) tab[idB[i]] += 2;
    for (int i = 0; i < nnames; ++i) {
        if (tab[i] == 1) m_ids[nm++] = i;
        if (tab[i] == 2) n_ids[nn++] = i;
        if (tab[i] == 3) k_ids[nk++] = i;
    }
    int at[ORC_MAXD], bt[ORC_MAXD], ct[ORC_MAXD];
    for (int i = 0; i < nm; ++i) { at[i] = m_ids[i]; ct[i] = m_ids[i]; }
    for (int i = 0; i < nk; ++i) { at[nm + i] = k_ids[i]; bt[i] = k_ids[i]; }
    for (int i = 0; i < nn; ++i) { bt[nk + i] = n_ids[i]; ct[nm + i] = n_ids[i]; }
    orc_dltc tA = {rA, idA, O, V, wbO, wbV, nocc};
    orc_dltc tB = {rB, idB, O, V, wbO, wbV, nocc};
    orc_dltc tC = {rC, idC, O, V, wbO, wbV, nocc};
    long wm = 1, wn = 1, wk = 1;
    for (int i = 0; i < nm; ++i) wm *= orc_wb(&tA, m_ids[i]);
    for (int i = 0; i < nn; ++i) wn *= orc_wb(&tA, n_ids[i]);
    for (int i = 0; i < nk; ++i) wk *= orc_wb(&tA, k_ids[i]);
    long a_size = wm * wk, b_size = wk * wn, c_size = wm * wn;
    double* buf_a = (double*)malloc(sizeof(double) * (size_t)a_size);
    double* buf_at = (double*)malloc(sizeof(double) * (size_t)a_size);
    double* buf_b = (double*)malloc(sizeof(double) * (size_t)b_size);
    double* buf_bt = (double*)malloc(sizeof(double) * (size_t)b_size);
    double* buf_ct = (double*)malloc(sizeof(double) * (size_t)c_size);
    double* buf_c = (double*)malloc(sizeof(double) * (size_t)c_size);
    int wa[ORC_MAXD], wbb[ORC_MAXD], wc[ORC_MAXD];
    orc_widths(&tA, idA, rA, wa);
    orc_widths(&tB, idB, rB, wbb);
    orc_widths(&tC, ct, rC, wc);
    int tc[64] = {0};
    int ext_hi[ORC_MAXD], k_hi[ORC_MAXD];
    for (int d = 0; d < rC; ++d) ext_hi[d] = orc_ext(&tC, idC[d]) / orc_wb(&tC, idC[d]);
    for (int d = 0; d < nk; ++d) k_hi[d] = orc_ext(&tA, k_ids[d]) / orc_wb(&tA, k_ids[d]);
    int ec[ORC_MAXD] = {0};
    for (;;) {                                   /* IndexLoops over C's tiles */
        for (int d = 0; d < rC; ++d) tc[idC[d]] = ec[d];
        memset(buf_ct, 0, sizeof(double) * (size_t)c_size);
        int kc[ORC_MAXD] = {0};
        for (;;) {                               /* IndexLoops over summed tiles */
            for (int d = 0; d < nk; ++d) tc[k_ids[d]] = kc[d];
            orc_get_tile(&tA, A, tc, buf_a);
            orc_dltc_transpose(buf_a, idA, buf_at, at, rA, wa);
            orc_get_tile(&tB, B, tc, buf_b);
            orc_dltc_transpose(buf_b, idB, buf_bt, bt, rB, wbb);
            orc_dltc_compute(wm, wn, wk, buf_at, buf_bt, buf_ct);
            int d = nk - 1;
            for (; d >= 0; --d) { if (++kc[d] < k_hi[d]) break; kc[d] = 0; }
            if (d < 0) break;
        }
        orc_dltc_transpose(buf_ct, ct, buf_c, idC, rC, wc);
        orc_acc_tile(&tC, C, tc, buf_c, coef);
        int d = rC - 1;
        for (; d >= 0; --d) { if (++ec[d] < ext_hi[d]) break; ec[d] = 0; }
        if (d < 0) break;
    }
    free(buf_a); free(buf_at); free(buf_b); free(buf_bt); free(buf_ct); free(buf_c);
    return 0;
}

/* task_sum, DLTC/task.cc:51-81: for every C tile, transpose the A tile to
 * C's index order and accumulate with coef. */
int orc_task_sum(double coef, int rC, const int* idC, double* C,
                 int rA, const int* idA, const double* A,
                 int O, int V, int wbO, int wbV, int nocc) {
    if (rC != rA || rC > ORC_MAXD) return -1;
    orc_dltc tA = {rA, idA, O, V, wbO, wbV, nocc};
    orc_dltc tC = {rC, idC, O, V, wbO, wbV, nocc};
    long n = 1;
    int wa[ORC_MAXD], hi[ORC_MAXD], ec[ORC_MAXD] = {0}, tc[64] = {0};
    for (int d = 0; d < rA; ++d) { wa[d] = orc_wb(&tA, idA[d]); n *= wa[d]; }
    for (int d = 0; d < rC; ++d) hi[d] = orc_ext(&tC, idC[d]) / orc_wb(&tC, idC[d]);
    double* buf_a = (double*)malloc(sizeof(double) * (size_t)n);
    double* buf_at = (double*)malloc(sizeof(double) * (size_t)n);
    for (;;) {
        for (int d = 0; d < rC; ++d) tc[idC[d]] = ec[d];
        orc_get_tile(&tA, A, tc, buf_a);
        orc_dltc_transpose(buf_a, idA, buf_at, idC, rA, wa);
        orc_acc_tile(&tC, C, tc, buf_at, coef);
        int d = rC - 1;
        for (; d >= 0; --d) { if (++ec[d] < hi[d]) break; ec[d] = 0; }
        if (d < 0) break;
    }
    free(buf_a); free(buf_at);
    return 0;
}

/* ---- RRR tile set -------------------------------------------------------- */

/* Tensor::generate_data / isValid / get_bound, tensor.cc:617-694, 761-783,
 * on one process: tiles are enumerated in lexicographic order of their block
 * address; an index whose symmetry character ('a'/'A' group 0, 'b'/'B' group 1)
 * repeats a previous index's group is bounded by that index (non-increasing
 * within a group).  Returns the tile count; addr receives dims ints per tile.
 * Pass addr = NULL to count only. */
long orc_rrr_tiles(const char* sym, const int* vgrid, int* addr) {
    int dims = (int)strlen(sym);
    int sg[ORC_MAXD], cur[ORC_MAXD];
    for (int i = 0; i < dims; ++i) {
        char c = sym[i];
        sg[i] = (c == 'a' || c == 'A') ? 0 : (c == 'b' || c == 'B') ? 1 : 3;
    }
    long n = 0;
    int d = 0;
    for (int i = 0; i < dims; ++i) cur[i] = 0;
    /* iterative odometer with per-index bounds */
    for (;;) {
        int ok = 1;
        for (int i = 0; i < dims && ok; ++i)
            for (int j = i + 1; j < dims; ++j)
                if (cur[i] < cur[j] && sg[i] == sg[j] && sg[i] != 3) { ok = 0; break; }
        if (ok) {
            if (addr) memcpy(addr + n * dims, cur, sizeof(int) * (size_t)dims);
            ++n;
        }
        for (d = dims - 1; d >= 0; --d) { if (++cur[d] < vgrid[d]) break; cur[d] = 0; }
        if (d < 0) break;
    }
    return n;
}
