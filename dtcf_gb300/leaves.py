"""Python mirror of the reference's leaf interface over the C ABI.

Arguments that the reference passes as device-resident buffers are torch CUDA
tensors (float64, contiguous); index arrays are Python sequences.  Each
function names the reference function it mirrors.
"""
import ctypes

import numpy as np
import torch

from ._lib import lib, check


def _ptr(t):
    assert t.is_cuda and t.dtype == torch.float64 and t.is_contiguous(), "need a contiguous float64 CUDA tensor"
    return ctypes.c_void_p(t.data_ptr())


def _iarr(seq):
    a = np.ascontiguousarray(np.asarray(seq, dtype=np.int32).reshape(-1))
    return a, a.ctypes.data_as(ctypes.c_void_p)


def _stream(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def transpose(inp, out, perm, widths, stream=None):
    """transpose (helper.cc:275): source dim i lands at output position perm[i]."""
    p, pp = _iarr(perm)
    w, wp = _iarr(widths)
    check(lib().gbx_transpose(_ptr(inp), _ptr(out), pp, len(p), wp, _stream(stream)))
    return out


def transpose_blocks(inp, out, perms, widths, stream=None):
    perms = np.asarray(perms, dtype=np.int32)
    p, pp = _iarr(perms)
    w, wp = _iarr(widths)
    check(lib().gbx_transpose_blocks(_ptr(inp), _ptr(out), perms.shape[0], pp, len(w), wp, _stream(stream)))
    return out


def dltc_transpose(x, ids_x, y, ids_y, wb_x, stream=None):
    """DLTC transpose (DLTC/transp.cc:3): x in index order ids_x -> y in ids_y."""
    a, ap = _iarr(ids_x)
    b, bp = _iarr(ids_y)
    w, wp = _iarr(wb_x)
    check(lib().gbx_dltc_transpose(_ptr(x), ap, _ptr(y), bp, len(a), wp, _stream(stream)))
    return y


def local_contraction(n_a, n_b, n_k, A, B, C, at, bt, alpha, stream=None):
    """local_contraction (localcontract.cc:3) with corrected leading dimensions."""
    check(lib().gbx_local_contraction(n_a, n_b, n_k, _ptr(A), _ptr(B), _ptr(C), at, bt, alpha, _stream(stream)))
    return C


def dltc_compute(c, a, b, m, n, k, stream=None):
    """DLTC compute (DLTC/compute.cc:3): c[m x n] += a[m x k] b[k x n]."""
    check(lib().gbx_dltc_compute(_ptr(c), _ptr(a), _ptr(b), m, n, k, _stream(stream)))
    return c


def create_big_matrix(vgrid, p_map, tiles, permuted_address, row_per_block, col_per_block, num_row_dim, big,
                      stream=None):
    """create_big_matrix (transpose_helper.cc:20); returns (nrows, ncols) block counts."""
    addr = np.asarray(permuted_address, dtype=np.int32)
    g, gp = _iarr(vgrid)
    pm, pmp = _iarr(p_map)
    a, ap = _iarr(addr)
    nr, nc = ctypes.c_int(), ctypes.c_int()
    check(lib().gbx_create_big_matrix(len(g), gp, pmp, addr.shape[0], _ptr(tiles), ap, row_per_block, col_per_block,
                                      num_row_dim, _ptr(big), ctypes.byref(nr), ctypes.byref(nc), _stream(stream)))
    return nr.value, nc.value


def create_big_matrix_nl(vgrid, p_map, tiles, permuted_address, row_per_block, col_per_block, num_row_dim,
                         address_to_location, big, stream=None):
    """create_big_matrix_nl (transpose_helper.cc:184): the tile data of each
    placed address comes from slot address_to_location[rank] of tiles (a dict
    or (ranks, slots) pairs); returns (nrows, ncols) block counts."""
    addr = np.asarray(permuted_address, dtype=np.int32)
    g, gp = _iarr(vgrid)
    pm, pmp = _iarr(p_map)
    a, ap = _iarr(addr)
    items = sorted(address_to_location.items()) if isinstance(address_to_location, dict) else address_to_location
    kr, krp = _iarr([k for k, _ in items])
    kv, kvp = _iarr([v for _, v in items])
    bs = row_per_block * col_per_block
    nr, nc = ctypes.c_int(), ctypes.c_int()
    check(lib().gbx_create_big_matrix_nl(len(g), gp, pmp, addr.shape[0], _ptr(tiles), tiles.numel() // max(1, bs), ap,
                                         row_per_block, col_per_block, num_row_dim, krp, kvp, len(kr), _ptr(big),
                                         ctypes.byref(nr), ctypes.byref(nc), _stream(stream)))
    return nr.value, nc.value


def revert_big_matrix(vgrid, p_map, permuted_address, row_per_block, col_per_block, num_row_dim, big, tiles,
                      stream=None):
    """revert_big_matrix (transpose_helper.cc:331)."""
    addr = np.asarray(permuted_address, dtype=np.int32)
    g, gp = _iarr(vgrid)
    pm, pmp = _iarr(p_map)
    a, ap = _iarr(addr)
    check(lib().gbx_revert_big_matrix(len(g), gp, pmp, addr.shape[0], ap, row_per_block, col_per_block, num_row_dim,
                                      _ptr(big), _ptr(tiles), _stream(stream)))
    return tiles


class Triple(ctypes.Structure):
    """gbx_triple (include/gbx.h)."""
    _fields_ = [("A", ctypes.c_void_p), ("B", ctypes.c_void_p), ("C", ctypes.c_void_p),
                ("a_rs", ctypes.c_int64), ("a_cs", ctypes.c_int64), ("b_rs", ctypes.c_int64),
                ("b_cs", ctypes.c_int64), ("c_rs", ctypes.c_int64),
                ("m", ctypes.c_int), ("n", ctypes.c_int), ("k", ctypes.c_int),
                ("alpha", ctypes.c_double), ("accumulate", ctypes.c_int)]


def grouped_gemm_f64(triples, stream=None):
    """All triples (Triple structs with device pointers) in one persistent launch."""
    arr = (Triple * len(triples))(*triples)
    check(lib().gbx_grouped_gemm_f64(ctypes.cast(arr, ctypes.c_void_p), len(triples), _stream(stream)))


def split_gemm(A, B, C, slices=0, stream=None):
    """C = A B^T (row-major FP64) on the split-precision tcgen05 engine."""
    M, K = A.shape
    N = B.shape[0]
    check(lib().gbx_split_gemm(_ptr(A), _ptr(B), _ptr(C), M, N, K, slices, _stream(stream)))
    return C


MODE_FP64, MODE_SPLIT, MODE_AUTO = 0, 1, 2


class Group:
    """A planned set of block triples (gbx_group_*): C_t (+)= alpha A_t B_t^T.

    ``triples`` are Triple structs over device memory that must outlive the
    group.  ``execute(per_triple=False)`` runs one persistent launch per
    kernel kind; ``per_triple=True`` launches each FP64 triple separately.
    """

    def __init__(self, triples, mode=MODE_AUTO, slices=0):
        self._arr = (Triple * len(triples))(*triples)
        self.n = len(triples)
        h = ctypes.c_void_p()
        check(lib().gbx_group_create(ctypes.cast(self._arr, ctypes.c_void_p), self.n, mode, slices,
                                     ctypes.byref(h)))
        self._h = h

    def execute(self, per_triple=False, stream=None):
        check(lib().gbx_group_execute(self._h, 1 if per_triple else 0, _stream(stream)))

    def autotune(self, reps=3, stream=None):
        check(lib().gbx_group_autotune(self._h, reps, _stream(stream)))

    def info(self):
        """(engines, params, flops): per-triple engine (0 FP64, 1 split) and tile parameter."""
        eng = (ctypes.c_int * max(self.n, 1))()
        par = (ctypes.c_int * max(self.n, 1))()
        fl = ctypes.c_double()
        check(lib().gbx_group_info(self._h, ctypes.cast(eng, ctypes.c_void_p), ctypes.cast(par, ctypes.c_void_p),
                                   ctypes.byref(fl)))
        return list(eng)[:self.n], list(par)[:self.n], fl.value

    def close(self):
        if getattr(self, "_h", None):
            lib().gbx_group_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
