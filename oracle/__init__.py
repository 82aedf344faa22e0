"""ORACLE -- CPU restatement of DTCF's node-local contraction path.

Test infrastructure only: tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU arm may import this package, as the checker or as the timed CPU baseline.
The product (``dtcf_gb300``) never imports it.

``liboracle.so`` (oracle/leaves.c) restates the reference leaves in C;
``_ref/libref.so`` is the reference's own leaf sources compiled in place by
oracle/Makefile when the DTCF tree is present.  Python wrappers below take and
return numpy arrays.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_ref = None
_ref_tried = False

_i = ctypes.c_int
_l = ctypes.c_long
_d = ctypes.c_double
_p = ctypes.c_void_p


def build(ref=True):
    """Compile liboracle.so, and oracle/_ref/libref.so when the reference tree
    exists.  The tree's location is the Makefile's REF (DTCF_REFERENCE, when
    set, overrides it); `make ref` reports a missing tree and builds nothing."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref:
        env = dict(os.environ)
        if "DTCF_REFERENCE" in env:
            env["REF"] = env["DTCF_REFERENCE"]
        probe = subprocess.run(["make", "-s", "-C", HERE, "ref-present"], env=env, capture_output=True, text=True)
        if probe.returncode == 0:
            subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True, env=env)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build(ref=False)
        _lib = ctypes.CDLL(path)
        _lib.orc_block_rank.restype = _l
        _lib.orc_create_big_matrix.restype = _l
        _lib.orc_revert_big_matrix.restype = _l
        _lib.orc_rrr_tiles.restype = _l
        _lib.orc_local_contraction.argtypes = [_l, _l, _l, _p, _p, _p, _i, _i, _d]
        _lib.orc_dltc_compute.argtypes = [_l, _l, _l, _p, _p, _p]
        _lib.orc_task_mul.argtypes = [_d, _i, _p, _p, _i, _p, _p, _i, _p, _p] + [_i] * 6
        _lib.orc_task_sum.argtypes = [_d, _i, _p, _p, _i, _p, _p] + [_i] * 5
        _lib.orc_cc_integrals.argtypes = [ctypes.c_uint64, _l, _p, _p] + [_l, _p] * 4 + [_p]
    return _lib


def ref():
    """The compiled reference leaves, or None when they are not built here."""
    global _ref, _ref_tried
    if not _ref_tried:
        _ref_tried = True
        path = os.path.join(HERE, "_ref", "libref.so")
        if os.path.exists(path):
            try:
                _ref = ctypes.CDLL(path)
                _ref.ref_block_rank.restype = _l
                _ref.ref_tensor_tiles.restype = _l
                _ref.ref_create_big_matrix.restype = _l
                _ref.ref_revert_big_matrix.restype = _l
                _ref.ref_local_contraction.argtypes = [_i, _i, _i, _p, _p, _p, _i, _i, _d]
            except OSError:
                _ref = None
    return _ref


def _ip(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return a.ctypes.data_as(_p)


# ---- restatement wrappers --------------------------------------------------

def transpose(block, perm):
    """RRR transpose (helper.cc:275): source dim i lands at output position perm[i]."""
    block = np.ascontiguousarray(block, dtype=np.float64)
    widths = _ip(block.shape)
    perm = _ip(perm)
    out_shape = [0] * block.ndim
    for i, p in enumerate(perm):
        out_shape[p] = block.shape[i]
    out = np.empty(out_shape, dtype=np.float64)
    lib().orc_transpose(_ptr(block), _ptr(out), _ptr(perm), _i(block.ndim), _ptr(widths))
    return out


def dltc_transpose(x, ids_x, ids_y):
    """DLTC transpose (DLTC/transp.cc:3): reorder block x from index order ids_x to ids_y."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    ix, iy = _ip(ids_x), _ip(ids_y)
    pos = [list(ids_x).index(n) for n in ids_y]
    y = np.empty([x.shape[p] for p in pos], dtype=np.float64)
    lib().orc_dltc_transpose(_ptr(x), _ptr(ix), _ptr(y), _ptr(iy), _i(x.ndim), _ptr(_ip(x.shape)))
    return y


def block_rank(addr, grid):
    a, g = _ip(addr), _ip(grid)
    return int(lib().orc_block_rank(_ptr(a), _i(len(a)), _ptr(g)))


def block_addr(rank, grid):
    g = _ip(grid)
    out = np.zeros(len(g), dtype=np.int32)
    lib().orc_block_addr(_l(rank), _i(len(g)), _ptr(g), _ptr(out))
    return out


def symm_permutation(tile_addr, sg):
    a, s = _ip(tile_addr), _ip(sg)
    out = np.zeros(len(a), dtype=np.int32)
    lib().orc_symm_permutation(_ptr(a), _ptr(s), _i(len(a)), _ptr(out))
    return out


def compose_p_maps(map1, map2):
    m1, m2 = _ip(map1), _ip(map2)
    out = np.zeros(len(m1), dtype=np.int32)
    lib().orc_compose_p_maps(_ptr(m1), _ptr(m2), _i(len(m1)), _ptr(out))
    return out


def generate_permutation_map(cntr_A, a2c, range_A, cntr_B, b2c, range_B, range_C, contr):
    """Contraction::generate_permutation_map (contraction.cc:164).  Returns a dict."""
    dA, dB, dC = len(cntr_A), len(cntr_B), len(range_C)
    pA, pB = np.zeros(dA, np.int32), np.zeros(dB, np.int32)
    pC, ipC, irC = np.zeros(dC, np.int32), np.zeros(dC, np.int32), np.zeros(dC, np.int32)
    na, nb, nk = _l(), _l(), _l()
    cl = _ip(np.array(contr, dtype=np.int32).reshape(-1))
    rc = lib().orc_generate_permutation_map(
        _i(dA), _ptr(_ip(cntr_A)), _ptr(_ip(a2c)), _ptr(_ip(range_A)),
        _i(dB), _ptr(_ip(cntr_B)), _ptr(_ip(b2c)), _ptr(_ip(range_B)),
        _ptr(_ip(range_C)), _i(len(contr)), _ptr(cl),
        _ptr(pA), _ptr(pB), _ptr(pC), _ptr(ipC), _ptr(irC),
        ctypes.byref(na), ctypes.byref(nb), ctypes.byref(nk))
    if rc != 0:
        raise ValueError("contracted extents of A and B differ")
    return dict(p_map_A=pA, p_map_B=pB, p_map_C=pC, inv_p_map_C=ipC, inv_range_C=irC,
                n_a=na.value, n_b=nb.value, n_k=nk.value)


def create_big_matrix(vgrid, p_map, tiles, permuted_address, row_per_block, col_per_block, num_row_dim):
    """create_big_matrix (transpose_helper.cc:20).  tiles: (num_tiles, block_size)."""
    tiles = np.ascontiguousarray(tiles, dtype=np.float64)
    addr = _ip(permuted_address)
    n = tiles.shape[0]
    big = np.zeros(tiles.size, dtype=np.float64)
    nr, nc = _i(), _i()
    r = lib().orc_create_big_matrix(_i(addr.shape[1]), _ptr(_ip(vgrid)), _ptr(_ip(p_map)), _i(n),
                                    _ptr(tiles), _ptr(addr), _i(row_per_block), _i(col_per_block),
                                    _i(num_row_dim), _ptr(big), ctypes.byref(nr), ctypes.byref(nc))
    if r < 0:
        raise ValueError("tile pattern is not rectangular")
    return big.reshape(nr.value * row_per_block, nc.value * col_per_block)


def create_big_matrix_nl(vgrid, p_map, tiles, permuted_address, row_per_block, col_per_block, num_row_dim,
                         address_to_location):
    """create_big_matrix_nl (transpose_helper.cc:184).  tiles: (slots, block_size);
    address_to_location: {rank in the permuted grid: slot}."""
    tiles = np.ascontiguousarray(tiles, dtype=np.float64)
    addr = _ip(permuted_address)
    n = addr.shape[0]
    items = sorted(address_to_location.items())
    kr, kv = _ip([k for k, _ in items]), _ip([v for _, v in items])
    big = np.zeros(n * tiles.shape[1], dtype=np.float64)
    nr, nc = _i(), _i()
    r = lib().orc_create_big_matrix_nl(_i(addr.shape[1]), _ptr(_ip(vgrid)), _ptr(_ip(p_map)), _i(n), _ptr(tiles),
                                       _ptr(addr), _i(row_per_block), _i(col_per_block), _i(num_row_dim), _ptr(kr),
                                       _ptr(kv), _i(len(items)), _ptr(big), ctypes.byref(nr), ctypes.byref(nc))
    if r == -2:
        raise KeyError("a placed tile has no location")
    if r < 0:
        raise ValueError("tile pattern is not rectangular")
    return big.reshape(nr.value * row_per_block, nc.value * col_per_block)


def revert_big_matrix(vgrid, p_map, permuted_address, row_per_block, col_per_block, num_row_dim, big):
    addr = _ip(permuted_address)
    n = addr.shape[0]
    big = np.ascontiguousarray(big, dtype=np.float64)
    tiles = np.zeros((n, row_per_block * col_per_block), dtype=np.float64)
    r = lib().orc_revert_big_matrix(_i(addr.shape[1]), _ptr(_ip(vgrid)), _ptr(_ip(p_map)), _i(n),
                                    _ptr(addr), _i(row_per_block), _i(col_per_block), _i(num_row_dim),
                                    _ptr(big), _ptr(tiles))
    if r < 0:
        raise ValueError("tile pattern is not rectangular")
    return tiles


def local_contraction(n_a, n_b, n_k, A, B, C, at, bt, alpha):
    """local_contraction (localcontract.cc:3) with corrected leading dimensions; C updated in place."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    assert C.flags.c_contiguous and C.dtype == np.float64
    lib().orc_local_contraction(n_a, n_b, n_k, _ptr(A), _ptr(B), _ptr(C), at, bt, alpha)
    return C


def dltc_compute(m, n, k, a, b, c):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    lib().orc_dltc_compute(m, n, k, _ptr(a), _ptr(b), _ptr(c))
    return c


def task_mul(coef, idC, C, idA, A, idB, B, O, V, wbO, wbV, nocc, nnames):
    """DLTC task_mul tile loop (DLTC/task.cc:83) over dense tensors; C updated in place."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    rc = lib().orc_task_mul(coef, len(idC), _ptr(_ip(idC)), _ptr(C), len(idA), _ptr(_ip(idA)), _ptr(A),
                            len(idB), _ptr(_ip(idB)), _ptr(B), O, V, wbO, wbV, nocc, nnames)
    if rc != 0:
        raise ValueError("bad task_mul arguments")
    return C


def task_sum(coef, idC, C, idA, A, O, V, wbO, wbV, nocc):
    A = np.ascontiguousarray(A, dtype=np.float64)
    rc = lib().orc_task_sum(coef, len(idC), _ptr(_ip(idC)), _ptr(C), len(idA), _ptr(_ip(idA)), _ptr(A),
                            O, V, wbO, wbV, nocc)
    if rc != 0:
        raise ValueError("bad task_sum arguments")
    return C


def rrr_tiles(sym, vgrid):
    """Tile addresses of an RRR tensor on one process (tensor.cc:617-694), (n, dims) int32."""
    g = _ip(vgrid)
    n = lib().orc_rrr_tiles(sym.encode(), _ptr(g), None)
    out = np.zeros((n, len(sym)), dtype=np.int32)
    lib().orc_rrr_tiles(sym.encode(), _ptr(g), _ptr(out))
    return out


def rrr_block_values(addr):
    """Tensor::get_value (tensor.cc:744): every element of a block is sum_d sin(addr_d)."""
    addr = np.asarray(addr)
    v = np.zeros(addr.shape[0], dtype=np.float64)
    for d in range(addr.shape[1] - 1, -1, -1):
        v += np.sin(addr[:, d].astype(np.float64))
    return v


# ---- drand48 (POSIX), used by the reference's checkM / checkS --------------

class Drand48:
    """POSIX drand48: X <- (0x5DEECE66D * X + 0xB) mod 2^48, value X / 2^48.
    The default state (no srand48 call) is 0x1234ABCD330E."""

    def __init__(self, seed=None):
        self.x = 0x1234ABCD330E if seed is None else ((seed << 16) | 0x330E) & ((1 << 48) - 1)

    def next(self, n):
        out = np.empty(n, dtype=np.float64)
        x = self.x
        for i in range(n):
            x = (0x5DEECE66D * x + 0xB) & ((1 << 48) - 1)
            out[i] = x / float(1 << 48)
        self.x = x
        return out


def cc_integrals(system, P, Q, R, S):
    """<pq||rs> of an oracle.cc.System over the outer product of four orbital
    index lists (oracle/cc_ints.c; the same values as System.integral_values)."""
    idx = [np.ascontiguousarray(x, dtype=np.int64).reshape(-1) for x in (P, Q, R, S)]
    mag = np.ascontiguousarray(system.mag, dtype=np.float64)
    irr = np.ascontiguousarray(system.irrep, dtype=np.int64)
    out = np.empty([len(x) for x in idx])
    args = []
    for x in idx:
        args += [len(x), _ptr(x)]
    lib().orc_cc_integrals(system.seed_int, system.n, _ptr(mag), _ptr(irr), *args, _ptr(out))
    return out
