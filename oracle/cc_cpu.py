"""ORACLE (test infrastructure only) -- CPU timing of one CC iteration along
the reference's node-local algorithm.

The reference executes each contraction as permute -> pack into one big
matrix -> one dgemm (Contraction::transpose_and_dgemm + kevin_dgemm,
contraction.cc:1779-2002; DLTC task_mul, DLTC/task.cc:83-137).  With spatial
symmetry the packed operands are block diagonal by irrep, so one contraction
is one dgemm per irrep h with M_h = number of external index tuples of A with
irrep product h, N_h likewise for B and K_h for the contracted tuples.  This
module derives those shapes from the synthetic system's irrep occupations
(independently of the product's planner) for the contraction list of one
CCSD / CCD iteration, and times the dgemms with numpy's multithreaded BLAS.
"""
import concurrent.futures
import ctypes
import glob
import os
import time

import numpy as np

SPACES = {"t1": "ov", "t2": "oovv", "tau": "oovv", "taut": "oovv", "Xa": "oovv", "Xb": "oovv", "Xj": "oovv",
          "Q": "oovv", "R2": "oovv",
          "R1": "ov", "Fae": "vv", "Fbe": "vv", "Fmi": "oo", "Fmj": "oo", "Fme": "ov", "Wmnij": "oooo",
          "Xoooo": "oooo", "Wmbej": "ovvo", "Zp": "ooov", "V3": "oovo", "Lad": "oovv"}

# Intermediates stored as canonical tiles only (antisymmetric index pairs, as
# RRR stores unique blocks, tensor.cc:617-640): C positions of each pair.
CANONICAL = {"Wmnij": [(0, 1), (2, 3)], "Lad": [(0, 1), (2, 3)], "Zp": [(0, 1)], "Xb": [(0, 1)], "Xj": [(2, 3)]}


def spaces(name):
    if name in SPACES:
        return SPACES[name]
    return name.lower()  # integral blocks, e.g. "OVVV" -> "ovvv"


def contraction_list(method="ccsd"):
    """(C, lc, A, la, B, lb) of one iteration, in execution order.

    Only contractions over at least one index are dgemms: the outer products
    t1 (x) t1 inside tau, taut and Q (no contracted index) are formed element
    by element together with those tensors, as are all permuted sums."""
    sd = method == "ccsd"
    L = []
    tau, taut = ("tau", "taut") if sd else ("t2", "t2")
    if sd:
        L += [("Fae", "ae", "t1", "mf", "OVVV", "mafe")]
    L += [("Fae", "ae", taut, "mnaf", "OOVV", "mnef")]
    if sd:
        L += [("Fmi", "mi", "t1", "ne", "OOOV", "mnie")]
    L += [("Fmi", "mi", taut, "inef", "OOVV", "mnef")]
    if sd:
        L += [("Fme", "me", "t1", "nf", "OOVV", "mnef"), ("Xoooo", "mnij", "t1", "je", "OOOV", "mnie")]
    L += [("Wmnij", "mnij", tau, "ijef", "OOVV", "mnef")]
    if sd:
        L += [("Wmbej", "mbej", "t1", "jf", "OVVV", "mbef"), ("Wmbej", "mbej", "t1", "nb", "OOVO", "mnej")]
    L += [("Wmbej", "mbej", "Q", "jnfb", "OOVV", "mnef")]
    if sd:
        L += [("R1", "ia", "t1", "ie", "Fae", "ae"), ("R1", "ia", "t1", "ma", "Fmi", "mi"),
              ("R1", "ia", "t2", "imae", "Fme", "me"), ("R1", "ia", "t1", "nf", "OVOV", "naif"),
              ("R1", "ia", "t2", "imef", "OVVV", "maef"), ("R1", "ia", "t2", "mnae", "OOVO", "nmei"),
              ("Fbe", "be", "t1", "mb", "Fme", "me"), ("Fmj", "mj", "t1", "je", "Fme", "me")]
    L += [("Xb", "ijab", "t2", "ijae", "Fbe" if sd else "Fae", "be"),
          ("Xj", "ijab", "t2", "imab", "Fmj" if sd else "Fmi", "mj"),
          ("Lad", "ijab", tau, "mnab", "Wmnij", "mnij"),
          ("Lad", "ijab", "VVVV", "abef", tau, "ijef")]
    if sd:
        L += [("Zp", "ijma", tau, "ijef", "OVVV", "maef"), ("Xb", "ijab", "Zp", "ijma", "t1", "mb")]
    L += [("Xa", "ijab", "t2", "imae", "Wmbej", "mbej")]
    if sd:
        L += [("V3", "imbj", "t1", "ie", "OVVO", "mbej"), ("Xa", "ijab", "t1", "ma", "V3", "imbj"),
              ("Xj", "ijab", "t1", "ie", "VVVO", "abej"), ("Xb", "ijab", "t1", "ma", "OVOO", "mbij")]
    return L


# Contractions whose two operands are both antisymmetric in a pair of
# contracted indices (tau, taut, t2, W_mnij and the <pq||rs> blocks): the
# product's planner runs their GEMMs over block pairs x >= y only (the
# off-diagonal pairs weighted 2).  Keyed by (C, la, lb).
PAIRS = {("Fae", "mnaf", "mnef"): "mn", ("Fmi", "inef", "mnef"): "ef", ("Wmnij", "ijef", "mnef"): "ef",
         ("R1", "imef", "maef"): "ef", ("R1", "mnae", "nmei"): "mn", ("Lad", "mnab", "mnij"): "mn",
         ("Lad", "abef", "ijef"): "ef", ("Zp", "ijef", "maef"): "ef"}


def _irrep_counts(system):
    n_irr = int(system.irrep.max()) + 1
    nirrep = 1
    while nirrep < n_irr:
        nirrep *= 2
    co = np.bincount(system.irrep[: system.o], minlength=nirrep)
    cv = np.bincount(system.irrep[system.o:], minlength=nirrep)
    return nirrep, {"o": co, "v": cv}


def _conv(counts, sp, nirrep):
    """Number of index tuples over the spaces sp with each irrep product."""
    out = np.zeros(nirrep, dtype=np.int64)
    out[0] = 1
    for c in sp:
        nxt = np.zeros(nirrep, dtype=np.int64)
        for h in range(nirrep):
            for g in range(nirrep):
                nxt[h ^ g] += out[h] * counts[c][g]
        out = nxt
    return out


def _conv_canonical(system, sp, pairs, nirrep):
    """_conv over block tuples of the spaces sp whose block indices are
    non-increasing on every position pair in pairs (element counts)."""
    blocks = {"o": system.occ_blocks, "v": system.vir_blocks}
    out = np.zeros(nirrep, dtype=np.int64)

    def rec(pos, idx, h, size):
        if pos == len(sp):
            out[h] += size
            return
        for b, (ext, irr) in enumerate(blocks[sp[pos]]):
            ok = all(not (j == pos and i < pos and idx[i] < b) and not (i == pos and j < pos and b < idx[j])
                     for i, j in pairs)
            if ok:
                idx.append(b)
                rec(pos + 1, idx, h ^ irr, size * ext)
                idx.pop()

    rec(0, [], 0, 1)
    return out


def _ext_counts(system, counts, nirrep, C, lc, X, lx):
    """Counts of the external index tuples of operand X (labels lx) that C needs."""
    sx = spaces(X)
    pos = [i for i, l in enumerate(lx) if l in lc]
    sp = "".join(sx[i] for i in pos)
    ext = [lx[i] for i in pos]
    pairs = [(ext.index(lc[ci]), ext.index(lc[cj])) for ci, cj in CANONICAL.get(C, [])
             if lc[ci] in ext and lc[cj] in ext]
    if not pairs:
        return _conv(counts, sp, nirrep)
    return _conv_canonical(system, sp, pairs, nirrep)


def gemm_shapes(system, method="ccsd", pairs=True):
    """Per-irrep (M, N, K) of every contraction of one iteration.  pairs:
    contracted extents over the block pairs x >= y of PAIRS, as the
    product's planner packs them; False: every contracted block tuple, as
    the reference's algorithm computes them."""
    nirrep, counts = _irrep_counts(system)
    shapes = []
    for C, lc, A, la, B, lb in contraction_list(method):
        sa = spaces(A)
        cl = [l for l in la if l in lb]
        con = "".join(sa[i] for i, l in enumerate(la) if l in lb)
        M = _ext_counts(system, counts, nirrep, C, lc, A, la)
        N = _ext_counts(system, counts, nirrep, C, lc, B, lb)
        pr = PAIRS.get((C, la, lb)) if pairs else None
        if pr:
            K = _conv_canonical(system, con, [(cl.index(pr[0]), cl.index(pr[1]))], nirrep)
        else:
            K = _conv(counts, con, nirrep)
        for h in range(nirrep):
            if M[h] and N[h] and K[h]:
                shapes.append((int(M[h]), int(N[h]), int(K[h])))
    return shapes


def flops(shapes):
    return float(sum(2.0 * m * n * k for m, n, k in shapes))


class IterationGemms:
    """Pre-allocated operands for the dgemms of one iteration."""

    def __init__(self, shapes, seed=0):
        rng = np.random.default_rng(seed)
        self.ops = []
        for m, n, k in shapes:
            a = rng.uniform(-1, 1, (m, k))
            b = rng.uniform(-1, 1, (n, k))
            self.ops.append((a, b, np.empty((m, n))))

    def run(self):
        for a, b, c in self.ops:
            np.matmul(a, b.T, out=c)

    def time(self, reps=1):
        self.run()
        t = time.perf_counter()
        for _ in range(reps):
            self.run()
        return (time.perf_counter() - t) / reps


def _factor(x, cap=64):
    """x = a * b with b the largest divisor of x not above cap."""
    for b in range(min(cap, x), 0, -1):
        if x % b == 0:
            return x // b, b
    return x, 1


class IterationLeaves:
    """The reference's node-local leaf algorithm for every packed GEMM of one
    iteration (Contraction::transpose_and_dgemm, contraction.cc:1779-2002;
    DLTC task_mul, DLTC/task.cc:83-137): both operands permuted from tile
    storage into the packed externals-by-contracted layout (the per-block
    transpose + create_big_matrix copy, done here as one strided copy per
    operand), one dgemm, and the product permuted back and accumulated into
    C's tile storage (revert_big_matrix + inverse transpose + accumulate, one
    strided pass).  Copies run on `threads` host threads (row slabs), the
    dgemm on BLAS's threads."""

    def __init__(self, shapes, seed=0, threads=None):
        rng = np.random.default_rng(seed)
        self.threads = threads or os.cpu_count() or 1
        self.pool = concurrent.futures.ThreadPoolExecutor(self.threads) if self.threads > 1 else None
        self.ops = []
        for m, n, k in shapes:
            ma, mb = _factor(m)
            ka, kb = _factor(k)
            na, nb = _factor(n)
            a_src = rng.uniform(-1, 1, (ma, ka, mb, kb))
            b_src = rng.uniform(-1, 1, (na, ka, nb, kb))
            c_dst = np.zeros((ma, na, mb, nb))
            self.ops.append((a_src, b_src, c_dst, np.empty((ma, mb, ka, kb)), np.empty((na, nb, ka, kb)),
                             np.empty((m, n)), (m, n, k)))

    def _par(self, fn, rows):
        if self.pool is None or rows < 2:
            fn(0, rows)
            return
        step = -(-rows // self.threads)
        list(self.pool.map(lambda lo: fn(lo, min(rows, lo + step)), range(0, rows, step)))

    def run(self):
        for a_src, b_src, c_dst, a_pk, b_pk, c, (m, n, k) in self.ops:
            def pack(lo, hi, src=a_src, dst=a_pk):
                dst[lo:hi] = src[lo:hi].transpose(0, 2, 1, 3)
            self._par(pack, a_src.shape[0])
            self._par(lambda lo, hi: pack(lo, hi, b_src, b_pk), b_src.shape[0])
            np.matmul(a_pk.reshape(m, k), b_pk.reshape(n, k).T, out=c)
            c4 = c.reshape(c_dst.shape[0], c_dst.shape[2], c_dst.shape[1], c_dst.shape[3])

            def unpack(lo, hi, c4=c4, dst=c_dst):
                dst[lo:hi] += c4[lo:hi].transpose(0, 2, 1, 3)
            self._par(unpack, c_dst.shape[0])

    def close(self):
        if self.pool is not None:
            self.pool.shutdown()


def blas_threads(n):
    """Set the thread count of numpy's bundled OpenBLAS (returns the previous
    count, or None when the library or its symbols are not found)."""
    import numpy
    libs = glob.glob(os.path.join(os.path.dirname(numpy.__file__), "..", "numpy.libs", "*openblas*"))
    for path in libs:
        try:
            lib = ctypes.CDLL(path)
        except OSError:
            continue
        for get_name, set_name in (("scipy_openblas_get_num_threads64_", "scipy_openblas_set_num_threads64_"),
                                   ("openblas_get_num_threads64_", "openblas_set_num_threads64_"),
                                   ("openblas_get_num_threads", "openblas_set_num_threads")):
            g, s = getattr(lib, get_name, None), getattr(lib, set_name, None)
            if g is not None and s is not None:
                g.restype = ctypes.c_int
                prev = g()
                s.argtypes = [ctypes.c_int]
                s(int(n))
                return prev
    return None
