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
import time

import numpy as np

SPACES = {"t1": "ov", "t2": "oovv", "tau": "oovv", "taut": "oovv", "Xa": "oovv", "Q": "oovv", "R2": "oovv",
          "R1": "ov", "Fae": "vv", "Fbe": "vv", "Fmi": "oo", "Fmj": "oo", "Fme": "ov", "Wmnij": "oooo",
          "Xoooo": "oooo", "Wmbej": "ovvo", "Zp": "ooov", "V3": "oovo", "Lad": "oovv"}

# Intermediates stored as canonical tiles only (antisymmetric index pairs, as
# RRR stores unique blocks, tensor.cc:617-640): C positions of each pair.
CANONICAL = {"Wmnij": [(0, 1), (2, 3)], "Lad": [(0, 1), (2, 3)], "Zp": [(0, 1)]}


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
    L += [("Xa", "ijab", "t2", "ijae", "Fbe" if sd else "Fae", "be"),
          ("Xa", "ijab", "t2", "imab", "Fmj" if sd else "Fmi", "mj"),
          ("Lad", "ijab", tau, "mnab", "Wmnij", "mnij"),
          ("Lad", "ijab", "VVVV", "abef", tau, "ijef")]
    if sd:
        L += [("Zp", "ijma", tau, "ijef", "OVVV", "maef"), ("Xa", "ijab", "Zp", "ijma", "t1", "mb")]
    L += [("Xa", "ijab", "t2", "imae", "Wmbej", "mbej")]
    if sd:
        L += [("V3", "imbj", "t1", "ie", "OVVO", "mbej"), ("Xa", "ijab", "t1", "ma", "V3", "imbj"),
              ("Xa", "ijab", "t1", "ie", "VVVO", "abej"), ("Xa", "ijab", "t1", "ma", "OVOO", "mbij")]
    return L


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


def gemm_shapes(system, method="ccsd"):
    """Per-irrep (M, N, K) of every contraction of one iteration."""
    nirrep, counts = _irrep_counts(system)
    shapes = []
    for C, lc, A, la, B, lb in contraction_list(method):
        sa = spaces(A)
        con = "".join(sa[i] for i, l in enumerate(la) if l in lb)
        M = _ext_counts(system, counts, nirrep, C, lc, A, la)
        N = _ext_counts(system, counts, nirrep, C, lc, B, lb)
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
