"""ORACLE (test infrastructure only) -- irrep-blocked FP64 coupled-cluster
iteration for systems too large for the dense oracle.

The same spin-orbital CCSD / CCD equations as ``oracle.cc`` (Stanton, Gauss,
Watts and Bartlett, J. Chem. Phys. 94, 4334 (1991), diagonal Fock operator,
explicit W_abef intermediate, Jacobi update from the MP2 guess), term for
term, but every tensor is stored as its nonzero irrep blocks: with the XOR
product rule a tensor element can be nonzero only when the irreps of its
indices multiply to the totally symmetric one, so a rank-r tensor is a dict
from irrep tuples (h_0, ..., h_{r-1}) with h_0 ^ ... ^ h_{r-1} = 0 to dense
blocks over the orbitals of those irreps.  Each contraction runs block pair
by block pair with numpy.tensordot (BLAS).  Orbitals of one irrep need not be
contiguous; block index arrays hold their orbital numbers.

The reference has no CC iteration (its DLTC tables DLTC/ccd-t2.cc:45-95,
DLTC/ccsd-t1.cc:40-109, DLTC/ccsd-t2.cc:55-216 are workload definitions), so
this is, like ``oracle.cc``, a restatement of a published formulation; its
integrals and orbitals come from ``oracle.cc.System``.  Pinned against the
dense oracle on small systems by tests/test_cc_blocks.py.
"""
import itertools
from collections import defaultdict

import numpy as np

from . import cc as occ


class Spaces:
    """Occupied / virtual orbitals of a system grouped by irrep."""

    def __init__(self, system):
        o = system.o
        irr = system.irrep
        nirrep = 1
        while nirrep < int(irr.max()) + 1:
            nirrep *= 2
        self.nirrep = nirrep
        self.system = system
        self.idx = {"o": [np.where(irr[:o] == h)[0] for h in range(nirrep)],
                    "v": [o + np.where(irr[o:] == h)[0] for h in range(nirrep)]}
        self.eps = system.eps
        self._keys = {}

    def keys(self, kinds):
        """Irrep tuples of the nonzero blocks of a tensor over these spaces."""
        if kinds not in self._keys:
            out = []
            for t in itertools.product(range(self.nirrep), repeat=len(kinds) - 1):
                h = 0
                for x in t:
                    h ^= x
                key = t + (h,)
                if all(len(self.idx[k][g]) for k, g in zip(kinds, key)):
                    out.append(key)
            self._keys[kinds] = out
        return self._keys[kinds]

    def shape(self, kinds, key):
        return tuple(len(self.idx[k][g]) for k, g in zip(kinds, key))

    def orbitals(self, kinds, key):
        """Orbital numbers along each index of a block, as broadcastable arrays."""
        r = len(kinds)
        out = []
        for d, (k, g) in enumerate(zip(kinds, key)):
            sh = [1] * r
            sh[d] = -1
            out.append(self.idx[k][g].astype(np.uint64).reshape(sh))
        return out


class BT:
    """A block tensor: kinds ('o'/'v' per index) and a dict of dense blocks."""

    def __init__(self, sp, kinds, blocks):
        self.sp, self.kinds, self.blocks = sp, kinds, blocks

    @staticmethod
    def zeros(sp, kinds):
        return BT(sp, kinds, {k: np.zeros(sp.shape(kinds, k)) for k in sp.keys(kinds)})

    @staticmethod
    def integrals(sp, kinds, fast=True):
        """Blocks of <pq||rs>: computed by oracle/cc_ints.c (fast) or by the
        numpy statement System.integral_values."""
        s = sp.system
        if fast:
            from . import cc_integrals
            return BT(sp, kinds, {k: cc_integrals(s, *[sp.idx[c][g] for c, g in zip(kinds, k)])
                                  for k in sp.keys(kinds)})
        return BT(sp, kinds, {k: s.integral_values(*sp.orbitals(kinds, k)) for k in sp.keys(kinds)})

    @staticmethod
    def from_dense(sp, kinds, dense, offsets):
        """Cut a dense tensor (index d over orbitals offsets[kind] + local) into blocks."""
        out = {}
        for k in sp.keys(kinds):
            ix = np.ix_(*[sp.idx[c][g] - offsets[c] for c, g in zip(kinds, k)])
            out[k] = np.ascontiguousarray(dense[ix])
        return BT(sp, kinds, out)

    def to_dense(self, offsets, sizes):
        d = np.zeros([sizes[c] for c in self.kinds])
        for k, b in self.blocks.items():
            d[np.ix_(*[self.sp.idx[c][g] - offsets[c] for c, g in zip(self.kinds, k)])] = b
        return d

    def map(self, f):
        return BT(self.sp, self.kinds, {k: f(b) for k, b in self.blocks.items()})

    def combine(self, other, f):
        assert self.kinds == other.kinds
        return BT(self.sp, self.kinds, {k: f(b, other.blocks[k]) for k, b in self.blocks.items()})

    def __add__(self, o):
        return self.combine(o, lambda x, y: x + y)

    def __sub__(self, o):
        return self.combine(o, lambda x, y: x - y)

    def __mul__(self, c):
        return self.map(lambda x: c * x)

    __rmul__ = __mul__

    def __truediv__(self, o):
        return self.combine(o, lambda x, y: x / y)

    def transpose(self, perm):
        kinds = "".join(self.kinds[p] for p in perm)
        return BT(self.sp, kinds, {tuple(k[p] for p in perm): np.transpose(b, perm) for k, b in self.blocks.items()})

    def vdot(self, o):
        return float(sum(np.sum(b * o.blocks[k]) for k, b in self.blocks.items()))

    def max_abs_diff_dense(self, dense, offsets):
        worst = 0.0
        for k, b in self.blocks.items():
            ix = np.ix_(*[self.sp.idx[c][g] - offsets[c] for c, g in zip(self.kinds, k)])
            if b.size:
                worst = max(worst, float(np.max(np.abs(dense[ix] - b))))
        return worst


def _parts(T, free, contr):
    """Blocks of T grouped by the irreps of its free indices, each block seen
    as a matrix (free x contracted, flag False) or (contracted x free, flag
    True) -- whichever its storage order gives without a copy -- sorted by
    the irreps of the contracted indices."""
    r = len(free) + len(contr)
    if free + contr == list(range(r)):
        order, tr = None, False
    elif contr + free == list(range(r)):
        order, tr = None, True
    else:
        order, tr = free + contr, False
    groups = defaultdict(list)
    for k, v in T.blocks.items():
        groups[tuple(k[i] for i in free)].append((tuple(k[i] for i in contr), v))
    out = {}
    for fk, lst in groups.items():
        lst.sort(key=lambda x: x[0])
        shp = [lst[0][1].shape[i] for i in free]
        F = int(np.prod(shp))
        mats = []
        for ck, v in lst:
            if order is not None:
                v = np.transpose(v, order)
            m = v.reshape((-1, F) if tr else (F, -1))
            mats.append((ck, m.T if tr else m))  # F x K_c (a view when tr)
        out[fk] = (shp, mats)
    return out


def einsum2(spec, A, B):
    """Two-operand contraction "ab,bc->ac" (every letter in exactly two of the
    three index lists) over block tensors.  For every output block (irreps of
    A's and of B's free indices) the block pairs over the matching contracted
    irreps are multiplied as matrices (BLAS) and summed -- or, when copying the
    operands is cheaper than summing the partial products, each operand's
    blocks are first packed side by side along the contracted index and every
    output block is one matrix product."""
    lhs, out = spec.split("->")
    la, lb = lhs.split(",")
    sp = A.sp
    kind = {c: A.kinds[i] for i, c in enumerate(la)}
    kind.update({c: B.kinds[i] for i, c in enumerate(lb)})
    out_kinds = "".join(kind[c] for c in out)
    shared = [c for c in la if c in lb]
    axA = [la.index(c) for c in shared]
    axB = [lb.index(c) for c in shared]
    freeA = [i for i, c in enumerate(la) if c not in shared]
    freeB = [i for i, c in enumerate(lb) if c not in shared]
    res = [la[i] for i in freeA] + [lb[i] for i in freeB]
    perm = [res.index(c) for c in out]
    ident = perm == list(range(len(perm)))
    PA = _parts(A, freeA, axA)
    PB = _parts(B, freeB, axB)
    # packed: operand bytes copied once; summed: every extra partial product
    # passes over its output block
    npairs = max(1, max((len(m) for _, m in PA.values()), default=1))
    size_a = sum(b.size for b in A.blocks.values())
    size_b = sum(b.size for b in B.blocks.values())
    size_c = sum(int(np.prod(sp.shape(out_kinds, k))) for k in sp.keys(out_kinds))
    pack = npairs > 1 and size_a + size_b < (npairs - 1) * size_c
    if pack:
        def packed(P):
            return {fk: (shp, [c for c, _ in mats], np.concatenate([m for _, m in mats], axis=1))
                    for fk, (shp, mats) in P.items()}
        QA, QB = packed(PA), packed(PB)
    C = {}
    for fa, (sa, ma) in PA.items():
        for fb, (sb, mb) in PB.items():
            if pack and QA[fa][1] == QB[fb][1]:
                r = QA[fa][2] @ QB[fb][2].T
            else:
                db = dict(mb)
                r = None
                for ck, a in ma:
                    b = db.get(ck)
                    if b is None:
                        continue
                    t = a @ b.T
                    if r is None:
                        r = t
                    else:
                        r += t
                if r is None:
                    continue
            irr = dict(zip([la[i] for i in freeA], fa))
            irr.update(zip([lb[i] for i in freeB], fb))
            kc = tuple(irr[c] for c in out)
            r = r.reshape(sa + sb)
            C[kc] = r if ident else np.ascontiguousarray(np.transpose(r, perm))
    for k in sp.keys(out_kinds):
        if k not in C:
            C[k] = np.zeros(sp.shape(out_kinds, k))
    return BT(sp, out_kinds, C)


def _pij(x):
    return x - x.transpose((1, 0, 2, 3))


def _pab(x):
    return x - x.transpose((0, 1, 3, 2))


INTEGRALS = ["oooo", "ooov", "oovv", "ovvo", "ovvv", "vvvv", "oovo", "ovov", "vvvo", "ovoo", "vovv"]


class CC:
    """Irrep-blocked CCD / CCSD Jacobi iteration from the MP2 guess; the same
    energies and amplitudes as oracle.cc.CC up to FP64 summation order."""

    def __init__(self, system, method="ccsd"):
        self.s, self.method = system, method
        sp = self.sp = Spaces(system)
        self.I = {k: BT.integrals(sp, k) for k in INTEGRALS}
        e = system.eps

        def denom(kinds, key):
            ix = sp.orbitals(kinds, key)
            out = 0.0
            for d, c in enumerate(kinds):
                ev = e[ix[d].astype(np.int64)]
                out = out + ev if c == "o" else out - ev
            return np.broadcast_to(out, sp.shape(kinds, key)).copy()

        self.D1 = BT(sp, "ov", {k: denom("ov", k) for k in sp.keys("ov")})
        self.D2 = BT(sp, "oovv", {k: denom("oovv", k) for k in sp.keys("oovv")})
        self.t1 = BT.zeros(sp, "ov")
        self.t2 = self.I["oovv"] / self.D2
        self.energies = [self.energy()]

    def taus(self):
        if self.method != "ccsd":
            return self.t2, self.t2
        t1 = self.t1
        x = einsum2("ia,jb->ijab", t1, t1) - einsum2("ib,ja->ijab", t1, t1)
        return self.t2 + x, self.t2 + 0.5 * x

    def energy(self):
        tau, _ = self.taus()
        return 0.25 * self.I["oovv"].vdot(tau)

    def iterate(self, niter=1):
        for _ in range(niter):
            R1, R2 = self.residuals()
            if self.method == "ccsd":
                self.t1 = R1 / self.D1
            self.t2 = R2 / self.D2
            self.energies.append(self.energy())
        return self.energies

    def residuals(self):
        I = self.I
        t2 = self.t2
        tau, taut = self.taus()
        sd = self.method == "ccsd"
        t1 = self.t1
        Fae = -0.5 * einsum2("mnaf,mnef->ae", taut, I["oovv"])
        Fmi = 0.5 * einsum2("inef,mnef->mi", taut, I["oovv"])
        Wmnij, Wabef, Wmbej, Q = I["oooo"], I["vvvv"], I["ovvo"], 0.5 * t2
        if sd:
            Fae = einsum2("mf,mafe->ae", t1, I["ovvv"]) + Fae
            Fmi = einsum2("ne,mnie->mi", t1, I["ooov"]) + Fmi
            Fme = einsum2("nf,mnef->me", t1, I["oovv"])
            X = einsum2("je,mnie->mnij", t1, I["ooov"])
            Wmnij = Wmnij + (X - X.transpose((0, 1, 3, 2)))
            X = einsum2("mb,amef->abef", t1, I["vovv"])
            XT = X.transpose((1, 0, 2, 3))
            W = {}
            for k, x in X.blocks.items():  # vvvv - (X - X^T), block by block
                w = x - XT.blocks[k]
                np.subtract(Wabef.blocks[k], w, out=w)
                W[k] = w
            Wabef = BT(self.sp, "vvvv", W)
            del X, XT
            Wmbej = Wmbej + einsum2("jf,mbef->mbej", t1, I["ovvv"]) - einsum2("nb,mnej->mbej", t1, I["oovo"])
            Q = Q + einsum2("jf,nb->jnfb", t1, t1)
        Wmnij = Wmnij + 0.25 * einsum2("ijef,mnef->mnij", tau, I["oovv"])
        T = einsum2("mnab,mnef->abef", tau, I["oovv"])
        if sd:
            for k, w in Wabef.blocks.items():  # in place: W += 0.25 T
                w += 0.25 * T.blocks[k]
        else:
            Wabef = Wabef + 0.25 * T
        del T
        Wmbej = Wmbej - einsum2("jnfb,mnef->mbej", Q, I["oovv"])
        R1 = None
        if sd:
            R1 = (einsum2("ie,ae->ia", t1, Fae) - einsum2("ma,mi->ia", t1, Fmi) + einsum2("imae,me->ia", t2, Fme)
                  - einsum2("nf,naif->ia", t1, I["ovov"]) - 0.5 * einsum2("imef,maef->ia", t2, I["ovvv"])
                  - 0.5 * einsum2("mnae,nmei->ia", t2, I["oovo"]))
            Fbe = Fae - 0.5 * einsum2("mb,me->be", t1, Fme)
            Fmj = Fmi + 0.5 * einsum2("je,me->mj", t1, Fme)
        else:
            Fbe, Fmj = Fae, Fmi
        inner = einsum2("imae,mbej->ijab", t2, Wmbej)
        if sd:
            Y = einsum2("ie,mbej->imbj", t1, I["ovvo"])
            inner = inner - einsum2("ma,imbj->ijab", t1, Y)
        R2 = (I["oovv"] + _pab(einsum2("ijae,be->ijab", t2, Fbe)) - _pij(einsum2("imab,mj->ijab", t2, Fmj))
              + 0.5 * einsum2("mnab,mnij->ijab", tau, Wmnij) + 0.5 * einsum2("ijef,abef->ijab", tau, Wabef)
              + _pij(_pab(inner)))
        if sd:
            R2 = R2 + _pij(einsum2("ie,abej->ijab", t1, I["vvvo"])) - _pab(einsum2("ma,mbij->ijab", t1, I["ovoo"]))
        return R1, R2

    def dense_t2(self):
        o, v = self.s.o, self.s.v
        return self.t2.to_dense({"o": 0, "v": o}, {"o": o, "v": v})

    def dense_t1(self):
        o, v = self.s.o, self.s.v
        return self.t1.to_dense({"o": 0, "v": o}, {"o": o, "v": v})


def system(nocc, nvir, nirrep=1, max_block=16, min_block=1, seed=1):
    return occ.System(nocc, nvir, nirrep=nirrep, max_block=max_block, min_block=min_block, seed=seed)
