"""ORACLE (test infrastructure only) -- dense FP64 coupled-cluster iteration.

The DTCF reference contains no CC iteration (its DLTC residual tables,
DLTC/ccd-t2.cc:45-95, DLTC/ccsd-t1.cc:40-109, DLTC/ccsd-t2.cc:55-216, are
workload definitions without permutation operators, coefficients or a Jacobi
update), so this oracle restates a published formulation instead: the
spin-orbital CCSD equations of Stanton, Gauss, Watts and Bartlett,
J. Chem. Phys. 94, 4334 (1991), with a diagonal Fock operator, written
directly with numpy.einsum on dense tensors -- including the explicit W_abef
intermediate that the GPU driver factorises away.  CCD is the same with
T1 = 0.  The synthetic system (orbital irreps, orbital energies, <pq||rs>) is
restated from its definition independently of the product code.
"""
import math

import numpy as np

M64 = (1 << 64) - 1
GOLD = 0x9E3779B97F4A7C15


def mix64(z):
    z &= M64
    z ^= z >> 30
    z = (z * 0xBF58476D1CE4E5B9) & M64
    z ^= z >> 27
    z = (z * 0x94D049BB133111EB) & M64
    z ^= z >> 31
    return z


class Stream:
    """splitmix64 stream k of a seed."""

    def __init__(self, seed, k):
        self.state = mix64(seed ^ ((GOLD * (k + 1)) & M64))

    def next(self):
        self.state = (self.state + GOLD) & M64
        return mix64(self.state)

    def uniform(self):
        return (self.next() >> 11) * 2.0 ** -53


def irrep_counts(n, nirrep, min_block, seed, stream):
    rng = Stream(seed, stream)
    need = min(min_block, n // nirrep)
    while True:
        c = [0] * nirrep
        for _ in range(n):
            h = min(int(rng.uniform() * nirrep), nirrep - 1)
            c[h] += 1
        if nirrep == 1 or min(c) >= need:
            return c


def blocks(counts, max_block):
    ext, irr = [], []
    for h, c in enumerate(counts):
        if c == 0:
            continue
        nb = -(-c // max_block)
        for k in range(nb):
            ext.append(c // nb + (1 if k < c % nb else 0))
            irr.append(h)
    return ext, irr


class System:
    """Orbitals, orbital energies and dense <pq||rs> of the synthetic system."""

    def __init__(self, nocc, nvir, nirrep=1, max_block=16, min_block=1, seed=1, eps_occ=(-2.0, -0.5),
                 eps_vir=(0.2, 3.0), v_scale=1e-2, v_decay=8.0):
        self.o, self.v, self.n = nocc, nvir, nocc + nvir
        eo, io = blocks(irrep_counts(nocc, nirrep, min_block, seed, 1), max_block)
        ev, iv = blocks(irrep_counts(nvir, nirrep, min_block, seed, 2), max_block)
        self.occ_blocks, self.vir_blocks = list(zip(eo, io)), list(zip(ev, iv))
        self.irrep = np.array([h for e, h in zip(eo, io) for _ in range(e)] +
                              [h for e, h in zip(ev, iv) for _ in range(e)], dtype=np.int64)
        so, sv, si = Stream(seed, 3), Stream(seed, 4), Stream(seed, 5)
        self.eps = np.array([eps_occ[0] + (eps_occ[1] - eps_occ[0]) * so.uniform() for _ in range(nocc)] +
                            [eps_vir[0] + (eps_vir[1] - eps_vir[0]) * sv.uniform() for _ in range(nvir)])
        self.seed_int = si.next()
        self.mag = np.array([v_scale * math.exp(-d / v_decay) for d in range(2 * self.n + 1)])

    def integrals(self):
        """Dense antisymmetrised <pq||rs>, shape (n, n, n, n)."""
        ar = np.arange(self.n, dtype=np.uint64)
        return self.integral_values(ar[:, None, None, None], ar[None, :, None, None], ar[None, None, :, None],
                                    ar[None, None, None, :])

    def integral_values(self, p, q, r, s):
        """<pq||rs> at broadcastable arrays of orbital indices (uint64)."""
        p, q, r, s = np.broadcast_arrays(*[np.asarray(x, dtype=np.uint64) for x in (p, q, r, s)])
        n = self.n
        sg = np.ones(p.shape)
        swap = p > q
        sg[swap] *= -1
        a, b = np.where(swap, q, p), np.where(swap, p, q)
        swap = r > s
        sg[swap] *= -1
        c, d = np.where(swap, s, r), np.where(swap, r, s)
        P, R = a * np.uint64(n) + b, c * np.uint64(n) + d
        P2, R2 = np.minimum(P, R), np.maximum(P, R)
        with np.errstate(over="ignore"):
            key = np.uint64(self.seed_int) ^ (P2 * np.uint64(GOLD) + R2 * np.uint64(0xC2B2AE3D27D4EB4F))
            z = key
            z = z ^ (z >> np.uint64(30))
            z = z * np.uint64(0xBF58476D1CE4E5B9)
            z = z ^ (z >> np.uint64(27))
            z = z * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        mag = self.mag[((b - a) + (d - c)).astype(np.int64)]
        val = np.where((z >> np.uint64(63)) != 0, -mag, mag) * sg
        ir = self.irrep
        zero = (p == q) | (r == s) | ((ir[p.astype(np.int64)] ^ ir[q.astype(np.int64)] ^ ir[r.astype(np.int64)]
                                       ^ ir[s.astype(np.int64)]) != 0)
        val[zero] = 0.0
        return val


def _pij(x):
    """P(ij) on an ijab-ordered tensor."""
    return x - x.transpose(1, 0, 2, 3)


def _pab(x):
    """P(ab) on an ijab-ordered tensor."""
    return x - x.transpose(0, 1, 3, 2)


class CC:
    """Dense CCD / CCSD Jacobi iteration from the MP2 guess."""

    def __init__(self, system, method="ccsd"):
        self.s, self.method = system, method
        o, n = system.o, system.n
        V = system.integrals()
        O, Vs = slice(0, o), slice(o, n)
        self.I = {}
        for name in ["oooo", "ooov", "oovv", "ovvo", "ovvv", "vvvv", "oovo", "ovov", "vvvo", "ovoo", "vovv"]:
            sl = tuple(O if c == "o" else Vs for c in name)
            self.I[name] = np.ascontiguousarray(V[sl])
        e = system.eps
        eo, ev = e[:o], e[o:]
        self.D1 = eo[:, None] - ev[None, :]
        self.D2 = ((eo[:, None, None, None] + eo[None, :, None, None]) - ev[None, None, :, None]) - ev[None, None, None, :]
        self.t1 = np.zeros((o, system.v))
        self.t2 = self.I["oovv"] / self.D2
        self.energies = [self.energy()]

    def taus(self):
        t1, t2 = self.t1, self.t2
        x = np.einsum("ia,jb->ijab", t1, t1) - np.einsum("ib,ja->ijab", t1, t1)
        return t2 + x, t2 + 0.5 * x

    def energy(self):
        tau, _ = self.taus()
        return 0.25 * float(np.sum(self.I["oovv"] * tau))

    def iterate(self, niter=1):
        for _ in range(niter):
            R1, R2 = self.residuals()
            if self.method == "ccsd":
                self.t1 = R1 / self.D1
            self.t2 = R2 / self.D2
            self.energies.append(self.energy())
        return self.energies

    def residuals(self):
        """Right-hand sides R1, R2 (T = R / D) at the current amplitudes."""
        I = self.I
        if True:
            t1, t2 = self.t1, self.t2
            tau, taut = self.taus()
            Fae = np.einsum("mf,mafe->ae", t1, I["ovvv"]) - 0.5 * np.einsum("mnaf,mnef->ae", taut, I["oovv"])
            Fmi = np.einsum("ne,mnie->mi", t1, I["ooov"]) + 0.5 * np.einsum("inef,mnef->mi", taut, I["oovv"])
            Fme = np.einsum("nf,mnef->me", t1, I["oovv"])
            X = np.einsum("je,mnie->mnij", t1, I["ooov"])
            Wmnij = I["oooo"] + (X - X.transpose(0, 1, 3, 2)) + 0.25 * np.einsum("ijef,mnef->mnij", tau, I["oovv"])
            X = np.einsum("mb,amef->abef", t1, I["vovv"])
            Wabef = I["vvvv"] - (X - X.transpose(1, 0, 2, 3)) + 0.25 * np.einsum("mnab,mnef->abef", tau, I["oovv"])
            Wmbej = (I["ovvo"] + np.einsum("jf,mbef->mbej", t1, I["ovvv"]) - np.einsum("nb,mnej->mbej", t1, I["oovo"])
                     - np.einsum("jnfb,mnef->mbej", 0.5 * t2 + np.einsum("jf,nb->jnfb", t1, t1), I["oovv"]))
            R1 = (np.einsum("ie,ae->ia", t1, Fae) - np.einsum("ma,mi->ia", t1, Fmi) + np.einsum("imae,me->ia", t2, Fme)
                  - np.einsum("nf,naif->ia", t1, I["ovov"]) - 0.5 * np.einsum("imef,maef->ia", t2, I["ovvv"])
                  - 0.5 * np.einsum("mnae,nmei->ia", t2, I["oovo"]))
            Fbe = Fae - 0.5 * np.einsum("mb,me->be", t1, Fme)
            Fmj = Fmi + 0.5 * np.einsum("je,me->mj", t1, Fme)
            R2 = (I["oovv"] + _pab(np.einsum("ijae,be->ijab", t2, Fbe)) - _pij(np.einsum("imab,mj->ijab", t2, Fmj))
                  + 0.5 * np.einsum("mnab,mnij->ijab", tau, Wmnij) + 0.5 * np.einsum("ijef,abef->ijab", tau, Wabef)
                  + _pij(_pab(np.einsum("imae,mbej->ijab", t2, Wmbej)
                              - np.einsum("ie,ma,mbej->ijab", t1, t1, I["ovvo"])))
                  + _pij(np.einsum("ie,abej->ijab", t1, I["vvvo"])) - _pab(np.einsum("ma,mbij->ijab", t1, I["ovoo"])))
            return R1, R2
