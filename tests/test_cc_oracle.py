"""CPU checks of the coupled-cluster oracle: the synthetic Hamiltonian has the
symmetries it claims, the iteration converges, and the factorised ladder the
GPU driver executes is algebraically the oracle's W_abef form."""
import numpy as np
import pytest

from oracle import cc


@pytest.fixture(scope="module")
def small():
    return cc.System(6, 14, nirrep=2, max_block=5, seed=3)


def test_integral_symmetries(small):
    V = small.integrals()
    assert np.array_equal(V, -V.transpose(1, 0, 2, 3))
    assert np.array_equal(V, -V.transpose(0, 1, 3, 2))
    assert np.array_equal(V, V.transpose(2, 3, 0, 1))
    ir = small.irrep
    nz = np.argwhere(V != 0)
    assert np.all((ir[nz[:, 0]] ^ ir[nz[:, 1]] ^ ir[nz[:, 2]] ^ ir[nz[:, 3]]) == 0)
    n = small.n
    p, q, r, s = 1, 4, 2, 7
    assert abs(abs(V[p, q, r, s]) - 1e-2 * np.exp(-((q - p) + (s - r)) / 8.0)) < 1e-18 or V[p, q, r, s] == 0


def test_orbital_generator_blocks():
    s = cc.System(48, 240, nirrep=8, max_block=40, min_block=4, seed=1)
    ext_o = [e for e, _ in s.occ_blocks]
    ext_v = [e for e, _ in s.vir_blocks]
    assert sum(ext_o) == 48 and sum(ext_v) == 240
    assert min(ext_o + ext_v) >= 4 and max(ext_o + ext_v) <= 40
    assert len(set(h for _, h in s.occ_blocks)) == 8


@pytest.mark.parametrize("method", ["ccd", "ccsd"])
def test_iteration_converges(small, method):
    c = cc.CC(small, method)
    e = c.iterate(12)
    d = np.abs(np.diff(e))
    assert d[-1] < 1e-9 and d[-1] < d[1]
    assert e[-1] < 0


def _factorised_R2(c):
    """The T2 residual as the GPU driver builds it (bare <ab||ef> ladder plus
    the Z' and folded W_mnij terms), restated in numpy."""
    I, t1, t2 = c.I, c.t1, c.t2
    tau, taut = c.taus()
    ein = np.einsum
    Fae = ein("mf,mafe->ae", t1, I["ovvv"]) - 0.5 * ein("mnaf,mnef->ae", taut, I["oovv"])
    Fmi = ein("ne,mnie->mi", t1, I["ooov"]) + 0.5 * ein("inef,mnef->mi", taut, I["oovv"])
    Fme = ein("nf,mnef->me", t1, I["oovv"])
    X = ein("je,mnie->mnij", t1, I["ooov"])
    W = I["oooo"] + X - X.transpose(0, 1, 3, 2) + 0.5 * ein("ijef,mnef->mnij", tau, I["oovv"])
    Wmbej = (I["ovvo"] + ein("jf,mbef->mbej", t1, I["ovvv"]) - ein("nb,mnej->mbej", t1, I["oovo"])
             - ein("jnfb,mnef->mbej", 0.5 * t2 + ein("jf,nb->jnfb", t1, t1), I["oovv"]))
    Fbe = Fae - 0.5 * ein("mb,me->be", t1, Fme)
    Fmj = Fmi + 0.5 * ein("je,me->mj", t1, Fme)
    R2 = I["oovv"].copy()
    Xa = ein("ijae,be->ijab", t2, Fbe)
    R2 += Xa - Xa.transpose(0, 1, 3, 2)
    Xa = ein("imab,mj->ijab", t2, Fmj)
    R2 += -Xa + Xa.transpose(1, 0, 2, 3)
    R2 += 0.5 * ein("mnab,mnij->ijab", tau, W)
    R2 += 0.5 * ein("abef,ijef->ijab", I["vvvv"], tau)
    Zp = ein("ijef,maef->ijma", tau, I["ovvv"])
    Xa = ein("ijma,mb->ijab", Zp, t1)
    R2 += 0.5 * Xa - 0.5 * Xa.transpose(0, 1, 3, 2)
    Xa = ein("imae,mbej->ijab", t2, Wmbej)
    V3 = ein("ie,mbej->imbj", t1, I["ovvo"])
    Xa -= ein("ma,imbj->ijab", t1, V3)
    R2 += Xa - Xa.transpose(1, 0, 2, 3) - Xa.transpose(0, 1, 3, 2) + Xa.transpose(1, 0, 3, 2)
    Xa = ein("ie,abej->ijab", t1, I["vvvo"])
    R2 += Xa - Xa.transpose(1, 0, 2, 3)
    Xa = ein("ma,mbij->ijab", t1, I["ovoo"])
    R2 += -Xa + Xa.transpose(0, 1, 3, 2)
    return R2


def test_factorised_ladder_equals_wabef_form(small):
    c = cc.CC(small, "ccsd")
    c.iterate(2)   # non-zero T1
    _, want = c.residuals()
    got = _factorised_R2(c)
    assert np.max(np.abs(got - want)) < 1e-15
