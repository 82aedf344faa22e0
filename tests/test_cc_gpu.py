"""GPU parity of the coupled-cluster driver against the dense FP64 oracle:
orbitals and energies of the synthetic system bit-identical, per-iteration
correlation energy within 1e-10 Eh, amplitudes within 1e-12."""
import numpy as np
import pytest

from oracle import cc as occ

pytestmark = pytest.mark.gpu

CASES = [
    dict(nocc=6, nvir=14, nirrep=2, max_block=5, seed=3),
    dict(nocc=8, nvir=24, nirrep=4, max_block=4, min_block=1, seed=7),
    dict(nocc=8, nvir=20, nirrep=1, max_block=8, seed=11),
]


def _system(c):
    return occ.System(c["nocc"], c["nvir"], nirrep=c["nirrep"], max_block=c["max_block"],
                      min_block=c.get("min_block", 1), seed=c["seed"])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("method", ["ccd", "ccsd"])
def test_cc_fp64_matches_oracle(case, method):
    from dtcf_gb300.cc import Job
    job = Job(method=method, engine="fp64", **case)
    sysm = _system(case)
    irr, eps = job.orbitals()
    assert np.array_equal(irr, sysm.irrep)
    assert np.array_equal(eps, sysm.eps)
    ref = occ.CC(sysm, method)
    e_ref = ref.iterate(6)
    e_gpu = np.concatenate([job.energies()[:1], job.iterate(6)])
    assert np.max(np.abs(e_gpu - np.array(e_ref))) <= 1e-10, (e_gpu, e_ref)
    t1, t2 = job.amplitudes()
    assert np.max(np.abs(t2 - ref.t2)) <= 1e-12
    assert np.max(np.abs(t1 - ref.t1)) <= 1e-12
    job.close()


def test_cc_graph_and_eager_identical():
    from dtcf_gb300.cc import Job
    case = CASES[1]
    a = Job(method="ccsd", use_graph=1, **case)
    b = Job(method="ccsd", use_graph=0, **case)
    ea, eb = a.iterate(4), b.iterate(4)
    assert np.array_equal(ea, eb)
    st = a.stats()
    from oracle import cc_cpu
    assert st.flops_per_iter > 0 and st.ncontractions == len(cc_cpu.contraction_list("ccsd"))


@pytest.mark.parametrize("method", ["ccd", "ccsd"])
def test_cc_split_engine_energy_within_1e10(method):
    """Split engine on every GEMM (6 slices): per-iteration correlation energy
    within 1e-10 Eh of the FP64 oracle."""
    from dtcf_gb300.cc import Job
    case = CASES[1]
    job = Job(method=method, engine="split", split_all=1, **case)
    ref = occ.CC(_system(case), method)
    e_ref = np.array(ref.iterate(6))
    e_gpu = np.concatenate([job.energies()[:1], job.iterate(6)])
    err = np.max(np.abs(e_gpu - e_ref))
    assert err <= 1e-10, err
    t1, t2 = job.amplitudes()
    assert np.max(np.abs(t2 - ref.t2)) <= 1e-9
    job.close()


def test_cc_large_tiles_match_oracle():
    """One irrep, 64-orbital virtual blocks: the (a, b) slabs of the o^2 v^2
    tensors hold 4096 elements, more than one work item of the fused residual
    sum, so items cover half slabs and the transposed terms are gathered.
    CCSD on both engines against the FP64 oracle."""
    from dtcf_gb300.cc import Job
    case = dict(nocc=4, nvir=64, nirrep=1, max_block=64, seed=5)
    ref = occ.CC(_system(case), "ccsd")
    e_ref = np.array(ref.iterate(4))
    for engine, tol_e, tol_t in (("fp64", 1e-10, 1e-12), ("split", 1e-10, 1e-9)):
        job = Job(method="ccsd", engine=engine, **case)
        e_gpu = np.concatenate([job.energies()[:1], job.iterate(4)])
        assert np.max(np.abs(e_gpu - e_ref)) <= tol_e, (engine, e_gpu, e_ref)
        t1, t2 = job.amplitudes()
        assert np.max(np.abs(t2 - ref.t2)) <= tol_t, engine
        assert np.max(np.abs(t1 - ref.t1)) <= tol_t, engine
        job.close()


@pytest.mark.parametrize("method", ["ccd", "ccsd"])
def test_cc_set_amplitudes_restarts_the_iteration(method):
    """Amplitudes set to zero: the next iteration is the MP2 guess again and
    the ones after it repeat a fresh job's energies bit for bit, so the
    amplitude combinations (tau, taut, Q) follow the amplitudes that were set."""
    import torch
    from dtcf_gb300.cc import Job
    case = CASES[1]
    fresh = Job(method=method, **case)
    e_fresh = np.concatenate([fresh.energies()[:1], fresh.iterate(3)])
    fresh.close()
    job = Job(method=method, **case)
    job.iterate(2)
    n1, n2 = job.amplitude_elems()
    z1, z2 = np.zeros(max(n1, 1)), np.zeros(n2)
    job.set_amplitudes(z1.ctypes.data if n1 else 0, z2.ctypes.data)
    torch.cuda.synchronize()
    e = job.iterate(3)
    assert np.array_equal(e, e_fresh[:3]), (e, e_fresh)
    job.close()


def test_cc_gemm_shapes_match_oracle_planner():
    """The packed GEMM shapes of one iteration equal the oracle's derivation
    from irrep occupations (the CPU arm times exactly these dgemms)."""
    from dtcf_gb300.cc import Job
    from oracle import cc_cpu
    case = dict(nocc=16, nvir=48, nirrep=8, max_block=6, min_block=1, seed=2)
    job = Job(method="ccsd", **case)
    got = sorted(map(tuple, job.gemm_shapes().tolist()))
    want = sorted(cc_cpu.gemm_shapes(_system(case), "ccsd"))
    assert got == want


def test_cc_split_autotune_keeps_energies():
    """The width autotuner changes tile shapes only: energies agree with the
    model-chosen plans to 1e-12 Eh and with the FP64 oracle to 1e-10 Eh."""
    from dtcf_gb300.cc import Job
    case = dict(nocc=12, nvir=60, nirrep=4, max_block=10, min_block=1, seed=13)
    a = Job(method="ccsd", engine="split", split_all=1, **case)
    b = Job(method="ccsd", engine="split", split_all=1, autotune=1, **case)
    ea, eb = a.iterate(3), b.iterate(3)
    assert np.max(np.abs(ea - eb)) <= 1e-12
    ref = occ.CC(_system(case), "ccsd")
    e_ref = np.array(ref.iterate(3)[1:])
    assert np.max(np.abs(eb - e_ref)) <= 1e-10
    a.close()
    b.close()


def test_ccd_config2_fp64_and_split_ten_iterations():
    """CCD at o=32, v=128, block 16 from the MP2 guess, 10 Jacobi iterations:
    the split path's energies stay within 1e-10 Eh of the FP64 path's at
    every iteration, and the iteration converges."""
    from dtcf_gb300.cc import Job
    case = dict(nocc=32, nvir=128, nirrep=1, max_block=16, min_block=1, seed=1, method="ccd")
    f = Job(engine="fp64", **case)
    s = Job(engine="split", slices=4, **case)
    ef = np.concatenate([f.energies()[:1], f.iterate(10)])
    es = np.concatenate([s.energies()[:1], s.iterate(10)])
    assert ef[0] == es[0]  # the MP2 guess is computed identically
    assert np.max(np.abs(ef - es)) <= 1e-10
    steps = np.abs(np.diff(ef))
    assert steps[-1] < steps[0] and np.all(np.isfinite(ef))
    f.close()
    s.close()
