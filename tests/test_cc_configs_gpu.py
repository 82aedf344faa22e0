"""The coupled-cluster configurations of the benchmark against the
irrep-blocked FP64 oracle (oracle/cc_blocks.py), not against the GPU's own
FP64 path:

* CCD, o = 32, v = 128, block 16, no spatial symmetry: 10 Jacobi iterations
  from the MP2 guess on the FP64 and split engines;
* CCSD, 8 irreps, o = 48, v = 240, uneven blocks 4..40 (the benchmark
  workload): the MP2 guess and two iterations on both engines.

Correlation energies within 1e-10 Eh of the oracle at every iteration;
FP64-engine amplitudes within 1e-12."""
import numpy as np
import pytest

from oracle import cc as occ, cc_blocks

pytestmark = pytest.mark.gpu

CFG2 = dict(nocc=32, nvir=128, nirrep=1, max_block=16, min_block=1, seed=1)
CFG3 = dict(nocc=48, nvir=240, nirrep=8, max_block=40, min_block=4, seed=1)


def _system(c):
    return occ.System(c["nocc"], c["nvir"], nirrep=c["nirrep"], max_block=c["max_block"],
                      min_block=c["min_block"], seed=c["seed"])


@pytest.fixture(scope="module")
def oracle_cfg2():
    ref = cc_blocks.CC(_system(CFG2), "ccd")
    ref.iterate(10)
    return ref


@pytest.fixture(scope="module")
def oracle_cfg3():
    ref = cc_blocks.CC(_system(CFG3), "ccsd")
    ref.iterate(2)
    return ref


@pytest.mark.parametrize("engine,slices", [("fp64", 0), ("split", 4)])
def test_ccd_config2_ten_iterations_vs_oracle(oracle_cfg2, engine, slices):
    from dtcf_gb300.cc import Job
    job = Job(method="ccd", engine=engine, slices=slices, **CFG2)
    e_gpu = np.concatenate([job.energies()[:1], job.iterate(10)])
    e_ref = np.array(oracle_cfg2.energies)
    err = np.abs(e_gpu - e_ref)
    assert np.max(err) <= 1e-10, err
    if engine == "fp64":
        t1, t2 = job.amplitudes()
        assert oracle_cfg2.t2.max_abs_diff_dense(t2, {"o": 0, "v": CFG2["nocc"]}) <= 1e-12
    job.close()


@pytest.mark.parametrize("engine,slices", [("fp64", 0), ("split", 4)])
def test_ccsd_config3_vs_oracle(oracle_cfg3, engine, slices):
    from dtcf_gb300.cc import Job
    job = Job(method="ccsd", engine=engine, slices=slices, **CFG3)
    irr, eps = job.orbitals()
    s = oracle_cfg3.s
    assert np.array_equal(irr, s.irrep) and np.array_equal(eps, s.eps)
    e_gpu = np.concatenate([job.energies()[:1], job.iterate(2)])
    e_ref = np.array(oracle_cfg3.energies)
    assert e_gpu[0] == pytest.approx(e_ref[0], abs=1e-12)  # the MP2 guess
    err = np.abs(e_gpu - e_ref)
    assert np.max(err) <= 1e-10, err
    if engine == "fp64":
        t1, t2 = job.amplitudes()
        off = {"o": 0, "v": CFG3["nocc"]}
        assert oracle_cfg3.t2.max_abs_diff_dense(t2, off) <= 1e-12
        assert oracle_cfg3.t1.max_abs_diff_dense(t1, off) <= 1e-12
    job.close()


def test_contraction_error_against_fp64_plans():
    """gbx_cc_contraction_error: an FP64 job's contractions agree with fresh
    FP64 plans to rounding; a split job (6 slices, split engine on every
    GEMM) stays within 1e-12 relative Frobenius error per contraction."""
    from dtcf_gb300.cc import Job
    case = dict(nocc=16, nvir=48, nirrep=8, max_block=6, min_block=1, seed=2, method="ccsd")
    f = Job(engine="fp64", **case)
    s = Job(engine="split", split_all=1, slices=6, **case)
    f.iterate(1)
    s.iterate(1)
    n = f.stats().ncontractions
    for c in range(n):
        rel, _ = f.contraction_error(c)
        assert rel <= 1e-14, (c, rel)
        rel, _ = s.contraction_error(c)
        assert rel <= 1e-12, (c, rel)
    # the job's state is untouched: the next iterations repeat a fresh job's
    g = Job(engine="split", split_all=1, slices=6, **case)
    assert np.array_equal(s.iterate(2), g.iterate(3)[1:])
    for j in (f, s, g):
        j.close()
