"""The persistent iteration program (use_graph=2): one coupled-cluster
iteration as a few persistent launches off a device-side work queue.

* bit-identical energies and amplitudes to the kernel-by-kernel CUDA graph
  (use_graph=1) on both engines, CCD and CCSD, with and without spatial
  symmetry, the pair-by-pair split kernel (5 slices), every GEMM on the
  split engine, and autotuned split tile widths;
* far fewer launches per iteration than the kernel graph (the bench
  workload: under 20);
* the bounded dependency wait: a wait that can never be met runs out,
  reports GBX_ETIMEOUT, and the context keeps working."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GBX_ETIMEOUT = -4

CASES = [
    dict(method="ccsd", engine="split", nocc=16, nvir=64, nirrep=8, max_block=8, seed=3),
    dict(method="ccd", engine="split", nocc=16, nvir=64, nirrep=4, max_block=8, seed=5),
    dict(method="ccsd", engine="fp64", nocc=12, nvir=48, nirrep=2, max_block=8, seed=7),
    dict(method="ccsd", engine="split", nocc=12, nvir=48, nirrep=1, max_block=12, slices=5, seed=9),
    dict(method="ccsd", engine="split", nocc=8, nvir=24, nirrep=4, max_block=4, split_all=1, seed=11),
    dict(method="ccsd", engine="split", nocc=32, nvir=160, nirrep=8, max_block=16, autotune=1, seed=1),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-%s-o%d-v%d-h%d" % (
    c["method"], c["engine"], c["nocc"], c["nvir"], c["nirrep"]))
def test_persistent_program_bit_identical_to_kernel_graph(case):
    from dtcf_gb300.cc import Job
    a = Job(use_graph=1, **case)
    b = Job(use_graph=2, **case)
    ea, eb = a.iterate(4), b.iterate(4)
    assert np.array_equal(ea, eb), (ea, eb)
    t1a, t2a = a.amplitudes()
    t1b, t2b = b.amplitudes()
    assert np.array_equal(t1a, t1b) and np.array_equal(t2a, t2b)
    info = b.program_info()
    sa, sb = a.stats(), b.stats()
    assert info["launches"] > 0 and info["levels"] >= 1
    # the graph of the persistent job holds its launches (zero fills that
    # stay memset nodes are launches of the program but not kernels)
    assert 0 < sb.launches_per_iter <= info["launches"]
    assert sb.launches_per_iter < sa.launches_per_iter
    a.close()
    b.close()


def test_bench_workload_under_20_launches_per_iteration():
    from dtcf_gb300.cc import Job
    job = Job(method="ccsd", engine="split", nocc=48, nvir=240, nirrep=8, max_block=40, min_block=4, slices=4,
              autotune=1, seed=1, use_graph=2)
    e = job.iterate(2)
    assert np.all(np.isfinite(e))
    info = job.program_info()
    st = job.stats()
    assert st.launches_per_iter < 20, (st.launches_per_iter, info)
    assert info["records"] > 100  # the iteration's kernels are now records of a few launches
    job.close()


def test_dependency_wait_that_runs_out_reports_timeout_and_context_survives():
    from dtcf_gb300._lib import lib
    from dtcf_gb300.cc import Job, program_selftest
    assert program_selftest(1_000_000) == GBX_ETIMEOUT
    assert b"bounded device wait ran out (code 31)" in lib().gbx_last_error()
    # the context still runs a persistent iteration, identical to the graph
    case = CASES[4]
    a = Job(use_graph=1, **case)
    b = Job(use_graph=2, **case)
    assert np.array_equal(a.iterate(2), b.iterate(2))


def test_selftest_rejects_bad_limits():
    from dtcf_gb300.cc import program_selftest
    assert program_selftest(0) == -1
    assert program_selftest(-5) == -1
