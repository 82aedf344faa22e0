"""Bounded device waits: a wait that runs out returns GBX_ETIMEOUT through
the C ABI and leaves the CUDA context usable.

The wait is made to run out without a fault: one CTA waits, through the same
bounded mbarrier wait as the split GEMM pipelines, on a barrier that nothing
arrives on, with a short limit.  A split GEMM run afterwards on the same
stream must still give correct results."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GBX_ETIMEOUT = -4


@pytest.mark.parametrize("limit", [0, 1_000_000])
def test_wait_that_runs_out_reports_timeout_and_context_survives(limit):
    from dtcf_gb300._lib import lib
    import dtcf_gb300
    L = lib()
    s = torch.cuda.current_stream()
    rc = L.gbx_wait_selftest(limit, ctypes.c_void_p(s.cuda_stream))
    assert rc == GBX_ETIMEOUT
    assert b"bounded device wait ran out (stage 31)" in L.gbx_last_error()
    # the context still runs the split engine correctly
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.rand(300, 200, dtype=torch.float64, device="cuda", generator=g) - 0.5
    B = torch.rand(150, 200, dtype=torch.float64, device="cuda", generator=g) - 0.5
    C = torch.zeros(300, 150, dtype=torch.float64, device="cuda")
    dtcf_gb300.split_gemm(A, B, C, slices=6)
    torch.cuda.synchronize()
    ref = (A @ B.T).cpu().numpy()
    assert np.max(np.abs(C.cpu().numpy() - ref)) <= 1e-13 * np.abs(ref).max()


def test_wait_limit_is_checked_on_the_host():
    from dtcf_gb300._lib import lib
    L = lib()
    assert L.gbx_wait_selftest(-1, None) == -1
    assert L.gbx_wait_selftest(10 ** 12, None) == -1
