"""The allocation-free entry point gbx_local_contraction_noalloc, called
through the C ABI, against gbx_local_contraction on the same inputs and
against the oracle's corrected local_contraction.

It serves callers that cannot let a library allocate device memory (a
framework that handed the GPU's memory to its own pool, or a latency-bound
loop that must not be stalled by cudaFree's device synchronisation); its
workspace is a fixed device array inside the library.  Two calls in a row check that the
shared array's leftover contents from the previous call do not leak into
the next.  This file sorts last so a stop-at-first-failure run has already
run every other test."""
import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

SHAPES = [
    (40, 30, 20000, 0, 1),   # small output, long K: split-K partials in the workspace
    (200, 150, 700, 0, 1),
    (5000, 6, 30, 0, 0),     # thin output, one thread per row
    (130, 70, 64, 1, 1),
    (64, 64, 4096, 1, 0),
    (6, 5000, 30, 0, 1),     # thin output, one thread per column
    (300, 200, 4, 1, 0),     # K <= 8: one thread per output element
    (50, 40, 0, 0, 0),       # K = 0: C unchanged
]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("na,nb,nk,at,bt", SHAPES)
def test_noalloc_matches_allocating_entry_point_twice(na, nb, nk, at, bt):
    from dtcf_gb300._lib import lib
    L = lib()
    rng = np.random.default_rng(na + nb + nk)
    A = torch.from_numpy(rng.standard_normal(na * nk)).cuda()
    B = torch.from_numpy(rng.standard_normal(nb * nk)).cuda()
    C0 = torch.from_numpy(rng.standard_normal(na * nb)).cuda()
    C_ref, C_new = C0.clone(), C0.clone()
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    want = C0.cpu().numpy().copy()
    a_h, b_h = A.cpu().numpy(), B.cpu().numpy()
    for call in range(2):
        assert L.gbx_local_contraction(na, nb, nk, _ptr(A), _ptr(B), _ptr(C_ref), at, bt, 0.75, sp) == 0
        rc = L.gbx_local_contraction_noalloc(na, nb, nk, _ptr(A), _ptr(B), _ptr(C_new), at, bt, 0.75, sp)
        assert rc == 0, L.gbx_last_error()
        oracle.local_contraction(na, nb, nk, a_h, b_h, want, at, bt, 0.75)
        torch.cuda.synchronize()
        ref, got = C_ref.cpu().numpy(), C_new.cpu().numpy()
        scale = max(1.0, float(np.abs(ref).max()))
        assert np.max(np.abs(got - ref)) <= 1e-12 * scale, (call, np.max(np.abs(got - ref)))
        # the oracle's loop sums in another order: 1e-13 of |A| |B| K
        tol = 1e-13 * float(np.abs(a_h).max(initial=1)) * float(np.abs(b_h).max(initial=1)) * max(nk, 1)
        assert np.max(np.abs(got - want)) <= tol, (call, np.max(np.abs(got - want)))


def test_noalloc_rejects_outputs_beyond_the_workspace():
    from dtcf_gb300._lib import lib
    L = lib()
    rc = L.gbx_local_contraction_noalloc(4096, 2049, 8, None, None, None, 0, 1, 1.0, None)
    assert rc == -1
    assert b"allocation-free workspace" in L.gbx_last_error()
