"""GPU checks of the split-precision tcgen05 GEMM: exact on inputs that the
slices represent exactly, FP64-level accuracy on random FP64 data."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (200, 100, 1000), (130, 70, 2500), (257, 190, 4100)])
def test_split_gemm_exact_on_integer_data(M, N, K):
    """Integers below 2^20 are held exactly by 6 slices; products and sums stay
    below 2^53, so the result must equal the exact integer GEMM bit for bit.
    K > 1024 exercises the chunked TMEM drains."""
    import dtcf_gb300
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-(1 << 20), 1 << 20, size=(M, K)).astype(np.float64)
    B = rng.integers(-(1 << 20), 1 << 20, size=(N, K)).astype(np.float64)
    want = (A.astype(np.int64) @ B.astype(np.int64).T).astype(np.float64)
    C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
    dtcf_gb300.split_gemm(dev(A), dev(B), C, slices=6)
    got = C.cpu().numpy()
    assert np.array_equal(got, want), np.max(np.abs(got - want))


@pytest.mark.parametrize("slices,tol", [(6, 1e-13), (7, 1e-15), (4, 1e-8)])
def test_split_gemm_random_fp64(slices, tol):
    import dtcf_gb300
    rng = np.random.default_rng(slices)
    M, N, K = 300, 150, 3000
    A = rng.uniform(-1, 1, (M, K))
    B = rng.uniform(-1, 1, (N, K))
    want = A @ B.T
    C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
    dtcf_gb300.split_gemm(dev(A), dev(B), C, slices=slices)
    got = C.cpu().numpy()
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < tol, err


@pytest.mark.parametrize("width", [32, 64, 128, 256])
@pytest.mark.parametrize("M,N,K", [(300, 270, 2100), (129, 33, 70)])
def test_split_gemm_exact_every_tile_width(width, M, N, K):
    """Every output tile width of the split kernel (forced through the tuning
    knob) gives the exact integer product."""
    import dtcf_gb300
    from dtcf_gb300._lib import lib
    rng = np.random.default_rng(M * N + K + width)
    A = rng.integers(-(1 << 20), 1 << 20, size=(M, K)).astype(np.float64)
    B = rng.integers(-(1 << 20), 1 << 20, size=(N, K)).astype(np.float64)
    want = (A.astype(np.int64) @ B.astype(np.int64).T).astype(np.float64)
    C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
    assert lib().gbx_split_set_width(width) == 0
    try:
        dtcf_gb300.split_gemm(dev(A), dev(B), C, slices=6)
    finally:
        lib().gbx_split_set_width(0)
    assert np.array_equal(C.cpu().numpy(), want)


@pytest.mark.parametrize("M,N,K", [(5000, 8, 38), (300, 1, 1), (1000, 32, 64), (129, 17, 5), (7000, 30, 30),
                                   (513, 32, 32), (200, 5, 16), (300, 20, 33)])
def test_split_gemm_thin_k_exact(M, N, K):
    """K <= 64 and N <= 32: the thin-K kernel (all slice products of a tile
    in per-level TMEM accumulators) is exact on integer data, with the
    64-element k-block (K > 32) and the 32-element one (K <= 32, 64-byte
    swizzled slices)."""
    import dtcf_gb300
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-(1 << 20), 1 << 20, size=(M, K)).astype(np.float64)
    B = rng.integers(-(1 << 20), 1 << 20, size=(N, K)).astype(np.float64)
    want = (A.astype(np.int64) @ B.astype(np.int64).T).astype(np.float64)
    C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
    dtcf_gb300.split_gemm(dev(A), dev(B), C, slices=6)
    assert np.array_equal(C.cpu().numpy(), want)
    Af = rng.uniform(-1, 1, (M, K))
    Bf = rng.uniform(-1, 1, (N, K))
    dtcf_gb300.split_gemm(dev(Af), dev(Bf), C, slices=7)
    ref = Af @ Bf.T
    assert np.linalg.norm(C.cpu().numpy() - ref) <= 1e-15 * max(np.linalg.norm(ref), 1e-300) * 10


@pytest.mark.parametrize("slices", [2, 3, 4])
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 270, 2100), (129, 33, 70), (100, 40, 40000), (257, 190, 4100),
                                   (128, 200, 40000), (70, 130, 300)])
def test_split_gemm_k_stationary_exact(slices, M, N, K):
    """Up to 4 slices the 64-column k-stationary kernel runs (all slice
    products of a k-block from one load of each slice, exact int64 sums):
    exact on integers whose digits all fall in the kept slice products
    (|x| < 2^(8 h - 2) with h = (slices + 1) // 2 leading digits), including
    several accumulation groups, ragged edges and a split K ((128, 200,
    40000) splits K over several column tiles)."""
    import dtcf_gb300
    rng = np.random.default_rng(M + N + K + slices)
    lim = 1 << (8 * ((slices + 1) // 2) - 2)
    A = rng.integers(-lim, lim, size=(M, K)).astype(np.float64)
    B = rng.integers(-lim, lim, size=(N, K)).astype(np.float64)
    want = (A.astype(np.int64) @ B.astype(np.int64).T).astype(np.float64)
    C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
    dtcf_gb300.split_gemm(dev(A), dev(B), C, slices=slices)
    assert np.array_equal(C.cpu().numpy(), want)


@pytest.mark.parametrize("K", [7, 30, 32, 33, 60])
def test_split_gemm_thin_k_four_slices_exact(K):
    """The thin-K kernel at 4 slices (the coupled-cluster setting) on both
    k-blocks: exact on integers whose digits fall in the kept products."""
    import dtcf_gb300
    rng = np.random.default_rng(K)
    M, N = 3000, 24
    A = rng.integers(-(1 << 14), 1 << 14, size=(M, K)).astype(np.float64)
    B = rng.integers(-(1 << 14), 1 << 14, size=(N, K)).astype(np.float64)
    want = (A.astype(np.int64) @ B.astype(np.int64).T).astype(np.float64)
    C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
    dtcf_gb300.split_gemm(dev(A), dev(B), C, slices=4)
    assert np.array_equal(C.cpu().numpy(), want)


def test_split_gemm_k_stationary_matches_pairwise_kernel():
    """Random FP64 at 4 slices: the k-stationary kernel (width 64) and the
    pair-by-pair kernel (width 128) keep the same slice products, so they
    agree to FP64 rounding; both are within 2^-28 of the FP64 product."""
    import dtcf_gb300
    from dtcf_gb300._lib import lib
    rng = np.random.default_rng(9)
    M, N, K = 400, 300, 5000
    A = rng.uniform(-1, 1, (M, K))
    B = rng.uniform(-1, 1, (N, K))
    want = A @ B.T
    out = []
    for w in (64, 128):
        C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
        assert lib().gbx_split_set_width(w) == 0
        try:
            dtcf_gb300.split_gemm(dev(A), dev(B), C, slices=4)
        finally:
            lib().gbx_split_set_width(0)
        out.append(C.cpu().numpy())
    scale = np.linalg.norm(want)
    assert np.linalg.norm(out[0] - out[1]) / scale < 1e-14
    assert np.linalg.norm(out[0] - want) / scale < 2.0 ** -28
