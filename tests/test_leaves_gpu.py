"""GPU parity of the leaf entry points against the reference fixtures and the
oracle: permutes and packs bit-exact, FP64 GEMMs within 1e-12 relative."""
import itertools

import numpy as np
import pytest
import torch

import oracle
import oracle.rrr  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gbx():
    import dtcf_gb300
    dtcf_gb300.lib()
    return dtcf_gb300


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_transpose_bit_exact_vs_reference(gbx, golden):
    for n in range(int(golden["tr_count"])):
        w, p = golden[f"tr{n}_widths"], golden[f"tr{n}_perm"]
        x = dev(golden[f"tr{n}_in"])
        y = torch.full_like(x, np.nan)
        gbx.transpose(x, y, p, w)
        assert np.array_equal(host(y), golden[f"tr{n}_out"]), (w, p)


def test_dltc_transpose_bit_exact_vs_reference(gbx, golden):
    for n in range(int(golden["dl_count"])):
        name = bytes(golden[f"dl{n}_name"]).decode()
        dims = golden[f"dl{n}_dims"]
        x = dev(golden[f"dl{n}_in"])
        y = torch.full_like(x, np.nan)
        letters = "ijkl"[: len(dims)]
        gbx.dltc_transpose(x, list(range(len(dims))), y, [letters.index(c) for c in name], dims)
        assert np.array_equal(host(y), golden[f"dl{n}_out"]), name


def test_dltc_identity_copies(gbx):
    """DLTC/transp.cc:16,24 leaves y unwritten for identity; the C ABI copies."""
    x = dev(np.arange(24.0))
    y = torch.zeros_like(x)
    gbx.dltc_transpose(x, [0, 1, 2, 3], y, [0, 1, 2, 3], [2, 3, 2, 2])
    assert np.array_equal(host(y), np.arange(24.0))


def test_big_matrix_bit_exact_vs_reference(gbx, golden):
    for b in range(int(golden["bm_count"])):
        pre = f"bm{b}_"
        vg, pm = golden[pre + "vgrid"], golden[pre + "p_map"]
        rpb, cpb, nrd = int(golden[pre + "rpb"]), int(golden[pre + "cpb"]), int(golden[pre + "nrd"])
        tiles = dev(golden[pre + "tiles"])
        big = torch.full_like(tiles, np.nan)
        gbx.create_big_matrix(vg, pm, tiles, golden[pre + "perm_addr"], rpb, cpb, nrd, big)
        assert np.array_equal(host(big), golden[pre + "big"])
        back = torch.full_like(tiles, np.nan)
        gbx.revert_big_matrix(vg, pm, golden[pre + "perm_addr"], rpb, cpb, nrd, dev(golden[pre + "big2"]), back)
        assert np.array_equal(host(back).reshape(golden[pre + "back"].shape), golden[pre + "back"])


def test_big_matrix_nl_bit_exact_vs_reference(gbx, golden):
    """create_big_matrix_nl: tile data in slots of a shuffled order (plus
    unused slots), found through address_to_location, as the compiled
    reference places them; a missing location is GBX_EINVAL."""
    for b in range(int(golden["nl_count"])):
        pre = f"nl{b}_"
        tiles = dev(golden[pre + "tiles"])
        big = torch.full((golden[pre + "big"].size,), np.nan, dtype=torch.float64, device="cuda")
        loc = dict(zip(golden[pre + "ranks"].tolist(), golden[pre + "slots"].tolist()))
        gbx.create_big_matrix_nl(golden[pre + "vgrid"], golden[pre + "p_map"], tiles, golden[pre + "perm_addr"],
                                 int(golden[pre + "rpb"]), int(golden[pre + "cpb"]), int(golden[pre + "nrd"]), loc, big)
        assert np.array_equal(host(big), golden[pre + "big"])
    pre = "nl0_"
    loc = dict(zip(golden[pre + "ranks"].tolist()[1:], golden[pre + "slots"].tolist()[1:]))
    with pytest.raises(Exception):
        gbx.create_big_matrix_nl(golden[pre + "vgrid"], golden[pre + "p_map"], dev(golden[pre + "tiles"]),
                                 golden[pre + "perm_addr"], int(golden[pre + "rpb"]), int(golden[pre + "cpb"]),
                                 int(golden[pre + "nrd"]), loc, torch.zeros(golden[pre + "big"].size,
                                                                           dtype=torch.float64, device="cuda"))


def test_big_matrix_rejects_ragged(gbx):
    tiles = dev(np.zeros(3 * 4))
    big = torch.zeros_like(tiles)
    with pytest.raises(Exception):
        gbx.create_big_matrix([2, 2], [0, 1], tiles, [[0, 0], [0, 1], [1, 0]], 2, 2, 1, big)


@pytest.mark.parametrize("na,nb,nk,at,bt", [(8, 8, 8, 0, 1), (3, 5, 7, 0, 1), (64, 48, 200, 0, 1), (7, 5, 9, 0, 0),
                                            (33, 65, 17, 1, 0), (130, 70, 64, 1, 1), (1, 1, 1, 0, 1), (5, 6, 0, 0, 1)])
def test_local_contraction_vs_oracle(gbx, na, nb, nk, at, bt):
    rng = np.random.default_rng(na * 1000 + nb * 10 + nk)
    A = rng.standard_normal(na * nk)
    B = rng.standard_normal(nb * nk)
    C = rng.standard_normal(na * nb)
    want = C.copy()
    oracle.local_contraction(na, nb, nk, A, B, want, at, bt, -0.75)
    dC = dev(C)
    gbx.local_contraction(na, nb, nk, dev(A), dev(B), dC, at, bt, -0.75)
    got = host(dC)
    scale = np.abs(A).max(initial=1) * np.abs(B).max(initial=1) * max(nk, 1)
    assert np.max(np.abs(got - want)) <= 1e-13 * scale


def test_local_contraction_vs_reference_fixtures(gbx, golden):
    for c in range(int(golden["lc_count"])):
        pre = f"lc{c}_"
        na, nb, nk, at, bt = [int(v) for v in golden[pre + "shape"]]
        dC = dev(golden[pre + "C_in"])
        gbx.local_contraction(na, nb, nk, dev(golden[pre + "A"]), dev(golden[pre + "B"]), dC, at, bt,
                              float(golden[pre + "alpha"]))
        np.testing.assert_allclose(host(dC), golden[pre + "C_out"], rtol=1e-12, atol=1e-12)


def test_grouped_gemm_triples(gbx):
    from dtcf_gb300.leaves import Triple
    rng = np.random.default_rng(5)
    keep, trip, want = [], [], []
    for _ in range(37):
        m, n, k = [int(x) for x in rng.integers(1, 90, size=3)]
        A, B, C = rng.standard_normal((m, k)), rng.standard_normal((n, k)), rng.standard_normal((m, n))
        dA, dB, dC = dev(A), dev(B), dev(C)
        keep += [dA, dB, dC]
        trip.append(Triple(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), k, 1, k, 1, n, m, n, k, 1.5, 1))
        want.append((dC, C + 1.5 * A @ B.T))
    gbx.grouped_gemm_f64(trip)
    for dC, w in want:
        np.testing.assert_allclose(host(dC).reshape(w.shape), w, rtol=1e-12, atol=1e-12)


def test_transpose_blocks_symmetric_unflip(gbx):
    """Per-block permutes of transpose_and_dgemm: get_symm_permutation composed
    with the p_map (contraction.cc:1824-1857), bit-exact."""
    rng = np.random.default_rng(9)
    addrs = [[1, 3, 0, 2], [3, 1, 2, 0], [2, 2, 1, 1], [0, 1, 1, 0]]
    sg = [0, 0, 1, 1]
    p_map = [2, 3, 0, 1]
    w = [4, 4, 3, 3]
    blocks = rng.standard_normal((len(addrs), int(np.prod(w))))
    perms = [oracle.compose_p_maps(oracle.symm_permutation(a, sg), p_map) for a in addrs]
    out = torch.full((blocks.size,), np.nan, dtype=torch.float64, device="cuda")
    gbx.transpose_blocks(dev(blocks), out, perms, w)
    got = host(out).reshape(blocks.shape)
    for i in range(len(addrs)):
        assert np.array_equal(got[i], oracle.transpose(blocks[i].reshape(w), perms[i]).reshape(-1))


def test_rrr_initialize_on_device_bit_exact_vs_reference(gbx, golden):
    """Tensor::initialize on one process (tensor.cc:315-335) on the device:
    the unique tile addresses in generation order and the block values,
    bit for bit as the compiled reference made them; counting only, and a
    too-small capacity, are checked too."""
    from dtcf_gb300.rrr import Tensor, unique_blocks
    for t in range(int(golden["tt_count"])):
        sym = bytes(golden[f"tt{t}_sym"]).decode()
        sizes, vgrid = golden[f"tt{t}_sizes"], golden[f"tt{t}_vgrid"]
        addr = unique_blocks(sym, vgrid)
        assert np.array_equal(addr.cpu().numpy(), golden[f"tt{t}_addr"]), sym
        T = Tensor(sym, sizes, vgrid).initialize()
        torch.cuda.synchronize()
        assert np.array_equal(T.addrs, golden[f"tt{t}_addr"])
        assert np.array_equal(host(T.tiles).reshape(golden[f"tt{t}_tiles"].shape), golden[f"tt{t}_tiles"]), sym
    import ctypes
    g = np.array([5, 5], dtype=np.int32)
    n = ctypes.c_int()
    lib = gbx.lib()
    assert lib.gbx_rrr_unique_tiles(2, b"aa", g.ctypes.data_as(ctypes.c_void_p), None, 0, ctypes.byref(n), None) == 0
    assert n.value == 15
    small = torch.zeros(4 * 2, dtype=torch.int32, device="cuda")
    rc = lib.gbx_rrr_unique_tiles(2, b"aa", g.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(small.data_ptr()), 4,
                                  ctypes.byref(n), None)
    assert rc != 0 and n.value == 15
    assert np.array_equal(small.cpu().numpy().reshape(4, 2), [[0, 0], [1, 0], [1, 1], [2, 0]])


def _rrr_case(sym_a, sym_b, sym_c, sizes, vgrids, seed):
    from dtcf_gb300.rrr import Tensor
    rng = np.random.default_rng(seed)
    T = [Tensor(s, z, v) for s, z, v in zip((sym_a, sym_b, sym_c), sizes, vgrids)]
    for t in T:
        t.tiles.copy_(torch.from_numpy(rng.uniform(-1, 1, t.tiles.numel())).cuda())
    return T


def _as_oracle(t):
    return dict(tiles=host(t.tiles).reshape(t.num_tiles, -1), addrs=t.addrs, sym=t.sym, block_range=t.block_range,
                vgrid=t.vgrid)


@pytest.mark.parametrize("sign", [1, -1])
def test_rrr_plan_ladder_small(gbx, sign):
    """C[a,b,i,j] += 0.5 sum_ef V[a,b,e,f] T[e,f,i,j] with unique blocks (aabb)."""
    from dtcf_gb300.rrr import Contraction
    o, v, blk = 8, 12, 4
    V, T, C = _rrr_case("aabb", "aabb", "aabb", [(v, v, v, v), (v, v, o, o), (v, v, o, o)],
                        [(v // blk,) * 4, (v // blk, v // blk, o // blk, o // blk), (v // blk, v // blk, o // blk, o // blk)],
                        11)
    want = oracle.rrr.contract(_as_oracle(V), _as_oracle(T), _as_oracle(C), "a,b,e,f", "e,f,i,j", "a,b,i,j", 0.5,
                               sign)
    Contraction(V, T, C, sign=sign).contract("a,b,e,f", "e,f,i,j", "a,b,i,j", 0.5)
    got = host(C.tiles).reshape(want.shape)
    assert np.max(np.abs(got - want)) <= 1e-12 * max(1.0, np.abs(want).max())


def test_rrr_plan_cntr4a_shape(gbx):
    """examples/cntr4a_4D-style C[a,b,m,n] = A[a,b,k,l] * B[m,n,k,l], no symmetry,
    block-constant initialize() values (tensor.cc:744-758)."""
    from dtcf_gb300.rrr import Tensor, Contraction
    n, nb = 16, 4
    A = Tensor("cccc", (n,) * 4, (nb,) * 4).initialize()
    B = Tensor("cccc", (n,) * 4, (nb,) * 4).initialize()
    C = Tensor("cccc", (n,) * 4, (nb,) * 4)
    want = oracle.rrr.contract(_as_oracle(A), _as_oracle(B), _as_oracle(C), "a,b,k,l", "m,n,k,l", "a,b,m,n", 1.0)
    ctr = Contraction(A, B, C)
    ctr.contract("a,b,k,l", "m,n,k,l", "a,b,m,n")
    got = host(C.tiles).reshape(want.shape)
    assert np.max(np.abs(got - want)) <= 1e-12 * np.abs(want).max()
    assert ctr.plan("a,b,k,l", "m,n,k,l", "a,b,m,n").flops == 2.0 * n ** 6


@pytest.mark.parametrize("mode", ["fp64", "split"])
@pytest.mark.parametrize("sign", [1, -1])
def test_rrr_plan_direct_engine(gbx, mode, sign):
    """C[a,b,i,j] += 0.5 sum_m A[a,b,i,m] B[m,j] with a contracted extent of 4
    per output element: the planner runs it on the direct FP64 kernel (no
    packing) in either mode; A and C keep unique (a, b) blocks, so reads go
    through the symmetric / antisymmetric un-flip with its sign."""
    from dtcf_gb300.rrr import Contraction
    o, v, m, blk = 8, 12, 4, 4
    A, B, C = _rrr_case("aabc", "ab", "aabc", [(v, v, o, m), (m, o), (v, v, o, o)],
                        [(v // blk, v // blk, o // blk, m // blk), (m // blk, o // blk),
                         (v // blk, v // blk, o // blk, o // blk)], 31)
    want = oracle.rrr.contract(_as_oracle(A), _as_oracle(B), _as_oracle(C), "a,b,i,m", "m,j", "a,b,i,j", 0.5, sign)
    Contraction(A, B, C, mode=mode, sign=sign).contract("a,b,i,m", "m,j", "a,b,i,j", 0.5)
    got = host(C.tiles).reshape(want.shape)
    assert np.max(np.abs(got - want)) <= 1e-13 * max(1.0, np.abs(want).max())


@pytest.mark.parametrize("sign", [1, -1])
def test_rrr_plan_split_engine(gbx, sign):
    """The same unique-block ladder on the split-precision engine (6 slices):
    within 1e-13 of the FP64 oracle relative to the largest element."""
    from dtcf_gb300.rrr import Contraction
    o, v, blk = 16, 48, 8
    V, T, C = _rrr_case("aabb", "aabb", "aabb", [(v, v, v, v), (v, v, o, o), (v, v, o, o)],
                        [(v // blk,) * 4, (v // blk, v // blk, o // blk, o // blk), (v // blk, v // blk, o // blk, o // blk)],
                        21)
    want = oracle.rrr.contract(_as_oracle(V), _as_oracle(T), _as_oracle(C), "a,b,e,f", "e,f,i,j", "a,b,i,j", 0.5,
                               sign)
    ctr = Contraction(V, T, C, mode="split", sign=sign)
    ctr.contract("a,b,e,f", "e,f,i,j", "a,b,i,j", 0.5)
    got = host(C.tiles).reshape(want.shape)
    assert np.max(np.abs(got - want)) <= 1e-13 * np.abs(want).max()
    # the unique-block flop count of this contraction (o=16, v=48, block 8)
    assert ctr.plan("a,b,e,f", "e,f,i,j", "a,b,i,j").flops == 2.0 * 63 * 4096 * 2304


@pytest.mark.parametrize("m,n,k", [(5000, 6, 30), (7, 3000, 20), (300, 32, 64), (40, 33, 64), (2000, 1, 1)])
def test_grouped_gemm_thin_shapes(gbx, m, n, k):
    """Thin problems (one output side <= 32, K <= 64) take the exact-shape
    CUDA-core FP64 path; results match numpy to FP64 rounding."""
    from dtcf_gb300.leaves import Triple
    rng = np.random.default_rng(m + n + k)
    A, B, C = rng.standard_normal((m, k)), rng.standard_normal((n, k)), rng.standard_normal((m, n))
    dA, dB, dC = dev(A), dev(B), dev(C)
    gbx.grouped_gemm_f64([Triple(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), k, 1, k, 1, n, m, n, k, -2.0, 1)])
    np.testing.assert_allclose(host(dC).reshape(m, n), C - 2.0 * A @ B.T, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("m,n,k", [(1475, 1475, 1), (300, 700, 8), (5, 9, 3)])
def test_grouped_gemm_small_k(gbx, m, n, k):
    """K <= 8 problems (outer products) take the per-element FP64 kernel."""
    from dtcf_gb300.leaves import Triple
    rng = np.random.default_rng(m + n + k)
    A, B, C = rng.standard_normal((m, k)), rng.standard_normal((n, k)), rng.standard_normal((m, n))
    dA, dB, dC = dev(A), dev(B), dev(C)
    gbx.grouped_gemm_f64([Triple(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), k, 1, k, 1, n, m, n, k, 0.5, 1)])
    np.testing.assert_allclose(host(dC).reshape(m, n), C + 0.5 * A @ B.T, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("m,n,k,acc", [(6, 6, 20000, 1), (16, 16, 8192, 0), (3, 11, 5000, 1), (16, 1, 4096, 0),
                                       (8, 8, 4096, 0), (1, 7, 4500, 1), (5, 2, 9001, 0), (7, 3, 12289, 1)])
def test_grouped_gemm_small_output_long_k(gbx, m, n, k, acc):
    """Outputs of at most 16 x 16 with K >= 4096: one CTA per K chunk holds the
    whole output, chunks reduced in a fixed order (odd shapes and K that is
    not a multiple of the chunk included)."""
    from dtcf_gb300.leaves import Triple
    rng = np.random.default_rng(m * n + k)
    A, B, C = rng.standard_normal((m, k)), rng.standard_normal((n, k)), rng.standard_normal((m, n))
    dA, dB, dC = dev(A), dev(B), dev(C)
    gbx.grouped_gemm_f64([Triple(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), k, 1, k, 1, n, m, n, k, -0.75, acc)])
    want = (C if acc else 0.0) - 0.75 * A @ B.T
    np.testing.assert_allclose(host(dC).reshape(m, n), want, rtol=1e-12, atol=1e-12 * np.sqrt(k))
    # and through the leaf entry point with a transposed A (strided operand reads)
    dC2 = dev(C)
    At = np.ascontiguousarray(A.T)
    gbx.local_contraction(m, n, k, dev(At), dB, dC2, 1, 1, -0.75)
    np.testing.assert_allclose(host(dC2).reshape(m, n), C - 0.75 * A @ B.T, rtol=1e-12, atol=1e-12 * np.sqrt(k))


@pytest.mark.parametrize("m,n,k", [(16, 16, 16), (256, 64, 256), (3, 70, 9), (100, 5, 2000), (1, 1, 1)])
def test_dltc_compute_vs_oracle(gbx, m, n, k):
    """DLTC compute (DLTC/compute.cc:3-36): c[m x n] += a[m x k] b[k x n],
    row-major, through gbx_dltc_compute, against the oracle's loop."""
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    a, b, c = rng.uniform(-1, 1, m * k), rng.uniform(-1, 1, k * n), rng.uniform(-1, 1, m * n)
    want = c.copy()
    oracle.dltc_compute(m, n, k, a, b, want)
    dc = dev(c)
    gbx.dltc_compute(dc, dev(a), dev(b), m, n, k)
    assert np.max(np.abs(host(dc) - want)) <= 1e-13 * k


def _antisym_pair(x):
    x = x - x.transpose(1, 0, 2, 3)
    return x - x.transpose(0, 1, 3, 2)


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_config1_ladder_exact_spec(gbx, mode):
    """The single 4-D contraction C[a,b,i,j] += 0.5 sum_ef V[a,b,e,f] T[e,f,i,j]
    at o=16, v=48, block 8: V antisymmetric in (a,b) and in (e,f) and
    pair-symmetric (V[ab,ef] = V[ef,ab]), T antisymmetric in (e,f) and (i,j),
    all drawn uniform(-1,1) (seed 1) before antisymmetrisation; only the
    unique blocks (non-increasing block coordinates per pair, RRR's order) are
    stored.  Checked against the dense oracle on every stored C block: FP64
    engine within 1e-12 relative, split engine (6 slices) within 1e-13 of the
    largest element."""
    from dtcf_gb300.rrr import Tensor, Contraction
    o, v, blk = 16, 48, 8
    rng = np.random.default_rng(1)
    Vd = _antisym_pair(rng.uniform(-1, 1, (v, v, v, v)))
    Vd = 0.5 * (Vd + Vd.transpose(2, 3, 0, 1))
    Td = _antisym_pair(rng.uniform(-1, 1, (v, v, o, o)))
    Cd = _antisym_pair(rng.uniform(-1, 1, (v, v, o, o)))
    assert np.array_equal(Vd, -Vd.transpose(1, 0, 2, 3)) and np.array_equal(Vd, Vd.transpose(2, 3, 0, 1))
    V = Tensor("aabb", (v,) * 4, (v // blk,) * 4)
    T = Tensor("aabb", (v, v, o, o), (v // blk, v // blk, o // blk, o // blk))
    C = Tensor("aabb", (v, v, o, o), (v // blk, v // blk, o // blk, o // blk))
    for t, d in ((V, Vd), (T, Td), (C, Cd)):
        t.tiles.copy_(torch.from_numpy(oracle.rrr.cut(d, t.addrs, t.block_range).reshape(-1)).cuda())
    assert (V.num_tiles, T.num_tiles) == (441, 63)
    want = oracle.rrr.cut(Cd + 0.5 * np.einsum("abef,efij->abij", Vd, Td), C.addrs, C.block_range)
    # the unique-block store expands back to the same dense operands (sign -1)
    assert np.array_equal(oracle.rrr.dense(host(T.tiles).reshape(T.num_tiles, -1), T.addrs, T.sym, T.block_range,
                                           T.vgrid, -1), Td)
    ctr = Contraction(V, T, C, mode=mode, sign=-1)
    ctr.contract("a,b,e,f", "e,f,i,j", "a,b,i,j", 0.5)
    got = host(C.tiles).reshape(want.shape)
    err = np.max(np.abs(got - want))
    if mode == "fp64":
        assert err <= 1e-12 * np.abs(want).max(), err
    else:
        assert err <= 1e-13 * np.abs(want).max(), err
    assert ctr.plan("a,b,e,f", "e,f,i,j", "a,b,i,j").flops == 1.189085184e9


@pytest.mark.parametrize("m,n,k,acc", [(1, 7200, 1440, 1), (2, 30, 345000, 0), (1, 40, 100000, 1), (2000, 1, 300, 1),
                                       (700, 2, 65, 0), (17, 1, 2000, 1), (3, 500, 100, 0)])
def test_grouped_gemm_matrix_vector_shapes(gbx, m, n, k, acc):
    """One side at most 2 with K above 64: one warp per output of the wide
    side, lanes striding K, fixed-order reduction; few outputs with long K
    split K into ranges reduced in a fixed order."""
    from dtcf_gb300.leaves import Triple
    rng = np.random.default_rng(m * 3 + n + k)
    A, B, C = rng.standard_normal((m, k)), rng.standard_normal((n, k)), rng.standard_normal((m, n))
    dA, dB, dC = dev(A), dev(B), dev(C)
    gbx.grouped_gemm_f64([Triple(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), k, 1, k, 1, n, m, n, k, 0.25, acc)])
    want = (C if acc else 0.0) + 0.25 * A @ B.T
    got = host(dC).reshape(m, n)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-13 * np.sqrt(k))
    # twice in a row: the same bits (deterministic reduction order)
    dC2 = dev(C)
    gbx.grouped_gemm_f64([Triple(dA.data_ptr(), dB.data_ptr(), dC2.data_ptr(), k, 1, k, 1, n, m, n, k, 0.25, acc)])
    assert np.array_equal(host(dC2).reshape(m, n), got)
    # strided operands through the leaf entry point (A transposed)
    dC3 = dev(C)
    gbx.local_contraction(m, n, k, dev(np.ascontiguousarray(A.T)), dB, dC3, 1, 1, 0.25)
    np.testing.assert_allclose(host(dC3).reshape(m, n), C + 0.25 * A @ B.T, rtol=1e-12, atol=1e-13 * np.sqrt(k))
