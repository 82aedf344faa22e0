"""Pins the oracle's C restatement (oracle/leaves.c) to the DTCF reference:
against the fixtures that tests/golden/make_golden.py wrote by running the
reference leaves, and -- where oracle/_ref/libref.so is built -- against the
reference leaves directly on fresh seeded inputs."""
import ctypes
import itertools

import numpy as np
import pytest

import oracle


def test_transpose_matches_reference_fixtures(golden):
    for n in range(int(golden["tr_count"])):
        w, p = golden[f"tr{n}_widths"], golden[f"tr{n}_perm"]
        x = golden[f"tr{n}_in"].reshape(w)
        y = oracle.transpose(x, p)
        assert np.array_equal(y.reshape(-1), golden[f"tr{n}_out"]), (w, p)


def test_dltc_kernels_match_reference_fixtures(golden):
    for n in range(int(golden["dl_count"])):
        name = bytes(golden[f"dl{n}_name"]).decode()
        dims = golden[f"dl{n}_dims"]
        x = golden[f"dl{n}_in"].reshape(dims)
        ids_x = list(range(len(dims)))
        ids_y = ["ijkl".index(c) for c in name]
        y = oracle.dltc_transpose(x, ids_x, ids_y)
        assert np.array_equal(y.reshape(-1), golden[f"dl{n}_out"]), name


def test_block_grid_matches_reference_fixtures(golden):
    for g in range(int(golden["bg_count"])):
        grid = golden[f"bg{g}_grid"]
        for r, a in zip(golden[f"bg{g}_ranks"], golden[f"bg{g}_addrs"]):
            assert oracle.block_rank(a, grid) == r
            assert np.array_equal(oracle.block_addr(int(r), grid), a)


def test_rrr_tiles_match_reference_fixtures(golden):
    for t in range(int(golden["tt_count"])):
        sym = bytes(golden[f"tt{t}_sym"]).decode()
        addr = oracle.rrr_tiles(sym, golden[f"tt{t}_vgrid"])
        assert np.array_equal(addr, golden[f"tt{t}_addr"]), sym
        vals = oracle.rrr_block_values(addr)
        tiles = golden[f"tt{t}_tiles"]
        assert np.array_equal(np.repeat(vals[:, None], tiles.shape[1], axis=1), tiles), sym


def test_big_matrix_matches_reference_fixtures(golden):
    for b in range(int(golden["bm_count"])):
        pre = f"bm{b}_"
        args = (golden[pre + "vgrid"], golden[pre + "p_map"])
        rpb, cpb, nrd = int(golden[pre + "rpb"]), int(golden[pre + "cpb"]), int(golden[pre + "nrd"])
        big = oracle.create_big_matrix(*args, golden[pre + "tiles"], golden[pre + "perm_addr"], rpb, cpb, nrd)
        assert np.array_equal(big.reshape(-1), golden[pre + "big"])
        back = oracle.revert_big_matrix(*args, golden[pre + "perm_addr"], rpb, cpb, nrd, golden[pre + "big2"])
        assert np.array_equal(back, golden[pre + "back"])
        # round trip, as test.cc:633-728 requires
        rt = oracle.revert_big_matrix(*args, golden[pre + "perm_addr"], rpb, cpb, nrd, big)
        assert np.array_equal(rt, golden[pre + "tiles"])



def test_big_matrix_nl_matches_reference_fixtures(golden):
    """create_big_matrix_nl (transpose_helper.cc:184-328): tile data looked
    up through address_to_location, against the compiled reference."""
    for b in range(int(golden["nl_count"])):
        pre = f"nl{b}_"
        loc = dict(zip(golden[pre + "ranks"].tolist(), golden[pre + "slots"].tolist()))
        big = oracle.create_big_matrix_nl(golden[pre + "vgrid"], golden[pre + "p_map"], golden[pre + "tiles"],
                                          golden[pre + "perm_addr"], int(golden[pre + "rpb"]), int(golden[pre + "cpb"]),
                                          int(golden[pre + "nrd"]), loc)
        assert np.array_equal(big.reshape(-1), golden[pre + "big"])
    # a placed address without a location is an error, as the reference asserts
    pre = "nl0_"
    loc = dict(zip(golden[pre + "ranks"].tolist()[1:], golden[pre + "slots"].tolist()[1:]))
    with pytest.raises(KeyError):
        oracle.create_big_matrix_nl(golden[pre + "vgrid"], golden[pre + "p_map"], golden[pre + "tiles"],
                                    golden[pre + "perm_addr"], int(golden[pre + "rpb"]), int(golden[pre + "cpb"]),
                                    int(golden[pre + "nrd"]), loc)

def test_local_contraction_matches_reference_fixtures(golden):
    for c in range(int(golden["lc_count"])):
        pre = f"lc{c}_"
        na, nb, nk, at, bt = [int(v) for v in golden[pre + "shape"]]
        C = golden[pre + "C_in"].copy()
        oracle.local_contraction(na, nb, nk, golden[pre + "A"], golden[pre + "B"], C, at, bt, float(golden[pre + "alpha"]))
        np.testing.assert_allclose(C, golden[pre + "C_out"], rtol=1e-13, atol=1e-13)


def test_local_contraction_defect_d1_is_corrected():
    """The reference passes n_b as the leading dimension of B^T; the
    restatement is right for every shape (checked against numpy)."""
    rng = np.random.default_rng(1)
    for na, nb, nk in [(3, 5, 7), (6, 4, 9), (8, 8, 2)]:
        A, B, C = rng.standard_normal((na, nk)), rng.standard_normal((nb, nk)), rng.standard_normal((na, nb))
        want = C + 0.75 * A @ B.T
        oracle.local_contraction(na, nb, nk, A, B, C, 0, 1, 0.75)
        np.testing.assert_allclose(C, want, rtol=1e-13, atol=1e-13)


def test_symm_permutation_and_permutation_map():
    # aabb tile [1,3,0,2]: group 0 pair flipped (1<3), group 1 pair flipped (0<2)
    assert list(oracle.symm_permutation([1, 3, 0, 2], [0, 0, 1, 1])) == [1, 0, 3, 2]
    assert list(oracle.symm_permutation([3, 1, 2, 0], [0, 0, 1, 1])) == [0, 1, 2, 3]
    assert list(oracle.symm_permutation([0, 1, 2, 3], [3, 3, 3, 3])) == [0, 1, 2, 3]
    assert list(oracle.compose_p_maps([1, 0, 3, 2], [2, 3, 0, 1])) == [3, 2, 1, 0]
    # C[a,b,m,n] = A[a,b,k,l] * B[m,n,k,l]  (examples/cntr1a_4D.cc:104-106)
    r = oracle.generate_permutation_map([0, 0, 1, 1], [0, 1, 0, 0], [4, 4, 5, 6],
                                        [0, 0, 1, 1], [2, 3, 0, 0], [2, 3, 5, 6], [4, 4, 2, 3],
                                        [(2, 2), (3, 3)])
    assert list(r["p_map_A"]) == [0, 1, 2, 3] and list(r["p_map_B"]) == [0, 1, 2, 3]
    assert list(r["p_map_C"]) == [0, 1, 2, 3] and (r["n_a"], r["n_b"], r["n_k"]) == (16, 6, 30)


def test_checkM_checkS_dense_loops_agree_with_tile_loop():
    """DLTC checkerM.cc:39-47 / checkerS.cc:35-41: O=V=4, tile width 1,
    inputs 2*drand48()-1 in the default drand48 state (A then B)."""
    O = V = 4
    H1, H2, H3, H4, P1, P2 = 0, 1, 2, 3, 6, 7
    rng = oracle.Drand48()
    A = 2 * rng.next(V * O * O * O) - 1
    B = 2 * rng.next(V * O * O * O) - 1
    sC = np.zeros(V * V * O * O)
    for a, b, i, j, k, l in itertools.product(range(V), range(V), range(O), range(O), range(O), range(O)):
        sC[a*V*O*O + b*O*O + i*O + j] += A[a*O*O*O + k*O*O + i*O + l] * B[b*O*O*O + l*O*O + j*O + k]
    pC = np.zeros_like(sC)
    oracle.task_mul(1.0, [P1, P2, H1, H2], pC, [P1, H4, H1, H3], A, [P2, H3, H2, H4], B, O, V, 1, 1, 6, 12)
    assert np.max(np.abs(sC - pC)) <= 1e-8       # checker.h:15 PRECISION
    # checkS: abij += baji
    X = 2 * oracle.Drand48().next(V * V * O * O) - 1
    sS = np.zeros(V * V * O * O)
    for a, b, i, j in itertools.product(range(V), range(V), range(O), range(O)):
        sS[a*V*O*O + b*O*O + i*O + j] += X[b*V*O*O + a*O*O + j*O + i]
    pS = np.zeros_like(sS)
    oracle.task_sum(1.0, [P1, P2, H1, H2], pS, [P2, P1, H2, H1], X, O, V, 1, 1, 6)
    assert np.array_equal(sS, pS)


def test_task_mul_wider_tiles_matches_einsum():
    rng = np.random.default_rng(3)
    O, V, wbO, wbV = 4, 6, 2, 3
    h1, h2, h3, h4, p1, p2 = 0, 1, 2, 3, 12, 13
    A = rng.standard_normal((V, O, O, O))   # (p1, h4, h1, h3)
    B = rng.standard_normal((V, O, O, O))   # (p2, h3, h2, h4)
    C = np.zeros((V, V, O, O))
    oracle.task_mul(0.5, [p1, p2, h1, h2], C, [p1, h4, h1, h3], A, [p2, h3, h2, h4], B, O, V, wbO, wbV, 12, 24)
    want = 0.5 * np.einsum("alik,bkjl->abij", A, B)
    np.testing.assert_allclose(C, want, rtol=1e-12, atol=1e-12)


ref = oracle.ref()
needs_ref = pytest.mark.skipif(ref is None, reason="reference leaves not built here (oracle/_ref)")


@needs_ref
def test_transpose_direct_against_reference_random_shapes():
    rng = np.random.default_rng(7)
    P = ctypes.c_void_p
    for _ in range(200):
        dims = int(rng.integers(2, 7))
        w = rng.integers(1, 6, size=dims).astype(np.int32)
        perm = rng.permutation(dims).astype(np.int32)
        x = rng.standard_normal(int(np.prod(w)))
        y = np.zeros_like(x)
        ref.ref_transpose(x.ctypes.data_as(P), y.ctypes.data_as(P), perm.ctypes.data_as(P), ctypes.c_int(dims),
                          w.ctypes.data_as(P))
        assert np.array_equal(oracle.transpose(x.reshape(w), perm).reshape(-1), y)
