"""Generate the golden fixtures in tests/golden/ by running the DTCF reference
leaves themselves (compiled in place from the read-only tree into
oracle/_ref/libref.so by oracle/Makefile).

Run from the repository root, where the reference tree is mounted:
    python tests/golden/make_golden.py
Writes tests/golden/ref_leaves.npz.  Inputs are seeded; outputs come only from
the reference's code, so the fixtures pin the oracle restatement on machines
where the reference tree is absent.
"""
import ctypes
import itertools
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

P = ctypes.c_void_p


def ptr(a):
    return a.ctypes.data_as(P)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def main():
    oracle.build(ref=True)
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("oracle/_ref/libref.so is not built (reference tree missing?)")
    rng = np.random.default_rng(20261203)
    out = {}

    # 1. RRR transpose (helper.cc:275): every 4-D permutation on odd and on
    #    block-8 extents, both 2-D permutations, a 3-D and some 5/6-D cases.
    cases = []
    for widths in [(3, 5, 2, 7), (4, 4, 4, 4), (4, 6, 4, 6)]:
        for perm in itertools.permutations(range(4)):
            cases.append((widths, perm))
    for perm in itertools.permutations(range(2)):
        cases.append(((5, 7), perm))
    for perm in itertools.permutations(range(3)):
        cases.append(((3, 4, 5), perm))
    for widths in [(2, 3, 4, 3, 2), (2, 3, 2, 2, 3, 2)]:
        for _ in range(6):
            cases.append((widths, tuple(rng.permutation(len(widths)))))
    for n, (widths, perm) in enumerate(cases):
        x = rng.standard_normal(int(np.prod(widths)))
        y = np.zeros_like(x)
        ref.ref_transpose(ptr(x), ptr(y), ptr(i32(perm)), ctypes.c_int(len(widths)), ptr(i32(widths)))
        out[f"tr{n}_widths"] = np.array(widths, np.int32)
        out[f"tr{n}_perm"] = np.array(perm, np.int32)
        out[f"tr{n}_in"] = x
        out[f"tr{n}_out"] = y
    out["tr_count"] = np.array(len(cases))

    # 2. DLTC fixed kernels (DLTC/transp-kernel-omp.cc): all 24 4-D output
    #    orders and the 2-D pair, extents odd and a multiple of the 4-tiling.
    n = 0
    for dims in [(3, 5, 2, 7), (4, 4, 8, 4), (5, 3, 4, 2)]:
        for order in itertools.permutations("ijkl"):
            name = "".join(order)
            x = rng.standard_normal(int(np.prod(dims)))
            y = np.zeros_like(x)
            rc = ref.ref_dltc_transpose4(name.encode(), ptr(x), ptr(y), *[ctypes.c_int(d) for d in dims])
            assert rc == 0
            out[f"dl{n}_name"] = np.frombuffer(name.encode(), np.uint8)
            out[f"dl{n}_dims"] = np.array(dims, np.int32)
            out[f"dl{n}_in"] = x
            out[f"dl{n}_out"] = y
            n += 1
    for dims in [(5, 7), (33, 40), (40, 32)]:
        for swap in (0, 1):
            x = rng.standard_normal(int(np.prod(dims)))
            y = np.zeros_like(x)
            ref.ref_dltc_transpose2(ptr(x), ptr(y), ctypes.c_int(dims[0]), ctypes.c_int(dims[1]), ctypes.c_int(swap))
            out[f"dl{n}_name"] = np.frombuffer(b"ji" if swap else b"ij", np.uint8)
            out[f"dl{n}_dims"] = np.array(dims, np.int32)
            out[f"dl{n}_in"] = x
            out[f"dl{n}_out"] = y
            n += 1
    out["dl_count"] = np.array(n)

    # 3. Block_Grid rank <-> address (block_grid.cc:22-67).
    grids = [np.array(g, np.int32) for g in [(6, 6, 2, 2), (3, 5, 2, 7), (4,), (2, 3, 4, 5, 6)]]
    for g_i, g in enumerate(grids):
        total = int(np.prod(g))
        ranks = np.arange(total, dtype=np.int64)
        addrs = np.zeros((total, len(g)), np.int32)
        for r in range(total):
            a = np.zeros(len(g), np.int32)
            ref.ref_block_addr(ctypes.c_long(r), ctypes.c_int(len(g)), ptr(g), ptr(a))
            addrs[r] = a
            back = ref.ref_block_rank(ptr(a), ctypes.c_int(len(g)), ptr(g))
            assert back == r
        out[f"bg{g_i}_grid"] = g
        out[f"bg{g_i}_addrs"] = addrs
        out[f"bg{g_i}_ranks"] = ranks
    out["bg_count"] = np.array(len(grids))

    # 4. RRR unique tiles and block-constant values (tensor.cc:315-335, 617-758).
    tcases = [("aabb", (48, 48, 16, 16), (6, 6, 2, 2)), ("abab", (24, 16, 24, 16), (3, 2, 3, 2)),
              ("cdaa", (8, 12, 20, 20), (2, 3, 5, 5)), ("aa", (40, 40), (5, 5)), ("cccc", (16, 16, 16, 16), (2, 2, 2, 2)),
              ("aaa", (12, 12, 12), (4, 4, 4))]
    for t_i, (sym, sizes, vgrid) in enumerate(tcases):
        dims = len(sym)
        bs = int(np.prod([s // v for s, v in zip(sizes, vgrid)]))
        cap = int(np.prod(vgrid))
        tiles = np.zeros(cap * bs)
        addr = np.zeros(cap * dims, np.int32)
        nt = ref.ref_tensor_tiles(sym.encode(), ptr(i32(sizes)), ptr(i32(vgrid)), ptr(tiles), ptr(addr), ctypes.c_long(cap))
        assert nt > 0
        out[f"tt{t_i}_sym"] = np.frombuffer(sym.encode(), np.uint8)
        out[f"tt{t_i}_sizes"] = np.array(sizes, np.int32)
        out[f"tt{t_i}_vgrid"] = np.array(vgrid, np.int32)
        out[f"tt{t_i}_addr"] = addr[: nt * dims].reshape(nt, dims)
        out[f"tt{t_i}_tiles"] = tiles[: nt * bs].reshape(nt, bs)
    out["tt_count"] = np.array(len(tcases))

    # 5. create_big_matrix / revert_big_matrix (transpose_helper.cc:20-409) on a
    #    full non-symmetric tile set with a permuting p_map, the shape of the
    #    round trip in test.cc:633-728.
    bcases = [("cccc", (12, 8, 12, 8), (3, 2, 3, 2), (0, 1, 2, 3), 2),
              ("cccc", (12, 8, 12, 8), (3, 2, 3, 2), (2, 0, 3, 1), 2),
              ("cccc", (6, 8, 10, 4), (3, 2, 5, 2), (1, 3, 0, 2), 1),
              ("ccc", (6, 8, 10), (3, 2, 5), (2, 0, 1), 2)]
    for b_i, (sym, sizes, vgrid, p_map, nrd) in enumerate(bcases):
        dims = len(sym)
        br = [s // v for s, v in zip(sizes, vgrid)]
        bs = int(np.prod(br))
        addrs = np.array(list(itertools.product(*[range(v) for v in vgrid])), np.int32)
        order = rng.permutation(len(addrs))
        addrs = addrs[order]
        perm_addr = np.zeros_like(addrs)
        for d in range(dims):
            perm_addr[:, p_map[d]] = addrs[:, d]
        tiles = rng.standard_normal((len(addrs), bs))
        pbr = [0] * dims
        for d in range(dims):
            pbr[p_map[d]] = br[d]
        rpb = int(np.prod(pbr[:nrd]))
        cpb = int(np.prod(pbr[nrd:]))
        big = np.zeros(tiles.size)
        ref.ref_create_big_matrix(sym.encode(), ptr(i32(sizes)), ptr(i32(vgrid)), ptr(tiles), ptr(i32(perm_addr)),
                                  ptr(i32(p_map)), ctypes.c_int(len(addrs)), ctypes.c_int(rpb), ctypes.c_int(cpb),
                                  ctypes.c_int(nrd), ptr(big))
        big2 = rng.standard_normal(tiles.size)
        back = np.zeros_like(tiles)
        ref.ref_revert_big_matrix(sym.encode(), ptr(i32(sizes)), ptr(i32(vgrid)), ptr(tiles), ptr(i32(perm_addr)),
                                  ptr(i32(p_map)), ctypes.c_int(len(addrs)), ctypes.c_int(rpb), ctypes.c_int(cpb),
                                  ctypes.c_int(nrd), ptr(big2), ptr(back))
        pre = f"bm{b_i}_"
        out[pre + "vgrid"] = np.array(vgrid, np.int32)
        out[pre + "p_map"] = np.array(p_map, np.int32)
        out[pre + "perm_addr"] = perm_addr
        out[pre + "tiles"] = tiles
        out[pre + "rpb"] = np.array(rpb)
        out[pre + "cpb"] = np.array(cpb)
        out[pre + "nrd"] = np.array(nrd)
        out[pre + "big"] = big
        out[pre + "big2"] = big2
        out[pre + "back"] = back
    out["bm_count"] = np.array(len(bcases))

    # 6. local_contraction (localcontract.cc:3) on shapes where its leading
    #    dimensions are right (n_b == n_k for bt=1), at=0, beta=1.
    lcases = [(8, 8, 8, 0, 1, 1.0), (12, 16, 16, 0, 1, 0.5), (64, 48, 48, 0, 1, -1.0), (7, 5, 9, 0, 0, 2.0),
              (30, 20, 20, 0, 1, 1.0)]
    for c_i, (na, nb, nk, at, bt, alpha) in enumerate(lcases):
        A = rng.standard_normal(na * nk)
        B = rng.standard_normal(nb * nk)
        C = rng.standard_normal(na * nb)
        C_in = C.copy()
        ref.ref_local_contraction(na, nb, nk, ptr(A), ptr(B), ptr(C), at, bt, alpha)
        pre = f"lc{c_i}_"
        out[pre + "shape"] = np.array([na, nb, nk, at, bt])
        out[pre + "alpha"] = np.array(alpha)
        out[pre + "A"] = A
        out[pre + "B"] = B
        out[pre + "C_in"] = C_in
        out[pre + "C_out"] = C
    out["lc_count"] = np.array(len(lcases))

    # 7. create_big_matrix_nl (transpose_helper.cc:184-328): the addresses in
    #    a shuffled order, the tile data in a second, independent order of
    #    slots (plus unused slots), the address_to_location map from each
    #    address's rank in the permuted grid to its slot -- as
    #    Contraction::contract builds it (contraction.cc:2399-2410).  Own
    #    generator, so the fixtures above stay as they were.
    rng7 = np.random.default_rng(20261204)
    ncases = [("cccc", (12, 8, 12, 8), (3, 2, 3, 2), (2, 0, 3, 1), 2),
              ("cccc", (6, 8, 10, 4), (3, 2, 5, 2), (1, 3, 0, 2), 1),
              ("ccc", (6, 8, 10), (3, 2, 5), (2, 0, 1), 2)]
    for n_i, (sym, sizes, vgrid, p_map, nrd) in enumerate(ncases):
        dims = len(sym)
        br = [s // v for s, v in zip(sizes, vgrid)]
        bs = int(np.prod(br))
        addrs = np.array(list(itertools.product(*[range(v) for v in vgrid])), np.int32)
        addrs = addrs[rng7.permutation(len(addrs))]
        perm_addr = np.zeros_like(addrs)
        for d in range(dims):
            perm_addr[:, p_map[d]] = addrs[:, d]
        grid_T = [0] * dims
        for d in range(dims):
            grid_T[p_map[d]] = vgrid[d]
        ranks = [int(ref.ref_block_rank(ptr(i32(a)), ctypes.c_int(dims), ptr(i32(grid_T)))) for a in perm_addr]
        nslots = len(addrs) + 3
        slots = rng7.permutation(nslots)[: len(addrs)]
        tiles = rng7.standard_normal((nslots, bs))
        pbr = [0] * dims
        for d in range(dims):
            pbr[p_map[d]] = br[d]
        rpb = int(np.prod(pbr[:nrd]))
        cpb = int(np.prod(pbr[nrd:]))
        big = np.zeros(len(addrs) * bs)
        ref.ref_create_big_matrix_nl(sym.encode(), ptr(i32(sizes)), ptr(i32(vgrid)), ptr(tiles), ptr(i32(perm_addr)),
                                     ptr(i32(p_map)), ctypes.c_int(len(addrs)), ctypes.c_int(rpb), ctypes.c_int(cpb),
                                     ctypes.c_int(nrd), ptr(i32(ranks)), ptr(i32(slots)), ctypes.c_int(len(addrs)),
                                     ptr(big))
        pre = f"nl{n_i}_"
        out[pre + "vgrid"] = np.array(vgrid, np.int32)
        out[pre + "p_map"] = np.array(p_map, np.int32)
        out[pre + "perm_addr"] = perm_addr
        out[pre + "ranks"] = np.array(ranks, np.int32)
        out[pre + "slots"] = np.array(slots, np.int32)
        out[pre + "tiles"] = tiles
        out[pre + "rpb"] = np.array(rpb)
        out[pre + "cpb"] = np.array(cpb)
        out[pre + "nrd"] = np.array(nrd)
        out[pre + "big"] = big
    out["nl_count"] = np.array(len(ncases))

    path = os.path.join(ROOT, "tests", "golden", "ref_leaves.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
