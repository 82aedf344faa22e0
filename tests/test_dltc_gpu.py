"""GPU parity of the DLTC executor against the oracle's tile loops
(oracle.task_mul / oracle.task_sum, the restatement of DLTC/task.cc:51-137):

* the reference's own correctness checks, checkM (abij += akil * bljk,
  DLTC/checkerM.cc:39-47) and checkS (abij += baji, DLTC/checkerS.cc:35-41),
  with O = V = 4, tile width 1 and 2 * drand48() - 1 inputs in the default
  drand48 state, through the CUDA path at the reference's 1e-8 tolerance;
* every expression of the three residual tables (DLTC/ccd-t2.cc,
  DLTC/ccsd-t1.cc, DLTC/ccsd-t2.cc) alone on seeded inputs, FP64 engine and
  split engine, within 1e-12 relative of the oracle;
* each table run whole as a program (layers in order, intermediates
  starting from zero) against the oracle running the same list;
* task ranges (a subset of tiles) against the tile loop's definition."""
import itertools

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

TABLES = ["ccd_t2", "ccsd_t1", "ccsd_t2"]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_checkM_checkS_through_the_gpu():
    from dtcf_gb300 import dltc
    O = V = 4
    H1, H2, H3, H4, P1, P2 = 0, 1, 2, 3, 6, 7  # check build: H1..H6 = 0..5, P1..P6 = 6..11
    d = dltc.dims(O, V, 1, 1, nocc_names=6)
    rng = oracle.Drand48()
    A = 2 * rng.next(V * O * O * O) - 1
    B = 2 * rng.next(V * O * O * O) - 1
    sC = np.zeros(V * V * O * O)  # checkerM.cc:39-47
    for a, b, i, j, k, l in itertools.product(range(V), range(V), range(O), range(O), range(O), range(O)):
        sC[a * V * O * O + b * O * O + i * O + j] += A[a * O * O * O + k * O * O + i * O + l] * \
            B[b * O * O * O + l * O * O + j * O + k]
    for mode in ("fp64", "split"):
        pC = torch.zeros(V * V * O * O, dtype=torch.float64, device="cuda")
        dltc.task_mul(1.0, [P1, P2, H1, H2], pC, [P1, H4, H1, H3], dev(A), [P2, H3, H2, H4], dev(B), d, mode=mode)
        got = host(pC)
        assert np.max(np.abs(got - sC)) <= 1e-8, mode  # checker.h:15 PRECISION
        want = np.zeros_like(sC)
        oracle.task_mul(1.0, [P1, P2, H1, H2], want, [P1, H4, H1, H3], A, [P2, H3, H2, H4], B, O, V, 1, 1, 6, 12)
        assert np.max(np.abs(got - want)) <= 1e-13, mode
    X = 2 * oracle.Drand48().next(V * V * O * O) - 1
    sS = np.zeros(V * V * O * O)  # checkerS.cc:35-41
    for a, b, i, j in itertools.product(range(V), range(V), range(O), range(O)):
        sS[a * V * O * O + b * O * O + i * O + j] += X[b * V * O * O + a * O * O + j * O + i]
    pS = torch.zeros(V * V * O * O, dtype=torch.float64, device="cuda")
    dltc.task_sum(1.0, [P1, P2, H1, H2], pS, [P2, P1, H2, H1], dev(X), d)
    assert np.array_equal(host(pS), sS)


DIMS = dict(O=8, V=12, wbO=4, wbV=6)


def _shape(ids, O, V):
    return [O if x < 12 else V for x in ids]


def _inputs(t, seed):
    rng = np.random.default_rng(seed)
    out = []
    for name, types in t["tensors"]:
        n = int(np.prod([DIMS["O"] if ty == 0 else DIMS["V"] for ty in types]))
        out.append(rng.uniform(-1, 1, n))
    return out


@pytest.mark.parametrize("which", TABLES)
@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_every_expression_alone_vs_oracle(which, mode):
    from dtcf_gb300 import dltc
    t = dltc.table(which)
    d = dltc.dims(DIMS["O"], DIMS["V"], DIMS["wbO"], DIMS["wbV"])
    data = _inputs(t, 11)
    O, V, wbO, wbV = DIMS["O"], DIMS["V"], DIMS["wbO"], DIMS["wbV"]
    for e in t["exprs"]:
        C = data[e["c"]].copy()
        dC = dev(C)
        if e["kind"] == dltc.MUL:
            dltc.task_mul(e["coef"], e["idC"], dC, e["idA"], dev(data[e["a"]]), e["idB"], dev(data[e["b"]]), d,
                          mode=mode)
            oracle.task_mul(e["coef"], e["idC"], C, e["idA"], data[e["a"]], e["idB"], data[e["b"]], O, V, wbO, wbV,
                            12, 24)
        else:
            dltc.task_sum(e["coef"], e["idC"], dC, e["idA"], dev(data[e["a"]]), d)
            oracle.task_sum(e["coef"], e["idC"], C, e["idA"], data[e["a"]], O, V, wbO, wbV, 12)
        got = host(dC)
        err = np.max(np.abs(got - C)) / max(1.0, np.abs(C).max())
        tol = 1e-12 if mode == "fp64" else 1e-12
        assert err <= tol, (which, e["kind"], e["index"], err)
        if e["kind"] == dltc.SUM:
            assert np.array_equal(got, C), (which, e["index"])


@pytest.mark.parametrize("which", TABLES)
@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_whole_table_program_vs_oracle(which, mode):
    """The table as DLTC runs it: inputs set, outputs and intermediates from
    zero, the layers in order; every tensor against the oracle running the
    same expression list on the host."""
    from dtcf_gb300 import dltc
    d = dltc.dims(DIMS["O"], DIMS["V"], DIMS["wbO"], DIMS["wbV"])
    prog = dltc.Program(which, d, mode=mode)
    t = prog.table
    written = {e["c"] for e in t["exprs"]}
    data = _inputs(t, 5)
    for i in range(len(t["tensors"])):
        if i in written:
            data[i][:] = 0.0
        prog.tensor(i).copy_(dev(data[i]))
    prog.run()
    prog.check()
    O, V, wbO, wbV = DIMS["O"], DIMS["V"], DIMS["wbO"], DIMS["wbV"]
    for e in t["exprs"]:
        if e["kind"] == dltc.MUL:
            oracle.task_mul(e["coef"], e["idC"], data[e["c"]], e["idA"], data[e["a"]], e["idB"], data[e["b"]], O, V,
                            wbO, wbV, 12, 24)
        else:
            oracle.task_sum(e["coef"], e["idC"], data[e["c"]], e["idA"], data[e["a"]], O, V, wbO, wbV, 12)
    for i, (name, _) in enumerate(t["tensors"]):
        got = host(prog.tensor(i))
        scale = max(1.0, np.abs(data[i]).max())
        assert np.max(np.abs(got - data[i])) <= 1e-12 * scale, (which, name)
    assert prog.flops > 0
    prog.close()


def test_task_ranges_match_the_tile_loop_definition():
    """task_mul / task_sum over a subset of tiles: only C tiles in the range
    change, and they receive the sum over the contracted tiles in the range."""
    from dtcf_gb300 import dltc
    O, V, wbO, wbV = 8, 12, 2, 3
    d = dltc.dims(O, V, wbO, wbV)
    h1, h2, h5, p3, p4, p6 = 0, 1, 4, 14, 15, 17
    rng = np.random.default_rng(4)
    # R[p3,p4,h1,h2] += 0.5 T[p3,p6,h1,h5] * I[h5,p6,h2,p4]
    idC, idA, idB = [p3, p4, h1, h2], [p3, p6, h1, h5], [h5, p6, h2, p4]
    A = rng.uniform(-1, 1, (V, V, O, O))
    B = rng.uniform(-1, 1, (O, V, O, V))
    C = rng.uniform(-1, 1, (V, V, O, O))
    lo = np.zeros(24, dtype=np.int32)
    hi = np.array([O // wbO] * 12 + [V // wbV] * 12, dtype=np.int32)
    lo[p3], hi[p3] = 1, 3
    lo[h2], hi[h2] = 2, 4
    lo[p6], hi[p6] = 0, 2
    lo[h5], hi[h5] = 1, 2
    dC = dev(C)
    dltc.task_mul(0.5, idC, dC, idA, dev(A), idB, dev(B), d, lo=lo, hi=hi)
    wb = [wbO] * 12 + [wbV] * 12
    sl = {x: slice(lo[x] * wb[x], hi[x] * wb[x]) for x in range(24)}
    want = C.copy()
    want[sl[p3], sl[p4], sl[h1], sl[h2]] += 0.5 * np.einsum(
        "acie,ecjb->abij", A[sl[p3], sl[p6], sl[h1], sl[h5]], B[sl[h5], sl[p6], sl[h2], sl[p4]])
    np.testing.assert_allclose(host(dC).reshape(C.shape), want, rtol=0, atol=1e-13)
    # task_sum over a range: C[p3,h1] += -1 * A[h1,p3] on the range's tiles only
    X = rng.uniform(-1, 1, (O, V))
    Y = rng.uniform(-1, 1, (V, O))
    dY = dev(Y)
    lo2, hi2 = lo.copy(), hi.copy()
    lo2[h1], hi2[h1] = 1, 3
    dltc.task_sum(-1.0, [p3, h1], dY, [h1, p3], dev(X), d, lo=lo2, hi=hi2)
    want = Y.copy()
    s3, s1 = slice(lo2[p3] * wbV, hi2[p3] * wbV), slice(lo2[h1] * wbO, hi2[h1] * wbO)
    want[s3, s1] += -1.0 * X[s1, s3].T
    assert np.array_equal(host(dY).reshape(Y.shape), want)
