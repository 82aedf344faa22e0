"""CPU checks of the DLTC executor's host side: the residual tables the
library carries are the reference's own (tests/golden/dltc_tables.json, read
from DLTC/ccd-t2.cc, DLTC/ccsd-t1.cc and DLTC/ccsd-t2.cc by
tests/golden/make_dltc_tables.py), and the Multiplication orders follow
DLTC/expr.cc:13-67."""
import itertools
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden_tables():
    return json.load(open(os.path.join(HERE, "golden", "dltc_tables.json")))


@pytest.mark.parametrize("which", ["ccd_t2", "ccsd_t1", "ccsd_t2"])
def test_tables_are_the_references(golden_tables, which):
    from dtcf_gb300 import dltc
    ref = golden_tables[which]
    t = dltc.table(which)
    assert [n for n, _ in t["tensors"]] == ref["tensors"]
    for n, ty in t["tensors"]:
        assert ty == [0 if x == "HOL" else 1 for x in ref["types"][n]], n
    names = ref["tensors"]
    got = [(("MUL" if e["kind"] == dltc.MUL else "SUM"), e["index"]) for e in t["exprs"]]
    want = [tuple(x) for layer in ref["layers"] for x in layer]
    assert got == want
    layers = [e["layer"] for e in t["exprs"]]
    assert layers == [i for i, layer in enumerate(ref["layers"]) for _ in layer]
    muls = {m["index"]: m for m in ref["muls"]}
    sums = {s["index"]: s for s in ref["sums"]}
    for e in t["exprs"]:
        r = muls[e["index"]] if e["kind"] == dltc.MUL else sums[e["index"]]
        assert names[e["c"]] == r["C"] and names[e["a"]] == r["A"]
        assert e["idC"] == r["idC"] and e["idA"] == r["idA"] and e["coef"] == r["coef"]
        if e["kind"] == dltc.MUL:
            assert names[e["b"]] == r["B"] and e["idB"] == r["idB"]
        else:
            assert e["b"] == -1


def _orders(idA, idB):
    """Restatement of the Multiplication constructor: names of A only, of B
    only, of both, each sorted."""
    return (sorted(set(idA) - set(idB)), sorted(set(idB) - set(idA)), sorted(set(idA) & set(idB)))


def test_mul_orders_follow_the_constructor(golden_tables):
    from dtcf_gb300 import dltc
    # the constructor's own example (DLTC/expr.h): abij += akil * bljk -> iajb += iakl * kljb,
    # in the check build's names H1..H6 = 0..5, P1..P6 = 6..11
    a, b, i, j, k, l = 6, 7, 0, 1, 2, 3
    m, n, kk = dltc.mul_orders([a, k, i, l], [b, l, j, k])
    assert m + n == [i, a, j, b] and m + kk == [i, a, k, l] and kk + n == [k, l, j, b]
    for t in golden_tables.values():
        for mu in t["muls"]:
            assert dltc.mul_orders(mu["idA"], mu["idB"]) == _orders(mu["idA"], mu["idB"])
    for idA, idB in itertools.product([[0, 1], [12, 0, 3, 14]], [[1, 2], [3, 14, 15, 16]]):
        assert dltc.mul_orders(idA, idB) == _orders(idA, idB)


def test_bad_expressions_are_rejected_on_the_host():
    from dtcf_gb300 import dltc
    from dtcf_gb300._lib import GbxError
    d = dltc.dims(4, 8, 2, 4)
    with pytest.raises(GbxError):
        dltc.mul_orders([0, 0], [1, 2])  # repeated name
    with pytest.raises(GbxError):
        dltc.Program(7, d)  # unknown table
    with pytest.raises(GbxError):
        dltc.Program("ccd_t2", dltc.dims(4, 8, 3, 4))  # O not a multiple of wbO
