"""CPU checks of the irrep-blocked CC oracle against the dense oracle: the
blocked integrals are the dense ones cut by irrep, and CCD / CCSD energies
and amplitudes agree at every iteration on small systems (1, 2, 4 and 8
irreps, uneven blocks)."""
import numpy as np
import pytest

from oracle import cc, cc_blocks

CASES = [
    dict(nocc=6, nvir=14, nirrep=2, max_block=5, seed=3),
    dict(nocc=8, nvir=24, nirrep=4, max_block=4, min_block=1, seed=7),
    dict(nocc=8, nvir=20, nirrep=1, max_block=8, seed=11),
    dict(nocc=10, nvir=30, nirrep=8, max_block=4, min_block=1, seed=5),
]


def _system(c):
    return cc.System(c["nocc"], c["nvir"], nirrep=c["nirrep"], max_block=c["max_block"],
                     min_block=c.get("min_block", 1), seed=c["seed"])


def test_blocked_integrals_are_the_dense_ones():
    s = _system(CASES[3])
    dense = s.integrals()
    sp = cc_blocks.Spaces(s)
    o, n = s.o, s.n
    for kinds in cc_blocks.INTEGRALS:
        sl = tuple(slice(0, o) if c == "o" else slice(o, n) for c in kinds)
        bt = cc_blocks.BT.integrals(sp, kinds)
        assert bt.max_abs_diff_dense(dense[sl], {"o": 0, "v": o}) == 0.0
        # the C generator and the numpy statement agree bit for bit (signs of zeros included)
        slow = cc_blocks.BT.integrals(sp, kinds, fast=False)
        for k, b in bt.blocks.items():
            assert b.tobytes() == slow.blocks[k].tobytes(), (kinds, k)
        # no nonzero element lives outside the irrep blocks
        back = bt.to_dense({"o": 0, "v": o}, {"o": o, "v": s.v})
        assert np.array_equal(back, dense[sl])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("method", ["ccd", "ccsd"])
def test_blocked_oracle_matches_dense_oracle(case, method):
    s = _system(case)
    d = cc.CC(s, method)
    b = cc_blocks.CC(s, method)
    ed, eb = np.array(d.iterate(5)), np.array(b.iterate(5))
    assert np.max(np.abs(ed - eb)) <= 1e-14, (ed, eb)
    assert np.max(np.abs(b.dense_t2() - d.t2)) <= 1e-15
    assert np.max(np.abs(b.dense_t1() - d.t1)) <= 1e-15
