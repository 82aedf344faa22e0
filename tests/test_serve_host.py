"""Host-side parts of job admission (no GPU): the planned footprint comes from
host planning alone, grows with the problem, and the server records it."""
import ctypes

import pytest

from dtcf_gb300 import GbxError
from dtcf_gb300._lib import lib
from dtcf_gb300.cc import config
from dtcf_gb300.serve import Server


def footprint(**kw):
    c = config(**kw)
    r, p, f = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    assert lib().gbx_cc_footprint(ctypes.byref(c), ctypes.byref(r), ctypes.byref(p), ctypes.byref(f)) == 0
    return r.value, p.value, f.value


def test_footprint_is_host_only_and_monotone():
    small = footprint(nocc=8, nvir=32, nirrep=1, max_block=8, method="ccsd", engine="split")
    big = footprint(nocc=12, nvir=48, nirrep=1, max_block=8, method="ccsd", engine="split")
    ccd = footprint(nocc=12, nvir=48, nirrep=1, max_block=8, method="ccd", engine="split")
    sym = footprint(nocc=12, nvir=48, nirrep=4, max_block=8, min_block=1, method="ccsd", engine="split")
    for r, p, f in (small, big, ccd, sym):
        assert 0 < r <= p and f > 0
    assert big[0] > small[0] and big[2] > small[2]
    assert ccd[2] < big[2]
    assert sym[0] < big[0] and sym[2] < big[2]


@pytest.mark.parametrize("method", ["ccd", "ccsd"])
@pytest.mark.parametrize("engine", ["fp64", "split"])
@pytest.mark.parametrize("nocc,nvir,nirrep,max_block,min_block", [
    (4, 64, 1, 64, 1),     # 64 x 64 (a, b) slabs: fused-sum items cover half slabs
    (6, 14, 2, 5, 1),      # ragged blocks, two irreps
    (8, 24, 4, 4, 1),      # blocks of 1..4 orbitals
    (16, 48, 8, 6, 1),     # eight irreps, uneven occupations
    (24, 120, 8, 40, 4),   # the bench system's blocking at a smaller size
])
def test_host_planning_of_every_step(method, engine, nocc, nvir, nirrep, max_block, min_block):
    """Every step of an iteration -- contraction plans on the packed or the
    direct engine, the fused permuted sums, the tau-family tile table -- is
    planned on the host (no device) for a range of blockings, and the peak
    covers the resident bytes."""
    r, p, f = footprint(nocc=nocc, nvir=nvir, nirrep=nirrep, max_block=max_block, min_block=min_block,
                        method=method, engine=engine, slices=4)
    assert 0 < r <= p and f > 0


def test_server_records_footprints_and_validates_requests():
    s = Server(budget_bytes=1e9, slots=2)
    j = s.add_job(config(nocc=8, nvir=32, nirrep=1, max_block=8, method="ccd", engine="fp64"))
    want = footprint(nocc=8, nvir=32, nirrep=1, max_block=8, method="ccd", engine="fp64")[0]
    assert s.footprints[j] == pytest.approx(want)
    s.submit(j, 0.0)
    with pytest.raises(GbxError):
        s.submit(j + 1, 0.0)
    with pytest.raises(GbxError):
        s.submit(j, -1.0)
    s.close()
    with pytest.raises(GbxError):
        Server(budget_bytes=0, slots=2)
