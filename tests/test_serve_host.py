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
