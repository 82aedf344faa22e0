"""The serving loop (gbx_server_*): each job's energies are the same alone,
in a mix of concurrent jobs of other sizes, and through the direct job API;
admission keeps the planned resident bytes within the budget and rejects a
job that cannot fit; the planned footprint matches the bytes a job holds."""
import ctypes

import numpy as np
import pytest

from dtcf_gb300._lib import lib
from dtcf_gb300.cc import Job, config
from dtcf_gb300.serve import Server

pytestmark = pytest.mark.gpu

LIMIT = 120.0  # every serving run here ends by itself well inside this
X = dict(nocc=8, nvir=24, nirrep=2, max_block=6, min_block=1, seed=21, method="ccsd", engine="split")
OTHERS = [
    dict(nocc=10, nvir=40, nirrep=1, max_block=8, min_block=1, seed=5, method="ccd", engine="split"),
    dict(nocc=12, nvir=52, nirrep=4, max_block=8, min_block=1, seed=6, method="ccsd", engine="split"),
    dict(nocc=6, nvir=30, nirrep=1, max_block=16, min_block=1, seed=7, method="ccsd", engine="split"),
    dict(nocc=16, nvir=64, nirrep=8, max_block=10, min_block=1, seed=8, method="ccd", engine="split"),
    dict(nocc=8, nvir=36, nirrep=2, max_block=9, min_block=1, seed=9, method="ccsd", engine="fp64"),
]
NIT = 4


def _energies(res, job):
    rows = sorted((r for r in res if r["job"] == job), key=lambda r: r["iteration"])
    assert all(r["status"] == 0 for r in rows), rows
    return np.array([r["energy"] for r in rows])


def test_job_alone_and_in_the_mix_identical():
    s = Server(budget_bytes=40e9, slots=4)
    jx = s.add_job(config(**X))
    for _ in range(NIT):
        s.submit(jx, 0.0)
    s.run(LIMIT)
    alone = _energies(s.results(), jx)
    s.close()
    direct = Job(**X)
    assert np.array_equal(alone, direct.iterate(NIT))
    direct.close()
    s = Server(budget_bytes=40e9, slots=4)
    ids = [s.add_job(config(**c)) for c in OTHERS]
    jx = s.add_job(config(**X))
    rng = np.random.default_rng(3)
    for j in ids + [jx]:
        for t in np.sort(rng.uniform(0.0, 0.05, NIT)):
            s.submit(j, t)
    s.run(LIMIT)
    res = s.results()
    st = s.stats()
    s.close()
    assert np.array_equal(alone, _energies(res, jx))
    assert st["completed"] == st["requests"] == NIT * (len(OTHERS) + 1)
    # requests of different jobs overlapped on the device
    busy = sorted((r["start"], r["end"]) for r in res)
    assert any(busy[i + 1][0] < busy[i][1] for i in range(len(busy) - 1))
    assert 0 < st["latency_p50_s"] <= st["latency_p99_s"] <= st["latency_max_s"]
    assert st["iter_per_s"] > 0


def test_admission_respects_the_budget_and_rejects_oversize():
    cfgs = [config(**c) for c in OTHERS[:4]]
    probe = Server(budget_bytes=1e12, slots=2)
    for c in cfgs:
        probe.add_job(c)
    budget = max(probe.footprints) * 1.5  # never two of the largest at once
    probe.close()
    s = Server(budget_bytes=budget, slots=3)
    ids = [s.add_job(c) for c in cfgs]
    big = s.add_job(config(nocc=24, nvir=120, nirrep=1, max_block=16, min_block=1, seed=2, method="ccsd",
                           engine="split"))
    assert s.footprints[big] > budget
    for j in ids + [big]:
        for _ in range(2):
            s.submit(j, 0.0)
    s.run(LIMIT)
    st = s.stats()
    res = s.results()
    s.close()
    assert st["peak_planned_bytes"] <= budget
    assert st["jobs_rejected"] == 1 and st["rejected"] == 2
    assert all(r["status"] == -2 for r in res if r["job"] == big)
    assert st["completed"] == 2 * len(ids)


@pytest.mark.parametrize("c", [OTHERS[1], OTHERS[3], OTHERS[4], X])
def test_planned_footprint_matches_measured_bytes(c):
    cfg = config(**c)
    res, peak = ctypes.c_double(), ctypes.c_double()
    assert lib().gbx_cc_footprint(ctypes.byref(cfg), ctypes.byref(res), ctypes.byref(peak), None) == 0
    job = Job(**c)
    got = job.stats().resident_bytes
    job.close()
    assert abs(got - res.value) <= 0.02 * res.value + (4 << 20), (got, res.value)
    assert peak.value >= res.value


def test_idle_jobs_are_evicted_and_restored_with_the_same_results():
    """A budget that holds about two of the jobs, requests of each job spread
    over time: jobs idle between their requests are evicted (amplitudes to
    pinned host memory) to admit the others and rebuilt when their next
    request arrives.  Every request completes, and every job's energies equal
    those of the job served alone."""
    cfgs = OTHERS[:4] + [X]
    probe = Server(budget_bytes=1e12, slots=2)
    for c in cfgs:
        probe.add_job(config(**c))
    fps = sorted(probe.footprints)
    probe.close()
    budget = fps[-1] + fps[-2]
    s = Server(budget_bytes=budget, slots=2)
    ids = [s.add_job(config(**c)) for c in cfgs]
    for n, j in enumerate(ids):
        for k in range(NIT):
            s.submit(j, 0.01 * n + 0.25 * k)
    s.run(LIMIT)
    res = s.results()
    st = s.stats()
    s.close()
    assert st["completed"] == st["requests"] == NIT * len(cfgs)
    assert st["peak_planned_bytes"] <= budget
    assert st["evictions"] >= 1 and st["restores"] >= 1, st
    for c, j in zip(cfgs, ids):
        direct = Job(**c)
        assert np.array_equal(_energies(res, j), direct.iterate(NIT)), c
        direct.close()
