"""Planned triple groups (gbx_group_*) against numpy FP64 on seeded triples
of the grouped-sweep kind: m, n, k log-uniform in [8, 256], entries
sign * 10^u with u uniform in [-6, 6] (a stress on the split engine's
per-row scaling)."""
import numpy as np
import pytest
import torch

from dtcf_gb300.leaves import Group, Triple, MODE_AUTO, MODE_FP64, MODE_SPLIT
from dtcf_gb300 import GbxError

pytestmark = pytest.mark.gpu


def make_set(n, seed, lo=8, hi=256, spread=6.0):
    rng = np.random.default_rng(seed)
    dims = np.exp(rng.uniform(np.log(lo), np.log(hi), size=(n, 3))).round().astype(np.int64)
    A, B, C = [], [], []
    for m, nn, k in dims:
        A.append(rng.choice([-1.0, 1.0], (m, k)) * 10.0 ** rng.uniform(-spread, spread, (m, k)))
        B.append(rng.choice([-1.0, 1.0], (nn, k)) * 10.0 ** rng.uniform(-spread, spread, (nn, k)))
        C.append(rng.standard_normal((m, nn)))
    return dims, A, B, C


class DeviceSet:
    """All operands of a triple set in three flat device buffers."""

    def __init__(self, dims, A, B, C):
        self.dims = dims
        self.oa = np.cumsum([0] + [a.size for a in A])
        self.ob = np.cumsum([0] + [b.size for b in B])
        self.oc = np.cumsum([0] + [c.size for c in C])
        self.A = torch.from_numpy(np.concatenate([a.ravel() for a in A])).cuda()
        self.B = torch.from_numpy(np.concatenate([b.ravel() for b in B])).cuda()
        self.C0 = np.concatenate([c.ravel() for c in C])
        self.C = torch.from_numpy(self.C0.copy()).cuda()

    def triples(self, alpha=1.0, accumulate=0):
        out = []
        for i, (m, n, k) in enumerate(self.dims):
            out.append(Triple(self.A.data_ptr() + 8 * int(self.oa[i]), self.B.data_ptr() + 8 * int(self.ob[i]),
                              self.C.data_ptr() + 8 * int(self.oc[i]), int(k), 1, int(k), 1, int(n),
                              int(m), int(n), int(k), alpha, accumulate))
        return out

    def result(self, i):
        m, n, _ = self.dims[i]
        return self.C.cpu().numpy()[self.oc[i]:self.oc[i + 1]].reshape(m, n)


def max_rel_frob(ds, A, B, C0, alpha=1.0, accumulate=0):
    got_all = ds.C.cpu().numpy()
    worst = 0.0
    for i, (m, n, _) in enumerate(ds.dims):
        ref = alpha * (A[i] @ B[i].T) + (C0[i] if accumulate else 0.0)
        got = got_all[ds.oc[i]:ds.oc[i + 1]].reshape(m, n)
        worst = max(worst, float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    return worst


@pytest.fixture(scope="module")
def tset():
    dims, A, B, C = make_set(300, seed=4)
    return dims, A, B, C


@pytest.mark.parametrize("mode,tol", [(MODE_FP64, 1e-13), (MODE_SPLIT, 1e-12), (MODE_AUTO, 1e-12)])
def test_group_modes_vs_numpy(tset, mode, tol):
    dims, A, B, C = tset
    ds = DeviceSet(dims, A, B, C)
    g = Group(ds.triples(), mode=mode)
    g.execute()
    torch.cuda.synchronize()
    assert max_rel_frob(ds, A, B, C) <= tol
    eng, _, fl = g.info()
    assert fl == pytest.approx(2.0 * float(np.sum(np.prod(dims.astype(float), axis=1))))
    if mode == MODE_FP64:
        assert set(eng) == {0}
    if mode == MODE_SPLIT:
        assert set(eng) == {1}


def test_group_accumulate_alpha_and_swapped_orientations(tset):
    dims, A, B, C = tset
    ds = DeviceSet(dims, A, B, C)
    g = Group(ds.triples(alpha=-0.375, accumulate=1), mode=MODE_SPLIT)
    g.execute()
    torch.cuda.synchronize()
    assert max_rel_frob(ds, A, B, C, alpha=-0.375, accumulate=1) <= 1e-12


def test_group_per_triple_launches_equal_persistent(tset):
    dims, A, B, C = tset
    ds = DeviceSet(dims, A, B, C)
    g = Group(ds.triples(), mode=MODE_FP64)
    g.execute(per_triple=False)
    torch.cuda.synchronize()
    one = ds.C.clone()
    ds.C.copy_(torch.from_numpy(ds.C0))
    g.execute(per_triple=True)
    torch.cuda.synchronize()
    assert torch.equal(one, ds.C)


def test_group_autotune_keeps_results(tset):
    dims, A, B, C = tset
    ds = DeviceSet(dims[:120], A[:120], B[:120], C[:120])
    g = Group(ds.triples(), mode=MODE_AUTO)
    g.autotune(reps=2)
    g.execute()
    torch.cuda.synchronize()
    assert max_rel_frob(ds, A[:120], B[:120], C[:120]) <= 1e-12
    # the tuned choice is valid: FP64 tile variants 0..3 or split widths 32..256
    eng, par, _ = g.info()
    for e, p in zip(eng, par):
        assert (e == 0 and -1 <= p <= 3) or (e == 1 and p // 2 in (32, 64, 128, 256))


def test_group_graph_replay_is_deterministic(tset):
    dims, A, B, C = tset
    ds = DeviceSet(dims, A, B, C)
    g = Group(ds.triples(), mode=MODE_AUTO)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g.execute(stream=s)  # warm-up outside the capture
    torch.cuda.synchronize()
    first = ds.C.clone()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        g.execute(stream=s)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(first, ds.C)


def test_group_split_rejects_strided_columns():
    A = torch.zeros(16, 16, dtype=torch.float64, device="cuda")
    t = Triple(A.data_ptr(), A.data_ptr(), A.data_ptr(), 1, 16, 16, 1, 16, 16, 16, 16, 1.0, 0)
    with pytest.raises(GbxError):
        Group([t], mode=MODE_SPLIT)
    # AUTO falls back to FP64 for it
    g = Group([t], mode=MODE_AUTO)
    assert g.info()[0] == [0]
