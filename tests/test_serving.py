"""Serving loop: admission under the memory budget and continuous batching
(host-only, with a stand-in forest), and on the GPU that every request's
result is the same alone and in the mix."""
import threading
import time

import numpy as np
import pytest

from afivo_gb300 import serving as S
from afivo_gb300 import workloads as W


class FakeTree:
    def __init__(self, cells):
        self.cells = cells

    def leaf_cells(self):
        return self.cells


class FakeForest:
    """Stands in for afivo_gb300.Forest: records how many forests are alive
    and busy at once and takes a little time per solve."""
    lock = threading.Lock()
    alive = 0
    peak = 0
    created = 0
    solving = 0
    peak_solving = 0

    def __init__(self, trees, device=0, mixed=True):
        self.n = len(trees)
        with FakeForest.lock:
            FakeForest.alive += 1
            FakeForest.created += 1
            FakeForest.peak = max(FakeForest.peak, FakeForest.alive)

    @classmethod
    def reset(cls):
        cls.alive = cls.peak = cls.created = cls.solving = cls.peak_solving = 0

    def zero_tree(self, i, var):
        assert 0 <= i < self.n

    def set_source_device(self, i, gauss, lpl=True):
        assert 0 <= i < self.n

    def solve(self, precision, tol, max_cycles, mg=None, check=True, mask=None):
        assert mask is not None and len(mask) == self.n and sum(mask) >= 1
        with FakeForest.lock:
            FakeForest.solving += 1
            FakeForest.peak_solving = max(FakeForest.peak_solving, FakeForest.solving)
        time.sleep(0.02)
        with FakeForest.lock:
            FakeForest.solving -= 1
        return np.full(self.n, 7), np.full(self.n, 1e-9), 0

    def get_var(self, i, var, interior_only=False):
        return np.zeros(4)

    def close(self):
        with FakeForest.lock:
            FakeForest.alive -= 1


def fake_requests(n, gap, shapes):
    """n requests over `shapes` distinct tree shapes (lvl_max stands for the shape)."""
    return [dict(name="r%d" % k, arrival=k * gap, gauss=np.zeros(5), dim=3, n_cell=8, coarsen_to=2,
                 dr=0.125, ix=[[1, 1, 1]], nb=[[-1] * 6], crit=W.AFV_REF_UNIFORM, thr=0.0,
                 lvl_max=3 + k % shapes) for k in range(n)]


def _server(monkeypatch, bytes_per_tree, **kw):
    monkeypatch.setattr(S, "forest_bytes", lambda t, mixed: bytes_per_tree)
    FakeForest.reset()
    return S.Server(forest_cls=FakeForest, build_tree=lambda spec: FakeTree(1000 * spec["lvl_max"]), **kw)


def test_resident_forest_is_reused(monkeypatch):
    """Requests of one shape share one resident forest, created once, across
    batches and across runs."""
    srv = _server(monkeypatch, 10, budget_bytes=1000, slots=2, max_batch=4, max_per_shape=1)
    reqs = fake_requests(12, 0.0, 1)
    res = srv.serve(reqs, realtime=False)
    assert all(r is not None for r in res)
    assert FakeForest.created == 1 and max(r.batch for r in res) <= 4
    assert sum(r.cold for r in res) <= 4  # the first batch only
    srv.serve(reqs, realtime=False)
    assert FakeForest.created == 1
    assert S.summary(res)["requests"] == 12


def test_admission_respects_budget(monkeypatch):
    """Twelve shapes of 100 bytes per tree slot under a 250-byte budget: at
    most two resident forests at once (idle ones are dropped for new shapes),
    every request served."""
    srv = _server(monkeypatch, 100, budget_bytes=250, slots=4, max_batch=1)
    res = srv.serve(fake_requests(12, 0.0, 12), realtime=False)
    assert all(r is not None for r in res)
    assert srv.last_peak_bytes <= 250 and FakeForest.peak <= 2


def test_continuous_batching_overlaps_forests(monkeypatch):
    srv = _server(monkeypatch, 10, budget_bytes=10000, slots=4, max_batch=3)
    res = srv.serve(fake_requests(24, 0.002, 4), realtime=True)
    assert FakeForest.peak_solving >= 2          # batches of several forests in flight at once
    assert max(r.batch for r in res) <= 3
    summ = S.summary(res)
    assert summ["requests"] == 24 and summ["p99_ms"] >= summ["p50_ms"] > 0
    assert summ["queue_p50_ms"] >= 0 and summ["service_p50_ms"] > 0


def test_batch_cell_cap(monkeypatch):
    """With max_batch_cells, a shape's forests hold at most that many leaf
    cells of trees (at least one tree): 3000-cell trees under a 7000-cell cap
    go two per batch, 1000-cell trees take the request cap of 4."""
    srv = _server(monkeypatch, 10, budget_bytes=10000, slots=2, max_batch=4, max_batch_cells=7000)
    reqs = [dict(r, lvl_max=3 if k % 2 else 1) for k, r in enumerate(fake_requests(16, 0.0, 1))]
    res = srv.serve(reqs, realtime=False)
    big = [r.batch for r, q in zip(res, reqs) if q["lvl_max"] == 3]
    small = [r.batch for r, q in zip(res, reqs) if q["lvl_max"] == 1]
    assert max(big) <= 2 and max(small) <= 4 and max(small) > 2
    assert S.summary(res)["requests"] == 16


def test_oversized_request_is_refused(monkeypatch):
    srv = _server(monkeypatch, 10 ** 12, budget_bytes=1000)
    with pytest.raises(ValueError, match="over the budget"):
        srv.serve(fake_requests(2, 0.0, 1), realtime=False)


def test_forest_bytes_estimate_grows_with_the_tree(afv):
    small = W.build_tree(W.c5_requests(n=1, seed=11, small=True)[0])
    spec = dict(W.c5_requests(n=1, seed=11, small=True)[0], lvl_max=4)
    big = W.build_tree(spec)
    assert S.forest_bytes(big, True) > S.forest_bytes(big, False) > 0
    assert S.forest_bytes(big, True) >= S.forest_bytes(small, True)


@pytest.mark.gpu
def test_served_results_equal_solo_results(gpu):
    """Each request's solution is bit-identical served in a batch among
    other requests (in a resident forest reused across batches) and solved
    alone; the estimate covers the real footprint."""
    reqs = W.c5_requests(n=12, seed=7, small=True)
    for r in reqs:
        r["lvl_max"] = min(r["lvl_max"], 4)
    srv = S.Server(budget_bytes=2 << 30, slots=3, max_batch=4, keep_phi=True)
    res = srv.serve(reqs, realtime=False)  # all waiting at once: batches form
    assert max(r.batch for r in res) >= 2
    res2 = srv.serve(reqs, realtime=False)  # again, on the resident forests
    assert not any(r.cold for r in res2)
    for r, r2, spec in zip(res, res2, reqs):
        tree = W.build_tree(spec)
        f = gpu.Forest([tree], mixed=True)
        assert f.info()["bytes"] <= S.forest_bytes(tree, True)
        f.set_source_device(0, spec["gauss"], lpl=True)
        cyc, rel, rc = f.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60, check=False)
        assert rc == 0 and int(cyc[0]) == r.cycles and r.rel_res <= 1e-8
        alone = f.get_var(0, gpu.AFV_PHI, interior_only=True)
        assert np.array_equal(alone, r.phi) and np.array_equal(alone, r2.phi)
        f.close()
    srv.close()


@pytest.mark.gpu
def test_served_result_matches_the_oracle(gpu):
    """Served requests (mixed precision) against the oracle's FP64 solve of
    the same tree and source: within 1e-6 of max |phi| over the leaves."""
    import oracle as O
    from helpers import interior_to_ghosted, leaf_error, oracle_solve, oracle_tree
    reqs = W.c5_requests(n=6, seed=9, small=True)
    for r in reqs:
        r["lvl_max"] = min(r["lvl_max"], 4)
    srv = S.Server(budget_bytes=2 << 30, slots=2, max_batch=3, keep_phi=True)
    res = srv.serve(reqs, realtime=False)
    for r, spec in zip(res, reqs):
        ot = oracle_tree(spec)
        ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
        ot.mg_init()
        oracle_solve(ot, 1e-10)
        from helpers import oracle_var
        got = interior_to_ghosted(r.phi, ot, 8, 3)
        assert leaf_error(got, oracle_var(ot, O.I_PHI, 8), ot, 8, 3) <= 1e-6
    srv.close()


@pytest.mark.gpu
def test_device_source_matches_host_source(gpu):
    spec = W.c5_requests(n=1, seed=3, small=True)[0]
    f = gpu.Forest([W.build_tree(spec)])
    f.set_source(0, spec["gauss"], lpl=True)
    host = f.get_var(0, gpu.AFV_RHS, interior_only=True)
    f.set_source_device(0, spec["gauss"], lpl=True)
    dev = f.get_var(0, gpu.AFV_RHS, interior_only=True)
    assert np.max(np.abs(dev - host)) <= 1e-13 * np.max(np.abs(host))
    f.close()
