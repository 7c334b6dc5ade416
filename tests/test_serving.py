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
    at once and takes a little time per solve."""
    lock = threading.Lock()
    alive = 0
    peak = 0

    def __init__(self, trees, device=0, mixed=True):
        self.n = len(trees)
        with FakeForest.lock:
            FakeForest.alive += 1
            FakeForest.peak = max(FakeForest.peak, FakeForest.alive)

    def set_source_device(self, i, gauss, lpl=True):
        pass

    def solve(self, precision, tol, max_cycles, mg=None, check=True):
        time.sleep(0.02)
        return np.full(self.n, 7), np.full(self.n, 1e-9), 0

    def get_var(self, i, var, interior_only=False):
        return np.zeros(4)

    def close(self):
        with FakeForest.lock:
            FakeForest.alive -= 1


def fake_requests(n, bytes_each, gap):
    reqs = [dict(name="r%d" % k, arrival=k * gap, gauss=np.zeros(5)) for k in range(n)]
    trees = [FakeTree(1000 * (k + 1)) for k in range(n)]
    return reqs, trees


def test_admission_respects_budget_and_order(monkeypatch):
    reqs, trees = fake_requests(12, 100, 0.0)
    monkeypatch.setattr(S, "forest_bytes", lambda t, mixed: 100)
    FakeForest.alive = FakeForest.peak = 0
    srv = S.Server(budget_bytes=250, slots=4, max_batch=8, forest_cls=FakeForest)
    res = srv.serve(reqs, trees, realtime=False)
    assert all(r is not None for r in res)
    assert srv.last_peak_bytes <= 250
    # at most two requests fit at a time: batches of <= 2, FIFO starts
    assert max(r.batch for r in res) <= 2
    starts = [r.start for r in sorted(res, key=lambda r: r.id)]
    assert starts == sorted(starts)


def test_continuous_batching_overlaps_forests(monkeypatch):
    reqs, trees = fake_requests(16, 10, 0.002)
    monkeypatch.setattr(S, "forest_bytes", lambda t, mixed: 10)
    FakeForest.alive = FakeForest.peak = 0
    srv = S.Server(budget_bytes=1000, slots=4, max_batch=3, forest_cls=FakeForest)
    res = srv.serve(reqs, trees, realtime=True)
    assert FakeForest.peak >= 2          # several forests in flight at once
    assert max(r.batch for r in res) <= 3
    summ = S.summary(res)
    assert summ["requests"] == 16 and summ["p99_ms"] >= summ["p50_ms"] > 0


def test_oversized_request_is_refused(monkeypatch):
    reqs, trees = fake_requests(2, 0, 0.0)
    monkeypatch.setattr(S, "forest_bytes", lambda t, mixed: 10 ** 12)
    with pytest.raises(ValueError, match="over the budget"):
        S.Server(budget_bytes=1000, forest_cls=FakeForest).serve(reqs, trees, realtime=False)


def test_forest_bytes_estimate_grows_with_the_tree(afv):
    small = W.build_tree(W.c5_requests(n=1, seed=11, small=True)[0])
    spec = dict(W.c5_requests(n=1, seed=11, small=True)[0], lvl_max=4)
    big = W.build_tree(spec)
    assert S.forest_bytes(big, True) > S.forest_bytes(big, False) > 0
    assert S.forest_bytes(big, True) >= S.forest_bytes(small, True)


@pytest.mark.gpu
def test_served_results_equal_solo_results(gpu):
    """Each request's solution is bit-identical served in a batch among
    other requests and solved alone; the estimate covers the real footprint."""
    reqs = W.c5_requests(n=10, seed=7, small=True)
    for r in reqs:
        r["lvl_max"] = min(r["lvl_max"], 4)
    trees = [W.build_tree(r) for r in reqs]
    srv = S.Server(budget_bytes=2 << 30, slots=3, max_batch=4, keep_phi=True)
    res = srv.serve(reqs, trees, realtime=False)  # all waiting at once: batches form
    assert max(r.batch for r in res) >= 2
    for r, spec, tree in zip(res, reqs, trees):
        f = gpu.Forest([W.build_tree(spec)], mixed=True)
        assert f.info()["bytes"] <= S.forest_bytes(tree, True)
        f.set_source_device(0, spec["gauss"], lpl=True)
        cyc, rel, rc = f.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60, check=False)
        assert rc == 0 and int(cyc[0]) == r.cycles and r.rel_res <= 1e-8
        assert np.array_equal(f.get_var(0, gpu.AFV_PHI, interior_only=True), r.phi)
        f.close()


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
