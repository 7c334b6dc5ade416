"""Serving loop for Poisson solves: requests of different tree sizes arrive
over time, are admitted against a device-memory budget, and are solved on the
GPU with their work overlapping.

Continuous batching. A fixed number of slots (worker threads) share one GPU.
A free slot takes the waiting requests, oldest first, that fit both the
memory budget and the batch limit, builds one forest of their trees (one
kernel launch per level and operator sweeps all of them), and solves it on its
own CUDA stream with per-tree convergence masks. Requests that arrive while
other slots are busy are admitted as soon as a slot and memory free up, so
the solves of several forests run on the device at the same time. Every tree
is computed independently of the others in its forest, so a request's result
is the same alone and in a batch (bit for bit, see tests/test_serving.py).

The C calls release the GIL (ctypes), so the slots overlap on the host too.
"""
import collections
import dataclasses
import threading
import time

import numpy as np

from . import AFV_PHI, AFV_PREC_MIXED, Forest, MgOpts, lib
from . import workloads as W


@dataclasses.dataclass
class Result:
    id: int
    name: str
    arrival: float       # s, relative to the start of the run
    start: float         # s, when its forest began to be built on the device
    done: float          # s, when its solution was back on the host
    cells: int
    cycles: int
    rel_res: float
    batch: int           # number of trees in its forest
    slot: int
    phi: np.ndarray = dataclasses.field(repr=False, default=None)

    @property
    def latency_ms(self):
        return (self.done - self.arrival) * 1e3


def forest_bytes(tree, mixed):
    """Device bytes a forest of this one tree allocates (an upper estimate of
    what afv_forest_create reserves: cell data in FP64, the FP32 copy when
    mixed, the per-slot tables and descriptors)."""
    info = tree.info()
    D, nc = info["dim"], info["n_cell"]
    total = 0
    for lvl in range(info["min_lvl"], info["highest_lvl"] + 1):
        n = len(tree.level(lvl)[0])
        ncl = tree.n_cell_at(lvl)
        sg, si = (ncl + 2) ** D, ncl ** D
        per = 8 * (2 * sg + si) + (4 * (2 * sg + si) if mixed else 0)
        per += 128 + 4 * 4 + 8 * 2 + 8 * 2 * D + 3 * 4  # descriptor, tables, lists
        total += n * per
    base = (nc + 2) ** D * 8 * 2  # FP64 copy of the coarsest level (mixed)
    return total + base + 64 * 8 + 4096


class Server:
    """Solve requests under a device-memory budget with `slots` concurrent
    forests of at most `max_batch` trees each."""

    def __init__(self, device=0, budget_bytes=8 << 30, slots=4, max_batch=8,
                 precision=AFV_PREC_MIXED, tol=1e-8, max_cycles=60, keep_phi=False,
                 autotune=False, forest_cls=Forest):
        self.device = device
        self.forest_cls = forest_cls  # the device forest type (a stand-in in host-only tests)
        self.budget = int(budget_bytes)
        self.slots = slots
        self.max_batch = max_batch
        self.precision = precision
        self.tol = tol
        self.max_cycles = max_cycles
        self.keep_phi = keep_phi
        self.autotune = autotune

    # -- scheduling ----------------------------------------------------------
    def _take(self, queue, in_use):
        """Oldest-first requests that fit the budget and the batch limit
        (stops at the first that does not fit, so nothing overtakes)."""
        batch, need = [], 0
        while queue and len(batch) < self.max_batch:
            r = queue[0]
            if in_use + need + r["bytes"] > self.budget:
                break
            batch.append(queue.popleft())
            need += r["bytes"]
        return batch, need

    def serve(self, requests, trees=None, realtime=True):
        """Run the request stream. requests: dicts with "arrival" (s) and a
        workload spec (workloads.c5_requests); trees: their host trees if
        already built (the client's side). Returns one Result per request."""
        mixed = self.precision == AFV_PREC_MIXED
        if trees is None:
            trees = [W.build_tree(r) for r in requests]
        items = []
        for k, (r, t) in enumerate(zip(requests, trees)):
            b = forest_bytes(t, mixed)
            if b > self.budget:
                raise ValueError(f"request {k} needs {b} bytes, over the budget {self.budget}")
            items.append(dict(id=k, spec=r, tree=t, bytes=b, arrival=float(r["arrival"])))
        order = sorted(items, key=lambda x: x["arrival"])
        queue = collections.deque()
        cond = threading.Condition()
        state = dict(in_use=0, arrived=0, finished=0, error=None, peak=0, peak_forests=0, forests=0)
        results = [None] * len(items)
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        def worker(slot):
            mg = MgOpts()
            while True:
                with cond:
                    while True:
                        if state["error"] is not None:
                            return
                        if queue:
                            batch, need = self._take(queue, state["in_use"])
                            if batch:
                                state["in_use"] += need
                                state["forests"] += 1
                                state["peak"] = max(state["peak"], state["in_use"])
                                state["peak_forests"] = max(state["peak_forests"], state["forests"])
                                break
                        if state["arrived"] == len(items) and not queue:
                            return
                        cond.wait(0.01)
                try:
                    start = now()
                    f = self.forest_cls([b["tree"] for b in batch], device=self.device, mixed=mixed)
                    try:
                        if self.autotune and mixed:
                            f.autotune()
                        for i, b in enumerate(batch):
                            f.set_source_device(i, b["spec"]["gauss"], lpl=b["spec"].get("lpl", True))
                        cyc, rel, rc = f.solve(self.precision, tol=self.tol,
                                               max_cycles=self.max_cycles, mg=mg, check=False)
                        if rc != 0:
                            raise RuntimeError(f"solve failed with status {rc}: "
                                               f"{lib().afv_last_error().decode()}")
                        phis = [f.get_var(i, AFV_PHI, interior_only=True) if self.keep_phi else None
                                for i in range(len(batch))]
                        done = now()
                    finally:
                        f.close()
                    for i, b in enumerate(batch):
                        results[b["id"]] = Result(
                            id=b["id"], name=b["spec"].get("name", str(b["id"])), arrival=b["arrival"],
                            start=start, done=done, cells=b["tree"].leaf_cells(), cycles=int(cyc[i]),
                            rel_res=float(rel[i]), batch=len(batch), slot=slot, phi=phis[i])
                except Exception as e:  # noqa: BLE001 - reported to the caller
                    with cond:
                        state["error"] = e
                        cond.notify_all()
                    return
                with cond:
                    state["in_use"] -= need
                    state["forests"] -= 1
                    state["finished"] += len(batch)
                    cond.notify_all()

        threads = [threading.Thread(target=worker, args=(s,), daemon=True) for s in range(self.slots)]
        for th in threads:
            th.start()
        for it in order:
            if realtime:
                wait = it["arrival"] - now()
                if wait > 0:
                    time.sleep(wait)
            with cond:
                it["arrival"] = it["arrival"] if realtime else now()
                queue.append(it)
                state["arrived"] += 1
                cond.notify_all()
        for th in threads:
            th.join()
        if state["error"] is not None:
            raise state["error"]
        self.last_peak_bytes = state["peak"]
        self.last_peak_forests = state["peak_forests"]
        return results


def summary(results):
    """p50 / p99 latency, throughput and batch sizes of a run."""
    lat = np.array([r.latency_ms for r in results])
    span = max(r.done for r in results) - min(r.arrival for r in results)
    cells = sum(r.cells * r.cycles for r in results)
    return {"requests": len(results), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "solves_per_s": len(results) / span, "unknowns_per_s": cells / span,
            "span_s": span, "mean_batch": float(np.mean([r.batch for r in results])),
            "max_rel_res": max(r.rel_res for r in results)}
