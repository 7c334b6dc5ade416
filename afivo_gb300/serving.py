"""Serving loop for Poisson solves: requests of different tree sizes arrive
over time, are admitted against a device-memory budget, and are solved on the
GPU with their work overlapping.

Resident forests. Requests whose trees have the same structure (the same
base boxes, refinement criterion and levels: the four uniform sizes of the
3-D request stream, for example) share a resident forest of K tree slots that
stays on the device between requests: serving a request puts its source into
a free slot (on the device), clears the slot's solution and solves the
occupied slots only (afv_mg_solve_trees), so no tree is rebuilt, uploaded or
allocated per request. A shape's first request builds its tree and creates the
forest, inside that request's latency. Forests are created under the memory
budget; idle forests of other shapes are dropped (least recently used first)
when a new shape needs the room.

Continuous batching. A fixed number of workers (host threads, each forest on
its own CUDA stream) take the oldest waiting request whose shape has an idle
forest (or room for a new one), together with up to K-1 more waiting requests
of that shape, and solve them as one batch. Requests that arrive while other
batches run are admitted as soon as a forest of their shape is idle, so the
solves of different forests run on the device at the same time. Trees are
computed independently of the other slots, so a request's result is the same
alone and in a batch (bit for bit, tests/test_serving.py).

Latency of a request = queueing (arrival to the start of its batch) + service
(its batch's set-up, solve and read-back, plus the tree build and forest
creation when its shape had no resident forest yet).

The C calls release the GIL (ctypes), so the workers overlap on the host too.
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
    start: float         # s, when its batch was taken by a worker
    done: float          # s, when its solution was back on the host
    cells: int
    cycles: int
    rel_res: float
    batch: int           # requests in its batch
    slot: int            # worker
    cold: bool = False   # its batch created the resident forest
    phi: np.ndarray = dataclasses.field(repr=False, default=None)

    @property
    def latency_ms(self):
        return (self.done - self.arrival) * 1e3

    @property
    def queue_ms(self):
        return (self.start - self.arrival) * 1e3

    @property
    def service_ms(self):
        return (self.done - self.start) * 1e3


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


_TREE_KEYS = ("dim", "n_cell", "coarsen_to", "dr", "crit", "lvl_max", "thr", "prob", "seed",
              "target_cells")


def shape_key(spec):
    """The fields that decide a request's tree: requests with equal keys have
    identical trees (the source enters only through a source criterion)."""
    key = [spec.get(k) for k in _TREE_KEYS]
    key.append(tuple(map(tuple, spec["ix"])))
    key.append(tuple(map(tuple, spec["nb"])))
    if spec.get("crit") == W.AFV_REF_SOURCE:
        key.append(tuple(np.asarray(spec["gauss"], dtype=float).ravel()))
        key.append(bool(spec.get("lpl", False)))
    return tuple(key)


class _Resident:
    """A forest of K slots for one tree shape."""

    def __init__(self, key, forest, k, nbytes, cells):
        self.key = key
        self.forest = forest
        self.k = k
        self.bytes = nbytes
        self.cells = cells
        self.busy = False
        self.last_used = 0.0


class Server:
    """Solve requests with resident per-shape forests under a device-memory
    budget; `slots` workers run batches of at most `max_batch` requests, and
    of at most `max_batch_cells` leaf cells where that is set (a batch of
    large trees takes about as long per request as one of two, so a smaller
    batch shortens the large requests' latency at little cost in rate)."""

    def __init__(self, device=0, budget_bytes=8 << 30, slots=4, max_batch=8,
                 precision=AFV_PREC_MIXED, tol=1e-8, max_cycles=60, keep_phi=False,
                 forest_cls=Forest, build_tree=W.build_tree, max_per_shape=2, max_batch_cells=None):
        self.device = device
        self.forest_cls = forest_cls  # the device forest type (a stand-in in host-only tests)
        self.build_tree = build_tree
        self.budget = int(budget_bytes)
        self.slots = slots
        self.max_batch = max_batch
        self.max_batch_cells = max_batch_cells
        self.max_per_shape = max_per_shape  # resident forests of one shape at most
        self.precision = precision
        self.tol = tol
        self.max_cycles = max_cycles
        self.keep_phi = keep_phi      # True, or a set of request ids whose solutions are kept
        self.pool = []                # resident forests, kept across serve() calls
        self.tree_bytes = {}          # shape -> (bytes per tree slot, leaf cells), once built
        self.last_peak_bytes = 0

    def close(self):
        for r in self.pool:
            r.forest.close()
        self.pool = []

    def resident_bytes(self):
        return sum(r.bytes for r in self.pool)

    def _batch_cap(self, cells):
        """Requests per batch for trees of `cells` leaf cells."""
        if not self.max_batch_cells:
            return self.max_batch
        return max(1, min(self.max_batch, int(self.max_batch_cells // max(1, cells))))

    def _keep(self, rid):
        return self.keep_phi is True or (self.keep_phi and rid in self.keep_phi)

    # -- scheduling (called with the lock held) -------------------------------
    def _choose(self, queue):
        """The oldest waiting request that can start now, its resident forest
        (or None: create one) and the batch of requests of its shape."""
        for it in queue:
            key = it["key"]
            mine = [r for r in self.pool if r.key == key]
            idle = [r for r in mine if not r.busy]
            if idle:
                res = idle[0]
                k = res.k
            elif len(mine) < self.max_per_shape:
                res = None
                per = self.tree_bytes.get(key)
                if per is not None:
                    k = max(1, min(self._batch_cap(per[1]), self.budget // per[0]))
                    need = k * per[0]
                else:
                    k, need = self.max_batch, 0  # sized once the tree is built
                if not self._make_room(need):
                    continue
            else:
                continue
            batch = [x for x in queue if x["key"] == key][:k]
            return res, batch
        return None, None

    def _make_room(self, need):
        """Drop idle forests (least recently used first) until `need` more
        bytes fit the budget; False if they cannot."""
        while self.resident_bytes() + need > self.budget:
            idle = sorted((r for r in self.pool if not r.busy), key=lambda r: r.last_used)
            if not idle:
                return False
            victim = idle[0]
            self.pool.remove(victim)
            victim.forest.close()
        return True

    def _create(self, res, spec, cond):
        """Build the shape's tree, reserve its slots under the budget (waiting
        for idle forests to be dropped if need be) and create a forest of K
        slots. The first batch's service time includes this."""
        mixed = self.precision == AFV_PREC_MIXED
        tree = self.build_tree(spec)
        per = forest_bytes(tree, mixed)
        if per > self.budget:
            raise ValueError(f"a request needs {per} bytes, over the budget {self.budget}")
        with cond:
            self.tree_bytes[res.key] = (per, tree.leaf_cells())
            while True:
                others = self.resident_bytes() - res.bytes
                k = min(self._batch_cap(tree.leaf_cells()), (self.budget - others) // per)
                if k < 1 and self._make_room(max(0, per - res.bytes)):
                    continue
                if k >= 1:
                    break
                cond.wait(0.005)
            res.k, res.bytes, res.cells = k, k * per, tree.leaf_cells()
        res.forest = self.forest_cls([tree] * k, device=self.device, mixed=mixed)

    def serve(self, requests, realtime=True):
        """Run the request stream. requests: workload specs with an
        "arrival" time (s), e.g. workloads.c5_requests. Returns one Result per
        request."""
        items = []
        for k, r in enumerate(requests):
            items.append(dict(id=k, spec=r, key=shape_key(r), arrival=float(r["arrival"])))
        order = sorted(items, key=lambda x: x["arrival"])
        queue = collections.deque()
        cond = threading.Condition()
        state = dict(arrived=0, error=None, peak=self.resident_bytes())
        results = [None] * len(items)
        t0 = time.perf_counter()
        mg = MgOpts()

        def now():
            return time.perf_counter() - t0

        def worker(slot):
            while True:
                with cond:
                    while True:
                        if state["error"] is not None:
                            return
                        res, batch = self._choose(queue) if queue else (None, None)
                        if batch:
                            for x in batch:
                                queue.remove(x)
                            if res is None:  # reserve the creation: a placeholder in the pool
                                res = _Resident(batch[0]["key"], None, 0, 0, 0)
                                per = self.tree_bytes.get(res.key)
                                if per is not None:
                                    res.k = max(1, min(self._batch_cap(per[1]), self.budget // per[0]))
                                    res.bytes = res.k * per[0]
                                self.pool.append(res)
                            res.busy = True
                            break
                        if state["arrived"] == len(items) and not queue:
                            return
                        cond.wait(0.005)
                start = now()
                cold = res.forest is None
                try:
                    if cold:
                        self._create(res, batch[0]["spec"], cond)
                        with cond:
                            state["peak"] = max(state["peak"], self.resident_bytes())
                            if len(batch) > res.k:  # sized now: give the rest back
                                for x in reversed(batch[res.k:]):
                                    queue.appendleft(x)
                                batch = batch[:res.k]
                                cond.notify_all()
                    f = res.forest
                    mask = np.zeros(res.k, np.int32)
                    for i, b in enumerate(batch):
                        f.zero_tree(i, AFV_PHI)
                        f.set_source_device(i, b["spec"]["gauss"], lpl=b["spec"].get("lpl", True))
                        mask[i] = 1
                    cyc, rel, rc = f.solve(self.precision, tol=self.tol, max_cycles=self.max_cycles,
                                           mg=mg, check=False, mask=mask)
                    if rc != 0:
                        raise RuntimeError(f"solve failed with status {rc}: "
                                           f"{lib().afv_last_error().decode()}")
                    phis = [f.get_var(i, AFV_PHI, interior_only=True) if self._keep(b["id"]) else None
                            for i, b in enumerate(batch)]
                    done = now()
                    for i, b in enumerate(batch):
                        results[b["id"]] = Result(
                            id=b["id"], name=b["spec"].get("name", str(b["id"])), arrival=b["arrival"],
                            start=start, done=done, cells=res.cells, cycles=int(cyc[i]),
                            rel_res=float(rel[i]), batch=len(batch), slot=slot, cold=cold, phi=phis[i])
                except Exception as e:  # noqa: BLE001 - reported to the caller
                    with cond:
                        state["error"] = e
                        if res in self.pool and res.forest is None:
                            self.pool.remove(res)
                        cond.notify_all()
                    return
                with cond:
                    res.busy = False
                    res.last_used = now()
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
        return results


def summary(results):
    """p50 / p99 latency (and its queueing and service parts), throughput and
    batch sizes of a run."""
    lat = np.array([r.latency_ms for r in results])
    que = np.array([r.queue_ms for r in results])
    svc = np.array([r.service_ms for r in results])
    span = max(r.done for r in results) - min(r.arrival for r in results)
    cells = sum(r.cells * r.cycles for r in results)
    return {"requests": len(results), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "queue_p50_ms": float(np.percentile(que, 50)), "queue_p99_ms": float(np.percentile(que, 99)),
            "service_p50_ms": float(np.percentile(svc, 50)),
            "service_p99_ms": float(np.percentile(svc, 99)),
            "solves_per_s": len(results) / span, "unknowns_per_s": cells / span,
            "span_s": span, "mean_batch": float(np.mean([r.batch for r in results])),
            "cold_batches": int(sum(1 for r in results if r.cold)),
            "max_rel_res": max(r.rel_res for r in results)}
