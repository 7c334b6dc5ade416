"""Online placement of independent solves (served requests, batches of
trees) on the GPUs of one node, one process per GPU.

Trees never exchange data, so the ranks share no data path: rank 0 admits
each request when it arrives and hands it to one rank, and the ranks report
back when a request is done. Admission is against a per-rank device-memory
budget: a request goes to the rank with the least outstanding work among
those with room for its bytes; when no rank has room it waits, first in,
first out, until completions free enough. The messages are small integer
tensors on a gloo process group (host memory; it can live beside an NCCL
group), so nothing of this touches a GPU.

`Admission` is the placement rule alone (deterministic for a given order of
arrivals and completions); `serve_ranks` runs it across the ranks of a
process group with a solve callback per rank: on rank 0 a thread solves its
own share and one thread per other rank receives that rank's completions
(blocking receives; the dispatching thread only sends).
"""
import collections
import queue
import threading
import time


class Admission:
    """Per-rank budget admission with a FIFO wait queue."""

    def __init__(self, n_ranks, budget_bytes):
        self.n = int(n_ranks)
        self.budget = int(budget_bytes)
        self.used = [0] * self.n        # bytes of the requests each rank holds
        self.load = [0.0] * self.n      # their work (e.g. leaf cells x cycles)
        self.peak = [0] * self.n
        self.waiting = collections.deque()
        self.where = {}
        self.waited = 0                 # requests that found no room on arrival

    def arrive(self, rid, work, need):
        """A request arrives; returns the (rid, rank) assignments it allows."""
        if need > self.budget:
            raise ValueError(f"request {rid} needs {need} bytes, over the per-rank budget {self.budget}")
        self.waiting.append((rid, float(work), int(need)))
        out = self._drain()
        if not any(r == rid for r, _ in out):
            self.waited += 1
        return out

    def complete(self, rid):
        """A request is done; returns the assignments the freed room allows."""
        rank, work, need = self.where.pop(rid)
        self.used[rank] -= need
        self.load[rank] -= work
        return self._drain()

    def _drain(self):
        out = []
        while self.waiting:
            rid, work, need = self.waiting[0]
            fits = [r for r in range(self.n) if self.used[r] + need <= self.budget]
            if not fits:
                break  # the oldest request waits; later ones do not overtake it
            r = min(fits, key=lambda q: (self.load[q], q))
            self.waiting.popleft()
            self.where[rid] = (r, work, need)
            self.used[r] += need
            self.load[r] += work
            self.peak[r] = max(self.peak[r], self.used[r])
            out.append((rid, r))
        return out

    def idle(self):
        return not self.where and not self.waiting


def serve_ranks(requests, solve, rank, world, budget_bytes, group=None, realtime=False):
    """Serve `requests` (dicts with "arrival" in s, "work" and "need" in
    bytes) over the ranks of `group` (a gloo group; None: the default group).
    Every rank calls this with the same list. `solve(request)` runs one
    request on the calling rank and returns its result; a solve that raises
    is reported with its request (as "error") instead of stopping the run.

    Returns on rank 0 a dict: per request its rank, start and done times (s
    from the start), result (rank 0's own requests) and error (or None), plus
    the admission's per-rank peak bytes and the count of requests that waited
    for room; on the other ranks the results of the requests they solved."""
    import torch
    import torch.distributed as dist

    t0 = time.perf_counter()
    now = lambda: time.perf_counter() - t0  # noqa: E731

    def run_one(rid):
        start = now()
        try:
            res, err = solve(requests[rid]), None
        except Exception as exc:  # reported to rank 0 with the request
            res, err = None, repr(exc)
        return rid, start, now(), res, err

    def send(value, dst):
        dist.send(torch.tensor([value], dtype=torch.int64), dst=dst, group=group)

    if rank != 0:
        done = {}
        msg = torch.zeros(1, dtype=torch.int64)
        while True:
            dist.recv(msg, src=0, group=group)
            rid = int(msg.item())
            if rid < 0:  # stop: acknowledge, which ends rank 0's receiver for this rank
                send(-1, 0)
                return done
            rid, _start, _end, res, err = run_one(rid)
            done[rid] = res
            send(rid if err is None else -2 - rid, 0)  # a failed request travels as -2 - rid

    # rank 0: the admission, its own worker thread, and one receiver per other rank
    adm = Admission(world, budget_bytes)
    local_q, finished = queue.Queue(), queue.Queue()
    out = {}

    def local_worker():
        while True:
            rid = local_q.get()
            if rid is None:
                return
            finished.put(run_one(rid))

    def receiver(r):  # completions of rank r, until its acknowledgement of the stop
        buf = torch.zeros(1, dtype=torch.int64)
        while True:
            dist.recv(buf, src=r, group=group)
            v = int(buf.item())
            if v == -1:
                return
            rid, err = (v, None) if v >= 0 else (-2 - v, "failed on rank %d" % r)
            finished.put((rid, None, now(), None, err))

    threads = [threading.Thread(target=local_worker, daemon=True)]
    threads += [threading.Thread(target=receiver, args=(r,), daemon=True) for r in range(1, world)]
    for th in threads:
        th.start()
    remote_start = {}

    def assign(pairs):
        for rid, r in pairs:
            out[rid] = {"rank": r}
            if r == 0:
                local_q.put(rid)
            else:
                remote_start[rid] = now()
                send(rid, r)

    order = sorted(range(len(requests)), key=lambda i: (requests[i]["arrival"], i))
    nxt, n_done = 0, 0
    while n_done < len(requests):
        if nxt < len(order) and (not realtime or now() >= requests[order[nxt]]["arrival"]):
            rid = order[nxt]
            assign(adm.arrive(rid, requests[rid]["work"], requests[rid]["need"]))
            nxt += 1
            continue
        # the next completion, or the next arrival's time
        wait = None
        if nxt < len(order) and realtime:
            wait = max(0.0, requests[order[nxt]]["arrival"] - now())
        try:
            rid, start, end, res, err = finished.get(timeout=wait)
        except queue.Empty:
            continue
        if start is None:
            start = remote_start.pop(rid)
        out[rid].update(start=start, done=end, result=res, error=err)
        n_done += 1
        assign(adm.complete(rid))
    local_q.put(None)
    for r in range(1, world):
        send(-1, r)
    for th in threads:
        th.join()
    return {"requests": out, "peak_bytes": list(adm.peak), "waited": adm.waited}
