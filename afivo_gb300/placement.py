"""Placement of independent trees (batched solves, served requests) on the
GPUs of one node. Trees never exchange data, so a multi-GPU run is one
process per GPU, each solving the trees placed on it; there is no data-path
collective. Placement is deterministic, so every rank computes the same
assignment on its own."""


def place(work, n_ranks, capacity=None, need=None):
    """Longest-processing-time-first placement: item i (work[i], e.g. leaf
    cells x cycles) goes to the rank with the least work so far among those
    with room for need[i] bytes under capacity (per rank). Returns the owner
    rank of every item; raises if an item fits no rank."""
    n = len(work)
    need = need if need is not None else [0] * n
    order = sorted(range(n), key=lambda i: (-work[i], i))
    load = [0.0] * n_ranks
    used = [0] * n_ranks
    owner = [-1] * n
    for i in order:
        fits = [r for r in range(n_ranks) if capacity is None or used[r] + need[i] <= capacity]
        if not fits:
            raise ValueError(f"item {i} ({need[i]} bytes) fits no rank")
        r = min(fits, key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += work[i]
        used[r] += need[i]
    return owner


def shard(items, work, rank, world, capacity=None, need=None):
    """The items placed on this rank, in their original order."""
    owner = place(work, world, capacity, need)
    return [it for it, o in zip(items, owner) if o == rank]
