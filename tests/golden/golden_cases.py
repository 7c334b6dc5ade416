"""Cases of the golden fixtures: trees grown by keyed random refinement and
right-hand sides from an integer hash, so that building them needs no
transcendental function and gives the same bits on every host. Shared by the
fixture generator (make_golden.py) and the tests that read the fixtures."""
import math

import numpy as np

CASES = {
    "random2d_nc8": dict(dim=2, n_cell=8, dr=1 / 8, coarsen_to=2, lvl_max=6, prob=0.45, seed=12345,
                         passes=5),
    "random3d_nc8": dict(dim=3, n_cell=8, dr=1 / 8, coarsen_to=2, lvl_max=4, prob=0.35, seed=777,
                         passes=3),
}
CYCLES = (1, 2, 5)


def hash_values(n, salt):
    """n values k / 2^20 - 1/2, k from a 64-bit mix of (salt, i): exact doubles."""
    i = np.arange(n, dtype=np.uint64)
    x = i * np.uint64(0x9E3779B97F4A7C15) + np.uint64(salt)
    x ^= x >> np.uint64(31)
    x *= np.uint64(0xBF58476D1CE4E5B9)
    x ^= x >> np.uint64(29)
    return (x >> np.uint64(44)).astype(np.float64) / 2.0 ** 20 - 0.5


def level_digest(a, nc, dim, interior=True):
    """Exact digest of one level's boxes: fsum, fsum of squares (as hex) and
    eight sampled cells."""
    if interior:
        sl = (slice(None),) + (slice(1, nc + 1),) * dim
        a = a[sl]
    flat = np.ascontiguousarray(a).ravel()
    idx = np.linspace(0, flat.size - 1, 8).astype(int) if flat.size else []
    return {"sum": math.fsum(flat).hex(), "sumsq": math.fsum(flat * flat).hex(),
            "samples": [float(flat[k]).hex() for k in idx]}
