"""The GPU FP64 V-cycle against the committed golden fixtures: same trees
(built by the library's host builder), same right-hand sides, same exact
digests of phi, tmp and rhs per level after 1, 2 and 5 V-cycles."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import golden_cases as GC  # noqa: E402

pytestmark = pytest.mark.gpu

with open(os.path.join(HERE, "golden", "golden.json")) as f:
    GOLDEN = json.load(f)


@pytest.mark.parametrize("name", sorted(GC.CASES))
def test_gpu_matches_golden(gpu, name):
    c = GC.CASES[name]
    g = GOLDEN[name]
    D, nc = c["dim"], c["n_cell"]
    t = gpu.Tree(D, nc, c["dr"], coarsen_to=c["coarsen_to"])
    t.set_base([[1] * D], [[-1] * (2 * D)])
    for _ in range(c["passes"]):
        t.adjust_builtin(gpu.AFV_REF_RANDOM, c["lvl_max"], prob=c["prob"], seed=c["seed"])
    b = t.boxes()
    boxes = [[int(l)] + [int(x) for x in ix] for l, ix, u in zip(b["lvl"], b["ix"], b["in_use"] != 0) if u]
    assert boxes == g["boxes"]
    levels = list(range(t.min_lvl, t.highest_lvl + 1))
    parts = []
    for l in levels:
        n = len(t.level(l)[0]) * (t.n_cell_at(l) + 2) ** D
        parts.append(GC.hash_values(n, 1000 + l))
    f = gpu.Forest([t])
    f.set_var(0, gpu.AFV_RHS, np.concatenate(parts))
    done = 0
    for k in GC.CYCLES:
        while done < k:
            f.vcycle(set_residual=True)
            done += 1
        for name_v, var in (("phi", gpu.AFV_PHI), ("tmp", gpu.AFV_TMP), ("rhs", gpu.AFV_RHS)):
            flat = f.get_var(0, var)
            off = 0
            for l in levels:
                ncl = t.n_cell_at(l)
                nb = len(t.level(l)[0])
                a = flat[off:off + nb * (ncl + 2) ** D].reshape((nb,) + (ncl + 2,) * D)
                off += a.size
                assert GC.level_digest(a, ncl, D) == g["cycles"][str(k)][name_v][str(l)], (name, k, name_v, l)
    f.close()
