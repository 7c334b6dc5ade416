"""Writes the golden fixtures (golden.json) from the oracle: per case the
tree's box list and, after 1, 2 and 5 FP64 V-cycles from phi = 0, exact
digests of phi, tmp and rhs per level. Run from the repository root:

    python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [HERE, os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

import golden_cases as GC  # noqa: E402
import oracle as O  # noqa: E402


def oracle_case(c):
    D = c["dim"]
    t = O.OracleTree(D, c["n_cell"], c["dr"], [[1] * D], [[-1] * (2 * D)], coarsen_to=c["coarsen_to"])
    for _ in range(c["passes"]):
        t.adjust_refinement(O.REF_RANDOM, c["lvl_max"], prob=c["prob"], seed=c["seed"])
    return t


def digest(t, c):
    out = {}
    for name, iv in (("phi", O.I_PHI), ("tmp", O.I_TMP), ("rhs", O.I_RHS)):
        out[name] = {str(l): GC.level_digest(t.get_level(l, iv, c["n_cell"]), t.n_cell_at(l, c["n_cell"]),
                                             c["dim"], interior=True)
                     for l in range(t.min_lvl, t.highest_lvl + 1)}
    return out


def set_rhs(t, c, salt):
    for l in range(t.min_lvl, t.highest_lvl + 1):
        a = t.get_level(l, O.I_RHS, c["n_cell"])
        t.set_level(l, O.I_RHS, GC.hash_values(a.size, salt + l).reshape(a.shape))


def main():
    O.build()
    res = {}
    for name, c in GC.CASES.items():
        t = oracle_case(c)
        b = t.boxes()
        used = b["in_use"] != 0
        res[name] = {"case": c, "min_lvl": t.min_lvl, "highest_lvl": t.highest_lvl,
                     "boxes": [[int(l)] + [int(x) for x in ix] for l, ix, u in zip(b["lvl"], b["ix"], used) if u],
                     "cycles": {}}
        set_rhs(t, c, 1000)
        t.mg_init()
        done = 0
        for k in GC.CYCLES:
            while done < k:
                t.vcycle(set_residual=True)
                done += 1
            res[name]["cycles"][str(k)] = digest(t, c)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(res, f, indent=0, sort_keys=True)


if __name__ == "__main__":
    main()
