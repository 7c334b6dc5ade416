"""GPU parity at the sizes the benchmark runs: the full 3-D adaptive tree
(34,907 boxes, 15.6 M leaf cells), the 4096^2 periodic uniform tree (87,384
boxes) with FMG, and all 256 random trees of the batched workload in one
forest. These reach the size-dependent paths of the kernels that small trees
never take: grid-stride loops once a level has more boxes than resident warps,
parents spread over more warps than the GPU holds, and reduction stripes over
many trees.

Bars: FP64 state within 1e-13 of the oracle (max |gpu - oracle| / max
|oracle|) after every V-cycle or FMG, compared per (level, ix, cell); the
mixed-precision solution within MIXED_TOL of the FP64 oracle's solution over
the leaf interiors, relative to max |phi| there."""
import numpy as np
import pytest

import oracle as O
from helpers import (compare_var, leaf_error, oracle_solve, oracle_tree, oracle_var,
                     same_tree)
from afivo_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13        # FP64 parity bar per cycle
MIXED_TOL = 1e-6   # mixed solution against the FP64 oracle's (relative to max |phi|)


def _state(afv, f, ot, nc, dim, tree=0):
    return {
        "phi": compare_var(f.get_var(tree, afv.AFV_PHI), oracle_var(ot, O.I_PHI, nc), ot, nc, dim,
                           False),
        "tmp": compare_var(f.get_var(tree, afv.AFV_TMP), oracle_var(ot, O.I_TMP, nc), ot, nc, dim,
                           True),
        "rhs": compare_var(f.get_var(tree, afv.AFV_RHS), oracle_var(ot, O.I_RHS, nc), ot, nc, dim,
                           True),
    }


@pytest.fixture(scope="module")
def c2(gpu):
    """The full 3-D workload on both sides, trees checked bit for bit."""
    spec = W.c2_poisson_3d()
    ot = oracle_tree(spec)
    pt = W.build_tree(spec)
    same_tree(pt, ot)
    ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    ot.mg_init()
    return spec, ot, pt


def test_c2_full_fp64_vcycles(gpu, c2):
    spec, ot, pt = c2
    assert pt.info()["n_boxes"] == 34907
    f = gpu.Forest([pt])
    f.set_var(0, gpu.AFV_RHS, oracle_var(ot, O.I_RHS, 8))
    ot.zero(O.I_PHI)
    ot.zero(O.I_TMP)
    for _ in range(3):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
        s = _state(gpu, f, ot, 8, 3)
        assert max(s.values()) <= TOL, s
    f.close()


def test_c2_full_fp64_solve_and_mixed_error(gpu, c2):
    """The FP64 GPU solve to 1e-8 takes the oracle's cycle count and ends on
    the oracle's bits; the mixed solve reaches 1e-8 with a solution within
    MIXED_TOL of the FP64 oracle solution."""
    spec, ot, pt = c2
    ot.zero(O.I_PHI)
    ot.zero(O.I_TMP)
    n = oracle_solve(ot, 1e-8)
    f = gpu.Forest([pt], mixed=True)
    f.set_var(0, gpu.AFV_RHS, oracle_var(ot, O.I_RHS, 8))
    cyc, rel, rc = f.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=40)
    assert rc == 0 and int(cyc[0]) == n and rel[0] <= 1e-8
    ref = oracle_var(ot, O.I_PHI, 8)
    assert compare_var(f.get_var(0, gpu.AFV_PHI), ref, ot, 8, 3, False) <= TOL
    f.zero(gpu.AFV_PHI)
    cyc, rel, rc = f.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=40)
    assert rc == 0 and rel[0] <= 1e-8
    err = leaf_error(f.get_var(0, gpu.AFV_PHI), ref, ot, 8, 3)
    print(f"C2 mixed: {int(cyc[0])} cycles, error against the FP64 oracle {err:.3e}")
    assert err <= MIXED_TOL, err
    f.close()


def _c3_rhs(ot, nc):
    """White noise (seed 3) on the finest level minus its mean, zero on the
    coarser levels: the periodic problem's source has zero mean."""
    rng = np.random.default_rng(3)
    for lvl in range(ot.min_lvl, ot.highest_lvl + 1):
        a = ot.get_level(lvl, O.I_RHS, nc).copy()
        a[...] = 0.0
        if lvl == ot.highest_lvl:
            inner = rng.standard_normal((a.shape[0], nc, nc))
            a[:, 1:nc + 1, 1:nc + 1] = inner - inner.mean()
        ot.set_level(lvl, O.I_RHS, a)


def test_c3_full_fmg_then_vcycles(gpu):
    spec = W.c3_uniform_2d(9)
    ot = oracle_tree(spec)
    pt = W.build_tree(spec)
    same_tree(pt, ot)
    assert pt.info()["n_boxes"] == 87384
    _c3_rhs(ot, 16)
    ot.mg_init()
    f = gpu.Forest([pt])
    f.set_var(0, gpu.AFV_RHS, oracle_var(ot, O.I_RHS, 16))
    ot.fmg(set_residual=True, have_guess=False)
    f.fmg(set_residual=True, have_guess=False)
    s = _state(gpu, f, ot, 16, 2)
    assert max(s.values()) <= TOL, s
    for _ in range(2):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
        s = _state(gpu, f, ot, 16, 2)
        assert max(s.values()) <= TOL, s
    f.close()


def test_c4_all_256_trees_vcycle(gpu):
    """All 256 random trees in one forest: each tree equals the oracle's bit
    for bit, and after one FP64 V-cycle each tree's state is the oracle's."""
    specs = W.c4_random_2d()
    pts = [W.build_tree(s) for s in specs]
    ots = []
    for s, pt in zip(specs, pts):
        ot = oracle_tree(s)
        same_tree(pt, ot)
        ot.fill_gauss(O.I_RHS, s["gauss"], lpl=True)
        ot.mg_init()
        ots.append(ot)
    f = gpu.Forest(pts)
    for k, ot in enumerate(ots):
        f.set_var(k, gpu.AFV_RHS, oracle_var(ot, O.I_RHS, 8))
    f.vcycle(set_residual=True)
    worst = 0.0
    for k, ot in enumerate(ots):
        ot.vcycle(set_residual=True)
        s = _state(gpu, f, ot, 8, 2, tree=k)
        worst = max(worst, max(s.values()))
        assert max(s.values()) <= TOL, (k, s)
    print(f"C4: 256 trees, worst FP64 difference {worst:.3e}")
    f.close()
