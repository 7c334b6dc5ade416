"""GPU parity of the general ghost-cell, transfer and output routines against
the oracle's restatement of the reference: a$D_gc_tree with every built-in
refinement-boundary and boundary method, a$D_prolong{0,1,2}_from with and
without add, a$D_restrict_tree, a$D_gc2_box, a$D_consistent_fluxes and
a$D_write_vtk, in Cartesian and cylindrical trees. Inputs are seeded random values in an extra cell variable (and
face variables) on every box, ghost cells included, on both sides; outputs
must be bit-identical (the VTK file byte for byte)."""
import os

import numpy as np
import pytest

import oracle as O
from helpers import cyl_spec, oracle_tree, oracle_var
from afivo_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = {
    "c1_2d": lambda: [W.c1_poisson_2d()],
    "adaptive_3d": lambda: [W.c2_poisson_3d(thr=3e-3, lvl_max=5)],
    "forest_2d": lambda: W.c4_random_2d(3, small=True),
    "cyl_2d": lambda: [cyl_spec(lvl_max=6)],  # weighted restriction and fluxes, r/z names
}


def _pair(afv, which, seed=5):
    """Library forest and oracle trees with random data in cell variables 3
    and 4 and in two face variables."""
    specs = CASES[which]()
    ots, trees = [], []
    for s in specs:
        ot = oracle_tree(s)
        ot.mg_init()
        ot.add_vars(2, 2)
        ots.append(ot)
        trees.append(W.build_tree(s))
    f = afv.Forest(trees)
    f.add_vars(2, 2)
    rng = np.random.default_rng(seed)
    nc = specs[0]["n_cell"]
    for k, ot in enumerate(ots):
        for iv in (3, 4):
            parts = []
            for lvl in range(ot.min_lvl, ot.highest_lvl + 1):
                a = rng.standard_normal(ot.get_level(lvl, iv, nc).shape)
                ot.set_level(lvl, iv, a)
                parts.append(a.ravel())
            f.set_var(k, iv, np.concatenate(parts))
        for ifc in (0, 1):
            v = rng.standard_normal(f.fc_count(k))
            ot.set_fc(ifc, v)
            f.set_fc(k, ifc, v)
    return specs, ots, f


def _same_var(afv, f, ots, specs, iv):
    for k, (ot, s) in enumerate(zip(ots, specs)):
        g = f.get_var(k, iv)
        o = oracle_var(ot, iv, s["n_cell"])
        assert np.array_equal(g, o), (k, iv, float(np.abs(g - o).max()))


@pytest.mark.parametrize("which", list(CASES))
@pytest.mark.parametrize("rb", [0, 1, 2, 3], ids=["mg", "prolong0", "interp", "interp_lim"])
@pytest.mark.parametrize("bc", [0, -1, -2], ids=["table", "dirichlet0", "neumann0"])
def test_gc_tree_var(gpu, which, rb, bc):
    specs, ots, f = _pair(gpu, which)
    for ot in ots:
        ot.gc_tree_var(3, rb, bc)
    f.gc_tree_var(3, rb, bc)
    _same_var(gpu, f, ots, specs, 3)


@pytest.mark.parametrize("which", list(CASES))
@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("add", [False, True])
def test_prolong_from_level(gpu, which, order, add):
    specs, ots, f = _pair(gpu, which)
    lmin = min(ot.min_lvl for ot in ots)
    lmax = max(ot.highest_lvl for ot in ots)
    for lp in range(lmin, lmax):
        for ot in ots:
            if lp < ot.highest_lvl:
                ot.prolong(lp, 3, 4, order, add)
        f.prolong(lp, 3, 4, order, add)
    _same_var(gpu, f, ots, specs, 4)
    # in place (iv_to = iv)
    for ot in ots:
        ot.prolong(ots[0].highest_lvl - 1 if len(ots) == 1 else 1, 3, 3, order, add)
    f.prolong(ots[0].highest_lvl - 1 if len(ots) == 1 else 1, 3, 3, order, add)
    _same_var(gpu, f, ots, specs, 3)


@pytest.mark.parametrize("which", list(CASES))
def test_restrict_tree(gpu, which):
    specs, ots, f = _pair(gpu, which)
    for ot in ots:
        ot.restrict_tree(3, 4)
    f.restrict_tree(3, 4)
    _same_var(gpu, f, ots, specs, 4)
    for ot in ots:
        ot.restrict_tree(3)
    f.restrict_tree(3)
    _same_var(gpu, f, ots, specs, 3)


@pytest.mark.parametrize("which", list(CASES))
def test_gc2(gpu, which):
    specs, ots, f = _pair(gpu, which)
    for k, (ot, s) in enumerate(zip(ots, specs)):
        for lvl in range(1, ot.highest_lvl + 1):
            assert np.array_equal(f.gc2_level(k, lvl, 3), ot.gc2_level(lvl, 3, s["n_cell"])), (k, lvl)


@pytest.mark.parametrize("which", list(CASES))
def test_consistent_fluxes(gpu, which):
    specs, ots, f = _pair(gpu, which)
    before = [f.get_fc(k, 1) for k in range(len(ots))]
    for ot in ots:
        ot.consistent_fluxes([1])
    f.consistent_fluxes([1])
    changed = 0
    for k, ot in enumerate(ots):
        g = f.get_fc(k, 1)
        o = ot.get_fc(1)
        assert np.array_equal(g, o), k
        assert np.array_equal(f.get_fc(k, 0), ot.get_fc(0))  # not selected: untouched
        changed += int((g != before[k]).sum())
    assert changed > 0  # the trees have refinement boundaries


@pytest.mark.parametrize("which", list(CASES))
def test_write_vtk_bytes(gpu, which, tmp_path):
    specs, ots, f = _pair(gpu, which)
    for k, ot in enumerate(ots):
        a = str(tmp_path / f"gpu_{k}")
        b = str(tmp_path / f"orc_{k}")
        f.write_vtk(k, a, [3, 4], ["u", "v"], [0, 1], ["flux", "g"], n_cycle=7, time=0.125)
        ot.write_vtk(b + ".vtu", [3, 4], ["u", "v"], [0, 1], ["flux", "g"], n_cycle=7, time=0.125)
        x = open(a + ".vtu", "rb").read()
        y = open(b + ".vtu", "rb").read()
        assert len(x) > 1000 and x == y, k
