"""Known answers for the oracle's variable-coefficient operators
(mg$D_box_*_lpld, src/m_aX_mg.f90:810-985) and the auto dispatch
(:562-706): with eps = 1 the auto dispatch is the Laplacian bit for bit, and
with a constant eps = c the lpld solve of c f equals the Laplacian solve of f
to round-off (the operator is c times the Laplacian)."""
import numpy as np
import pytest

import oracle as O
from helpers import oracle_solve, oracle_tree, oracle_var
from afivo_gb300 import workloads as W


def _tree(spec, eps, scale=1.0):
    ot = oracle_tree(spec)
    ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    ot.mg_init()
    ot.add_vars(1, 0)
    for lvl in range(ot.min_lvl, ot.highest_lvl + 1):
        a = ot.get_level(lvl, 3, spec["n_cell"])
        ot.set_level(lvl, 3, np.full(a.shape, eps))
        r = ot.get_level(lvl, O.I_RHS, spec["n_cell"])
        ot.set_level(lvl, O.I_RHS, r * scale)
    return ot


@pytest.mark.parametrize("spec", [W.c1_poisson_2d(), W.c2_poisson_3d(thr=3e-3, lvl_max=4)],
                         ids=["2d", "3d"])
def test_auto_unit_eps_is_laplacian(oracle_lib, spec):
    a = _tree(spec, 1.0)
    b = _tree(spec, 1.0)
    b.set_operator(2, 3)
    for _ in range(3):
        a.vcycle()
        b.vcycle()
    nc = spec["n_cell"]
    assert np.array_equal(oracle_var(a, O.I_PHI, nc), oracle_var(b, O.I_PHI, nc))


@pytest.mark.parametrize("spec", [W.c1_poisson_2d(), W.c2_poisson_3d(thr=3e-3, lvl_max=4)],
                         ids=["2d", "3d"])
@pytest.mark.parametrize("op", [1, 2], ids=["lpld", "auto"])
def test_constant_eps_scales_the_solution(oracle_lib, spec, op):
    a = _tree(spec, 1.0)
    b = _tree(spec, 4.0, scale=4.0)
    b.set_operator(op, 3)
    oracle_solve(a, 1e-10)
    oracle_solve(b, 1e-10)
    nc = spec["n_cell"]
    pa, pb = oracle_var(a, O.I_PHI, nc), oracle_var(b, O.I_PHI, nc)
    assert np.abs(pa - pb).max() <= 1e-8 * np.abs(pa).max()
