"""Known answers for the oracle's cylindrical operators (mg2_box_*_clpl /
_clpld, src/m_aX_mg.f90:1323-1443), the cylindrical restriction
(src/m_aX_restrict.f90:90-103) and the level-set operators
(mg$D_box_*_lpllsf, :987-1321), and the auto tags (mg$D_set_box_tag,
:672-706). The discrete cylindrical Laplacian of r^2 + z^2 is 6 exactly, an
r-weighted average of 1/r over a cell is 1/r at its centre, and the level-set
operator is exact for linear functions whose interface value is the
function's."""
import numpy as np
import pytest

import oracle as O
from helpers import (bval_field, centres, cyl_spec, fill_from_centres, lsf_sphere, oracle_tree,
                     oracle_var)
from afivo_gb300 import workloads as W

I_EPS, I_LSF, I_BVAL = 3, 4, 5


def _interiors(t, iv, nc):
    out = []
    for lvl in range(t.min_lvl, t.highest_lvl + 1):
        a = t.get_level(lvl, iv, nc)
        out.append(a[(slice(None),) + (slice(1, -1),) * t.dim].ravel())
    return np.concatenate(out)


@pytest.mark.parametrize("op", [0, 2, 3, 4], ids=["lpl", "auto", "clpl", "clpld"])
def test_cylindrical_laplacian_of_r2_z2(oracle_lib, op):
    spec = cyl_spec(lvl_max=5)
    t = oracle_tree(spec)
    t.mg_init()
    t.add_vars(3, 0)
    nc = spec["n_cell"]
    fill_from_centres(t, O.I_PHI, lambda r: r[..., 0] ** 2 + r[..., 1] ** 2, nc)
    fill_from_centres(t, O.I_RHS, lambda r: 0 * r[..., 0], nc)
    fill_from_centres(t, I_EPS, lambda r: 2.5 + 0 * r[..., 0], nc)
    assert t.set_operator(op, I_EPS if op in (2, 4) else -1)
    lib = O.lib()
    lib.orc_residual_all(t.h)
    res = _interiors(t, O.I_TMP, nc)
    if op == 0:  # the Cartesian operator on r^2 + z^2 is 4, not 6
        assert np.allclose(res, -4.0, rtol=0, atol=1e-6)
    else:
        want = -6.0 * (2.5 if op in (2, 4) else 1.0)
        assert np.allclose(res, want, rtol=0, atol=1e-6 * abs(want)), np.abs(res - want).max()


def test_cylindrical_restriction_of_inverse_radius(oracle_lib):
    """Parent cells covered by a leaf child whose quadrant starts at the
    parent's low-x edge get 1/r of their own centre. Children in the outer
    quadrant take the weights of the quadrant-local index, as
    a2_restrict_box passes i rather than i_c (src/m_aX_restrict.f90:
    98-99): there the average is not the r-weighted one, and the oracle
    keeps that."""
    spec = cyl_spec(lvl_max=5)
    t = oracle_tree(spec)
    t.mg_init()
    t.add_vars(1, 0)
    nc = spec["n_cell"]
    fill_from_centres(t, 3, lambda r: 1.0 / r[..., 0], nc)
    t.restrict_tree(3, 3)
    b = t.boxes()
    n_exact = n_quirk = 0
    for lvl in range(t.min_lvl, t.highest_lvl):
        ncl = t.n_cell_at(lvl, nc)
        ids, _, _ = t.level(lvl)
        got = t.get_level(lvl, 3, nc)
        want = 1.0 / centres(t, lvl, ncl, 2)[..., 0]
        for k, p in enumerate(ids):
            for c in b["children"][p - 1]:
                if c <= 0 or b["children"][c - 1][0] > 0:
                    continue  # no child, or a child that was itself restricted
                hnc = b["n_cell"][c - 1] // 2
                xb, yb = ((b["ix"][c - 1] - 1) & 1) if b["lvl"][c - 1] > 1 else (0, 0)
                sl = (k, slice(1 + yb * hnc, 1 + yb * hnc + hnc), slice(1 + xb * hnc, 1 + xb * hnc + hnc))
                rel = np.abs(got[sl] / want[sl] - 1).max()
                if xb == 0:
                    assert rel <= 1e-14, (lvl, p, rel)
                    n_exact += 1
                else:
                    assert rel > 1e-6
                    n_quirk += 1
    assert n_exact > 0 and n_quirk > 0


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("op", [5, 2], ids=["lpllsf", "auto"])
def test_level_set_operator_is_exact_for_linear_functions(oracle_lib, dim, op):
    spec = W.c1_poisson_2d() if dim == 2 else W.c2_poisson_3d(thr=3e-3, lvl_max=4)
    spec = dict(spec, lvl_max=min(spec["lvl_max"], 5))
    t = oracle_tree(spec)
    t.mg_init()
    t.add_vars(3, 0)
    nc = spec["n_cell"]
    lin = lambda r: 1.0 + 0.5 * r[..., 0]  # noqa: E731  (equals bval_field)
    fill_from_centres(t, O.I_PHI, lin, nc)
    fill_from_centres(t, O.I_RHS, lambda r: 0 * r[..., 0], nc)
    fill_from_centres(t, I_LSF, lsf_sphere, nc)
    fill_from_centres(t, I_BVAL, bval_field, nc)
    assert t.set_operator(op, -1, I_LSF, I_BVAL)
    O.lib().orc_residual_all(t.h)
    res = _interiors(t, O.I_TMP, nc)
    # |phi| <= 1.5 with 1 / dx^2 up to 2^14 (2-D) : round-off only
    assert np.abs(res).max() <= 1e-7, np.abs(res).max()


def test_level_set_operator_sees_the_interface(oracle_lib):
    """phi = 0 everywhere with bval = 1: the boxes the interface crosses get
    a nonzero operator, every other box 0."""
    spec = dict(W.c1_poisson_2d(), lvl_max=4)
    t = oracle_tree(spec)
    t.mg_init()
    t.add_vars(3, 0)
    nc = spec["n_cell"]
    fill_from_centres(t, O.I_PHI, lambda r: 0 * r[..., 0], nc)
    fill_from_centres(t, O.I_RHS, lambda r: 0 * r[..., 0], nc)
    lsf = fill_from_centres(t, I_LSF, lsf_sphere, nc)
    fill_from_centres(t, I_BVAL, lambda r: 1 + 0 * r[..., 0], nc)
    assert t.set_operator(5, -1, I_LSF, I_BVAL)
    O.lib().orc_residual_all(t.h)
    res = _interiors(t, O.I_TMP, nc)
    assert (res < 0).any() and np.abs(res).max() > 1.0
    # cells with every face neighbour on their own side see only phi = 0
    far = np.abs(_interiors(t, I_LSF, nc)) > 2 * 0.125
    assert np.all(res[far] == 0)


def test_auto_tags_refuse_two_kinds_in_one_box(oracle_lib):
    spec = dict(W.c1_poisson_2d(), lvl_max=3)
    t = oracle_tree(spec)
    t.mg_init()
    t.add_vars(3, 0)
    nc = spec["n_cell"]
    fill_from_centres(t, I_LSF, lsf_sphere, nc)
    fill_from_centres(t, I_BVAL, bval_field, nc)
    fill_from_centres(t, I_EPS, lambda r: 1 + 0 * r[..., 0], nc)
    assert t.set_operator(2, I_EPS, I_LSF, I_BVAL)
    fill_from_centres(t, I_EPS, lambda r: np.where(r[..., 0] > 0.5, 3.0, 1.0), nc)
    assert not t.set_operator(2, I_EPS, I_LSF, I_BVAL)
