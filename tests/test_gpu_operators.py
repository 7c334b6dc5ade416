"""GPU parity of the operator variants behind the FAS V-cycle: the
variable-coefficient operator div(eps grad phi) of mg$D_box_*_lpld
(src/m_aX_mg.f90:810-985) on every box, and the per-box dispatch of
mg$D_auto_* (src/m_aX_mg.f90:562-706) where boxes with eps = 1 take the
Laplacian. eps jumps by a factor 100 across a plane (as in
examples/poisson_cyl_dielectric.f90:140-157), so a tree holds all three box
tags. Bar: 1e-13 relative per V-cycle or FMG against the oracle (FP64)."""
import numpy as np
import pytest

import oracle as O
from helpers import compare_var, oracle_solve, oracle_tree, oracle_var
from afivo_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13
I_EPS = 3


def _centres(ot, lvl, nc, dim):
    b = ot.boxes()
    ids, _, _ = ot.level(lvl)
    g = np.arange(nc + 2) - 0.5
    out = np.zeros((len(ids),) + (nc + 2,) * dim + (dim,))
    grids = np.meshgrid(*([g] * dim), indexing="ij")[::-1]
    for n, i in enumerate(ids):
        for d in range(dim):
            out[n, ..., d] = b["r_min"][i - 1][d] + grids[d] * b["dr"][i - 1]
    return out


def _eps(r):
    return np.where(r[..., 0] > 0.53, 100.0, 1.0)


SPECS = {"2d": W.c1_poisson_2d(), "3d": W.c2_poisson_3d(thr=3e-3, lvl_max=5)}


def _pair(afv, which, op, eps_fn=None):
    eps_fn = eps_fn or _eps
    spec = SPECS[which]
    nc, dim = spec["n_cell"], spec["dim"]
    ot = oracle_tree(spec)
    ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    ot.mg_init()
    ot.add_vars(1, 0)
    f = afv.Forest([W.build_tree(spec)], mixed=True)
    f.add_vars(1, 0)
    parts = []
    for lvl in range(ot.min_lvl, ot.highest_lvl + 1):
        ncl = nc if lvl >= 1 else nc >> (1 - lvl)
        e = eps_fn(_centres(ot, lvl, ncl, dim))
        ot.set_level(lvl, I_EPS, e)
        parts.append(e.ravel())
    f.set_var(0, I_EPS, np.concatenate(parts))
    f.set_var(0, afv.AFV_RHS, oracle_var(ot, O.I_RHS, nc))
    ot.set_operator(op, I_EPS)
    f.set_operator(op, I_EPS)
    return spec, ot, f


def _check(afv, f, ot, spec):
    nc, dim = spec["n_cell"], spec["dim"]
    out = {
        "phi": compare_var(f.get_var(0, afv.AFV_PHI), oracle_var(ot, O.I_PHI, nc), ot, nc, dim, False),
        "tmp": compare_var(f.get_var(0, afv.AFV_TMP), oracle_var(ot, O.I_TMP, nc), ot, nc, dim, True),
        "rhs": compare_var(f.get_var(0, afv.AFV_RHS), oracle_var(ot, O.I_RHS, nc), ot, nc, dim, True),
    }
    assert max(out.values()) <= TOL, out


@pytest.mark.parametrize("which", ["2d", "3d"])
@pytest.mark.parametrize("op", [1, 2], ids=["lpld", "auto"])
def test_vcycles_match_oracle(gpu, which, op):
    spec, ot, f = _pair(gpu, which, op)
    for _ in range(4):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
        _check(gpu, f, ot, spec)


@pytest.mark.parametrize("which", ["2d", "3d"])
@pytest.mark.parametrize("op", [1, 2], ids=["lpld", "auto"])
def test_fmg_matches_oracle(gpu, which, op):
    spec, ot, f = _pair(gpu, which, op)
    for i in range(2):
        ot.fmg(set_residual=True, have_guess=i > 0)
        f.fmg(set_residual=True, have_guess=i > 0)
        _check(gpu, f, ot, spec)


@pytest.mark.parametrize("op", [1, 2], ids=["lpld", "auto"])
def test_single_operators(gpu, op):
    spec, ot, f = _pair(gpu, "2d", op)
    ot.vcycle()
    f.vcycle()
    top = ot.highest_lvl
    ot.gsrb_level(top, 2)
    f.gsrb_level(top, 2)
    ot.update_coarse(top)
    f.update_coarse(top)
    ot.correct_children(top - 1)
    f.correct_children(top - 1)
    _check(gpu, f, ot, spec)


@pytest.mark.parametrize("op", [1, 2], ids=["lpld", "auto"])
def test_fp64_solve(gpu, op):
    """The FP64 solve loop takes the oracle's cycle count and ends on its
    values; a mixed-precision solve is refused for these operators."""
    spec, ot, f = _pair(gpu, "2d", op)
    n = oracle_solve(ot, 1e-8)
    cyc, rel, rc = f.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=60)
    assert rc == 0 and int(cyc[0]) == n and rel[0] <= 1e-8
    _check(gpu, f, ot, spec)
    cyc, rel, rc = f.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60, check=False)
    assert rc == gpu.AFV_ERR_UNSUPPORTED


def test_auto_with_unit_eps_is_the_laplacian(gpu):
    """Every box tagged normal: the auto dispatch gives the constant-
    coefficient solver's bits (its fused kernels)."""
    spec = SPECS["2d"]
    ot = oracle_tree(spec)
    ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    rhs = oracle_var(ot, O.I_RHS, 8)
    out = []
    for op in (0, 2):
        f = gpu.Forest([W.build_tree(spec)])
        f.add_vars(1, 0)
        f.set_var(0, I_EPS, np.ones_like(rhs))
        f.set_var(0, gpu.AFV_RHS, rhs)
        if op:
            f.set_operator(op, I_EPS)
        for _ in range(3):
            f.vcycle(set_residual=True)
        out.append(f.get_var(0, gpu.AFV_PHI))
    assert np.array_equal(out[0], out[1])


def _scale_eps(ot, f, spec, factor):
    """eps times factor on both sides (ghost cells and coarse levels included)."""
    nc, dim = spec["n_cell"], spec["dim"]
    parts = []
    for lvl in range(ot.min_lvl, ot.highest_lvl + 1):
        ncl = nc if lvl >= 1 else nc >> (1 - lvl)
        e = factor * _eps(_centres(ot, lvl, ncl, dim))
        ot.set_level(lvl, I_EPS, e)
        parts.append(e.ravel())
    f.set_var(0, I_EPS, np.concatenate(parts))


def test_eps_changed_between_calls(gpu):
    """The reference's lpld operators read eps at every use: eps changed
    after the operator was set is seen by the next V-cycle and by the next
    solve of a cached solve graph."""
    spec, ot, f = _pair(gpu, "3d", 1)
    for _ in range(2):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
    _scale_eps(ot, f, spec, 3.0)
    for _ in range(2):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
    _check(gpu, f, ot, spec)
    spec, ot, f = _pair(gpu, "2d", 1)
    for factor in (1.0, 0.25):
        _scale_eps(ot, f, spec, factor)
        n = oracle_solve(ot, 1e-8)
        cyc, rel, rc = f.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=60)
        assert rc == 0 and int(cyc[0]) == n
        _check(gpu, f, ot, spec)


@pytest.mark.parametrize("scale", [1.0, 2.0 ** -450, 1e-160], ids=["unit", "tiny", "subnormal_products"])
@pytest.mark.parametrize("which", ["2d", "3d"])
def test_lpld_face_weights_all_branches(gpu, which, scale):
    """eps of 0.1 (its square is inexact: the face weight divides), 3 (an
    exact square: eps / 2 directly) and a smooth eps (unequal neighbours) in
    one tree, and the same times 2^-450 (below the range of the shortcut)
    and times 1e-160 (products of neighbouring eps below the normal range,
    where the sweep divides instead of doubling the stored weight): V-cycles
    give the oracle's values, all finite."""
    def eps(r):
        x = r[..., 0]
        return scale * np.where(x < 0.3, 0.1, np.where(x < 0.6, 3.0, 1.0 + r[..., 1]))
    spec, ot, f = _pair(gpu, which, 1, eps_fn=eps)
    for _ in range(2):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
        _check(gpu, f, ot, spec)
    for v in (gpu.AFV_PHI, gpu.AFV_TMP):
        assert np.isfinite(f.get_var(0, v, interior_only=True)).all()
    assert np.isfinite(f.get_var(0, gpu.AFV_RHS)).all()


def test_lpld_masked_solves(gpu):
    """Masked FP64 solves with the variable-coefficient operator on a forest
    of two copies of a tree: the leading tree alone (the solve limited to the
    leading slots, face weights of those trees only) and the trailing tree
    alone each give the solo forest's bits, and leave the other tree as it
    was."""
    spec, ot, solo = _pair(gpu, "2d", 1)
    eps, rhs = solo.get_var(0, I_EPS), solo.get_var(0, gpu.AFV_RHS)
    cyc, rel, rc = solo.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=60)
    assert rc == 0
    ref = solo.get_var(0, gpu.AFV_PHI)
    for mask in ([1, 0], [0, 1]):
        g = gpu.Forest([W.build_tree(spec), W.build_tree(spec)])
        g.add_vars(1, 0)
        for t in (0, 1):
            g.set_var(t, I_EPS, eps)
            g.set_var(t, gpu.AFV_RHS, rhs)
        g.set_operator(1, I_EPS)
        before = [g.get_var(t, gpu.AFV_PHI) for t in (0, 1)]
        c, r, rc = g.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=60, mask=mask)
        assert rc == 0
        on, off = mask.index(1), mask.index(0)
        assert int(c[on]) == int(cyc[0])
        assert np.array_equal(g.get_var(on, gpu.AFV_PHI), ref)
        assert np.array_equal(g.get_var(off, gpu.AFV_PHI), before[off])
        g.close()
