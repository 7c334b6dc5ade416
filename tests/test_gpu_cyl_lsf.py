"""GPU parity of the cylindrical and level-set operators behind the FAS
V-cycle: mg2_box_*_clpl / _clpld (src/m_aX_mg.f90:1323-1443) with the
weighted restriction of a2_restrict_box (src/m_aX_restrict.f90:90-103), the
internal-boundary operators mg$D_box_*_lpllsf with their masked restriction
and correction (:987-1321), and the auto dispatch over normal, eps and
level-set boxes (:562-706). The cylindrical case is examples/poisson_cyl.f90's
set-up (Neumann 0 on the axis); the level set is a sphere (circle) with a
position-dependent boundary value. Bar: 1e-13 relative per V-cycle or FMG
against the oracle (FP64); every tree holds each box kind the case names."""
import numpy as np
import pytest

import oracle as O
from helpers import (bval_field, compare_var, cyl_bc_table, cyl_spec, fill_from_centres, lsf_sphere,
                     oracle_solve, oracle_tree, oracle_var)
from afivo_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13
I_EPS, I_LSF, I_BVAL = 3, 4, 5


def _eps_jump(r):
    return np.where(r[..., 0] > 0.53, 100.0, 1.0)


def _pair(afv, spec, op, eps=None, lsf=False, cyl_bc=False):
    nc = spec["n_cell"]
    ot = oracle_tree(spec)
    ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    ot.mg_init()
    ot.add_vars(3, 0)
    tree = W.build_tree(spec)
    f = afv.Forest([tree], mixed=True)
    f.add_vars(3, 0)
    i_eps = i_lsf = i_bval = -1
    if eps is not None:
        f.set_var(0, I_EPS, fill_from_centres(ot, I_EPS, eps, nc))
        i_eps = I_EPS
    if lsf:
        f.set_var(0, I_LSF, fill_from_centres(ot, I_LSF, lsf_sphere, nc))
        f.set_var(0, I_BVAL, fill_from_centres(ot, I_BVAL, bval_field, nc))
        i_lsf, i_bval = I_LSF, I_BVAL
    f.set_var(0, afv.AFV_RHS, oracle_var(ot, O.I_RHS, nc))
    if cyl_bc:
        ids, faces, types, vals = cyl_bc_table(tree)
        ot.set_bc_table(ids, faces, types, vals)
        f.set_bc_faces(0, types, vals)
    assert ot.set_operator(op, i_eps, i_lsf, i_bval)
    f.set_operator(op, i_eps, i_lsf, i_bval)
    return ot, f


def _check(afv, f, ot, spec):
    nc, dim = spec["n_cell"], spec["dim"]
    out = {
        "phi": compare_var(f.get_var(0, afv.AFV_PHI), oracle_var(ot, O.I_PHI, nc), ot, nc, dim, False),
        "tmp": compare_var(f.get_var(0, afv.AFV_TMP), oracle_var(ot, O.I_TMP, nc), ot, nc, dim, True),
        "rhs": compare_var(f.get_var(0, afv.AFV_RHS), oracle_var(ot, O.I_RHS, nc), ot, nc, dim, True),
    }
    assert max(out.values()) <= TOL, out


# (operator, eps) in a cylindrical tree: the Cartesian Laplacian with the
# weighted restriction, auto without eps (every box clpl), clpl, clpld with
# an eps jump, auto with the jump (clpl and clpld boxes)
CYL = {
    "lpl": (0, None),
    "auto_normal": (2, None),
    "clpl": (3, None),
    "clpld": (4, _eps_jump),
    "auto_eps": (2, _eps_jump),
}


@pytest.mark.parametrize("case", list(CYL))
def test_cylindrical_cycles_match_oracle(gpu, case):
    op, eps = CYL[case]
    spec = cyl_spec(lvl_max=7)
    ot, f = _pair(gpu, spec, op, eps=eps, cyl_bc=True)
    for _ in range(3):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
        _check(gpu, f, ot, spec)


@pytest.mark.parametrize("case", ["lpl", "clpl", "auto_eps"])
def test_cylindrical_fmg_matches_oracle(gpu, case):
    op, eps = CYL[case]
    spec = cyl_spec(lvl_max=7)
    ot, f = _pair(gpu, spec, op, eps=eps, cyl_bc=True)
    for i in range(2):
        ot.fmg(set_residual=True, have_guess=i > 0)
        f.fmg(set_residual=True, have_guess=i > 0)
        _check(gpu, f, ot, spec)


def test_cylindrical_fp64_solve(gpu):
    """poisson_cyl's loop: the FP64 solve takes the oracle's cycle count and
    ends on its values; the mixed-precision solve is refused."""
    spec = cyl_spec(lvl_max=7)
    ot, f = _pair(gpu, spec, 2, cyl_bc=True)
    n = oracle_solve(ot, 1e-8)
    cyc, rel, rc = f.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=60)
    assert rc == 0 and int(cyc[0]) == n and rel[0] <= 1e-8
    _check(gpu, f, ot, spec)
    cyc, rel, rc = f.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60, check=False)
    assert rc == gpu.AFV_ERR_UNSUPPORTED


def _lsf_spec(dim):
    return W.c1_poisson_2d() if dim == 2 else W.c2_poisson_3d(thr=3e-3, lvl_max=5)


# (operator, eps) with the level set: lpllsf on every box, auto with the
# level set (normal and lsf boxes). A varying eps cannot join a level set
# under auto: the coarsest box holds both and mg$D_set_box_tag stops.
LSF = {"lpllsf": (5, None), "auto_lsf": (2, None)}


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("case", list(LSF))
def test_level_set_cycles_match_oracle(gpu, dim, case):
    op, eps = LSF[case]
    spec = _lsf_spec(dim)
    ot, f = _pair(gpu, spec, op, eps=eps, lsf=True)
    for _ in range(3):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
        _check(gpu, f, ot, spec)


@pytest.mark.parametrize("dim", [2, 3])
def test_level_set_fmg_and_solve(gpu, dim):
    spec = _lsf_spec(dim)
    ot, f = _pair(gpu, spec, 2, lsf=True)
    for i in range(2):
        ot.fmg(set_residual=True, have_guess=i > 0)
        f.fmg(set_residual=True, have_guess=i > 0)
        _check(gpu, f, ot, spec)
    ot2, f2 = _pair(gpu, spec, 5, lsf=True)
    n = oracle_solve(ot2, 1e-8)
    cyc, rel, rc = f2.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=60)
    assert rc == 0 and int(cyc[0]) == n and rel[0] <= 1e-8
    _check(gpu, f2, ot2, spec)


def test_single_operators_level_set_2d(gpu):
    spec = _lsf_spec(2)
    ot, f = _pair(gpu, spec, 2, lsf=True)
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


def test_auto_refuses_two_tags_in_one_box(gpu):
    """A box with both a level-set crossing and a varying eps is refused,
    where mg$D_set_box_tag stops; the forest keeps its operator."""
    spec = dict(W.c1_poisson_2d(), lvl_max=4)
    ot = oracle_tree(spec)
    ot.mg_init()
    ot.add_vars(3, 0)
    tree = W.build_tree(spec)
    f = gpu.Forest([tree])
    f.add_vars(3, 0)
    nc = spec["n_cell"]
    f.set_var(0, I_LSF, fill_from_centres(ot, I_LSF, lsf_sphere, nc))
    f.set_var(0, I_BVAL, fill_from_centres(ot, I_BVAL, bval_field, nc))
    f.set_var(0, I_EPS, fill_from_centres(ot, I_EPS, lambda r: np.where(r[..., 0] > 0.5, 3.0, 1.0), nc))
    assert not ot.set_operator(2, I_EPS, I_LSF, I_BVAL)
    with pytest.raises(gpu.AfivoError) as e:
        f.set_operator(2, I_EPS, I_LSF, I_BVAL)
    assert e.value.code == gpu.AFV_ERR_INVALID
    with pytest.raises(gpu.AfivoError):
        f.set_operator(3)  # clpl in a Cartesian tree


def test_device_tree_keeps_coordinates(gpu):
    """A cylindrical tree refined on the device and downloaded into a
    Cartesian host tree comes back cylindrical, and solves like the tree
    refined on the host."""
    spec = cyl_spec(lvl_max=6)
    base = gpu.Tree(2, spec["n_cell"], spec["dr"], coarsen_to=spec["coarsen_to"]).set_coord(1)
    d = gpu.DeviceTree(base.set_base(spec["ix"], spec["nb"]))
    d.refine_builtin(spec["crit"], spec["lvl_max"], thr=spec["thr"], gauss=spec["gauss"], lpl=spec["lpl"])
    host = gpu.Tree(2, spec["n_cell"], spec["dr"], coarsen_to=spec["coarsen_to"]).set_base(spec["ix"], spec["nb"])
    d.download(host)
    d.close()
    out = []
    for tree in (host, W.build_tree(spec)):
        ot = oracle_tree(spec)
        ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
        f = gpu.Forest([tree])
        f.set_operator(3)  # accepted for cylindrical trees only
        f.set_var(0, gpu.AFV_RHS, oracle_var(ot, O.I_RHS, spec["n_cell"]))
        f.vcycle(set_residual=True)
        out.append(f.get_var(0, gpu.AFV_PHI))
    assert np.array_equal(out[0], out[1])
