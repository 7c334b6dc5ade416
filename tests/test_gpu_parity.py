"""GPU parity: the sm_103a kernels against the CPU oracle on the same trees,
right-hand sides and cycle schedules. The FP64 path must agree within
1e-13 relative (max |gpu - oracle| / max |oracle|) after every V-cycle; the
tree and index work is compared bit for bit in test_tree_build.py."""
import numpy as np
import pytest

import oracle as O
from helpers import compare_var, oracle_solve, oracle_tree, oracle_var, setup_pair
from afivo_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13  # FP64 parity bar per cycle


def assert_state(afv, f, ot, spec, tol=TOL, tree=0, what=("phi", "tmp", "rhs")):
    nc, dim = spec["n_cell"], spec["dim"]
    out = {}
    if "phi" in what:
        out["phi"] = compare_var(f.get_var(tree, afv.AFV_PHI), oracle_var(ot, O.I_PHI, nc), ot, nc,
                                 dim, False)
    if "tmp" in what:
        out["tmp"] = compare_var(f.get_var(tree, afv.AFV_TMP), oracle_var(ot, O.I_TMP, nc), ot, nc,
                                 dim, True)
    if "rhs" in what:
        out["rhs"] = compare_var(f.get_var(tree, afv.AFV_RHS), oracle_var(ot, O.I_RHS, nc), ot, nc,
                                 dim, True)
    for k, v in out.items():
        assert v <= tol, (k, out)
    return out


def test_vcycle_c1_every_cycle(gpu):
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec)
    for _ in range(10):
        ot.vcycle(set_residual=True)
        f.vcycle(set_residual=True)
        assert_state(gpu, f, ot, spec)


def test_single_operators_c1(gpu):
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec)
    ot.vcycle()
    f.vcycle()
    top = ot.highest_lvl
    # gsrb_boxes on the finest level (includes refinement-boundary ghosts)
    ot.gsrb_level(top, 2)
    f.gsrb_level(top, 2)
    assert_state(gpu, f, ot, spec, what=("phi",))
    ot.update_coarse(top)
    f.update_coarse(top)
    assert_state(gpu, f, ot, spec, what=("phi", "rhs"))
    ot.gsrb_level(top - 1, 1)
    f.gsrb_level(top - 1, 1)
    ot.correct_children(top - 1)
    f.correct_children(top - 1)
    ot.fill_gc_level(top)
    f.fill_gc_level(top)
    assert_state(gpu, f, ot, spec, what=("phi",))


def test_fmg_c1(gpu):
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec)
    for i in range(3):
        ot.fmg(set_residual=True, have_guess=i > 0)
        f.fmg(set_residual=True, have_guess=i > 0)
        assert_state(gpu, f, ot, spec)
    # residual norm over the leaves (a$D_tree_max_cc / a$D_tree_min_cc)
    r_o = ot.max_abs_residual()
    r_g = f.max_abs(0, gpu.AFV_TMP)
    assert abs(r_o - r_g) <= TOL * max(r_o, 1e-300)


def test_vcycle_3d(gpu):
    spec = W.c2_poisson_3d(thr=3e-3, lvl_max=6)
    f, ot, _ = setup_pair(gpu, spec)
    for _ in range(4):
        ot.vcycle()
        f.vcycle()
        assert_state(gpu, f, ot, spec)


def test_fmg_3d(gpu):
    spec = W.c2_poisson_3d(thr=3e-3, lvl_max=6)
    f, ot, _ = setup_pair(gpu, spec)
    for i in range(2):
        ot.fmg(set_residual=True, have_guess=i > 0)
        f.fmg(set_residual=True, have_guess=i > 0)
        assert_state(gpu, f, ot, spec)


def test_dirichlet_values(gpu):
    """Non-zero boundary values from the sides_bc hook
    (examples/poisson_basic_2d.f90:167-203)."""
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec, bc_gauss=True)
    for i in range(2):
        ot.fmg(set_residual=True, have_guess=i > 0)
        f.fmg(set_residual=True, have_guess=i > 0)
        assert_state(gpu, f, ot, spec)
    ot.vcycle()
    f.vcycle()
    assert_state(gpu, f, ot, spec)


def _bc_table(tree):
    """Mixed per-face boundary records: Neumann with a smooth flux on x
    faces, Dirichlet with smooth values on y (and z) faces."""
    ids, faces, types, vals = [], [], [], []
    for i, fc, cen in tree.bc_faces():
        ids.append(i)
        faces.append(fc)
        types.append(-2 if fc // 2 == 0 else -1)
        vals.append(np.sin(3.0 * cen[:, 0]) + np.cos(2.0 * cen[:, 1]) * (0.5 if fc % 2 else -1.0))
    return ids, faces, types, np.concatenate(vals)


def test_bc_faces_hook(gpu):
    """A sampled sides_bc hook with a type and values per face
    (afv_forest_set_bc_faces) against the oracle's hook returning the same."""
    spec = W.c1_poisson_2d()
    f, ot, pt = setup_pair(gpu, spec)
    ids, faces, types, vals = _bc_table(pt)
    ot.set_bc_table(ids, faces, types, vals)
    f.set_bc_faces(0, types, vals)
    for _ in range(3):
        ot.vcycle()
        f.vcycle()
        assert_state(gpu, f, ot, spec)
    ot.fmg(set_residual=True, have_guess=True)
    f.fmg(set_residual=True, have_guess=True)
    assert_state(gpu, f, ot, spec)


def test_bc_faces_hook_3d(gpu):
    spec = W.c2_poisson_3d(thr=3e-3, lvl_max=5)
    f, ot, pt = setup_pair(gpu, spec)
    ids, faces, types, vals = _bc_table(pt)
    ot.set_bc_table(ids, faces, types, vals)
    f.set_bc_faces(0, types, vals)
    for _ in range(2):
        ot.vcycle()
        f.vcycle()
        assert_state(gpu, f, ot, spec)


def test_neumann(gpu):
    spec = dict(W.c3_uniform_2d(4), nb=[[-1] * 4], n_cell=8, dr=1 / 8, name="neumann")
    ot = oracle_tree(spec)
    pt = W.build_tree(spec)
    rng = np.random.default_rng(7)
    for l in range(ot.min_lvl, ot.highest_lvl + 1):
        a = ot.get_level(l, O.I_RHS, 8).copy()
        a[...] = rng.standard_normal(a.shape)
        ot.set_level(l, O.I_RHS, a)
    ot.mg_init(bc_kind=O.BC_NEUMANN_ZERO)
    f = gpu.Forest([pt])
    f.set_var(0, gpu.AFV_RHS, oracle_var(ot, O.I_RHS, 8))
    f.set_bc(0, gpu.AFV_BC_NEUMANN)
    for _ in range(3):
        ot.vcycle()
        f.vcycle()
        assert_state(gpu, f, ot, spec)


def test_periodic_uniform_2d(gpu):
    spec = W.c3_uniform_2d(4)
    f, ot, _ = setup_pair(gpu, spec)
    for _ in range(4):
        ot.vcycle()
        f.vcycle()
        assert_state(gpu, f, ot, spec)


def _uniform_3d(lvl, periodic):
    return dict(name="uniform3d_nc8_lvl%d" % lvl, dim=3, n_cell=8, coarsen_to=2, dr=1 / 8,
                ix=[[1, 1, 1]], nb=[[1] * 6] if periodic else [[-1] * 6], gauss=None, lpl=False,
                crit=W.AFV_REF_UNIFORM, thr=0.0, lvl_max=lvl, bc=W.AFV_BC_DIRICHLET)


def test_periodic_uniform_3d(gpu):
    """3-D, the base box its own neighbour on all six faces."""
    spec = _uniform_3d(4, periodic=True)
    f, ot, _ = setup_pair(gpu, spec)
    for _ in range(3):
        ot.vcycle()
        f.vcycle()
        assert_state(gpu, f, ot, spec)


def test_neumann_3d(gpu):
    spec = _uniform_3d(4, periodic=False)
    ot = oracle_tree(spec)
    pt = W.build_tree(spec)
    rng = np.random.default_rng(11)
    for l in range(ot.min_lvl, ot.highest_lvl + 1):
        a = ot.get_level(l, O.I_RHS, 8).copy()
        a[...] = rng.standard_normal(a.shape)
        ot.set_level(l, O.I_RHS, a)
    ot.mg_init(bc_kind=O.BC_NEUMANN_ZERO)
    f = gpu.Forest([pt])
    f.set_var(0, gpu.AFV_RHS, oracle_var(ot, O.I_RHS, 8))
    f.set_bc(0, gpu.AFV_BC_NEUMANN)
    for _ in range(3):
        ot.vcycle()
        f.vcycle()
        assert_state(gpu, f, ot, spec)


def test_forest_matches_single_trees(gpu):
    """Several trees of different depth in one forest give, per tree, the same
    bits as the tree alone and the oracle's values."""
    specs = W.c4_random_2d(4, small=True)
    trees = [W.build_tree(s) for s in specs]
    ots = []
    forest = gpu.Forest(trees)
    alone = []
    for k, s in enumerate(specs):
        ot = oracle_tree(s)
        ot.fill_gauss(O.I_RHS, s["gauss"], lpl=True)
        ot.mg_init()
        ots.append(ot)
        rhs = oracle_var(ot, O.I_RHS, 8)
        forest.set_var(k, gpu.AFV_RHS, rhs)
        f1 = gpu.Forest([W.build_tree(s)])
        f1.set_var(0, gpu.AFV_RHS, rhs)
        alone.append(f1)
    for _ in range(3):
        forest.vcycle()
        for f1 in alone:
            f1.vcycle()
        for ot in ots:
            ot.vcycle()
    for k, s in enumerate(specs):
        a = forest.get_var(k, gpu.AFV_PHI)
        b = alone[k].get_var(0, gpu.AFV_PHI)
        # Each tree alone is a forest whose highest level may be lower than the
        # forest's; the V-cycle of a tree starts at its own highest level.
        assert np.array_equal(a, b)
        assert_state(gpu, forest, ots[k], s, tree=k)


def test_fp64_solve_matches_oracle_cycle_count(gpu):
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec)
    fmax = ot.max_abs(O.I_RHS)
    ot.residual_all()
    n = 0
    while ot.max_abs_residual() > 1e-8 * fmax:
        ot.vcycle()
        n += 1
    cyc, rel, rc = f.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=40)
    assert rc == 0 and cyc[0] == n and rel[0] <= 1e-8
    assert_state(gpu, f, ot, spec)


def test_mixed_solve_reaches_tolerance(gpu):
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec, mixed=True)
    cyc, rel, rc = f.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
    assert rc == 0 and rel[0] <= 1e-8
    # error against the FP64 oracle solution solved to 1e-12
    for _ in range(40):
        ot.vcycle()
    ref = oracle_var(ot, O.I_PHI, 8)
    got = f.get_var(0, gpu.AFV_PHI)
    err = compare_var(got, ref, ot, 8, 2, True)
    assert err < 1e-6, err


def test_mixed_batch_alone_vs_mix(gpu):
    """Continuous-batching invariant: a tree solved inside a forest gets the
    same bits as solved alone (inactive trees are masked out per launch)."""
    specs = W.c4_random_2d(3, small=True)
    forest = gpu.Forest([W.build_tree(s) for s in specs], mixed=True)
    outs = []
    for k, s in enumerate(specs):
        forest.set_source(k, s["gauss"], lpl=True)
    cyc_f, rel_f, _ = forest.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
    for k, s in enumerate(specs):
        f1 = gpu.Forest([W.build_tree(s)], mixed=True)
        f1.set_source(0, s["gauss"], lpl=True)
        c1, r1, _ = f1.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
        assert c1[0] == cyc_f[k]
        assert np.array_equal(f1.get_var(0, gpu.AFV_PHI), forest.get_var(k, gpu.AFV_PHI))
        outs.append(r1[0])
    assert max(outs) <= 1e-8


@pytest.mark.parametrize("which", ["c1", "c1_nc16", "3d"])
def test_sweep_kernel_variants_agree(gpu, which):
    """Every sweep kernel variant (block-pipelined, warp-per-box with bulk
    copies in four warp / stage shapes, warp-per-box with per-lane copies)
    gives the oracle's bits, FP64 and mixed."""
    spec = {"c1": W.c1_poisson_2d, "c1_nc16": lambda: dict(W.c1_poisson_2d(), n_cell=16, dr=1 / 16, lvl_max=6),
            "3d": lambda: W.c2_poisson_3d(thr=3e-3, lvl_max=5)}[which]()
    f, ot, _ = setup_pair(gpu, spec)
    for _ in range(2):
        ot.vcycle()
    ref = oracle_var(ot, O.I_PHI, spec["n_cell"])
    rhs = f.get_var(0, gpu.AFV_RHS)
    mixed = []
    for sk in (0, 1, 2, 3, 4, 5):
        g = gpu.Forest([W.build_tree(spec)], mixed=True)
        g.set_var(0, gpu.AFV_RHS, rhs)
        g.set_option(gpu.AFV_OPT_SWEEP_KERNEL, sk)
        for _ in range(2):
            g.vcycle()
        assert compare_var(g.get_var(0, gpu.AFV_PHI), ref, ot, spec["n_cell"], spec["dim"], False) == 0.0
        g.zero(gpu.AFV_PHI)
        g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=30)
        mixed.append(g.get_var(0, gpu.AFV_PHI))
        g.close()
    for m in mixed[1:]:
        assert np.array_equal(mixed[0], m)


def test_sweep_kernel_variants_agree_batch(gpu):
    """A forest of trees of different depths (a warp's boxes from several
    trees): every sweep variant gives the same bits in FP64 V-cycles and
    mixed solves, per tree."""
    specs = W.c4_random_2d(5, small=True)
    out = []
    for sk in (0, 1, 2, 3, 4, 5):
        g = gpu.Forest([W.build_tree(s) for s in specs], mixed=True)
        for t, s in enumerate(specs):
            g.set_source(t, s["gauss"], lpl=True)
        g.set_option(gpu.AFV_OPT_SWEEP_KERNEL, sk)
        for _ in range(2):
            g.vcycle()
        v = [g.get_var(t, gpu.AFV_PHI) for t in range(len(specs))]
        g.zero(gpu.AFV_PHI)
        cyc, rel, rc = g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
        assert rc == 0 and max(rel) <= 1e-8
        v += [g.get_var(t, gpu.AFV_PHI) for t in range(len(specs))]
        out.append((list(cyc), v))
        g.close()
    for cyc, v in out[1:]:
        assert cyc == out[0][0]
        for a, b in zip(v, out[0][1]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("which", ["c1", "3d"])
def test_restrict_kernel_variants_agree(gpu, which):
    """Warp-per-box and block-staged residual restriction give the same bits
    (FP64 V-cycles and mixed solves)."""
    spec = W.c1_poisson_2d() if which == "c1" else W.c2_poisson_3d(thr=3e-3, lvl_max=5)
    f, ot, _ = setup_pair(gpu, spec)
    rhs = f.get_var(0, gpu.AFV_RHS)
    out = []
    for rk in (1, 0):
        g = gpu.Forest([W.build_tree(spec)], mixed=True)
        g.set_var(0, gpu.AFV_RHS, rhs)
        g.set_option(gpu.AFV_OPT_RESTRICT_KERNEL, rk)
        for _ in range(2):
            g.vcycle(set_residual=True)
        v = [g.get_var(0, x) for x in (gpu.AFV_PHI, gpu.AFV_TMP, gpu.AFV_RHS)]
        g.zero(gpu.AFV_PHI)
        g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=30)
        v.append(g.get_var(0, gpu.AFV_PHI))
        out.append(v)
        g.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("which", ["c1", "3d"])
def test_small_level_sweeps_agree(gpu, which):
    """All half-sweeps of a small level in one block (the default) and launched
    one by one give the same bits (FP64 V-cycles and mixed solves)."""
    spec = W.c1_poisson_2d() if which == "c1" else W.c2_poisson_3d(thr=3e-3, lvl_max=5)
    f, ot, _ = setup_pair(gpu, spec)
    rhs = f.get_var(0, gpu.AFV_RHS)
    out = []
    for opt in (1, 0):
        g = gpu.Forest([W.build_tree(spec)], mixed=True)
        g.set_var(0, gpu.AFV_RHS, rhs)
        g.set_option(gpu.AFV_OPT_SMALL_SWEEPS, opt)
        for _ in range(2):
            g.vcycle(set_residual=True)
        v = [g.get_var(0, x) for x in (gpu.AFV_PHI, gpu.AFV_TMP, gpu.AFV_RHS)]
        g.zero(gpu.AFV_PHI)
        g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=30)
        v.append(g.get_var(0, gpu.AFV_PHI))
        out.append(v)
        g.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def _steep_spec(dim):
    """A near-delta source the tree does not resolve: one Gaussian of width
    0.01 centred on a cell centre (its Laplacian as the source, values
    spanning many orders of magnitude inside a box) on a tree refined to
    level 4 (2-D, cells of 0.016) or 3 (3-D, 0.031) uniformly."""
    c = (0.5078125, 0.4921875, 0.5078125)[:dim]
    base = W.c1_poisson_2d() if dim == 2 else W.c2_poisson_3d()
    return dict(base, name="steep%dd" % dim, gauss=W.gauss_records([c], [1.0], [0.01]),
                crit=W.AFV_REF_UNIFORM, lvl_max=4 if dim == 2 else 3)


@pytest.mark.parametrize("which", ["c1", "c1_nc4", "3d", "steep2d", "steep3d"])
def test_defect_kernels_agree(gpu, which):
    """The mixed solve's defect with the fixed-point Laplacian (default) and
    with the FP64 sum: same cycle counts, residuals within float rounding,
    solutions within the solve tolerance of each other and of the oracle,
    also for a source with steep jumps inside boxes."""
    spec = {"c1": W.c1_poisson_2d, "c1_nc4": lambda: dict(W.c1_poisson_2d(), n_cell=4, dr=0.25, lvl_max=8, thr=1e-6),
            "3d": lambda: W.c2_poisson_3d(thr=3e-3, lvl_max=5),
            "steep2d": lambda: _steep_spec(2), "steep3d": lambda: _steep_spec(3)}[which]()
    f, ot, _ = setup_pair(gpu, spec)
    rhs = f.get_var(0, gpu.AFV_RHS)
    out = []
    for opt in (1, 0):
        g = gpu.Forest([W.build_tree(spec)], mixed=True)
        g.set_var(0, gpu.AFV_RHS, rhs)
        g.set_option(gpu.AFV_OPT_DEFECT_KERNEL, opt)
        assert g.get_option(gpu.AFV_OPT_DEFECT_KERNEL) == opt
        cyc, rel, rc = g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
        assert rc == 0 and rel[0] <= 1e-8
        out.append((int(cyc[0]), float(rel[0]), g.get_var(0, gpu.AFV_PHI)))
        g.close()
    (c1, r1, p1), (c0, r0, p0) = out
    assert c1 == c0
    assert abs(r1 - r0) <= 1e-3 * r0
    scale = np.abs(p0).max()
    assert np.abs(p1 - p0).max() <= 1e-7 * scale
    for _ in range(40):
        ot.vcycle()
    ref = oracle_var(ot, O.I_PHI, spec["n_cell"])
    assert compare_var(p1, ref, ot, spec["n_cell"], spec["dim"], True) < 1e-6


@pytest.mark.parametrize("which", ["c1", "c1_nc4", "3d", "3d_nc4", "batch"])
def test_defect_cells_agree(gpu, which):
    """The fixed-point defect with 1, 2 and 4 cells per thread (one leaf or
    several per block iteration, 16 or more threads per leaf: two leaves per
    warp at 16) gives the same bits: each leaf's sums and exponent do not
    depend on how its cells are spread over threads. The autotuner keeps one
    of the shapes the boxes allow."""
    if which == "batch":
        specs = W.c4_random_2d(3, small=True)
    elif which == "c1":
        specs = [W.c1_poisson_2d()]
    elif which == "c1_nc4":
        specs = [dict(W.c1_poisson_2d(), n_cell=4, dr=0.25, lvl_max=8, thr=1e-6)]
    elif which == "3d_nc4":
        specs = [dict(W.c2_poisson_3d(thr=3e-3, lvl_max=6), n_cell=4, dr=0.25)]
    else:
        specs = [W.c2_poisson_3d(thr=3e-3, lvl_max=5)]
    out = []
    for cells in (1, 2, 4):
        g = gpu.Forest([W.build_tree(s) for s in specs], mixed=True)
        for t, s in enumerate(specs):
            g.set_source(t, s["gauss"], lpl=True)
        g.set_option(gpu.AFV_OPT_DEFECT_CELLS, cells)
        assert g.get_option(gpu.AFV_OPT_DEFECT_CELLS) == cells
        cyc, rel, rc = g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
        assert rc == 0 and max(rel) <= 1e-8
        out.append((list(cyc), list(rel), [g.get_var(t, gpu.AFV_PHI) for t in range(len(specs))]))
        if cells == 4:
            choice, ms = g.autotune_defect()
            assert choice in ms and g.get_option(gpu.AFV_OPT_DEFECT_CELLS) == choice
            assert all(v > 0 for v in ms.values())
        g.close()
    for o in out[1:]:
        assert o[0] == out[0][0] and o[1] == out[0][1]
        for a, b in zip(o[2], out[0][2]):
            assert np.array_equal(a, b)


def test_mixed_solve_scale_invariant(gpu):
    """Scaling the right-hand side by 2^k scales every value of the mixed
    solve exactly (the fixed-point defect shifts its scale with the box's
    largest exponent), so the solution is the unscaled one times 2^k, bit for
    bit, and the cycle count is the same."""
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec)
    rhs = f.get_var(0, gpu.AFV_RHS)
    out = {}
    for k in (0, -40, 40):
        g = gpu.Forest([W.build_tree(spec)], mixed=True)
        g.set_var(0, gpu.AFV_RHS, np.ldexp(rhs, k))
        cyc, rel, rc = g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
        assert rc == 0 and rel[0] <= 1e-8
        out[k] = (int(cyc[0]), float(rel[0]), g.get_var(0, gpu.AFV_PHI))
        g.close()
    for k in (-40, 40):
        assert out[k][0] == out[0][0] and out[k][1] == out[0][1]
        assert np.array_equal(out[k][2], np.ldexp(out[0][2], k))


def test_defect_nonfinite_reports_divergence(gpu):
    """A box holding a NaN takes the FP64 sum, which carries the NaN into the
    residual: both defect kernels report the solve as diverged (the fixed-
    point one also with several leaves per block, the others in fixed point)."""
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec)
    rhs = f.get_var(0, gpu.AFV_RHS)
    phi = np.zeros_like(f.get_var(0, gpu.AFV_PHI, interior_only=True))
    phi[-1] = np.nan  # a cell of the last box, a leaf on the finest level
    for opt, cells in ((1, 1), (1, 2), (0, 0)):
        g = gpu.Forest([W.build_tree(spec)], mixed=True)
        g.set_var(0, gpu.AFV_RHS, rhs)
        g.set_var(0, gpu.AFV_PHI, phi, interior_only=True)
        g.set_option(gpu.AFV_OPT_DEFECT_KERNEL, opt)
        g.set_option(gpu.AFV_OPT_DEFECT_CELLS, cells)
        cyc, rel, rc = g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=5, check=False)
        assert rc == gpu.AFV_ERR_DIVERGED
        g.close()


@pytest.mark.parametrize("which", ["c1", "3d", "batch"])
def test_coarse_end_agrees(gpu, which):
    """The correction cycle's levels <= 1 in one launch (k_coarse_end, the
    default) and as one launch per operator give the same bits: mixed solves
    of a 2-D and a 3-D tree with coarsened levels, and of a forest of trees."""
    if which == "batch":
        specs = W.c4_random_2d(3, small=True)
    else:
        specs = [W.c1_poisson_2d() if which == "c1" else W.c2_poisson_3d(thr=3e-3, lvl_max=5)]
    out = []
    for opt in (1, 0):
        g = gpu.Forest([W.build_tree(s) for s in specs], mixed=True)
        for k, s in enumerate(specs):
            g.set_source(k, s["gauss"], lpl=True)
        g.set_option(gpu.AFV_OPT_COARSE_END, opt)
        assert g.get_option(gpu.AFV_OPT_COARSE_END) == opt
        cyc, rel, rc = g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
        assert rc == 0 and max(rel) <= 1e-8
        out.append((list(cyc), [g.get_var(k, gpu.AFV_PHI) for k in range(len(specs))]))
        g.close()
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)


def test_pinned_host_exchange(gpu):
    """Page-locked host buffers are read and written by the device directly
    (no staging copy): the same values as through pageable memory, both
    ways, ghosted and interior."""
    torch = pytest.importorskip("torch")
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec)
    for interior in (False, True):
        ref = f.get_var(0, gpu.AFV_RHS, interior_only=interior)
        pinned = torch.empty(ref.size, dtype=torch.float64, pin_memory=True)
        f.get_var(0, gpu.AFV_RHS, interior_only=interior, out=pinned.numpy())
        assert np.array_equal(pinned.numpy(), ref)
        src = torch.empty(ref.size, dtype=torch.float64, pin_memory=True)
        src.numpy()[:] = np.arange(ref.size, dtype=np.float64) * 0.5
        f.set_var(0, gpu.AFV_PHI, src.numpy(), interior_only=interior)
        back = f.get_var(0, gpu.AFV_PHI, interior_only=interior)
        if interior:
            assert np.array_equal(back, src.numpy())
        else:
            assert np.array_equal(back, src.numpy())


def test_wait_limit_error_path(gpu):
    """A wait limit of 0 makes every kernel's wait for its own copies give up
    at once: the kernels set the device error word and return after their
    copies in flight have landed, the solve stops and reports AFV_ERR_TIMEOUT
    and the word is cleared. With the default limit back, the next solve
    succeeds and matches the oracle, bit for bit in FP64."""
    spec = W.c2_poisson_3d(thr=3e-3, lvl_max=5)
    f, ot, _ = setup_pair(gpu, spec, mixed=True)
    default = f.get_option(gpu.AFV_OPT_WAIT_LIMIT_US)
    assert default == 2000000
    for prec in (gpu.AFV_PREC_MIXED, gpu.AFV_PREC_FP64):
        f.set_option(gpu.AFV_OPT_WAIT_LIMIT_US, 0)
        assert f.get_option(gpu.AFV_OPT_WAIT_LIMIT_US) == 0
        f.zero(gpu.AFV_PHI)
        cyc, rel, rc = f.solve(prec, tol=1e-8, max_cycles=5, check=False)
        assert rc == gpu.AFV_ERR_TIMEOUT, (prec, rc, cyc, rel)
        with pytest.raises(gpu.AfivoError) as e:
            f.vcycle()
        assert e.value.code == gpu.AFV_ERR_TIMEOUT
        f.set_option(gpu.AFV_OPT_WAIT_LIMIT_US, default)
        f.zero(gpu.AFV_PHI)
        f.zero(gpu.AFV_TMP)
        cyc, rel, rc = f.solve(prec, tol=1e-8, max_cycles=40)
        assert rc == 0 and rel[0] <= 1e-8
    # FP64 solve from zero again, against the oracle's loop
    n = oracle_solve(ot, 1e-8)
    f.zero(gpu.AFV_PHI)
    f.zero(gpu.AFV_TMP)
    cyc, rel, rc = f.solve(gpu.AFV_PREC_FP64, tol=1e-8, max_cycles=40)
    assert rc == 0 and int(cyc[0]) == n
    assert compare_var(f.get_var(0, gpu.AFV_PHI), oracle_var(ot, O.I_PHI, 8), ot, 8, 3, False) <= TOL


def test_not_converged_is_its_own_code(gpu):
    """Running out of cycles is AFV_ERR_NOT_CONVERGED, not a timeout."""
    spec = W.c1_poisson_2d()
    f, ot, _ = setup_pair(gpu, spec, mixed=True)
    for prec in (gpu.AFV_PREC_MIXED, gpu.AFV_PREC_FP64):
        f.zero(gpu.AFV_PHI)
        cyc, rel, rc = f.solve(prec, tol=1e-8, max_cycles=2, check=False)
        assert rc == gpu.AFV_ERR_NOT_CONVERGED and int(cyc[0]) == 2 and rel[0] > 1e-8


def test_autotune_all_keeps_results(gpu):
    """The full tuning pass picks a sweep kernel and the two fusion switches,
    reports a time for every setting, and a solve with the choice gives the
    same bits as one with the defaults."""
    specs = W.c4_random_2d(3, small=True)
    out = []
    for tune in (False, True):
        g = gpu.Forest([W.build_tree(s) for s in specs], mixed=True)
        for k, s in enumerate(specs):
            g.set_source(k, s["gauss"], lpl=True)
        if tune:
            choice, times = g.autotune_all()
            assert 0 <= choice["sweep_kernel"] <= 5 and len(times) == 10
            assert all(t > 0 for t in times.values())
            assert g.get_option(gpu.AFV_OPT_SWEEP_KERNEL) == choice["sweep_kernel"]
            assert g.get_option(gpu.AFV_OPT_SMALL_SWEEPS) == choice["small_sweeps"]
            assert g.get_option(gpu.AFV_OPT_COARSE_END) == choice["coarse_end"]
        cyc, rel, rc = g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=60)
        out.append([g.get_var(k, gpu.AFV_PHI) for k in range(len(specs))])
        g.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("which", ["c1", "3d", "batch"])
def test_direct_sweeps_agree(gpu, which):
    """The unstaged half-sweep (AFV_OPT_DIRECT_BOXES) on every level and the
    staged sweeps give the same bits: FP64 V-cycles and mixed solves, with
    refinement boundaries, coarsened levels and a forest of trees."""
    if which == "batch":
        specs = W.c4_random_2d(3, small=True)
    else:
        specs = [W.c1_poisson_2d() if which == "c1" else W.c2_poisson_3d(thr=3e-3, lvl_max=5)]
    out = []
    for nb in (0, 1 << 30):
        g = gpu.Forest([W.build_tree(s) for s in specs], mixed=True)
        for k, s in enumerate(specs):
            g.set_source(k, s["gauss"], lpl=True)
        g.set_option(gpu.AFV_OPT_DIRECT_BOXES, nb)
        assert g.get_option(gpu.AFV_OPT_DIRECT_BOXES) == nb
        for _ in range(2):
            g.vcycle(set_residual=True)
        v = [g.get_var(k, x) for k in range(len(specs)) for x in (gpu.AFV_PHI, gpu.AFV_TMP)]
        g.zero(gpu.AFV_PHI)
        g.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=30)
        v += [g.get_var(k, gpu.AFV_PHI) for k in range(len(specs))]
        out.append(v)
        g.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_masked_solves_leading_and_scattered(gpu, prec):
    """Masked solves of a 4-tree forest: a mask of leading trees (run over
    those trees' boxes only) and a scattered mask give every selected tree
    the bits of its solve alone, leave the other trees' phi untouched, and a
    full solve afterwards is unaffected."""
    p = gpu.AFV_PREC_MIXED if prec == "mixed" else gpu.AFV_PREC_FP64
    specs = W.c4_random_2d(4, small=True)
    alone = []
    for s in specs:
        f1 = gpu.Forest([W.build_tree(s)], mixed=True)
        f1.set_source(0, s["gauss"], lpl=True)
        c1, _, _ = f1.solve(p, tol=1e-8, max_cycles=60)
        alone.append((int(c1[0]), f1.get_var(0, gpu.AFV_PHI)))
        f1.close()
    f = gpu.Forest([W.build_tree(s) for s in specs], mixed=True)
    for k, s in enumerate(specs):
        f.set_source(k, s["gauss"], lpl=True)
    for mask in ([1, 1, 0, 0], [1, 0, 0, 0], [0, 1, 0, 1], [1, 1, 1, 0]):
        f.zero(gpu.AFV_PHI)
        marker = [f.get_var(k, gpu.AFV_PHI) + (k + 1) for k in range(4)]
        for k in range(4):
            if not mask[k]:
                f.set_var(k, gpu.AFV_PHI, marker[k])  # must survive the masked solve
        cyc, rel, rc = f.solve(p, tol=1e-8, max_cycles=60, mask=mask)
        assert rc == 0
        for k in range(4):
            got = f.get_var(k, gpu.AFV_PHI)
            if mask[k]:
                assert int(cyc[k]) == alone[k][0]
                assert np.array_equal(got, alone[k][1]), (mask, k)
            else:
                assert np.array_equal(got, marker[k]), (mask, k)
    f.zero(gpu.AFV_PHI)
    cyc, rel, rc = f.solve(p, tol=1e-8, max_cycles=60)
    for k in range(4):
        assert np.array_equal(f.get_var(k, gpu.AFV_PHI), alone[k][1])
    f.close()


def test_host_exchange_routes_agree(gpu):
    """Page-locked host arrays exchanged by kernel loads and stores
    (AFV_OPT_ZERO_COPY 1, the default) and through the staging buffer on the
    copy engines (0) carry the same bits, ghosted and interior-only."""
    torch = pytest.importorskip("torch")
    spec = W.c1_poisson_2d()
    f = gpu.Forest([W.build_tree(spec)], mixed=True)
    f.set_source(0, spec["gauss"], lpl=True)
    rng = np.random.default_rng(11)
    for interior in (True, False):
        n = f._n_values(0, interior)
        src = torch.from_numpy(rng.standard_normal(n)).pin_memory()
        outs = []
        for zc in (1, 0):
            f.set_option(gpu.AFV_OPT_ZERO_COPY, zc)
            assert f.get_option(gpu.AFV_OPT_ZERO_COPY) == zc
            f.set_var(0, gpu.AFV_PHI, src.numpy(), interior_only=interior)
            dst = torch.empty(n, dtype=torch.float64).pin_memory()
            f.get_var(0, gpu.AFV_PHI, interior_only=interior, out=dst.numpy())
            outs.append(dst.numpy().copy())
        assert np.array_equal(outs[0], outs[1])
        if interior:
            assert np.array_equal(outs[0], src.numpy())
    f.close()
