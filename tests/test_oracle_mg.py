"""The oracle's multigrid against properties the reference solver has: the
V-cycle contraction, the V-cycle's fixed point at the discrete solution, and
second-order convergence to the manufactured solution of
examples/poisson_basic_2d.f90."""
import numpy as np

import oracle as O
from helpers import oracle_tree
from afivo_gb300 import workloads as W


def test_vcycle_contraction_c1(oracle_lib):
    spec = W.c1_poisson_2d()
    t = oracle_tree(spec)
    t.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    t.mg_init()
    fmax = t.max_abs(O.I_RHS)
    prev = None
    for k in range(8):
        t.vcycle()
        r = t.max_abs_residual() / fmax
        if prev is not None:
            assert r < 0.2 * prev
        prev = r
    assert prev < 1e-8


def test_fixed_point(oracle_lib):
    spec = W.c2_poisson_3d(thr=3e-3, lvl_max=6)
    t = oracle_tree(spec)
    t.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    t.mg_init()
    for _ in range(30):
        t.vcycle()
    before = [t.get_level(l, O.I_PHI, 8).copy() for l in range(1, t.highest_lvl + 1)]
    t.vcycle()
    after = [t.get_level(l, O.I_PHI, 8) for l in range(1, t.highest_lvl + 1)]
    scale = max(np.abs(b).max() for b in before)
    diff = max(np.abs(a - b).max() for a, b in zip(after, before))
    assert diff <= 1e-12 * scale


def test_manufactured_solution_second_order(oracle_lib):
    g = W.c1_poisson_2d()["gauss"].copy()
    g[1::4] = 0.1  # wider Gaussians so that the coarse grids resolve them
    errs = []
    for lvl in (3, 4, 5):
        t = O.OracleTree(2, 8, 1 / 8, [[1, 1]], [[-1] * 4], coarsen_to=2)
        t.refine_until_done(O.REF_UNIFORM, lvl)
        t.fill_gauss(O.I_RHS, g, lpl=True)
        t.mg_init(bc_kind=O.BC_DIRICHLET_GAUSS, bc_gauss=g)
        for i in range(4):
            t.fmg(set_residual=True, have_guess=i > 0)
        phi = t.get_level(lvl, O.I_PHI, 8)[:, 1:-1, 1:-1]
        ids, _, _ = t.level(lvl)
        b = t.boxes()
        err = 0.0
        for n, i in enumerate(ids):
            dr = b["dr"][i - 1]
            x = b["r_min"][i - 1, 0] + (np.arange(1, 9) - 0.5) * dr
            y = b["r_min"][i - 1, 1] + (np.arange(1, 9) - 0.5) * dr
            u = np.zeros((8, 8))
            for a_, s, cx, cy in g.reshape(-1, 4):
                # boxes are stored x fastest: array index [j, i]
                u += a_ * np.exp(-(((x[None, :] - cx) / s) ** 2 + ((y[:, None] - cy) / s) ** 2))
            err = max(err, np.abs(phi[n] - u).max())
        errs.append(err)
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5, errs


def test_bc_table_matches_builtin_hooks(oracle_lib):
    """Per-face records that restate a built-in hook give the same bits."""
    spec = W.c1_poisson_2d()
    for kind, typ in ((O.BC_DIRICHLET_ZERO, -1), (O.BC_NEUMANN_ZERO, -2)):
        a = oracle_tree(spec)
        b = oracle_tree(spec)
        for t in (a, b):
            t.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
        a.mg_init(bc_kind=kind)
        b.mg_init()
        pt = W.build_tree(spec)
        fl = pt.bc_faces()
        b.set_bc_table([x[0] for x in fl], [x[1] for x in fl], [typ] * len(fl),
                       np.zeros(sum(len(x[2]) for x in fl)))
        for _ in range(2):
            a.vcycle()
            b.vcycle()
        for lvl in range(a.min_lvl, a.highest_lvl + 1):
            assert np.array_equal(a.get_level(lvl, O.I_PHI, 8), b.get_level(lvl, O.I_PHI, 8))
