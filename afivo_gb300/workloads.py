"""Seeded synthetic workloads: the five Poisson configurations the path is
measured and checked on. No public data set is involved; every input is made
here from fixed seeds.

The Gaussian records are (amplitude, sigma, centre...). Following the
reference's example examples/poisson_basic_2d.f90 (which these configurations
paraphrase), the Gaussians are the manufactured solution and the source
(right-hand side) is their Laplacian, gauss_lpl (examples/m_gaussians.f90:
90-102); a box is refined where any cell centre has |source| * dx^2 > thr.
"""
import numpy as np

from . import (AFV_BC_DIRICHLET, AFV_REF_RANDOM, AFV_REF_SOURCE, AFV_REF_UNIFORM, Tree)


def gauss_records(centres, amps, sigmas):
    recs = []
    for c, a, s in zip(centres, amps, sigmas):
        recs.extend([float(a), float(s), *[float(x) for x in c]])
    return np.array(recs)


def c1_poisson_2d():
    """2-D, 8x8 boxes on the unit square, Dirichlet 0, two Gaussians of
    amplitude 1 and width 0.04 at (0.25,0.25) and (0.75,0.75); refine where
    |source| dx^2 > 1e-3 up to level 8; 10 V-cycles."""
    g = gauss_records([(0.25, 0.25), (0.75, 0.75)], [1.0, 1.0], [0.04, 0.04])
    return dict(name="poisson2d_nc8_lvl8_gauss2", dim=2, n_cell=8, coarsen_to=2, dr=1 / 8,
                ix=[[1, 1]], nb=[[-1] * 4], gauss=g, lpl=True, crit=AFV_REF_SOURCE, thr=1e-3,
                lvl_max=8, bc=AFV_BC_DIRICHLET)


def c2_poisson_3d(seed=2, thr=7e-4, lvl_max=9):
    """3-D, 8^3 boxes on the unit cube, Dirichlet 0, four Gaussians with
    centres U(0.1,0.9)^3, amplitudes U(0.5,1), widths U(0.02,0.08) drawn from
    numpy's PCG64 with this seed; refine where |source| dx^2 > 7e-4 up to
    level 9 (1.564e7 leaf cells for seed 2)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.1, 0.9, (4, 3))
    a = rng.uniform(0.5, 1.0, 4)
    s = rng.uniform(0.02, 0.08, 4)
    return dict(name="poisson3d_nc8_gauss4_seed%d" % seed, dim=3, n_cell=8, coarsen_to=2,
                dr=1 / 8, ix=[[1, 1, 1]], nb=[[-1] * 6], gauss=gauss_records(c, a, s), lpl=True,
                crit=AFV_REF_SOURCE, thr=thr, lvl_max=lvl_max, bc=AFV_BC_DIRICHLET)


def c3_uniform_2d(lvl=9):
    """2-D, 16x16 boxes refined uniformly to `lvl` (4096^2 cells at 9),
    periodic (the base box is its own neighbour)."""
    return dict(name="uniform2d_nc16_lvl%d_periodic" % lvl, dim=2, n_cell=16, coarsen_to=2,
                dr=1 / 16, ix=[[1, 1]], nb=[[1, 1, 1, 1]], gauss=None, lpl=False,
                crit=AFV_REF_UNIFORM, thr=0.0, lvl_max=lvl, bc=AFV_BC_DIRICHLET)


def c4_random_2d(n_trees=256, seed=4, small=False):
    """Batched 2-D solves: trees of 8x8 boxes grown by keyed random refinement
    (probability 0.3 per leaf per pass) to a target size log-uniform in
    [1e4, 1e6] cells, maximum level U{6..9}; 3 Gaussians per tree, Dirichlet 0."""
    out = []
    for t in range(n_trees):
        rng = np.random.default_rng(seed + t)
        lo, hi = (1e3, 3e4) if small else (1e4, 1e6)
        target = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        lvl_max = int(rng.integers(6, 10))
        c = rng.uniform(0.1, 0.9, (3, 2))
        a = rng.uniform(0.5, 1.0, 3)
        s = rng.uniform(0.02, 0.08, 3)
        out.append(dict(name="random2d_t%d" % t, dim=2, n_cell=8, coarsen_to=2, dr=1 / 8,
                        ix=[[1, 1]], nb=[[-1] * 4], gauss=gauss_records(c, a, s), lpl=True,
                        crit=AFV_REF_RANDOM, prob=0.3, seed=seed * 1000003 + t,
                        lvl_max=lvl_max, target_cells=target, bc=AFV_BC_DIRICHLET))
    return out


def c5_requests(n=64, seed=5, small=False):
    """Serving: 3-D requests, 8^3 boxes, uniform trees from 32^3 to 256^3
    cells (log-uniform) with seeded Gaussian sources; Poisson arrivals of mean
    rate 200/s."""
    rng = np.random.default_rng(seed)
    reqs = []
    t = 0.0
    for k in range(n):
        t += rng.exponential(1 / 200.0)
        side = float(np.exp(rng.uniform(np.log(32), np.log(128 if small else 256))))
        # smallest uniform level whose cell count reaches side^3
        lvl = 1
        while 8 * 2 ** (lvl - 1) < side:
            lvl += 1
        c = rng.uniform(0.1, 0.9, (3, 3))
        a = rng.uniform(0.5, 1.0, 3)
        s = rng.uniform(0.02, 0.08, 3)
        reqs.append(dict(name="req%d" % k, arrival=t, dim=3, n_cell=8, coarsen_to=2, dr=1 / 8,
                         ix=[[1, 1, 1]], nb=[[-1] * 6], gauss=gauss_records(c, a, s), lpl=True,
                         crit=AFV_REF_UNIFORM, thr=0.0, lvl_max=lvl, bc=AFV_BC_DIRICHLET))
    return reqs


def build_tree(spec, max_passes=100):
    """Build the host tree of a workload with the library's tree builder."""
    t = Tree(spec["dim"], spec["n_cell"], spec["dr"], coarsen_to=spec["coarsen_to"])
    if spec.get("coord", 0):
        t.set_coord(spec["coord"])
    t.set_base(spec["ix"], spec["nb"])
    if spec["crit"] == AFV_REF_RANDOM and "target_cells" in spec:
        for _ in range(max_passes):
            if t.leaf_cells() >= spec["target_cells"]:
                break
            t.adjust_builtin(AFV_REF_RANDOM, spec["lvl_max"], prob=spec["prob"], seed=spec["seed"])
    else:
        t.refine_builtin(spec["crit"], spec["lvl_max"], thr=spec.get("thr", 0.0),
                         prob=spec.get("prob", 0.0), seed=spec.get("seed", 0),
                         gauss=spec.get("gauss"), lpl=spec.get("lpl", False),
                         max_passes=max_passes)
    return t
