"""Shared setup for parity tests: build the same tree with the library and
with the CPU oracle, feed both the same inputs, and compare per (level, ix)."""
import numpy as np

import oracle as O
from afivo_gb300 import workloads as W


def oracle_tree(spec, max_passes=100):
    t = O.OracleTree(spec["dim"], spec["n_cell"], spec["dr"], spec["ix"], spec["nb"],
                     coarsen_to=spec["coarsen_to"])
    if spec.get("coord", 0):
        t.set_coord(spec["coord"])
    if "target_cells" in spec:
        for _ in range(max_passes):
            if leaf_boxes(t) * spec["n_cell"] ** spec["dim"] >= spec["target_cells"]:
                break
            t.adjust_refinement(O.REF_RANDOM, spec["lvl_max"], prob=spec["prob"], seed=spec["seed"])
    else:
        t.refine_until_done(spec["crit"], spec["lvl_max"], thr=spec.get("thr", 0.0),
                            prob=spec.get("prob", 0.0), seed=spec.get("seed", 0),
                            gauss=spec.get("gauss"), lpl=spec.get("lpl", False))
    return t


def leaf_boxes(t):
    return sum(len(t.level(l)[1]) for l in range(t.min_lvl, t.highest_lvl + 1))


def oracle_var(t, iv, n_cell):
    """Concatenation over levels of the oracle's boxes (the library's host layout)."""
    parts = [t.get_level(l, iv, n_cell).ravel() for l in range(t.min_lvl, t.highest_lvl + 1)]
    return np.concatenate(parts)


def split_boxes(flat, t, n_cell, dim):
    """Split a host-layout array into per-level box arrays."""
    out = {}
    off = 0
    for l in range(t.min_lvl, t.highest_lvl + 1):
        n = len(t.level(l)[0])
        nc = n_cell if l >= 1 else n_cell >> (1 - l)
        sz = n * (nc + 2) ** dim
        out[l] = flat[off:off + sz].reshape((n,) + (nc + 2,) * dim)
        off += sz
    return out


def face_mask(nc, dim):
    """Interior plus face ghost cells (corners and edges excluded)."""
    g = nc + 2
    idx = np.indices((g,) * dim)
    inner = [(a >= 1) & (a <= nc) for a in idx]
    n_out = sum((~m).astype(int) for m in inner)
    return n_out <= 1


def interior_mask(nc, dim):
    g = nc + 2
    idx = np.indices((g,) * dim)
    m = np.ones((g,) * dim, bool)
    for a in idx:
        m &= (a >= 1) & (a <= nc)
    return m


def compare_var(gpu_flat, ora_flat, t, n_cell, dim, interior_only):
    """Max relative difference over the compared cells of all boxes."""
    g = split_boxes(gpu_flat, t, n_cell, dim)
    o = split_boxes(ora_flat, t, n_cell, dim)
    worst = 0.0
    scale = max(np.abs(ora_flat).max(), 1e-300)
    for l in g:
        nc = n_cell if l >= 1 else n_cell >> (1 - l)
        m = interior_mask(nc, dim) if interior_only else face_mask(nc, dim)
        a, b = g[l][:, m], o[l][:, m]
        # identical values (infinities and NaNs included) differ by 0; a
        # non-finite value against another value by infinity
        same = (a == b) | (np.isnan(a) & np.isnan(b))
        with np.errstate(invalid="ignore"):
            d = np.where(same, 0.0, np.abs(a - b))
        d[np.isnan(d)] = np.inf
        if d.size:
            worst = max(worst, float(d.max()) / scale)
    return worst


def setup_pair(afv, spec, mixed=False, bc_gauss=False):
    """Library forest + oracle tree with identical trees and right-hand sides."""
    ot = oracle_tree(spec)
    pt = W.build_tree(spec)
    if spec.get("gauss") is not None:
        ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=spec.get("lpl", False))
    else:
        rng = np.random.default_rng(3)
        for l in range(ot.min_lvl, ot.highest_lvl + 1):
            a = ot.get_level(l, O.I_RHS, spec["n_cell"]).copy()
            a[...] = rng.standard_normal(a.shape)
            ot.set_level(l, O.I_RHS, a)
    bc_kind = O.BC_DIRICHLET_GAUSS if bc_gauss else O.BC_DIRICHLET_ZERO
    ot.mg_init(bc_kind=bc_kind, bc_gauss=spec["gauss"] if bc_gauss else None)
    f = afv.Forest([pt], mixed=mixed)
    f.set_var(0, afv.AFV_RHS, oracle_var(ot, O.I_RHS, spec["n_cell"]))
    if bc_gauss:
        f.set_bc(0, afv.AFV_BC_DIRICHLET, gauss=spec["gauss"], lpl=False)
    return f, ot, pt


def leaf_interiors(flat, t, n_cell, dim):
    """Interior values of the leaves only, concatenated over the levels, from
    a ghosted host-layout array (boxes in level-list order)."""
    boxes = split_boxes(flat, t, n_cell, dim)
    parts = []
    for l, arr in boxes.items():
        ids, leaves, _ = t.level(l)
        if not len(leaves):
            continue
        nc = n_cell if l >= 1 else n_cell >> (1 - l)
        rows = np.isin(ids, leaves)
        parts.append(arr[rows][:, interior_mask(nc, dim)].ravel())
    return np.concatenate(parts) if parts else np.zeros(0)


def leaf_error(gpu_flat, ora_flat, t, n_cell, dim):
    """max |gpu - oracle| over leaf interiors / max |oracle| there: the error
    of a solution against the oracle's, relative to the solution's size."""
    g = leaf_interiors(gpu_flat, t, n_cell, dim)
    o = leaf_interiors(ora_flat, t, n_cell, dim)
    return float(np.abs(g - o).max() / max(np.abs(o).max(), 1e-300))


def oracle_solve(ot, tol, max_cycles=80):
    """The reference's solve loop (examples/poisson_basic_2d.f90:84-92) on the
    oracle: V-cycles with the residual until max |r| <= tol * max |f| over the
    leaves; returns the number of V-cycles."""
    fmax = ot.max_abs(O.I_RHS)
    ot.residual_all()
    n = 0
    while ot.max_abs_residual() > tol * fmax and n < max_cycles:
        ot.vcycle(set_residual=True)
        n += 1
    return n


def same_tree(a, o):
    """The library's host tree equals the oracle's bit for bit: per-id
    topology (lvl, ix, parent, children, neighbours, n_cell, dr, r_min,
    in_use) and the level lists (ids, leaves, parents)."""
    ba, bo = a.boxes(), o.boxes()
    for k in bo:
        assert np.array_equal(ba[k], bo[k]), k
    for l in range(o.min_lvl, o.highest_lvl + 2):
        for x, y in zip(a.level(l), o.level(l)):
            assert np.array_equal(x, y), l


def interior_to_ghosted(flat_int, t, n_cell, dim):
    """A host-layout interior-only array (cc(1:nc,...) per box) spread into the
    ghosted layout, ghost cells zero."""
    parts, off = [], 0
    for l in range(t.min_lvl, t.highest_lvl + 1):
        n = len(t.level(l)[0])
        nc = n_cell if l >= 1 else n_cell >> (1 - l)
        g = np.zeros((n,) + (nc + 2,) * dim)
        sl = (slice(None),) + (slice(1, nc + 1),) * dim
        g[sl] = flat_int[off:off + n * nc ** dim].reshape((n,) + (nc,) * dim)
        off += n * nc ** dim
        parts.append(g.ravel())
    return np.concatenate(parts)


def centres(t, lvl, nc, dim):
    """Cell-centre coordinates of every box of a level of the oracle tree,
    ghost cells included: array (boxes, (nc+2)^dim..., dim), x fastest."""
    b = t.boxes()
    ids, _, _ = t.level(lvl)
    g = np.arange(nc + 2) - 0.5
    out = np.zeros((len(ids),) + (nc + 2,) * dim + (dim,))
    grids = np.meshgrid(*([g] * dim), indexing="ij")[::-1]
    for n, i in enumerate(ids):
        for d in range(dim):
            out[n, ..., d] = b["r_min"][i - 1][d] + grids[d] * b["dr"][i - 1]
    return out


def fill_from_centres(t, iv, fn, n_cell):
    """Variable iv of every box (ghost cells included) as fn(centres); returns
    the concatenation over levels (the library's host layout)."""
    parts = []
    for lvl in range(t.min_lvl, t.highest_lvl + 1):
        nc = t.n_cell_at(lvl, n_cell)
        v = np.ascontiguousarray(fn(centres(t, lvl, nc, t.dim)), dtype=np.float64)
        t.set_level(lvl, iv, v)
        parts.append(v.ravel())
    return np.concatenate(parts)


def cyl_spec(lvl_max=6):
    """The 2-D Gaussian workload in cylindrical coordinates (x the radius
    from the axis at 0, y the axis), as examples/poisson_cyl.f90 sets up."""
    s = W.c1_poisson_2d()
    s.update(name="poisson2d_cyl_nc8_lvl%d" % lvl_max, coord=1, lvl_max=lvl_max)
    return s


def cyl_bc_table(tree):
    """poisson_cyl's sides_bc: Neumann 0 on the axis (the low-x faces at
    r = 0), Dirichlet with smooth values on the other faces."""
    ids, faces, types, vals = [], [], [], []
    for i, fc, cen in tree.bc_faces():
        ids.append(i)
        faces.append(fc)
        types.append(-2 if fc == 0 else -1)
        vals.append(np.zeros(len(cen)) if fc == 0 else 0.1 * np.cos(2.0 * cen[:, 1]) + 0.05 * cen[:, 0])
    return ids, faces, types, np.concatenate(vals)


LSF_CENTRE = (0.45, 0.55, 0.5)
LSF_RADIUS = 0.23


def lsf_sphere(r):
    """Level set of a sphere (circle) around LSF_CENTRE: negative inside."""
    d = r.shape[-1]
    c = np.asarray(LSF_CENTRE[:d])
    return np.sqrt(((r - c) ** 2).sum(-1)) - LSF_RADIUS


def bval_field(r):
    """Boundary value at the interface, position dependent: 1 + 0.5 x."""
    return 1.0 + 0.5 * r[..., 0]
