"""Known answers for the oracle's restatement of the general ghost-cell,
transfer and output routines (src/m_aX_prolong.f90, m_aX_restrict.f90,
m_aX_gc.f90, m_aX_core.f90:811-945, m_aX_io.f90:115-310): the linear and
quadratic fields each stencil reproduces exactly, and the VTK file's own
structure. These pin the restatement to the mathematics of the reference,
which holds no golden vectors for these routines."""
import re
import struct

import numpy as np
import pytest

import oracle as O
from helpers import oracle_tree
from afivo_gb300 import workloads as W


def _centres(ot, lvl, nc, dim, ghost=True):
    """Cell-centre coordinates of every box of a level, ghost cells included:
    array (n_box, (nc+2)^dim..., dim)."""
    b = ot.boxes()
    ids, _, _ = ot.level(lvl)
    g = np.arange(nc + 2) - 0.5
    out = np.zeros((len(ids),) + (nc + 2,) * dim + (dim,))
    for n, i in enumerate(ids):
        rmin, dr = b["r_min"][i - 1], b["dr"][i - 1]
        grids = np.meshgrid(*([g] * dim), indexing="ij")[::-1]  # last axis = x
        for d in range(dim):
            out[n, ..., d] = rmin[d] + grids[d] * dr
    return out


def _fill(ot, iv, nc, dim, fn):
    for lvl in range(ot.min_lvl, ot.highest_lvl + 1):
        ncl = nc if lvl >= 1 else nc >> (1 - lvl)
        r = _centres(ot, lvl, ncl, dim)
        ot.set_level(lvl, iv, fn(r))


def _lin(r):
    return 0.3 + 1.7 * r[..., 0] - 0.9 * r[..., 1] + (0.4 * r[..., 2] if r.shape[-1] == 3 else 0)


def _quad(r):
    # quadratic in each direction separately (no cross terms)
    return 0.2 + 1.1 * r[..., 0] ** 2 - 0.7 * r[..., 1] ** 2 + (0.5 * r[..., 2] ** 2 if r.shape[-1] == 3 else 0)


SPECS = [W.c1_poisson_2d(), W.c2_poisson_3d(thr=3e-3, lvl_max=4)]


def _interior(ot, lvl, iv, nc, dim):
    a = ot.get_level(lvl, iv, nc)
    sl = (slice(None),) + (slice(1, nc + 1),) * dim
    return a[sl]


@pytest.mark.parametrize("spec", SPECS, ids=["2d", "3d"])
@pytest.mark.parametrize("order,fn", [(0, None), (1, _lin), (2, _lin), (2, _quad)])
def test_prolongation_reproduces_fields(oracle_lib, spec, order, fn):
    nc, dim = spec["n_cell"], spec["dim"]
    ot = oracle_tree(spec)
    ot.add_vars(2, 0)
    f = fn or (lambda r: np.full(r.shape[:-1], 2.5))  # injection: constants
    _fill(ot, 3, nc, dim, f)
    for lvl in range(1, ot.highest_lvl):
        ot.prolong(lvl, 3, 4, order, False)
    for lvl in range(2, ot.highest_lvl + 1):
        ids, _, _ = ot.level(lvl)
        want = f(_centres(ot, lvl, nc, dim))[(slice(None),) + (slice(1, nc + 1),) * dim]
        got = _interior(ot, lvl, 4, nc, dim)
        assert np.abs(got - want).max() <= 1e-12 * max(1.0, np.abs(want).max()), lvl


@pytest.mark.parametrize("spec", SPECS, ids=["2d", "3d"])
def test_restriction_of_linear_field(oracle_lib, spec):
    nc, dim = spec["n_cell"], spec["dim"]
    ot = oracle_tree(spec)
    ot.add_vars(1, 0)
    _fill(ot, 3, nc, dim, _lin)
    before = {l: ot.get_level(l, 3, nc).copy() for l in range(ot.min_lvl, ot.highest_lvl + 1)}
    ot.restrict_tree(3)
    for lvl in range(ot.min_lvl, ot.highest_lvl):
        got = ot.get_level(lvl, 3, nc)
        assert np.abs(got - before[lvl]).max() <= 1e-12


@pytest.mark.parametrize("spec", SPECS, ids=["2d", "3d"])
@pytest.mark.parametrize("rb", [2, 3], ids=["interp", "interp_lim"])
def test_interp_ghosts_of_linear_field(oracle_lib, spec, rb):
    """a$D_gc_interp reproduces a linear field in the refinement-boundary
    ghost cells (and the limiter does not act on a positive linear field)."""
    nc, dim = spec["n_cell"], spec["dim"]
    ot = oracle_tree(spec)
    ot.add_vars(1, 0)
    pos = lambda r: 5.0 + _lin(r)  # noqa: E731
    _fill(ot, 3, nc, dim, pos)
    ot.gc_tree_var(3, rb, -2)
    b = ot.boxes()
    checked = 0
    for lvl in range(2, ot.highest_lvl + 1):
        ids, _, _ = ot.level(lvl)
        want = pos(_centres(ot, lvl, nc, dim))
        got = ot.get_level(lvl, 3, nc)
        for n, i in enumerate(ids):
            for fc in range(2 * dim):
                if b["neighbors"][i - 1, fc] != 0:
                    continue
                d, hi = fc // 2, fc % 2
                # tangential end cells can read the coarse neighbour's own
                # ghost cells (physical-boundary values): left out
                idx = [slice(2, nc)] * dim
                idx[dim - 1 - d] = nc + 1 if hi else 0
                sl = (n,) + tuple(idx)
                assert np.abs(got[sl] - want[sl]).max() <= 1e-12
                checked += 1
    assert checked > 0


def test_vtk_structure(oracle_lib, tmp_path):
    spec = W.c1_poisson_2d()
    ot = oracle_tree(spec)
    ot.add_vars(1, 1)
    _fill(ot, 3, 8, 2, _lin)
    path = str(tmp_path / "t.vtu")
    ot.write_vtk(path, [3], ["u"], [0], ["flux"], n_cycle=3, time=0.5)
    data = open(path, "rb").read()
    head, raw = data.split(b'<AppendedData encoding="raw">\n_', 1)
    text = head.decode()
    npts = int(re.search(r'NumberOfPoints="(\d+)"', text).group(1))
    ncell = int(re.search(r'NumberOfCells="(\d+)"', text).group(1))
    leaves = sum(len(ot.level(l)[1]) for l in range(1, ot.highest_lvl + 1))
    assert ncell == leaves * 64 and npts == leaves * 81
    offs = [int(x) for x in re.findall(r'offset="(\d+)"', text)]
    sizes = [12 * npts, 16 * ncell, 4 * ncell, 4 * ncell, 8 * ncell, 8 * ncell, 8 * ncell]
    assert len(offs) == len(sizes)
    for o, n in zip(offs, sizes):
        assert struct.unpack("<i", raw[o:o + 4])[0] == n
    # the first cell array is u on the leaves, level by level
    o = offs[4]
    u = np.frombuffer(raw[o + 4:o + 4 + 8 * ncell], dtype="<f8")
    want = np.concatenate([_interior(ot, l, 3, 8, 2)[np.isin(ot.level(l)[0], ot.level(l)[1])].ravel()
                           for l in range(1, ot.highest_lvl + 1)])
    assert np.array_equal(u, want)
    assert data.endswith(b"\n  </AppendedData>\n</VTKFile>\n")
