"""ctypes wrapper of the CPU oracle (oracle/afivo_oracle.cpp).

Test infrastructure only: tests/, __graft_entry__.smoke() and the CPU legs of
bench.py import this module, to check the GPU results and as the timed CPU baseline. The
afivo_gb300 product never imports it.

The oracle restates the Afivo reference's tree build (src/m_aX_core.f90,
src/m_morton.f90) and FAS multigrid (src/m_aX_mg.f90, m_aX_gc.f90,
m_aX_prolong.f90, m_aX_restrict.f90, m_aX_utils.f90). Parity is unpinned by
reference outputs (no Fortran compiler, no golden vectors in the reference);
see afivo_oracle.cpp for what pins it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libafivo_oracle.so")

I_PHI, I_RHS, I_TMP = 0, 1, 2
REF_UNIFORM, REF_GAUSS, REF_RANDOM, REF_RANDOM_RM = 0, 1, 2, 3
BC_DIRICHLET_ZERO, BC_NEUMANN_ZERO, BC_DIRICHLET_GAUSS, BC_TABLE = 0, 1, 2, 3

_lib = None


def build():
    """Compile the oracle with its Makefile (g++ -O2 -fopenmp -ffp-contract=off)."""
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO):
            build()
        L = ctypes.CDLL(_SO)
        P = ctypes.c_void_p
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_tree_new.restype = P
        L.orc_tree_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ip, ip]
        L.orc_tree_free.argtypes = [P]
        L.orc_adjust_refinement.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_ulonglong, ctypes.c_int,
                                            ctypes.c_int, dp, ip, ip]
        for f in ("orc_min_lvl", "orc_highest_lvl", "orc_highest_id"):
            getattr(L, f).argtypes = [P]
        L.orc_export_boxes.argtypes = [P, ip, ip, ip, ip, ip, ip, dp, dp, ip]
        L.orc_level_sizes.argtypes = [P, ctypes.c_int, ip]
        L.orc_level_lists.argtypes = [P, ctypes.c_int, ip, ip, ip]
        L.orc_get_level_cc.argtypes = [P, ctypes.c_int, ctypes.c_int, dp]
        L.orc_set_level_cc.argtypes = [P, ctypes.c_int, ctypes.c_int, dp]
        L.orc_fill_gauss.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        L.orc_mg_init.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, dp]
        L.orc_zero_var.argtypes = [P, ctypes.c_int]
        L.orc_mg_set_bc_table.argtypes = [P, ctypes.c_int, ip, ip, ip, dp]
        L.orc_vcycle.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_fmg.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_gsrb_level.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_fill_gc_level.argtypes = [P, ctypes.c_int]
        L.orc_update_coarse.argtypes = [P, ctypes.c_int]
        L.orc_correct_children.argtypes = [P, ctypes.c_int]
        L.orc_gc_tree.argtypes = [P]
        L.orc_residual_all.argtypes = [P]
        for f in ("orc_tree_max_cc", "orc_tree_min_cc", "orc_leaf_mean"):
            getattr(L, f).argtypes = [P, ctypes.c_int]
            getattr(L, f).restype = ctypes.c_double
        L.orc_morton_from_ix.argtypes = [ctypes.c_int, ip]
        L.orc_morton_from_ix.restype = ctypes.c_ulonglong
        L.orc_morton_to_ix.argtypes = [ctypes.c_int, ctypes.c_ulonglong, ip]
        L.orc_ix_to_ichild.argtypes = [ctypes.c_int, ip]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_add_vars.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_mg_set_operator.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_mg_set_operator.restype = ctypes.c_int
        L.orc_set_coord.argtypes = [P, ctypes.c_int]
        L.orc_set_coord.restype = ctypes.c_int
        L.orc_fc_count.argtypes = [P]
        L.orc_fc_count.restype = ctypes.c_longlong
        L.orc_get_fc.argtypes = [P, ctypes.c_int, dp]
        L.orc_set_fc.argtypes = [P, ctypes.c_int, dp]
        L.orc_prolong_from_level.argtypes = [P] + [ctypes.c_int] * 5
        L.orc_restrict_tree.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_gc_tree_var.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_gc2_level.argtypes = [P, ctypes.c_int, ctypes.c_int, dp]
        L.orc_consistent_fluxes.argtypes = [P, ctypes.c_int, ip]
        cpp = ctypes.POINTER(ctypes.c_char_p)
        L.orc_write_vtk.argtypes = [P, ctypes.c_char_p, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_int, ip, cpp, ctypes.c_int, ip, cpp]
        _lib = L
    return _lib


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return lib().orc_max_threads()


class OracleTree:
    """One reference tree (a$D_t) with three cell variables: phi, rhs, tmp."""

    def __init__(self, dim, n_cell, dr, ix_list, nb_list, r_min=None, lvl_limit=30,
                 coarsen_to=-1):
        self.dim = dim
        L = lib()
        ix = np.ascontiguousarray(np.asarray(ix_list, dtype=np.int32).reshape(-1, dim))
        nb = np.ascontiguousarray(np.asarray(nb_list, dtype=np.int32).reshape(-1, 2 * dim))
        rm = np.zeros(dim) if r_min is None else np.asarray(r_min, dtype=np.float64)
        self.h = L.orc_tree_new(dim, n_cell, dr, _dp(rm), lvl_limit, coarsen_to, ix.shape[0],
                                _ip(ix), _ip(nb))
        if not self.h:
            raise ValueError("orc_tree_new failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_tree_free(self.h)
            self.h = None

    # tree build ------------------------------------------------------------
    def adjust_refinement(self, kind, lvl_max, thr=0.0, prob=0.0, seed=0, gauss=None, lpl=False):
        g = np.zeros(1) if gauss is None else np.ascontiguousarray(gauss, dtype=np.float64)
        n_g = 0 if gauss is None else g.size // (2 + self.dim)
        na = ctypes.c_int(0)
        nr = ctypes.c_int(0)
        rc = lib().orc_adjust_refinement(self.h, kind, lvl_max, thr, prob, seed, int(lpl), n_g,
                                         _dp(g), ctypes.byref(na), ctypes.byref(nr))
        if rc != 0:
            raise RuntimeError(f"orc_adjust_refinement failed: {rc}")
        return na.value, nr.value

    def refine_until_done(self, kind, lvl_max, thr=0.0, prob=0.0, seed=0, gauss=None,
                          lpl=False, max_passes=100):
        for _ in range(max_passes):
            na, _ = self.adjust_refinement(kind, lvl_max, thr, prob, seed, gauss, lpl)
            if na == 0:
                break

    @property
    def min_lvl(self):
        return lib().orc_min_lvl(self.h)

    @property
    def highest_lvl(self):
        return lib().orc_highest_lvl(self.h)

    @property
    def highest_id(self):
        return lib().orc_highest_id(self.h)

    def boxes(self):
        """Per-id topology arrays (row id-1)."""
        n, D = self.highest_id, self.dim
        out = dict(lvl=np.zeros(n, np.int32), ix=np.zeros((n, D), np.int32),
                   parent=np.zeros(n, np.int32), children=np.zeros((n, 2 ** D), np.int32),
                   neighbors=np.zeros((n, 2 * D), np.int32), n_cell=np.zeros(n, np.int32),
                   dr=np.zeros(n), r_min=np.zeros((n, D)), in_use=np.zeros(n, np.int32))
        lib().orc_export_boxes(self.h, _ip(out["lvl"]), _ip(out["ix"]), _ip(out["parent"]),
                               _ip(out["children"]), _ip(out["neighbors"]), _ip(out["n_cell"]),
                               _dp(out["dr"]), _dp(out["r_min"]), _ip(out["in_use"]))
        return out

    def level(self, lvl):
        sz = np.zeros(3, np.int32)
        lib().orc_level_sizes(self.h, lvl, _ip(sz))
        ids, lv, pa = (np.zeros(max(int(s), 1), np.int32) for s in sz)
        lib().orc_level_lists(self.h, lvl, _ip(ids), _ip(lv), _ip(pa))
        return ids[:sz[0]].copy(), lv[:sz[1]].copy(), pa[:sz[2]].copy()

    def n_cell_at(self, lvl, n_cell):
        return n_cell if lvl >= 1 else n_cell >> (1 - lvl)

    # data --------------------------------------------------------------------
    def get_level(self, lvl, iv, n_cell):
        ids, _, _ = self.level(lvl)
        nc = self.n_cell_at(lvl, n_cell)
        buf = np.zeros(len(ids) * (nc + 2) ** self.dim)
        if len(ids):
            lib().orc_get_level_cc(self.h, lvl, iv, _dp(buf))
        return buf.reshape((len(ids),) + (nc + 2,) * self.dim)

    def set_level(self, lvl, iv, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        lib().orc_set_level_cc(self.h, lvl, iv, _dp(a))

    def fill_gauss(self, iv, gauss, lpl=False):
        g = np.ascontiguousarray(gauss, dtype=np.float64)
        lib().orc_fill_gauss(self.h, iv, int(lpl), g.size // (2 + self.dim), _dp(g))

    # multigrid ---------------------------------------------------------------
    def mg_init(self, n_down=-1, n_up=-1, n_base=-1, bc_kind=BC_DIRICHLET_ZERO, bc_gauss=None):
        g = np.zeros(1) if bc_gauss is None else np.ascontiguousarray(bc_gauss, dtype=np.float64)
        n_g = 0 if bc_gauss is None else g.size // (2 + self.dim)
        lib().orc_mg_init(self.h, n_down, n_up, n_base, bc_kind, n_g, _dp(g))

    def set_bc_table(self, ids, faces, types, values):
        """Per-face boundary records (kind BC_TABLE): face i of box ids[i]
        (0-based face), type types[i] (-1 Dirichlet, -2 Neumann), values of all
        faces concatenated (first tangential index fastest)."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        types = np.ascontiguousarray(types, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64)
        lib().orc_mg_set_bc_table(self.h, ids.size, _ip(ids), _ip(faces), _ip(types), _dp(v))

    def vcycle(self, highest_lvl=None, set_residual=True):
        hl = self.highest_lvl if highest_lvl is None else highest_lvl
        lib().orc_vcycle(self.h, hl, int(set_residual))

    def fmg(self, set_residual=True, have_guess=False):
        lib().orc_fmg(self.h, int(set_residual), int(have_guess))

    def gsrb_level(self, lvl, n_cycle):
        lib().orc_gsrb_level(self.h, lvl, n_cycle)

    def fill_gc_level(self, lvl):
        lib().orc_fill_gc_level(self.h, lvl)

    def update_coarse(self, lvl):
        lib().orc_update_coarse(self.h, lvl)

    def correct_children(self, lvl_parent):
        lib().orc_correct_children(self.h, lvl_parent)

    def gc_tree(self):
        lib().orc_gc_tree(self.h)

    def residual_all(self):
        lib().orc_residual_all(self.h)

    def zero(self, iv):
        lib().orc_zero_var(self.h, iv)

    def max_abs_residual(self):
        L = lib()
        return max(abs(L.orc_tree_max_cc(self.h, I_TMP)), abs(L.orc_tree_min_cc(self.h, I_TMP)))

    def max_abs(self, iv):
        L = lib()
        return max(abs(L.orc_tree_max_cc(self.h, iv)), abs(L.orc_tree_min_cc(self.h, iv)))

    def leaf_mean(self, iv):
        return lib().orc_leaf_mean(self.h, iv)

    def set_operator(self, op, i_eps=-1, i_lsf=-1, i_bval=-1):
        """mg%box_op / box_gsrb / box_corr / box_rstr: 0 lpl, 1 lpld, 2 auto,
        3 clpl, 4 clpld, 5 lpllsf, with mg%i_eps, mg%i_lsf, mg%i_bval.
        Returns False when a box would take two auto tags."""
        return lib().orc_mg_set_operator(self.h, op, i_eps, i_lsf, i_bval) == 0

    def set_coord(self, coord):
        """a$D_init's coord: 0 Cartesian, 1 cylindrical (2-D; before refinement)."""
        if lib().orc_set_coord(self.h, coord) != 0:
            raise ValueError("cylindrical coordinates need a 2-D tree")

    # general ghost cells, transfers and output ---------------------------------
    def add_vars(self, n_cc=0, n_fc=0):
        lib().orc_add_vars(self.h, n_cc, n_fc)

    def get_fc(self, ifc):
        out = np.zeros(lib().orc_fc_count(self.h))
        lib().orc_get_fc(self.h, ifc, _dp(out))
        return out

    def set_fc(self, ifc, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        lib().orc_set_fc(self.h, ifc, _dp(a))

    def prolong(self, lvl_parent, iv, iv_to=None, order=2, add=False):
        lib().orc_prolong_from_level(self.h, lvl_parent, iv, iv if iv_to is None else iv_to,
                                     order, int(add))

    def restrict_tree(self, iv, iv_to=None):
        lib().orc_restrict_tree(self.h, iv, iv if iv_to is None else iv_to)

    def gc_tree_var(self, iv, rb=0, bc=0):
        lib().orc_gc_tree_var(self.h, iv, rb, bc)

    def gc2_level(self, lvl, iv, n_cell):
        n = len(self.level(lvl)[0]) * 2 * self.dim * n_cell ** (self.dim - 1)
        out = np.zeros(n)
        lib().orc_gc2_level(self.h, lvl, iv, _dp(out))
        return out

    def consistent_fluxes(self, f_ixs):
        a = np.ascontiguousarray(f_ixs, dtype=np.int32)
        lib().orc_consistent_fluxes(self.h, a.size, _ip(a))

    def write_vtk(self, path, ixs_cc, cc_names, ixs_fc=(), fc_names=(), n_cycle=0, time=0.0):
        icc = np.ascontiguousarray(ixs_cc, dtype=np.int32)
        ifc = np.ascontiguousarray(ixs_fc, dtype=np.int32)
        cn = (ctypes.c_char_p * max(1, len(cc_names)))(*[n.encode() for n in cc_names])
        fn = (ctypes.c_char_p * max(1, len(fc_names)))(*[n.encode() for n in fc_names])
        rc = lib().orc_write_vtk(self.h, path.encode(), n_cycle, float(time), icc.size, _ip(icc),
                                 cn, ifc.size, _ip(ifc), fn)
        if rc != 0:
            raise OSError(f"cannot write {path}")


def morton_from_ix(ix):
    a = np.ascontiguousarray(ix, dtype=np.int32)
    return lib().orc_morton_from_ix(a.size, _ip(a))


def morton_to_ix(dim, m):
    a = np.zeros(dim, np.int32)
    lib().orc_morton_to_ix(dim, m, _ip(a))
    return a
