"""afivo_gb300: GB300 (sm_103a) FAS multigrid for Poisson problems on
quadtree/octree block grids, behind the C ABI of include/afivo_gb300.h.

This module is the Python host side of that ABI. Its names follow the Afivo
reference's Fortran API for this path:

=========================  ===============================================
here                       reference (src/...)
=========================  ===============================================
``a2_init`` / ``a3_init``  ``a$D_init`` (m_aX_core.f90:24-131)
``Tree.set_base``          ``a$D_set_base`` (m_aX_core.f90:152-235)
``Tree.adjust_refinement`` ``a$D_adjust_refinement`` (m_aX_core.f90:452-541)
``Forest``                 the device copy of one or more ``a$D_t`` trees
``mg2_init_mg``            ``mg$D_init_mg`` (m_aX_mg.f90:130-154)
``mg2_fas_vcycle``         ``mg$D_fas_vcycle`` (m_aX_mg.f90:208-255)
``mg2_fas_fmg``            ``mg$D_fas_fmg`` (m_aX_mg.f90:164-203)
``a2_gc_tree``             ``a$D_gc_tree`` (m_aX_gc.f90:28-46)
``a2_tree_max_abs_cc``     ``a$D_tree_max_cc``/``min_cc`` (m_aX_utils.f90:468-571)
=========================  ===============================================

Errors: every C call returns a status; a negative status raises AfivoError
with the library's message (the reference calls ``stop`` instead).
The CUDA library must have been built (``afivo_gb300.build.build()``); there is
no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libafivo_gb300.so")

AFV_OK = 0
AFV_ERR_INVALID, AFV_ERR_CUDA, AFV_ERR_NOMEM = -1, -2, -3
AFV_ERR_UNSUPPORTED, AFV_ERR_TIMEOUT, AFV_ERR_STATE, AFV_ERR_BUDGET = -4, -5, -6, -7
AFV_ERR_DIVERGED, AFV_ERR_NOT_CONVERGED = -8, -9
AFV_RM_REF, AFV_KEEP_REF, AFV_DO_REF = -1, 0, 1
AFV_PHI, AFV_RHS, AFV_TMP = 0, 1, 2
AFV_BC_DIRICHLET, AFV_BC_NEUMANN = -1, -2
AFV_REF_UNIFORM, AFV_REF_SOURCE, AFV_REF_RANDOM, AFV_REF_RANDOM_RM = 0, 1, 2, 3
AFV_PREC_FP64, AFV_PREC_MIXED = 0, 1
AFV_OPT_SWEEP_KERNEL, AFV_OPT_GRAPHS, AFV_OPT_RESTRICT_KERNEL, AFV_OPT_SMALL_SWEEPS = 0, 1, 2, 3
AFV_OPT_PROFILE_LEAD_US, AFV_OPT_DEFECT_KERNEL, AFV_OPT_COARSE_END = 4, 5, 6
AFV_OPT_WAIT_LIMIT_US, AFV_OPT_DIRECT_BOXES, AFV_OPT_ZERO_COPY, AFV_OPT_DEFECT_CELLS = 7, 8, 9, 10
OPTION_NAMES = ("sweep_kernel", "graphs", "restrict_kernel", "small_sweeps", "profile_lead_us",
                "defect_kernel", "coarse_end", "wait_limit_us", "direct_boxes",
                "zero_copy", "defect_cells")  # AFV_OPT_* in order
AFV_RB_MG, AFV_RB_PROLONG0, AFV_RB_INTERP, AFV_RB_INTERP_LIM = 0, 1, 2, 3
AFV_BCM_TABLE, AFV_BCM_DIRICHLET_ZERO, AFV_BCM_NEUMANN_ZERO = 0, -1, -2
AFV_OP_LPL, AFV_OP_LPLD, AFV_OP_AUTO = 0, 1, 2
AFV_OP_CLPL, AFV_OP_CLPLD, AFV_OP_LPLLSF = 3, 4, 5
AFV_COORD_XYZ, AFV_COORD_CYL = 0, 1
KERNEL_KINDS = ("sweep", "fill", "restrict", "coarse_rhs", "correct", "residual", "defect",
                "accumulate", "coarse_end")

# Refinement flags under the reference's names (src/m_aX_t.f90:17-24)
a5_rm_ref, a5_keep_ref, a5_do_ref = AFV_RM_REF, AFV_KEEP_REF, AFV_DO_REF
a5_bc_dirichlet, a5_bc_neumann = AFV_BC_DIRICHLET, AFV_BC_NEUMANN


class AfivoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"afivo_gb300 error {code}: {msg}")
        self.code = code


class BoxView(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int), ("lvl", ctypes.c_int), ("n_cell", ctypes.c_int),
                ("dim", ctypes.c_int), ("ix", ctypes.c_int * 3), ("dr", ctypes.c_double),
                ("r_min", ctypes.c_double * 3), ("pass_", ctypes.c_int)]


REF_FN = ctypes.CFUNCTYPE(None, ctypes.POINTER(BoxView), ctypes.POINTER(ctypes.c_int),
                          ctypes.c_void_p)


class RefCrit(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("lvl_max", ctypes.c_int), ("thr", ctypes.c_double),
                ("prob", ctypes.c_double), ("seed", ctypes.c_ulonglong),
                ("src_lpl", ctypes.c_int), ("n_gauss", ctypes.c_int),
                ("gauss", ctypes.POINTER(ctypes.c_double))]


class MgOpts(ctypes.Structure):
    """The mg$D_t options of src/m_aX_mg.f90:20-52 (cycle counts)."""
    _fields_ = [("n_cycle_down", ctypes.c_int), ("n_cycle_up", ctypes.c_int),
                ("n_cycle_base", ctypes.c_int)]

    def __init__(self, n_cycle_down=-1, n_cycle_up=-1, n_cycle_base=-1):
        super().__init__(n_cycle_down, n_cycle_up, n_cycle_base)


class ForestOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("mixed_buffers", ctypes.c_int)]


_lib = None


def lib():
    """Load the in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with afivo_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        Dd = ctypes.c_double
        ip = ctypes.POINTER(I)
        dp = ctypes.POINTER(Dd)
        llp = ctypes.POINTER(ctypes.c_longlong)
        LL = ctypes.c_longlong
        sig = {
            "afv_last_error": (ctypes.c_char_p, []),
            "afv_version": (I, []),
            "afv_tree_create": (I, [I, I, Dd, dp, I, I, Dd, ctypes.POINTER(P)]),
            "afv_tree_set_base": (I, [P, I, ip, ip]),
            "afv_tree_set_coord": (I, [P, I]),
            "afv_tree_adjust_refinement": (I, [P, REF_FN, P, ip, ip]),
            "afv_tree_adjust_builtin": (I, [P, ctypes.POINTER(RefCrit), ip, ip]),
            "afv_tree_refine_builtin": (I, [P, ctypes.POINTER(RefCrit), I, ip]),
            "afv_tree_destroy": (None, [P]),
            "afv_tree_get_info": (I, [P, ip]),
            "afv_tree_export": (I, [P, ip, ip, ip, ip, ip, ip, dp, dp, ip]),
            "afv_tree_level": (I, [P, I, ip, ip, ip, ip]),
            "afv_forest_create": (I, [I, ctypes.POINTER(P), ctypes.POINTER(ForestOpts),
                                      ctypes.POINTER(P)]),
            "afv_forest_destroy": (None, [P]),
            "afv_forest_get_info": (I, [P, llp]),
            "afv_forest_set_var": (I, [P, I, I, dp, I]),
            "afv_forest_get_var": (I, [P, I, I, dp, I]),
            "afv_forest_set_source": (I, [P, I, I, I, dp]),
            "afv_forest_set_bc_faces": (I, [P, I, LL, ip, LL, dp]),
            "afv_forest_set_bc": (I, [P, I, I, I, I, dp]),
            "afv_forest_zero": (I, [P, I]),
            "afv_forest_sync": (I, [P]),
            "afv_forest_get_stream": (I, [P, ctypes.POINTER(P)]),
            "afv_mg_init": (I, [ctypes.POINTER(MgOpts)]),
            "afv_mg_fas_vcycle": (I, [P, ctypes.POINTER(MgOpts), I, I]),
            "afv_mg_fas_fmg": (I, [P, ctypes.POINTER(MgOpts), I, I]),
            "afv_gc_tree": (I, [P]),
            "afv_tree_max_abs_cc": (I, [P, I, I, dp]),
            "afv_forest_profile_entries": (I, [P, LL, ip, ip, dp, dp, ip, llp]),
            "afv_forest_set_option": (I, [P, I, I]),
            "afv_forest_set_source_device": (I, [P, I, I, I, dp]),
            "afv_forest_autotune": (I, [P, ip, ctypes.POINTER(ctypes.c_float)]),
            "afv_forest_autotune_all": (I, [P, ip, ctypes.POINTER(ctypes.c_float)]),
            "afv_forest_autotune_defect": (I, [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)]),
            "afv_forest_get_option": (I, [P, I, ip]),
            "afv_tree_max_abs_cc_noalloc": (I, [P, I, I, dp]),
            "afv_mg_solve": (I, [P, ctypes.POINTER(MgOpts), I, Dd, I, ip, dp]),
            "afv_mg_solve_trees": (I, [P, ctypes.POINTER(MgOpts), I, Dd, I, ip, ip, dp]),
            "afv_forest_zero_tree": (I, [P, I, I]),
            "afv_mg_gsrb_level": (I, [P, I, I]),
            "afv_fill_gc_level": (I, [P, I]),
            "afv_mg_update_coarse": (I, [P, I]),
            "afv_mg_correct_children": (I, [P, I]),
            "afv_mg_residual_all": (I, [P]),
            "afv_forest_profile": (I, [P, I]),
            "afv_forest_profile_read": (I, [P, I, llp, dp, dp]),
            "afv_forest_add_vars": (I, [P, I, I]),
            "afv_dtree_create": (I, [P, I, ctypes.POINTER(P)]),
            "afv_dtree_destroy": (None, [P]),
            "afv_dtree_adjust_builtin": (I, [P, ctypes.POINTER(RefCrit), ip, ip]),
            "afv_dtree_refine_builtin": (I, [P, ctypes.POINTER(RefCrit), I, ip]),
            "afv_dtree_download": (I, [P, P]),
            "afv_dtree_get_info": (I, [P, ip]),
            "afv_mg_set_operator": (I, [P, I, I]),
            "afv_mg_set_operator_lsf": (I, [P, I, I, I, I]),
            "afv_forest_set_fc": (I, [P, I, I, dp, LL]),
            "afv_forest_get_fc": (I, [P, I, I, dp, LL]),
            "afv_prolong_from_level": (I, [P, I, I, I, I, I]),
            "afv_restrict_tree": (I, [P, I, I]),
            "afv_gc_tree_var": (I, [P, I, I, I]),
            "afv_gc2_level": (I, [P, I, I, I, dp, LL]),
            "afv_consistent_fluxes": (I, [P, I, ip]),
            "afv_write_vtk": (I, [P, I, ctypes.c_char_p, I, Dd, I, ip,
                                  ctypes.POINTER(ctypes.c_char_p), I, ip,
                                  ctypes.POINTER(ctypes.c_char_p), ctypes.c_char_p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != AFV_OK:
        raise AfivoError(rc, lib().afv_last_error().decode())
    return rc


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _crit(kind, lvl_max, thr=0.0, prob=0.0, seed=0, gauss=None, lpl=False):
    g = None if gauss is None else np.ascontiguousarray(gauss, dtype=np.float64)
    c = RefCrit(kind, lvl_max, thr, prob, seed, int(lpl), 0, None)
    if g is not None:
        c.gauss = _dp(g)
    return c, g


class Tree:
    """Host tree of NxN(xN) boxes, the reference's a$D_t (src/m_aX_t.f90:189-207)."""

    def __init__(self, dim, n_cell, dr, r_min=None, lvl_limit=30, coarsen_to=-1,
                 mem_limit_gb=64.0):
        self.dim = dim
        rm = np.zeros(dim) if r_min is None else np.ascontiguousarray(r_min, dtype=np.float64)
        h = ctypes.c_void_p()
        _check(lib().afv_tree_create(dim, n_cell, float(dr), _dp(rm), lvl_limit, coarsen_to,
                                     float(mem_limit_gb), ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.afv_tree_destroy(self.h)
            self.h = None

    def set_coord(self, coord):
        """a$D_init's coord (AFV_COORD_XYZ or AFV_COORD_CYL); before set_base."""
        _check(lib().afv_tree_set_coord(self.h, coord))
        return self

    def set_base(self, ix_list, nb_list):
        ix = np.ascontiguousarray(np.asarray(ix_list, dtype=np.int32).reshape(-1, self.dim))
        nb = np.ascontiguousarray(np.asarray(nb_list, dtype=np.int32).reshape(-1, 2 * self.dim))
        _check(lib().afv_tree_set_base(self.h, ix.shape[0], _ip(ix), _ip(nb)))
        return self

    def adjust_refinement(self, ref_fn):
        """One a$D_adjust_refinement pass with a Python ref_subr(box, flag) -> flag."""
        def cb(view_p, flag_p, _user):
            v = view_p.contents
            flag_p[0] = int(ref_fn(v, flag_p[0]))
        c = REF_FN(cb)
        na, nr = ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().afv_tree_adjust_refinement(self.h, c, None, ctypes.byref(na), ctypes.byref(nr)))
        return na.value, nr.value

    def adjust_builtin(self, kind, lvl_max, thr=0.0, prob=0.0, seed=0, gauss=None, lpl=False):
        c, _keep = _crit(kind, lvl_max, thr, prob, seed, gauss, lpl)
        if gauss is not None:
            c.n_gauss = len(gauss) // (2 + self.dim)
        na, nr = ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().afv_tree_adjust_builtin(self.h, ctypes.byref(c), ctypes.byref(na),
                                             ctypes.byref(nr)))
        return na.value, nr.value

    def refine_builtin(self, kind, lvl_max, thr=0.0, prob=0.0, seed=0, gauss=None, lpl=False,
                       max_passes=100):
        c, _keep = _crit(kind, lvl_max, thr, prob, seed, gauss, lpl)
        if gauss is not None:
            c.n_gauss = len(gauss) // (2 + self.dim)
        n = ctypes.c_int(0)
        _check(lib().afv_tree_refine_builtin(self.h, ctypes.byref(c), max_passes, ctypes.byref(n)))
        return n.value

    def info(self):
        out = np.zeros(8, np.int32)
        _check(lib().afv_tree_get_info(self.h, _ip(out)))
        keys = ("dim", "n_cell", "min_lvl", "highest_lvl", "highest_id", "n_boxes", "n_leaves",
                "lvl_limit")
        return dict(zip(keys, (int(x) for x in out)))

    @property
    def min_lvl(self):
        return self.info()["min_lvl"]

    @property
    def highest_lvl(self):
        return self.info()["highest_lvl"]

    def boxes(self):
        n, D = self.info()["highest_id"], self.dim
        out = dict(lvl=np.zeros(n, np.int32), ix=np.zeros((n, D), np.int32),
                   parent=np.zeros(n, np.int32), children=np.zeros((n, 2 ** D), np.int32),
                   neighbors=np.zeros((n, 2 * D), np.int32), n_cell=np.zeros(n, np.int32),
                   dr=np.zeros(n), r_min=np.zeros((n, D)), in_use=np.zeros(n, np.int32))
        _check(lib().afv_tree_export(self.h, _ip(out["lvl"]), _ip(out["ix"]), _ip(out["parent"]),
                                     _ip(out["children"]), _ip(out["neighbors"]),
                                     _ip(out["n_cell"]), _dp(out["dr"]), _dp(out["r_min"]),
                                     _ip(out["in_use"])))
        return out

    def level(self, lvl):
        sz = np.zeros(3, np.int32)
        _check(lib().afv_tree_level(self.h, lvl, _ip(sz), None, None, None))
        ids, lv, pa = (np.zeros(max(int(s), 1), np.int32) for s in sz)
        _check(lib().afv_tree_level(self.h, lvl, _ip(sz), _ip(ids), _ip(lv), _ip(pa)))
        return ids[:sz[0]].copy(), lv[:sz[1]].copy(), pa[:sz[2]].copy()

    def bc_faces(self):
        """Physical-boundary faces in the order afv_forest_set_bc_faces takes
        them: list of (id, face, centres), centres an (nc^(D-1), D) array of the
        face-cell centres (first tangential index fastest)."""
        b = self.boxes()
        D = self.dim
        out = []
        for lvl in range(self.min_lvl, self.highest_lvl + 1):
            ids, _, _ = self.level(lvl)
            for i in ids:
                k = int(i) - 1
                nc, dr, rmin = int(b["n_cell"][k]), float(b["dr"][k]), b["r_min"][k]
                for f in range(2 * D):
                    if b["neighbors"][k, f] >= 0:
                        continue
                    dim, low = f // 2, f % 2 == 0
                    tang = [e for e in range(D) if e != dim]
                    idx = np.arange(1, nc + 1, dtype=np.float64)
                    grids = np.meshgrid(*([idx] * (D - 1)), indexing="xy") if D == 3 else [idx]
                    cen = np.empty((nc ** (D - 1), D))
                    cen[:, dim] = rmin[dim] + ((0.5 if low else nc + 0.5) - 0.5) * dr
                    for e, g in zip(tang, grids):
                        cen[:, e] = rmin[e] + (g.ravel() - 0.5) * dr
                    out.append((int(i), f, cen))
        return out

    def n_cell_at(self, lvl):
        nc = self.info()["n_cell"]
        return nc if lvl >= 1 else nc >> (1 - lvl)

    def leaf_cells(self):
        i = self.info()
        return i["n_leaves"] * i["n_cell"] ** self.dim


class DeviceTree:
    """A copy of a host tree in device memory, refined there
    (afv_dtree_*): a$D_adjust_refinement with the built-in criteria."""

    def __init__(self, tree, device=0):
        self.dim = tree.dim
        h = ctypes.c_void_p()
        _check(lib().afv_dtree_create(tree.h, device, ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.afv_dtree_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def adjust_builtin(self, kind, lvl_max, thr=0.0, prob=0.0, seed=0, gauss=None, lpl=False):
        c, _keep = _crit(kind, lvl_max, thr, prob, seed, gauss, lpl)
        if gauss is not None:
            c.n_gauss = len(gauss) // (2 + self.dim)
        na, nr = ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().afv_dtree_adjust_builtin(self.h, ctypes.byref(c), ctypes.byref(na),
                                              ctypes.byref(nr)))
        return na.value, nr.value

    def refine_builtin(self, kind, lvl_max, thr=0.0, prob=0.0, seed=0, gauss=None, lpl=False,
                       max_passes=100):
        c, _keep = _crit(kind, lvl_max, thr, prob, seed, gauss, lpl)
        if gauss is not None:
            c.n_gauss = len(gauss) // (2 + self.dim)
        n = ctypes.c_int(0)
        _check(lib().afv_dtree_refine_builtin(self.h, ctypes.byref(c), max_passes, ctypes.byref(n)))
        return n.value

    def download(self, tree):
        """Copy the device tree's state into host tree `tree`."""
        _check(lib().afv_dtree_download(self.h, tree.h))
        return tree

    def info(self):
        out = np.zeros(5, np.int32)
        _check(lib().afv_dtree_get_info(self.h, _ip(out)))
        return dict(zip(("highest_lvl", "highest_id", "passes", "n_boxes", "n_leaves"),
                        (int(x) for x in out)))


def a2_init(n_cell, dr, r_min=None, lvl_limit=30, coarsen_to=-1, mem_limit_gb=64.0):
    """a2_init (src/m_aX_core.f90:24-131) for phi, rhs and tmp."""
    return Tree(2, n_cell, dr, r_min, lvl_limit, coarsen_to, mem_limit_gb)


def a3_init(n_cell, dr, r_min=None, lvl_limit=30, coarsen_to=-1, mem_limit_gb=64.0):
    """a3_init (src/m_aX_core.f90:24-131) for phi, rhs and tmp."""
    return Tree(3, n_cell, dr, r_min, lvl_limit, coarsen_to, mem_limit_gb)


class Forest:
    """One or more trees resident on a GPU, swept together by every launch."""

    def __init__(self, trees, device=0, mixed=False):
        self.trees = list(trees)
        self.dim = self.trees[0].dim
        arr = (ctypes.c_void_p * len(self.trees))(*[t.h for t in self.trees])
        opts = ForestOpts(device, int(mixed))
        h = ctypes.c_void_p()
        _check(lib().afv_forest_create(len(self.trees), arr, ctypes.byref(opts), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.afv_forest_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def info(self):
        out = np.zeros(8, np.int64)
        _check(lib().afv_forest_get_info(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))))
        keys = ("n_trees", "dim", "n_cell", "min_lvl", "max_lvl", "n_boxes", "leaf_cells", "bytes")
        return dict(zip(keys, (int(x) for x in out)))

    def _n_values(self, tree, interior):
        """Values of a tree's variable in the host layout (the forest's boxes
        are fixed when it is created, so the count is kept)."""
        key = (tree, bool(interior))
        cache = self.__dict__.setdefault("_n_values_cache", {})
        if key not in cache:
            t = self.trees[tree]
            n = 0
            for lvl in range(t.min_lvl, t.highest_lvl + 1):
                ids, _, _ = t.level(lvl)
                nc = t.n_cell_at(lvl)
                n += len(ids) * ((nc if interior else nc + 2) ** self.dim)
            cache[key] = n
        return cache[key]

    def set_var(self, tree, var, values, interior_only=False):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        if a.size != self._n_values(tree, interior_only):
            raise ValueError("values do not match the tree's box layout")
        _check(lib().afv_forest_set_var(self.h, tree, var, _dp(a), int(interior_only)))

    def get_var(self, tree, var, interior_only=False, out=None):
        n = self._n_values(tree, interior_only)
        a = np.empty(n) if out is None else out
        _check(lib().afv_forest_get_var(self.h, tree, var, _dp(a), int(interior_only)))
        return a

    def set_source(self, tree, gauss, lpl=False):
        g = np.ascontiguousarray(gauss, dtype=np.float64)
        _check(lib().afv_forest_set_source(self.h, tree, int(lpl), g.size // (2 + self.dim), _dp(g)))

    def set_source_device(self, tree, gauss, lpl=False):
        """set_source evaluated on the device (may differ in the last bit)."""
        g = np.ascontiguousarray(gauss, dtype=np.float64)
        _check(lib().afv_forest_set_source_device(self.h, tree, int(lpl), g.size // (2 + self.dim),
                                                  _dp(g)))

    def set_bc_faces(self, tree, bc_types, values):
        """Sampled sides_bc hook: one AFV_BC_* per physical face and the face
        values, in the order of Tree.bc_faces()."""
        t = np.ascontiguousarray(bc_types, dtype=np.int32).ravel()
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        _check(lib().afv_forest_set_bc_faces(self.h, tree, t.size, _ip(t), v.size, _dp(v)))

    def set_bc(self, tree, bc_type=AFV_BC_DIRICHLET, gauss=None, lpl=False):
        if gauss is None:
            _check(lib().afv_forest_set_bc(self.h, tree, bc_type, 0, 0, None))
        else:
            g = np.ascontiguousarray(gauss, dtype=np.float64)
            _check(lib().afv_forest_set_bc(self.h, tree, bc_type, int(lpl),
                                           g.size // (2 + self.dim), _dp(g)))

    def zero(self, var):
        _check(lib().afv_forest_zero(self.h, var))

    def zero_tree(self, tree, var):
        _check(lib().afv_forest_zero_tree(self.h, tree, var))

    def sync(self):
        _check(lib().afv_forest_sync(self.h))

    def stream(self):
        """The cudaStream_t (as an int) that orders this forest's work."""
        s = ctypes.c_void_p()
        _check(lib().afv_forest_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def launches(self):
        return self.profile_read(-1)[0]

    def vcycle(self, mg=None, highest_lvl=None, set_residual=True):
        mg = mg or MgOpts()
        hl = self.info()["max_lvl"] if highest_lvl is None else highest_lvl
        _check(lib().afv_mg_fas_vcycle(self.h, ctypes.byref(mg), hl, int(set_residual)))

    def fmg(self, mg=None, set_residual=True, have_guess=False):
        mg = mg or MgOpts()
        _check(lib().afv_mg_fas_fmg(self.h, ctypes.byref(mg), int(set_residual), int(have_guess)))

    def gc_tree(self):
        _check(lib().afv_gc_tree(self.h))

    def max_abs(self, tree, var):
        out = ctypes.c_double(0)
        _check(lib().afv_tree_max_abs_cc(self.h, tree, var, ctypes.byref(out)))
        return out.value

    def max_abs_noalloc(self, tree, var):
        """max_abs with static device scratch: allocates nothing (forests of <= 1024 trees)."""
        out = ctypes.c_double(0)
        _check(lib().afv_tree_max_abs_cc_noalloc(self.h, tree, var, ctypes.byref(out)))
        return out.value

    def solve(self, precision=AFV_PREC_FP64, tol=1e-8, max_cycles=50, mg=None, check=True,
              mask=None):
        """Solve every tree (or the trees with a nonzero mask entry)."""
        mg = mg or MgOpts()
        n = len(self.trees)
        cyc = np.zeros(n, np.int32)
        rel = np.zeros(n)
        if mask is None:
            rc = lib().afv_mg_solve(self.h, ctypes.byref(mg), precision, float(tol), max_cycles,
                                    _ip(cyc), _dp(rel))
        else:
            m = np.ascontiguousarray(mask, dtype=np.int32)
            if m.size != n:
                raise ValueError("mask must have one entry per tree")
            rc = lib().afv_mg_solve_trees(self.h, ctypes.byref(mg), precision, float(tol),
                                          max_cycles, _ip(m), _ip(cyc), _dp(rel))
        if check and rc != AFV_OK:
            _check(rc)
        return cyc, rel, rc

    # general ghost cells, transfers and output (src/m_aX_gc.f90,
    # m_aX_prolong.f90, m_aX_restrict.f90, m_aX_core.f90, m_aX_io.f90)
    def add_vars(self, n_cc=0, n_fc=0):
        """Extra cell variables (numbered 3, 4, ...) and face variables."""
        _check(lib().afv_forest_add_vars(self.h, n_cc, n_fc))
        self.__dict__["_n_fc"] = self.__dict__.get("_n_fc", 0) + n_fc

    def set_operator(self, op, i_eps=-1, i_lsf=-1, i_bval=-1):
        """mg%box_op / box_gsrb / box_corr / box_rstr with mg%i_eps, mg%i_lsf
        and mg%i_bval (AFV_OP_*)."""
        if i_lsf < 0 and i_bval < 0:
            _check(lib().afv_mg_set_operator(self.h, op, i_eps))
        else:
            _check(lib().afv_mg_set_operator_lsf(self.h, op, i_eps, i_lsf, i_bval))

    def fc_count(self, tree):
        t = self.trees[tree]
        n = 0
        for lvl in range(t.min_lvl, t.highest_lvl + 1):
            nc = t.n_cell_at(lvl)
            n += len(t.level(lvl)[0]) * self.dim * (nc + 1) * nc ** (self.dim - 1)
        return n

    def set_fc(self, tree, ifc, values):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        _check(lib().afv_forest_set_fc(self.h, tree, ifc, _dp(a), a.size))

    def get_fc(self, tree, ifc):
        a = np.empty(self.fc_count(tree))
        _check(lib().afv_forest_get_fc(self.h, tree, ifc, _dp(a), a.size))
        return a

    def prolong(self, lvl_parent, iv, iv_to=None, order=2, add=False):
        """a$D_prolong{order}_from on every parent of lvl_parent."""
        iv_to = iv if iv_to is None else iv_to
        _check(lib().afv_prolong_from_level(self.h, lvl_parent, iv, iv_to, order, int(add)))

    def restrict_tree(self, iv, iv_to=None):
        _check(lib().afv_restrict_tree(self.h, iv, iv if iv_to is None else iv_to))

    def gc_tree_var(self, iv, rb=AFV_RB_MG, bc=AFV_BCM_TABLE):
        _check(lib().afv_gc_tree_var(self.h, iv, rb, bc))

    def gc2_level(self, tree, lvl, iv):
        t = self.trees[tree]
        nc = t.n_cell_at(lvl)
        n = len(t.level(lvl)[0]) * 2 * self.dim * nc ** (self.dim - 1)
        out = np.empty(n)
        _check(lib().afv_gc2_level(self.h, tree, lvl, iv, _dp(out), n))
        return out

    def consistent_fluxes(self, f_ixs):
        ix = np.ascontiguousarray(f_ixs, dtype=np.int32)
        _check(lib().afv_consistent_fluxes(self.h, ix.size, _ip(ix)))

    def write_vtk(self, tree, filename, ixs_cc, cc_names, ixs_fc=(), fc_names=(), n_cycle=0,
                  time=0.0, dir=None):
        """a$D_write_vtk: leaves of one tree to filename.vtu."""
        icc = np.ascontiguousarray(ixs_cc, dtype=np.int32)
        ifc = np.ascontiguousarray(ixs_fc, dtype=np.int32)
        cn = (ctypes.c_char_p * max(1, len(cc_names)))(*[n.encode() for n in cc_names])
        fn = (ctypes.c_char_p * max(1, len(fc_names)))(*[n.encode() for n in fc_names])
        _check(lib().afv_write_vtk(self.h, tree, filename.encode(), n_cycle, float(time), icc.size,
                                   _ip(icc), cn, ifc.size, _ip(ifc), fn,
                                   None if dir is None else dir.encode()))

    # single operators
    def gsrb_level(self, lvl, n_cycle):
        _check(lib().afv_mg_gsrb_level(self.h, lvl, n_cycle))

    def fill_gc_level(self, lvl):
        _check(lib().afv_fill_gc_level(self.h, lvl))

    def update_coarse(self, lvl):
        _check(lib().afv_mg_update_coarse(self.h, lvl))

    def correct_children(self, lvl_parent):
        _check(lib().afv_mg_correct_children(self.h, lvl_parent))

    def residual_all(self):
        _check(lib().afv_mg_residual_all(self.h))

    # event profiler
    def profile(self, mask):
        _check(lib().afv_forest_profile(self.h, mask))

    def autotune(self):
        """Pick the fastest sweep kernel for this forest; returns (choice,
        {variant: ms per FP32 V-cycle})."""
        c = ctypes.c_int(0)
        ms = (ctypes.c_float * 3)()
        _check(lib().afv_forest_autotune(self.h, ctypes.byref(c), ms))
        return c.value, {1: ms[0], 2: ms[1], 0: ms[2]}

    def autotune_all(self):
        """Full tuning pass: (sweep kernel, small sweeps, coarse end) chosen,
        and the ms per FP32 V-cycle of every setting timed."""
        c = np.zeros(3, np.int32)
        ms = (ctypes.c_float * 10)()
        _check(lib().afv_forest_autotune_all(self.h, _ip(c), ms))
        times = {"sweep_kernel_%d" % k: ms[k] for k in range(6)}
        for k in range(4):
            times["small_%d_coarse_end_%d" % (k >> 1, k & 1)] = ms[6 + k]
        return {"sweep_kernel": int(c[0]), "small_sweeps": int(c[1]), "coarse_end": int(c[2]),
                "defect_cells": self.get_option(AFV_OPT_DEFECT_CELLS)}, times

    def autotune_defect(self):
        """Times the fixed-point defect with 1, 2 and 4 cells per thread and
        keeps the fastest: (choice, {cells: ms per launch} of the shapes the
        boxes allow)."""
        c = ctypes.c_int(0)
        ms = (ctypes.c_float * 3)()
        _check(lib().afv_forest_autotune_defect(self.h, ctypes.byref(c), ms))
        return int(c.value), {cr: ms[k] for k, cr in enumerate((1, 2, 4)) if ms[k] >= 0}

    def set_option(self, option, value):
        _check(lib().afv_forest_set_option(self.h, option, int(value)))

    def get_option(self, option):
        v = ctypes.c_int(0)
        _check(lib().afv_forest_get_option(self.h, option, ctypes.byref(v)))
        return v.value

    def profile_entries(self):
        """Profiled event pairs: dict of arrays kind, level, ms, bytes, launches."""
        n = ctypes.c_longlong(0)
        _check(lib().afv_forest_profile_entries(self.h, 0, None, None, None, None, None, ctypes.byref(n)))
        m = max(int(n.value), 1)
        kind, level, cnt = np.zeros(m, np.int32), np.zeros(m, np.int32), np.zeros(m, np.int32)
        ms, by = np.zeros(m), np.zeros(m)
        _check(lib().afv_forest_profile_entries(self.h, m, _ip(kind), _ip(level), _dp(ms), _dp(by),
                                                _ip(cnt), ctypes.byref(n)))
        k = int(n.value)
        return dict(kind=kind[:k], level=level[:k], ms=ms[:k], bytes=by[:k], launches=cnt[:k])

    def profile_read(self, kind):
        n, ms, b = ctypes.c_longlong(0), ctypes.c_double(0), ctypes.c_double(0)
        _check(lib().afv_forest_profile_read(self.h, kind, ctypes.byref(n), ctypes.byref(ms),
                                             ctypes.byref(b)))
        return n.value, ms.value, b.value


def mg2_init_mg(mg=None):
    """mg$D_init_mg (src/m_aX_mg.f90:130-154): negative cycle counts become 2."""
    mg = mg or MgOpts()
    _check(lib().afv_mg_init(ctypes.byref(mg)))
    return mg


mg3_init_mg = mg2_init_mg


def mg2_fas_vcycle(forest, mg, highest_lvl, set_residual):
    forest.vcycle(mg, highest_lvl, set_residual)


def mg2_fas_fmg(forest, mg, set_residual, have_guess):
    forest.fmg(mg, set_residual, have_guess)


mg3_fas_vcycle, mg3_fas_fmg = mg2_fas_vcycle, mg2_fas_fmg


def a2_gc_tree(forest):
    forest.gc_tree()


a3_gc_tree = a2_gc_tree


def a2_tree_max_abs_cc(forest, tree, var):
    return forest.max_abs(tree, var)


a3_tree_max_abs_cc = a2_tree_max_abs_cc
