"""The C ABI without a GPU: the library loads, exports every function the
header declares, and the host-side entry points (tree build, options, errors)
behave as documented."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "afivo_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(afv_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("afv_tree_create", "afv_forest_create", "afv_mg_fas_vcycle", "afv_mg_fas_fmg",
              "afv_mg_solve", "afv_forest_set_bc_faces", "afv_tree_max_abs_cc_noalloc"):
        assert n in names
    assert len(names) >= 39


def test_library_exports_every_declared_function(afv):
    lib = ctypes.CDLL(afv.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_errors_are_codes_not_aborts(afv):
    lib = afv.lib()
    h = ctypes.c_void_p()
    rc = lib.afv_tree_create(4, 8, 0.1, None, 30, -1, 1.0, ctypes.byref(h))
    assert rc == afv.AFV_ERR_INVALID
    assert len(lib.afv_last_error()) > 0
    with pytest.raises(afv.AfivoError):
        afv.Tree(2, 7, 0.1)  # odd block size


def test_tree_build_host_only(afv):
    t = afv.Tree(2, 8, 1 / 8, coarsen_to=2)
    t.set_base([[1, 1]], [[-1, -1, -1, -1]])
    t.refine_builtin(afv.AFV_REF_UNIFORM, lvl_max=3)
    info = t.info()
    assert info["dim"] == 2 and info["n_cell"] == 8 and info["highest_lvl"] == 3
    assert info["min_lvl"] == -1  # coarsen_to = 2 with nc = 8: sub-levels 0 and -1
    faces = t.bc_faces()
    assert all(len(c) == t.n_cell_at(t.boxes()["lvl"][i - 1]) for i, _, c in faces)


def test_mg_init_defaults(afv):
    mg = afv.MgOpts()
    afv._check(afv.lib().afv_mg_init(ctypes.byref(mg)))
    assert (mg.n_cycle_down, mg.n_cycle_up, mg.n_cycle_base) == (2, 2, 2)


def test_python_constants_match_the_header(afv):
    """Every enumerator the header gives a value has the same value in the
    Python module, and the profiler's kernel kinds are in the header's order."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    values = {n: int(v) for n, v in re.findall(r"\b(AFV_[A-Z0-9_]+)\s*=\s*(-?\d+)", text)}
    assert len(values) >= 30
    kinds = {n: v for n, v in values.items() if n.startswith("AFV_KERNEL_")}
    for n, v in values.items():
        if n in kinds:
            continue
        assert hasattr(afv, n), n
        assert getattr(afv, n) == v, (n, getattr(afv, n), v)
    assert len(afv.KERNEL_KINDS) == len(kinds)
    for n, v in kinds.items():
        assert afv.KERNEL_KINDS[v] == n[len("AFV_KERNEL_"):].lower(), (n, v)
