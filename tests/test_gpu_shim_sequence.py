"""The call sequences of the Fortran drop-in (fortran/m_aX_gb300.f90) through
the C ABI: the default one (every call uploads phi, rhs and tmp and downloads
all three, so the caller's tree ends as the reference's routine leaves it) and
the lean one (the device keeps the state; a call uploads only when the
caller's data generation changed, and downloads phi, plus tmp with
set_residual). Both give the oracle's phi after every V-cycle, and the lean
one re-uploads after the caller changes its data."""
import numpy as np
import pytest

import oracle as O
from helpers import compare_var, oracle_var, setup_pair
from afivo_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13


def test_default_and_lean_sequences_match_the_oracle(gpu):
    spec = W.c1_poisson_2d()
    full, ot, _ = setup_pair(gpu, spec)
    lean = gpu.Forest([W.build_tree(spec)])
    V = (gpu.AFV_PHI, gpu.AFV_RHS, gpu.AFV_TMP)
    host = {v: full.get_var(0, v) for v in V}        # the default caller's arrays
    lean_host = {v: a.copy() for v, a in host.items()}  # the lean caller's arrays
    gen, lean_gen, uploads = 0, -1, 0
    for cycle in range(8):
        set_residual = cycle % 2 == 0
        if cycle == 5:  # both callers scale rhs on the host; the lean one bumps its generation
            host[gpu.AFV_RHS] = host[gpu.AFV_RHS] * 1.5
            lean_host[gpu.AFV_RHS] = lean_host[gpu.AFV_RHS] * 1.5
            for lvl in range(ot.min_lvl, ot.highest_lvl + 1):
                ot.set_level(lvl, O.I_RHS, ot.get_level(lvl, O.I_RHS, 8) * 1.5)
            gen += 1
        # default sequence: upload all, cycle, download all
        for v in V:
            full.set_var(0, v, host[v])
        full.vcycle(set_residual=set_residual)
        for v in V:
            host[v] = full.get_var(0, v)
        # lean sequence: upload only for a new generation; phi (and tmp) back
        if gen != lean_gen:
            for v in V:
                lean.set_var(0, v, lean_host[v])
            lean_gen = gen
            uploads += 1
        lean.vcycle(set_residual=set_residual)
        lean_host[gpu.AFV_PHI] = lean.get_var(0, gpu.AFV_PHI)
        if set_residual:
            lean_host[gpu.AFV_TMP] = lean.get_var(0, gpu.AFV_TMP)
        ot.vcycle(set_residual=set_residual)
        ref = oracle_var(ot, O.I_PHI, 8)
        assert compare_var(host[gpu.AFV_PHI], ref, ot, 8, 2, False) <= TOL
        assert compare_var(lean_host[gpu.AFV_PHI], ref, ot, 8, 2, False) <= TOL
        if set_residual:
            assert compare_var(lean_host[gpu.AFV_TMP], oracle_var(ot, O.I_TMP, 8), ot, 8, 2, True) <= TOL
    assert uploads == 2


def test_operator_hooks_sequence_matches_the_oracle(gpu):
    """The drop-in's sequence for the reference's built-in operator hooks in
    a cylindrical tree (examples/poisson_cyl.f90 with mg2_auto_*, and eps):
    extra variables 3-5 added once, eps uploaded beside phi, rhs and tmp with
    every upload, the operator set after it (tags from the uploaded eps),
    then the cycle; phi after every V-cycle is the oracle's."""
    from helpers import cyl_spec, fill_from_centres, oracle_tree
    spec = cyl_spec(lvl_max=6)
    nc = spec["n_cell"]
    ot = oracle_tree(spec)
    ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    ot.mg_init()
    ot.add_vars(3, 0)
    eps = fill_from_centres(ot, 3, lambda r: np.where(r[..., 0] > 0.53, 100.0, 1.0), nc)
    assert ot.set_operator(2, 3)  # mg2_auto_op / _gsrb / _corr with mg%i_eps
    f = gpu.Forest([W.build_tree(spec)])
    host = {v: oracle_var(ot, v, nc) for v in (gpu.AFV_PHI, gpu.AFV_RHS, gpu.AFV_TMP)}
    added = False
    for cycle in range(4):
        for v, a in host.items():
            f.set_var(0, v, a)
        if not added:
            f.add_vars(3, 0)
            added = True
        f.set_var(0, 3, eps)
        f.set_operator(gpu.AFV_OP_AUTO, 3, -1, -1)
        f.vcycle(set_residual=True)
        host = {v: f.get_var(0, v) for v in host}
        ot.vcycle(set_residual=True)
        assert compare_var(host[gpu.AFV_PHI], oracle_var(ot, O.I_PHI, nc), ot, nc, 2, False) <= TOL
