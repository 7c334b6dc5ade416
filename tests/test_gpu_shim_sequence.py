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
