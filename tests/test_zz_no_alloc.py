"""afv_tree_max_abs_cc_noalloc (static device scratch, no allocation) against
afv_tree_max_abs_cc (forest-owned scratch). Collected last so that it runs
both alone and after every other test of the session."""
import numpy as np
import pytest

from afivo_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# Both entry points take the same per-box maxima and fold them with max, which
# is exact, so the values agree bit for bit; the tolerance is written anyway.
REL_TOL = 0.0


def _specs(which):
    if which == "2d":
        return W.c4_random_2d(3, small=True)
    # 3-D trees of different depth (leaves on levels 2 to 5) in one forest
    return [W.c2_poisson_3d(seed=s, thr=3e-3, lvl_max=l) for s, l in ((2, 5), (3, 4), (5, 3))]


def _forest(afv, which="2d"):
    specs = _specs(which)
    trees = [W.build_tree(s) for s in specs]
    f = afv.Forest(trees)
    rng = np.random.default_rng(11)
    for k in range(len(trees)):
        rhs = f.get_var(k, afv.AFV_RHS)
        f.set_var(k, afv.AFV_RHS, rng.standard_normal(rhs.size) * (k + 1))
    for _ in range(2):
        f.vcycle(set_residual=True)
    return f, len(trees)


@pytest.mark.parametrize("which", ["2d", "3d"])
def test_noalloc_matches_max_abs_twice(gpu, which):
    f, nt = _forest(gpu, which)
    for var in (gpu.AFV_PHI, gpu.AFV_RHS, gpu.AFV_TMP):
        for t in range(nt):
            want = f.max_abs(t, var)
            first = f.max_abs_noalloc(t, var)
            second = f.max_abs_noalloc(t, var)
            assert want > 0
            for got in (first, second):
                assert abs(got - want) <= REL_TOL * abs(want), (var, t, got, want)
    f.close()


def test_noalloc_rejects_too_many_trees(gpu):
    trees = []
    for _ in range(1025):
        t = gpu.Tree(2, 4, 0.25)
        t.set_base([[1, 1]], [[-1, -1, -1, -1]])
        trees.append(t)
    f = gpu.Forest(trees)
    with pytest.raises(gpu.AfivoError, match="at most 1024"):
        f.max_abs_noalloc(0, gpu.AFV_PHI)
    # The forest-scratch entry point has no such limit.
    assert f.max_abs(1024, gpu.AFV_PHI) == 0.0
    f.close()
