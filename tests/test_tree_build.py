"""Tree build: invariants of the oracle's trees, and the library's host tree
builder bit-exact against the oracle (same ids, links and level lists), for
the configurations the solver runs on and for refine/derefine sequences that
trigger the Morton renumbering of a$D_tidy_up."""
import numpy as np
import pytest

import oracle as O
from helpers import oracle_tree, same_tree
from afivo_gb300 import workloads as W


def check_invariants(t):
    b = t.boxes()
    dim = t.dim
    nch, nnb = 2 ** dim, 2 * dim
    rev = [2, 1, 4, 3, 6, 5]
    for l in range(t.min_lvl, t.highest_lvl + 1):
        ids, leaves, parents = t.level(l)
        assert sorted(ids) == sorted(np.concatenate([leaves, parents]))
        for i in ids:
            k = i - 1
            assert b["in_use"][k] == 1 and b["lvl"][k] == l
            for nb in range(nnb):
                v = b["neighbors"][k, nb]
                if v > 0:  # symmetric links on the same level
                    assert b["neighbors"][v - 1, rev[nb] - 1] == i
                    assert b["lvl"][v - 1] == l
                elif v == 0:  # refinement boundary: 2:1 balance
                    p = b["parent"][k]
                    assert b["neighbors"][p - 1, nb] > 0
                    assert b["children"][k, 0] == 0
            if l >= 1 and b["children"][k, 0] > 0:
                for c in range(nch):
                    cid = b["children"][k, c]
                    assert b["parent"][cid - 1] == i
                    # child index from its position (src/m_aX_t.f90:378-387)
                    ix = b["ix"][cid - 1]
                    ic = nch - sum((int(ix[d]) & 1) << d for d in range(dim))
                    assert ic == c + 1


SPECS = [W.c1_poisson_2d(), W.c3_uniform_2d(5), W.c2_poisson_3d(thr=3e-3, lvl_max=7)] + \
    W.c4_random_2d(3, small=True)


@pytest.mark.parametrize("spec", SPECS, ids=lambda s: s["name"])
def test_library_tree_matches_oracle(afv, oracle_lib, spec):
    o = oracle_tree(spec)
    check_invariants(o)
    a = W.build_tree(spec)
    same_tree(a, o)


@pytest.mark.parametrize("dim", [2, 3])
def test_refine_derefine_and_tidy_up(afv, oracle_lib, dim):
    """Random refine / derefine passes (examples/random_refinement_2d.f90:85-100
    with a keyed generator) until ids have holes and tidy_up renumbers them."""
    nb = [[1] * (2 * dim)]
    ix = [[1] * dim]
    o = O.OracleTree(dim, 4, 0.25, ix, nb, coarsen_to=2)
    a = afv.Tree(dim, 4, 0.25, coarsen_to=2).set_base(ix, nb)
    seen_tidy = False
    n_up, lmax = (7, 8) if dim == 2 else (5, 5)
    for p in range(n_up + 8):
        prob = 0.9 if p < n_up else 0.02
        before = o.highest_id
        na_o, nr_o = o.adjust_refinement(O.REF_RANDOM_RM, lmax, prob=prob, seed=11)
        na_a, nr_a = a.adjust_builtin(afv.AFV_REF_RANDOM_RM, lmax, prob=prob, seed=11)
        assert (na_o, nr_o) == (na_a, nr_a)
        same_tree(a, o)
        check_invariants(o)
        if o.highest_id < before + na_o:  # ids were compacted by tidy_up
            seen_tidy = True
    # the sequence must have exercised the renumbering at least once
    assert seen_tidy


def test_invalid_inputs(afv):
    with pytest.raises(afv.AfivoError):
        afv.Tree(2, 7, 0.1)  # odd n_cell (src/m_aX_core.f90:62)
    with pytest.raises(afv.AfivoError):
        afv.Tree(2, 8, 0.1, coarsen_to=3)  # cannot coarsen to 3 (:79-80)
    t = afv.Tree(2, 8, 0.1)
    with pytest.raises(afv.AfivoError):
        t.set_base([[0, 1]], [[-1] * 4])  # ix must be > 0 (:159)
    t = afv.Tree(2, 8, 0.1)
    with pytest.raises(afv.AfivoError):
        t.set_base([[1, 1], [2, 1]], [[-1, 0, -1, -1], [0, -1, -1, -1]])  # unresolved (:174)
    t = afv.Tree(2, 8, 0.1)
    with pytest.raises(afv.AfivoError):
        t.adjust_builtin(afv.AFV_REF_UNIFORM, 3)  # before set_base
    t.set_base([[1, 1]], [[-1] * 4])

    def bad(view, flag):
        return 7
    with pytest.raises(afv.AfivoError):
        t.adjust_refinement(bad)  # invalid flag (:662-663)


def test_memory_limit(afv):
    t = afv.Tree(2, 8, 0.1, mem_limit_gb=1e-5)
    t.set_base([[1, 1]], [[-1] * 4])
    with pytest.raises(afv.AfivoError) as e:
        for _ in range(10):
            t.adjust_builtin(afv.AFV_REF_UNIFORM, 10)
    assert e.value.code == afv.AFV_ERR_BUDGET


def test_python_callback_matches_builtin(afv):
    spec = W.c1_poisson_2d()
    a = W.build_tree(spec)
    t = afv.Tree(2, 8, 1 / 8, coarsen_to=2).set_base(spec["ix"], spec["nb"])
    g = spec["gauss"].reshape(-1, 4)

    def ref(box, flag):
        if box.lvl >= 8:
            return flag
        nc, dr = box.n_cell, box.dr
        i = np.arange(1, nc + 1) - 0.5
        x = box.r_min[0] + i[:, None] * dr
        y = box.r_min[1] + i[None, :] * dr
        f = np.zeros((nc, nc))
        for a_, s, cx, cy in g:
            xr2 = ((x - cx) / s) ** 2 + ((y - cy) / s) ** 2
            f += a_ * (4 / s ** 2 * (xr2 - 1.0) * np.exp(-xr2))
        return afv.AFV_DO_REF if (np.abs(f) * dr * dr > 1e-3).any() else flag
    for _ in range(30):
        na, _ = t.adjust_refinement(ref)
        if na == 0:
            break
    assert t.info()["n_leaves"] == a.info()["n_leaves"]


@pytest.mark.parametrize("which", ["c2_full", "c3_lvl9", "c4_256"])
def test_library_tree_matches_oracle_full_size(afv, oracle_lib, which):
    """The trees the benchmark runs on, at their full sizes: the 3-D adaptive
    tree (34,907 boxes), the 4096^2 uniform tree (87,384 boxes) and all 256
    random trees of the batched workload, bit for bit."""
    specs = {"c2_full": [W.c2_poisson_3d()], "c3_lvl9": [W.c3_uniform_2d(9)],
             "c4_256": W.c4_random_2d()}[which]
    boxes = 0
    for spec in specs:
        o = oracle_tree(spec)
        a = W.build_tree(spec)
        same_tree(a, o)
        boxes += a.info()["n_boxes"]
    assert boxes == {"c2_full": 34907, "c3_lvl9": 87384, "c4_256": 1166416}[which]
