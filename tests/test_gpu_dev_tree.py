"""The tree build on the device (afv_dtree_*: a$D_adjust_refinement with
consistent_ref_flags, add/remove_children, set_neighbs and the Morton
renumbering of a$D_tidy_up, src/m_aX_core.f90:238-787) against the host
builder and the oracle: ids, links and level lists bit for bit, on the
workload trees and on refine/derefine sequences that trigger the
renumbering."""
import numpy as np
import pytest

import oracle as O
from helpers import oracle_tree, same_tree
from afivo_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _base(afv, spec):
    return afv.Tree(spec["dim"], spec["n_cell"], spec["dr"], coarsen_to=spec["coarsen_to"]).set_base(
        spec["ix"], spec["nb"])


def _device_built(afv, spec):
    """The workload's tree refined on the device, downloaded into a host tree."""
    d = afv.DeviceTree(_base(afv, spec))
    if spec["crit"] == afv.AFV_REF_RANDOM and "target_cells" in spec:
        for _ in range(100):
            if d.info()["n_leaves"] * spec["n_cell"] ** spec["dim"] >= spec["target_cells"]:
                break
            d.adjust_builtin(afv.AFV_REF_RANDOM, spec["lvl_max"], prob=spec["prob"], seed=spec["seed"])
    else:
        d.refine_builtin(spec["crit"], spec["lvl_max"], thr=spec.get("thr", 0.0), prob=spec.get("prob", 0.0),
                         seed=spec.get("seed", 0), gauss=spec.get("gauss"), lpl=spec.get("lpl", False))
    out = _base(afv, spec)
    d.download(out)
    d.close()
    return out


SPECS = [W.c1_poisson_2d(), W.c3_uniform_2d(6), W.c2_poisson_3d(thr=3e-3, lvl_max=7),
         W.c2_poisson_3d()] + W.c4_random_2d(8, small=True)


@pytest.mark.parametrize("spec", SPECS, ids=lambda s: s["name"] + ("_full" if s.get("thr") == 7e-4 else ""))
def test_device_tree_matches_host_and_oracle(gpu, spec):
    dev = _device_built(gpu, spec)
    same_tree(dev, W.build_tree(spec))
    same_tree(dev, oracle_tree(spec))


def test_device_tree_all_256_batch_trees(gpu):
    for spec in W.c4_random_2d(256):
        same_tree(_device_built(gpu, spec), W.build_tree(spec))


@pytest.mark.parametrize("dim", [2, 3])
def test_device_refine_derefine_and_tidy_up(gpu, dim):
    """Random refine / derefine passes until ids have holes and tidy_up
    renumbers them; the device tree equals the host tree and the oracle
    after every pass."""
    nb = [[1] * (2 * dim)]
    ix = [[1] * dim]
    o = O.OracleTree(dim, 4, 0.25, ix, nb, coarsen_to=2)
    h = gpu.Tree(dim, 4, 0.25, coarsen_to=2).set_base(ix, nb)
    d = gpu.DeviceTree(gpu.Tree(dim, 4, 0.25, coarsen_to=2).set_base(ix, nb))
    seen_tidy = False
    n_up, lmax = (7, 8) if dim == 2 else (5, 5)
    for p in range(n_up + 8):
        prob = 0.9 if p < n_up else 0.02
        before = o.highest_id
        r_o = o.adjust_refinement(O.REF_RANDOM_RM, lmax, prob=prob, seed=11)
        r_h = h.adjust_builtin(gpu.AFV_REF_RANDOM_RM, lmax, prob=prob, seed=11)
        r_d = d.adjust_builtin(gpu.AFV_REF_RANDOM_RM, lmax, prob=prob, seed=11)
        assert r_o == r_h == r_d
        got = d.download(gpu.Tree(dim, 4, 0.25, coarsen_to=2).set_base(ix, nb))
        same_tree(got, h)
        same_tree(got, o)
        if o.highest_id < before + r_o[0]:
            seen_tidy = True
    assert seen_tidy


def test_device_tree_feeds_a_forest(gpu):
    """A forest made from the downloaded device tree solves like one made
    from the host tree (bit for bit)."""
    spec = W.c1_poisson_2d()
    out = []
    for tree in (_device_built(gpu, spec), W.build_tree(spec)):
        f = gpu.Forest([tree], mixed=True)
        f.set_source(0, spec["gauss"], lpl=True)
        cyc, rel, rc = f.solve(gpu.AFV_PREC_MIXED, tol=1e-8, max_cycles=40)
        assert rc == 0
        out.append(f.get_var(0, gpu.AFV_PHI))
    assert np.array_equal(out[0], out[1])
