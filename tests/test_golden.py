"""Golden fixtures (tests/golden/golden.json, written by
tests/golden/make_golden.py from the oracle): the oracle rebuilt here must
reproduce them bit for bit, so the fixtures pin the oracle across hosts and
compilers; the GPU path is checked against the same fixtures in
tests/test_gpu_golden.py."""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import golden_cases as GC  # noqa: E402

with open(os.path.join(HERE, "golden", "golden.json")) as f:
    GOLDEN = json.load(f)


@pytest.mark.parametrize("name", sorted(GC.CASES))
def test_oracle_reproduces_golden(oracle_lib, name):
    import make_golden as MG
    O = oracle_lib
    c = GC.CASES[name]
    g = GOLDEN[name]
    t = MG.oracle_case(c)
    b = t.boxes()
    boxes = [[int(l)] + [int(x) for x in ix] for l, ix, u in zip(b["lvl"], b["ix"], b["in_use"] != 0) if u]
    assert boxes == g["boxes"]
    MG.set_rhs(t, c, 1000)
    t.mg_init()
    done = 0
    for k in GC.CYCLES:
        while done < k:
            t.vcycle(set_residual=True)
            done += 1
        assert MG.digest(t, c) == g["cycles"][str(k)], (name, k)


def test_hash_values_are_exact():
    v = GC.hash_values(1000, 7)
    assert ((v + 0.5) * 2 ** 20 == ((v + 0.5) * 2 ** 20).round()).all()
    assert v.min() >= -0.5 and v.max() < 0.5
