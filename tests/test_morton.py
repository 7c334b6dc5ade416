"""Morton keys (src/m_morton.f90) against tests/test_morton.f90's round trip
and hand-checked interleavings, in the oracle and in the library's planner."""
import numpy as np


def interleave(ix):
    m = 0
    for b in range(21):
        for d, v in enumerate(ix):
            m |= ((int(v) >> b) & 1) << (len(ix) * b + d)
    return m


def test_reference_known_answer(oracle_lib):
    # tests/test_morton.f90:9-14: ix = (15, 2047) -> morton -> ix
    m = oracle_lib.morton_from_ix([15, 2047])
    assert m == interleave([15, 2047]) == 2796287
    assert list(oracle_lib.morton_to_ix(2, m)) == [15, 2047]


def test_hand_checked(oracle_lib):
    assert oracle_lib.morton_from_ix([1, 0]) == 1
    assert oracle_lib.morton_from_ix([0, 1]) == 2
    assert oracle_lib.morton_from_ix([1, 1]) == 3
    assert oracle_lib.morton_from_ix([1, 0, 0]) == 1
    assert oracle_lib.morton_from_ix([0, 1, 0]) == 2
    assert oracle_lib.morton_from_ix([0, 0, 1]) == 4


def test_round_trip_random(oracle_lib):
    rng = np.random.default_rng(0)
    for _ in range(200):
        ix = rng.integers(0, 2 ** 20, 2)
        m = oracle_lib.morton_from_ix(ix)
        assert m == interleave(ix)
        assert list(oracle_lib.morton_to_ix(2, m)) == list(ix)
        ix3 = rng.integers(0, 2 ** 21, 3)
        m3 = oracle_lib.morton_from_ix(ix3)
        assert m3 == interleave(ix3)
        assert list(oracle_lib.morton_to_ix(3, m3)) == list(ix3)
