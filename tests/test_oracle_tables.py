"""The oracle's topology functions against the literal tables of the
reference's src/m_aX_t.f90:54-149."""
import numpy as np


def fortran_reshape(vals, shape):
    return np.array(vals).reshape(shape[::-1]).T


REF2 = dict(
    child_dix=fortran_reshape([0, 0, 1, 0, 0, 1, 1, 1], (2, 4)),            # :65
    child_rev=fortran_reshape([2, 1, 4, 3, 3, 4, 1, 2], (4, 2)),            # :67
    child_adj_nb=fortran_reshape([1, 3, 2, 4, 1, 2, 3, 4], (2, 4)),         # :69
    neighb_dix=fortran_reshape([-1, 0, 1, 0, 0, -1, 0, 1], (2, 4)),         # :82
    neighb_rev=np.array([2, 1, 4, 3]),                                      # :91
)
REF3 = dict(
    child_dix=fortran_reshape([0, 0, 0, 1, 0, 0, 0, 1, 0, 1, 1, 0,
                               0, 0, 1, 1, 0, 1, 0, 1, 1, 1, 1, 1], (3, 8)),  # :111-113
    child_rev=fortran_reshape([2, 1, 4, 3, 6, 5, 8, 7, 3, 4, 1, 2, 7, 8, 5, 6,
                               5, 6, 7, 8, 1, 2, 3, 4], (8, 3)),            # :115-116
    child_adj_nb=fortran_reshape([1, 3, 5, 7, 2, 4, 6, 8, 1, 2, 5, 6, 3, 4, 7, 8,
                                  1, 2, 3, 4, 5, 6, 7, 8], (4, 6)),         # :118-119
    neighb_dix=fortran_reshape([-1, 0, 0, 1, 0, 0, 0, -1, 0, 0, 1, 0, 0, 0, -1, 0, 0, 1],
                               (3, 6)),                                     # :136-137
    neighb_rev=np.array([2, 1, 4, 3, 6, 5]),                                # :146
)


def test_tables_match_reference(oracle_lib):
    L = oracle_lib.lib()
    for dim, ref in ((2, REF2), (3, REF3)):
        nch, nnb = 2 ** dim, 2 * dim
        for c in range(1, nch + 1):
            for d in range(1, dim + 1):
                assert L.orc_child_dix(dim, d, c) == ref["child_dix"][d - 1, c - 1]
                assert L.orc_child_rev(dim, c, d) == ref["child_rev"][c - 1, d - 1]
        for nb in range(1, nnb + 1):
            assert L.orc_neighb_rev(dim, nb) == ref["neighb_rev"][nb - 1]
            for d in range(1, dim + 1):
                assert L.orc_neighb_dix(dim, d, nb) == ref["neighb_dix"][d - 1, nb - 1]
            for k in range(1, nch // 2 + 1):
                assert L.orc_child_adj_nb(dim, k, nb) == ref["child_adj_nb"][k - 1, nb - 1]


def test_ix_to_ichild(oracle_lib):
    import ctypes
    L = oracle_lib.lib()
    # a$D_ix_to_ichild, src/m_aX_t.f90:378-387: odd indices are low children
    for ix, c in (((1, 1), 1), ((2, 1), 2), ((1, 2), 3), ((2, 2), 4), ((7, 10), 3)):
        a = (ctypes.c_int * 2)(*ix)
        assert L.orc_ix_to_ichild(2, a) == c
    for ix, c in (((1, 1, 1), 1), ((2, 2, 2), 8), ((1, 2, 2), 7), ((2, 1, 1), 2)):
        a = (ctypes.c_int * 3)(*ix)
        assert L.orc_ix_to_ichild(3, a) == c
