"""CPU checks of the product library: exports, host-built SG4 tables against the
oracle, and argument validation (no device work)."""
import ctypes
import re
import os

import numpy as np
import pytest

from elvibrot_gb300 import EVRError, SG4Basis, lib
from oracle.oracle import OracleSG4

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "evr_sg4.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(evr_\w+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    L = lib()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n


@pytest.mark.parametrize("D,L,A,B,Aq,Bq", [(3, 6, 1, 1, 2, 1), (6, 8, 1, 1, 2, 1), (6, 3, 1, 2, 1, 2),
                                            (21, 2, 1, 2, 1, 2), (4, 7, 1, 1, 2, 1), (2, 4, 2, 1, 3, 2)])
def test_tables_match_oracle(D, L, A, B, Aq, Bq):
    s = np.linspace(0.3, 0.9, D)
    Bs = SG4Basis(D, L, L, A, B, Aq, Bq, scaleQ=s)
    O = OracleSG4(D, L, L, A, B, Aq, Bq, scaleQ=s)
    assert (Bs.N, Bs.nb_SG, Bs.sum_nb, Bs.sum_nq) == (O.N, O.nb_SG, O.sum_nb, O.sum_nq)
    tl, w, m = Bs.tables()
    tl2, w2, m2, _ = O.tables()
    np.testing.assert_array_equal(tl, tl2)
    np.testing.assert_array_equal(w, w2)
    np.testing.assert_array_equal(m, m2)
    for mode in range(D):
        for l in range(L + 1):
            x, y = Bs.basis1d(mode, l), O.basis1d(mode, l)
            for k1, k2 in (("x", "x"), ("RGB", "d0"), ("RBGwrho", "bgw"), ("d1GG", "d1gg"), ("d2GG", "d2gg")):
                ref = y[k2]
                assert np.max(np.abs(x[k1] - ref)) <= 4e-15 * max(1.0, np.max(np.abs(ref))), (mode, l, k1)
    np.testing.assert_allclose(Bs.grid_points(), O.grid_points(), rtol=0, atol=1e-14)


def test_reduced_basis_level():
    # LB < L: packed set is smaller, the map gets zeros (the reference warns)
    Bs = SG4Basis(3, 5, 3, 1, 1, 2, 1)
    O = OracleSG4(3, 5, 3, 1, 1, 2, 1)
    assert Bs.N == O.N
    np.testing.assert_array_equal(Bs.tables()[2], O.tables()[2])
    assert (Bs.tables()[2] == 0).any()


@pytest.mark.parametrize("args", [(0, 3, 3, 1, 1, 2, 1), (3, -1, 3, 1, 1, 2, 1), (3, 3, 3, 0, 1, 2, 1),
                                  (3, 3, 3, 3, 1, 2, 1), (3, 20, 20, 1, 1, 2, 1), (40, 2, 2, 1, 1, 2, 1)])
def test_build_rejects_bad_arguments(args):
    with pytest.raises(EVRError) as e:
        SG4Basis(*args)
    assert e.value.code == 1


def test_weights_sum_to_one_and_map_covers_packed_basis():
    for D, L in ((2, 5), (5, 4), (9, 3)):
        Bs = SG4Basis(D, L)
        tl, w, m = Bs.tables()
        assert abs(w.sum() - 1.0) < 1e-12
        assert set(m[m > 0]) == set(range(1, Bs.N + 1))
