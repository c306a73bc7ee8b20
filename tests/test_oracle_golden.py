"""Pins the CPU oracle to the reference's own known answers.

* Gauss-Hermite nodes/weights against Internal_data/HermQuadra (the files
  sub_quadra_herm.f90 reads).
* Henon-Heiles SG4 levels (6-D L=3, 21-D L=2; Working_tests/MPI_tests/*_S0/
  benchmark) from a dense diagonalisation of the oracle's H.psi.  The
  reference's Davidson converged to a residual of 5e-4 au, which bounds its
  eigenvalue error near 1e-7 au; the tolerance below is 2e-7 au.
"""
import json
import os

import numpy as np
import pytest

from oracle.oracle import OracleSG4, gauss_hermite

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_hermquadra_bitwise():
    d = json.load(open(os.path.join(GOLD, "hermquadra.json")))["nq"]
    worst, exact, tot = 0.0, 0, 0
    for nq_s, ref in d.items():
        nq = int(nq_s)
        x, w, wr = gauss_hermite(nq)
        for a, b in ((x, ref["x"]), (wr, ref["wrho"]), (w, ref["w"])):
            b = np.array(b)
            err = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
            worst = max(worst, float(err.max()))
            exact += int(np.sum(a == b))
            tot += nq
    # nodes and weights are correctly rounded doubles of the 50-digit tables,
    # except for rare 1-ulp ties
    assert worst <= 2.3e-16, worst
    assert exact >= tot - 8, (exact, tot)


def hh_potential(Q, lam):
    """Henon-Heiles V of Working_tests/MPI_tests/*/sub_system_HenonHeiles.f."""
    V = 0.5 * np.sum(Q ** 2, axis=1)
    for i in range(Q.shape[1] - 1):
        V += lam * (Q[:, i] ** 2 * Q[:, i + 1] - Q[:, i + 1] ** 3 / 3.0)
    return V


@pytest.mark.parametrize("case", ["6D_Davidson_S0", "21D_Davidson_S0"])
def test_henon_heiles_levels(case):
    c = json.load(open(os.path.join(GOLD, "hh_levels.json")))["cases"][case]
    D, L, B = c["D"], c["L"], c["L_TO_nq_B"]
    o = OracleSG4(D, L, c["LB"], A_nb=c["L_TO_nq_A"], B_nb=B, A_nq=c["L_TO_nq_A"], B_nq=B)
    V = hh_potential(o.grid_points(), c["lambda"])
    H = o.hpsi(np.eye(o.N), type_op=1, V=V, F2=(-0.5 * np.eye(D)).ravel())
    assert np.max(np.abs(H - H.T)) < 1e-12
    ev = np.sort(np.linalg.eigvalsh(0.5 * (H + H.T)))
    ref = np.array(c["levels_au"])
    assert np.max(np.abs(ev[: len(ref)] - ref)) < 2e-7


def test_sizes_match_index_set_formulas():
    # N = C(L+D, D) and term counts for nb(l)=l+1, nq(l)=l+2
    from math import comb
    for D, L, nsg in ((3, 6, 64), (6, 8, 2975), (4, 7, 295)):
        o = OracleSG4(D, L, L, 1, 1, 2, 1)
        assert o.N == comb(L + D, D)
        assert o.nb_SG == nsg
        tab_l, w, m, p = o.tables()
        assert abs(w.sum() - 1.0) < 1e-12
        assert np.all((m >= 0) & (m <= o.N))
        # every packed function is reached by at least one term
        assert set(m[m > 0]) == set(range(1, o.N + 1))


def test_type10_invariances():
    # constant Jac and rho cancel in the type-10 formula
    o = OracleSG4(3, 3, 3, 1, 1, 2, 1)
    rng = np.random.default_rng(1)
    V = rng.normal(size=o.sum_nq)
    psi = rng.normal(size=(o.N, 2))
    h0 = o.hpsi(psi, type_op=10, V=V)
    c = np.full(o.sum_nq, 2.5)
    h1 = o.hpsi(psi, type_op=10, V=V, Jac=c, sqRho=np.ones(o.sum_nq))
    assert np.max(np.abs(h1 - h0)) <= 1e-13 * np.max(np.abs(h0))
    G = np.zeros(o.sum_nq * 9)
    oq = 0
    for t in range(o.nb_SG):
        pass
    # identity G given explicitly equals G=None
    tab_l = o.tables()[0]
    off = 0
    for t in range(o.nb_SG):
        nq = int(np.prod(tab_l[t] + 2))
        for i in range(3):
            G[off * 9 + nq * (i + 3 * i): off * 9 + nq * (i + 3 * i) + nq] = 1.0
        off += nq
    h2 = o.hpsi(psi, type_op=10, V=V, G=G)
    assert np.max(np.abs(h2 - h0)) <= 1e-14 * np.max(np.abs(h0))


def pyrazine_model(g, O):
    """The 2-state pyrazine model of Working_tests/MPI_tests/12D_propagation_S0
    (sub_system_pyrazine.f: V11, V22, V12 on the oracle's grid points, in
    hartree; calc_f2_f1Q.f90: Tdef2(i,i) = -1/2 omega_i)."""
    ev = g["eV_to_hartree"]
    w, k1, k2 = (np.array(g[k]) for k in ("omega_eV", "kappa1_eV", "kappa2_eV"))
    Q = O.grid_points()
    v0 = 0.5 * (Q * Q) @ w
    V11 = (v0 - g["delta_eV"] + Q @ k1) * ev
    V22 = (v0 + g["delta_eV"] + Q @ k2) * ev
    V12 = g["lambda_eV"] * Q[:, 0] * ev
    F2 = np.diag(-0.5 * w * ev)
    return V11, V22, V12, F2


def pyrazine_oracle(g):
    A, B = g["L_TO_nq_A"], g["L_TO_nq_B"]
    return OracleSG4(g["D"], g["L"], g["LB"], A_nb=A, B_nb=B, A_nq=A, B_nq=B)   # Hm: nb(l) = nq(l)


def test_pyrazine_autocorrelation_golden():
    """H of the nb0=2 vibronic system from the oracle: the electronic blocks
    are T + V11, V12, V21 = V12, T + V22, each applied per Smolyak term as the
    reference does with V(:,ie,je); exp(-iHt) psi0 then reproduces the
    reference's 61-point autocorrelation to its own criterion (1e-8)."""
    from scipy.linalg import expm
    g = json.load(open(os.path.join(GOLD, "pyrazine12d.json")))
    O = pyrazine_oracle(g)
    assert O.N == 1 + sum(g["L_TO_nq_B"])      # ground state + one excited mode (LB = 1)
    V11, V22, V12, F2 = pyrazine_model(g, O)
    I = np.eye(O.N)
    H11 = O.hpsi(I, type_op=1, V=V11, F2=F2.ravel())
    H22 = O.hpsi(I, type_op=1, V=V22, F2=F2.ravel())
    H12 = O.hpsi(I, type_op=0, V=V12)
    H = np.block([[H11, H12], [H12, H22]])
    psi0 = np.zeros(2 * O.N, dtype=complex)
    assert g["psi0"]["nDval"] == [1] * 12 and g["psi0"]["i_e"] == 2
    psi0[O.N + 0] = complex(*g["psi0"]["coef"])    # packed index 1 = all modes in their first function
    ac = g["autocorr"]
    t = np.array(ac["t_au"])
    U1 = expm(-1j * H * (t[1] - t[0]))
    psi = psi0.copy()
    got = []
    for k in range(len(t)):
        got.append(np.vdot(psi0, psi))
        psi = U1 @ psi
    got = np.array(got)
    err = max(np.max(np.abs(got.real - ac["re"])), np.max(np.abs(got.imag - ac["im"])))
    print(f"pyrazine 12-D L=1 autocorrelation: max error {err:.2e} over {len(t)} times")
    assert err <= g["criterion"]


def test_oracle_analytic_fields_match_grid_fields():
    """The oracle's term-by-term evaluation of a polynomial V and an affine G
    (no stored grids: what the large 12-D checks need) gives the operator of
    the same fields passed as grids."""
    from elvibrot_gb300.configs import make_model
    m = make_model(4, 4, 10, 99)
    O = OracleSG4(m.D, m.L, m.L, 1, 1, 2, 1, scaleQ=m.scaleQ)
    Q = O.grid_points()
    nq = np.prod(O.tables()[0] + 2, axis=1)
    psi = np.random.default_rng(4).normal(size=(O.N, 3))
    ref = O.hpsi(psi, type_op=10, V=m.V(Q), G=m.G_grid(Q, nq))
    got = O.hpsi(psi, type_op=10, V_poly=(m.V.coef, m.V.expo), G0=m.G0, G1=m.G1)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    # type 1 with the polynomial V
    m1 = make_model(3, 5, 1, 98)
    O1 = OracleSG4(m1.D, m1.L, m1.L, 1, 1, 2, 1, scaleQ=m1.scaleQ)
    psi1 = np.random.default_rng(5).normal(size=(O1.N, 2))
    r1 = O1.hpsi(psi1, type_op=1, V=m1.V(O1.grid_points()), F2=m1.F2.ravel())
    g1 = O1.hpsi(psi1, type_op=1, V_poly=(m1.V.coef, m1.V.expo), F2=m1.F2.ravel())
    assert np.max(np.abs(g1 - r1)) <= 1e-13 * np.max(np.abs(r1))


def test_oracle_type1_coefficient_grids():
    """Type-1 coefficients given as grids (OpGrid(iterm)%Grid): a grid equal
    to the constant everywhere gives the constant-coefficient operator bit
    for bit, a grid zero everywhere drops its term (grid_zero), and a
    Q-dependent grid multiplies its term's derivatives point by point.  One
    thread: the reference's atomic scatter makes the sum order, and so the
    last bits, depend on the thread schedule."""
    D, L = 3, 4
    O = OracleSG4(D, L, L, 1, 1, 2, 1, scaleQ=np.full(D, 0.5))
    rng = np.random.default_rng(12)
    snq = O.sum_nq
    V = rng.normal(size=snq)
    F2 = np.triu(rng.normal(size=(D, D)))
    F1 = rng.normal(size=D)
    psi = rng.normal(size=(O.N, 2))
    ref = O.hpsi(psi, type_op=1, V=V, F2=F2.ravel(), F1=F1, nthreads=1)
    F2g = np.repeat(F2[:, :, None], snq, axis=2)
    F1g = np.repeat(F1[:, None], snq, axis=1)
    assert np.array_equal(O.hpsi(psi, type_op=1, V=V, F2_grid=F2g, F1_grid=F1g, nthreads=1), ref)
    F2z = F2.copy()
    F2z[0, 1] = 0.0
    F2gz = F2g.copy()
    F2gz[0, 1] = 0.0
    assert np.array_equal(O.hpsi(psi, type_op=1, V=V, F2_grid=F2gz, F1_grid=F1g, nthreads=1),
                          O.hpsi(psi, type_op=1, V=V, F2=F2z.ravel(), F1=F1, nthreads=1))
    # a coefficient that is a sum of two grids: the operator is linear in it
    g1 = rng.normal(size=snq)
    g2 = rng.normal(size=snq)
    def one(g):
        G = np.zeros((D, D, snq))
        G[1, 2] = g
        return O.hpsi(psi, type_op=1, F2_grid=G)
    np.testing.assert_allclose(one(g1 + g2), one(g1) + one(g2), rtol=0, atol=1e-12 * np.abs(one(g1 + g2)).max())
