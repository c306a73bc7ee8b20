"""Several channels (electronic states, nb0 > 1) through the GPU path.

A vector holds nb0 blocks of the packed basis (RvecB((ie-1)*Max_nDI + iB));
the operator's V is an nb0 x nb0 matrix on the grid and the derivative terms
act on every channel.  The oracle builds the same H block by block (T + V_aa
on the diagonal, V_ab off it, each applied per Smolyak term), which is how the
CPU test pins it to the reference's 2-state pyrazine autocorrelation; here the
GPU operator must match that H to 1e-12 and its Chebyshev propagation must
reproduce the reference's autocorrelation to the reference's 1e-8.
"""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elvibrot_gb300 import EVRError, ParamOp, SG4Basis
from oracle.oracle import OracleSG4

from test_oracle_golden import pyrazine_model, pyrazine_oracle

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def oracle_blocks(O, Vm, F2, type_op):
    """Dense nb0 N x nb0 N H from the oracle, one block per channel pair."""
    nb0 = Vm.shape[0]
    I = np.eye(O.N)
    rows = []
    for a in range(nb0):
        row = []
        for b in range(nb0):
            if a == b and type_op == 1:
                row.append(O.hpsi(I, type_op=1, V=Vm[a, a], F2=F2.ravel()))
            else:
                row.append(O.hpsi(I, type_op=0, V=Vm[a, b]))
        rows.append(row)
    return np.block(rows)


def gpu_dense(op, n, cplx=False, transpose=False):
    E = torch.eye(n, dtype=torch.complex128 if cplx else torch.float64, device="cuda")
    if cplx:
        E = E * (0.6 + 0.8j)
    out = torch.empty_like(E)
    op.hpsi_dev(E.contiguous(), out, transpose=transpose)
    torch.cuda.synchronize()
    H = out.cpu().numpy().T
    return H / (0.6 + 0.8j) if cplx else H


def pyrazine_gpu(g):
    A, B = g["L_TO_nq_A"], g["L_TO_nq_B"]
    basis = SG4Basis(g["D"], g["L"], g["LB"], A_nb=A, B_nb=B, A_nq=A, B_nq=B, nb0=2)
    O = pyrazine_oracle(g)
    V11, V22, V12, F2 = pyrazine_model(g, O)
    Vm = np.array([[V11, V12], [V12, V22]])
    return basis, O, Vm, F2


def test_pyrazine_operator_matches_oracle_blocks():
    need_cuda()
    g = json.load(open(os.path.join(GOLD, "pyrazine12d.json")))
    basis, O, Vm, F2 = pyrazine_gpu(g)
    assert basis.N == O.N and basis.nvec == 2 * O.N
    np.testing.assert_allclose(basis.grid_points(), O.grid_points(), rtol=0, atol=1e-14)
    op = ParamOp(basis, 1, V=Vm.reshape(4, -1), F2=F2)
    Href = oracle_blocks(O, Vm, F2, 1)
    scale = np.max(np.abs(Href))
    for cplx, tr in ((False, False), (True, False), (False, True)):
        H = gpu_dense(op, basis.nvec, cplx, tr)
        ref = Href.T if tr else Href
        err = np.max(np.abs(H - ref)) / scale
        print(f"pyrazine nb0=2 cplx={cplx} transpose={tr}: {err:.2e}")
        assert err <= 1e-12


def test_pyrazine_chebyshev_autocorrelation_golden():
    need_cuda()
    g = json.load(open(os.path.join(GOLD, "pyrazine12d.json")))
    basis, O, Vm, F2 = pyrazine_gpu(g)
    op = ParamOp(basis, 1, V=Vm.reshape(4, -1), F2=F2)
    w = np.linalg.eigvals(oracle_blocks(O, Vm, F2, 1)).real
    ac = g["autocorr"]
    t = np.array(ac["t_au"])
    psi = torch.zeros((1, basis.nvec), dtype=torch.complex128, device="cuda")
    psi[0, basis.N] = complex(*g["psi0"]["coef"])   # channel 2, all modes in their first function
    margin = 0.05 * (w.max() - w.min())
    got, used = op.cheby_propagate(psi, w.min() - margin, w.max() + margin, float(t[1] - t[0]), npoly=300,
                                   nsteps=len(t) - 1, poly_tol=1e-16)
    got = np.asarray(got)[:, 0]
    err = max(np.max(np.abs(got.real - ac["re"])), np.max(np.abs(got.imag - ac["im"])))
    print(f"GPU Chebyshev pyrazine autocorrelation: max error {err:.2e} (npoly used {used})")
    assert err <= g["criterion"]


def test_three_channels_random_coupling():
    need_cuda()
    D, L, nb0 = 4, 4, 3
    basis = SG4Basis(D, L, L, 1, 1, 2, 1, nb0=nb0)
    O = OracleSG4(D, L, L, 1, 1, 2, 1)
    Q = O.grid_points()
    rng = np.random.default_rng(31)
    Vm = np.empty((nb0, nb0, len(Q)))
    for a in range(nb0):
        for b in range(nb0):
            c = rng.normal(size=D + 1)
            Vm[a, b] = c[0] + Q @ c[1:] + (0.5 * (Q * Q).sum(axis=1) if a == b else 0.0)
    F2 = -0.5 * np.diag(rng.uniform(0.5, 1.5, size=D))
    for type_op in (0, 1):
        op = ParamOp(basis, type_op, V=Vm.reshape(nb0 * nb0, -1), F2=F2 if type_op == 1 else None)
        Href = oracle_blocks(O, Vm, F2, type_op)
        scale = np.max(np.abs(Href))
        for cplx, tr in ((False, False), (True, True)):
            H = gpu_dense(op, basis.nvec, cplx, tr)
            ref = Href.T if tr else Href
            assert np.max(np.abs(H - ref)) / scale <= 1e-12, (type_op, cplx, tr)
        # a block of 5 vectors (odd, so the last work items hold one channel group)
        P = torch.from_numpy(rng.normal(size=(5, basis.nvec))).cuda()
        out = torch.empty_like(P)
        op.hpsi_dev(P, out, E0=0.3, Esc=1.5)
        want = (Href @ P.cpu().numpy().T - 0.3 * P.cpu().numpy().T) / 1.5
        assert np.max(np.abs(out.cpu().numpy().T - want)) / np.max(np.abs(want)) <= 1e-12


def test_channels_type10_matches_oracle_blocks():
    """Type 10 with two and three channels: V couples them (the reference's
    VPsi(:,ib0) = sum_jb0 V(:,ib0,jb0) psi_jb0, formed before the rho
    rescaling), the G-dependent kinetic operator acts on each channel; with
    and without Jac/rho (the in-place and separate-V.x layouts)."""
    need_cuda()
    from elvibrot_gb300.configs import make_model
    for D, L, nb0, with_rho in ((3, 4, 2, False), (4, 3, 3, True)):
        m = make_model(D, L, 10, 4300 + D)
        basis = SG4Basis(D, L, L, 1, 1, 2, 1, nb0=nb0)
        O = OracleSG4(D, L, L, 1, 1, 2, 1)
        Q = O.grid_points()
        nq = np.prod(O.tables()[0] + 2, axis=1)
        G = m.G_grid(Q, nq)
        rng = np.random.default_rng(44 + D)
        Vm = np.empty((nb0, nb0, len(Q)))
        for a in range(nb0):
            for b in range(nb0):
                c = rng.normal(size=D + 1) * 0.1
                Vm[a, b] = c[0] + Q @ c[1:] + (0.5 * (Q * Q).sum(axis=1) if a == b else 0.0)
        extra = {}
        if with_rho:
            extra = dict(Jac=1.0 + 0.1 * np.cos(Q.sum(axis=1)), sqRho=1.0 + 0.05 * np.sin(Q[:, 0]))
        I = np.eye(O.N)
        Href = np.block([[O.hpsi(I, type_op=10, V=Vm[a, a], G=G, **extra) if a == b else O.hpsi(I, type_op=0, V=Vm[a, b])
                          for b in range(nb0)] for a in range(nb0)])
        op = ParamOp(basis, 10, V=Vm.reshape(nb0 * nb0, -1), G=G, **extra)
        scale = np.max(np.abs(Href))
        for cplx, tr in ((False, False), (True, False), (False, True)):
            H = gpu_dense(op, basis.nvec, cplx, tr)
            ref = Href.T if tr else Href
            err = np.max(np.abs(H - ref)) / scale
            print(f"type 10, {D}-D L={L}, nb0={nb0}, rho={with_rho}, cplx={cplx}, transpose={tr}: {err:.2e}")
            assert err <= 1e-12


def test_channels_polynomial_v_matches_grid_v():
    """The nb0 x nb0 electronic matrix given as polynomials (one coefficient
    block per element over shared monomials, evaluated on the device) gives
    the operator of the same matrix given as grids, for types 1 and 10; the
    grid form is itself checked against the oracle's channel blocks above."""
    need_cuda()
    from elvibrot_gb300 import Polynomial
    D, L, nb0 = 3, 5, 3
    basis = SG4Basis(D, L, L, 1, 1, 2, 1, nb0=nb0)
    Q = basis.grid_points()
    rng = np.random.default_rng(71)
    expo = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [2, 0, 0], [0, 2, 0], [0, 0, 2], [1, 1, 1]],
                     dtype=np.int32)
    coef = rng.normal(0.0, 0.05, size=(nb0 * nb0, len(expo)))
    for a in range(nb0):
        coef[a * nb0 + a, 4:7] += 0.5                              # harmonic diagonal elements
    Vg = np.stack([Polynomial(coef[k], expo)(Q) for k in range(nb0 * nb0)])
    G1 = 0.02 * rng.normal(size=(D, D, D))
    G1 = 0.5 * (G1 + G1.transpose(1, 0, 2))
    for type_op in (1, 10):
        kw = dict(F2=-0.5 * np.eye(D)) if type_op == 1 else dict(G0=np.eye(D), G1=G1)
        a_op = ParamOp(basis, type_op, V_poly=Polynomial(coef, expo), **kw)
        b_op = ParamOp(basis, type_op, V=Vg.reshape(nb0 * nb0, -1), **kw)
        for cplx, tr in ((False, False), (True, True)):
            Ha = gpu_dense(a_op, basis.nvec, cplx, tr)
            Hb = gpu_dense(b_op, basis.nvec, cplx, tr)
            err = np.max(np.abs(Ha - Hb)) / np.max(np.abs(Hb))
            print(f"type {type_op}, nb0={nb0}, cplx={cplx}, transpose={tr}: polynomial vs grid V {err:.2e}")
            assert err <= 1e-13
    with pytest.raises(EVRError):                                  # wrong number of coefficients
        ParamOp(basis, 1, V_poly=Polynomial(coef[0], expo), F2=-0.5 * np.eye(D))


def test_channel_coupled_derivative_terms_match_oracle_blocks():
    """Type-1 derivative terms whose coefficient grids couple channels
    (GridOp(:,a,b,iterm) with a != b: non-adiabatic derivative couplings):
    the dense GPU H, real and complex, H and H^T, against the oracle's
    blocks H_ab = V_ab + sum_t GridOp_t(:,a,b) Der_t, each a one-channel
    type-1 operator with coefficient grids."""
    need_cuda()
    D, L, nb0 = 3, 4, 2
    basis = SG4Basis(D, L, L, 1, 1, 2, 1, nb0=nb0)
    O = OracleSG4(D, L, L, 1, 1, 2, 1)
    Q = O.grid_points()
    snq = len(Q)
    rng = np.random.default_rng(77)
    Vm = np.empty((nb0, nb0, snq))
    F2g = np.zeros((D, D, nb0, nb0, snq))
    F1g = np.zeros((D, nb0, nb0, snq))
    for a in range(nb0):
        for b in range(nb0):
            c = rng.normal(size=D + 1)
            Vm[a, b] = c[0] + Q @ c[1:] + (0.5 * (Q * Q).sum(axis=1) if a == b else 0.0)
            for i in range(D):
                for j in range(i, D):
                    if a == b or (i, j) == (0, 1):   # kinetic terms on each channel, one coupled mixed term
                        F2g[i, j, a, b] = (-0.5 if i == j else 0.1) * rng.uniform(0.5, 1.5) * (1 + 0.1 * np.cos(Q[:, j]))
            if a != b:                                # first-derivative couplings
                F1g[:, a, b] = rng.normal(size=(D, 1)) * 0.2 * (1 + 0.1 * Q.T)
    op = ParamOp(basis, 1, V=Vm.reshape(nb0 * nb0, -1), F2_grid=F2g.reshape(-1), F1_grid=F1g.reshape(-1))
    I = np.eye(O.N)
    Href = np.block([[O.hpsi(I, type_op=1, V=Vm[a, b], F2_grid=F2g[:, :, a, b], F1_grid=F1g[:, a, b])
                      for b in range(nb0)] for a in range(nb0)])
    scale = np.max(np.abs(Href))
    for cplx, tr in ((False, False), (False, True), (True, False), (True, True)):
        H = gpu_dense(op, basis.nvec, cplx, tr)
        ref = Href.T if tr else Href
        assert np.max(np.abs(H - ref)) / scale <= 1e-12, (cplx, tr)
