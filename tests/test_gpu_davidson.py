"""Device block Davidson (sub_propagation_Davidson) against dense diagonalisation.

Bar: eigenvalues within 1e-6 cm^-1 (4.556e-12 hartree) of the dense
eigenvalues of the same operator -- H itself when it is symmetric (type 1),
its symmetric part (H + H^T)/2 otherwise (type 10 on nq > nb grids is not
symmetric; the reference symmetrises the projected matrix, sub_hermitic_H).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elvibrot_gb300.configs import make_model
from oracle.oracle import OracleSG4

pytestmark = pytest.mark.gpu
CM1 = 4.556335252767e-6          # hartree per cm^-1
TOL_E = 1e-6 * CM1


def need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def dense_h_oracle(m):
    O = OracleSG4(m.D, m.L, m.L, 1, 1, 2, 1, scaleQ=m.scaleQ)
    Q = O.grid_points()
    kw = dict(V=m.V(Q), type_op=m.type_op)
    if m.type_op == 1:
        kw["F2"] = m.F2.ravel()
    else:
        kw["G"] = m.G_grid(Q, np.prod(O.tables()[0] + 2, axis=1))
    return O.hpsi(np.eye(O.N), **kw)


def dense_h_gpu(op):
    N = op.basis.N
    H = np.empty((N, N))
    for n0 in range(0, N, 256):
        m = min(256, N - n0)
        E = torch.zeros((m, N), dtype=torch.float64, device="cuda")
        E[torch.arange(m), torch.arange(n0, n0 + m)] = 1.0
        out = torch.empty_like(E)
        op.hpsi_dev(E, out)
        torch.cuda.synchronize()
        H[:, n0:n0 + m] = out.cpu().numpy().T
    return H


def test_davidson_3d_type1_10_levels():
    need_cuda()
    m = make_model(3, 6, 1, 20261203)       # the 3-D L=6 workload
    op = m.operator()
    ev, vec, rs, its = op.davidson(10, conv_resi=1e-9, max_it=300)
    ref = np.linalg.eigvalsh(dense_h_oracle(m))[:10]
    assert np.max(np.abs(ev - ref)) <= TOL_E, (ev - ref)
    assert np.all(rs < 1e-9)


def test_davidson_type10_symmetrised_with_preconditioner():
    need_cuda()
    m = make_model(6, 5, 10, 77)
    op = m.operator()
    H = dense_h_oracle(m)
    ref = np.linalg.eigvalsh(0.5 * (H + H.T))[:20]
    d = op.diagonal()
    np.testing.assert_allclose(d.cpu().numpy(), np.diag(H), rtol=0, atol=1e-12 * np.abs(np.diag(H)).max())
    ev, vec, rs, its = op.davidson(20, max_subspace=60, conv_resi=1e-8, symmetrize=True, diag=d, max_it=500)
    assert np.max(np.abs(ev - ref)) <= TOL_E, (ev - ref)
    # Ritz vectors are orthonormal eigenvectors of the symmetric part
    X = vec.cpu().numpy().T
    assert np.max(np.abs(X.T @ X - np.eye(20))) < 1e-10
    Hs = 0.5 * (H + H.T)
    assert np.max(np.linalg.norm(Hs @ X - X * ev, axis=0)) < 2e-8


def test_davidson_benchmark_6d_20_levels():
    """The 6-D L=8 benchmark operator: 20 levels, restart at 60, residual 1e-8."""
    need_cuda()
    m = make_model(6, 8, 10, 20261204)
    op = m.operator()
    d = op.diagonal()
    ev, vec, rs, its = op.davidson(20, max_subspace=60, conv_resi=1e-8, symmetrize=True, diag=d, max_it=1000)
    H = dense_h_gpu(op)                     # GPU operator, itself parity-checked in test_gpu_parity
    ref = np.linalg.eigvalsh(0.5 * (H + H.T))[:20]
    print(f"6-D L=8 Davidson: {its} iterations, max |dE| {np.max(np.abs(ev - ref)):.2e} hartree")
    assert np.max(np.abs(ev - ref)) <= TOL_E


def test_davidson_graph_replay_is_bit_identical():
    """Each iteration replays two recorded CUDA graphs (Ritz vectors and
    residual norms; the expansion with its H.psi and projected matrix); the
    same steps launched one by one give the same bits."""
    need_cuda()
    m = make_model(5, 6, 10, 78)
    op = m.operator()
    d = op.diagonal()
    runs = [op.davidson(12, block=6, max_subspace=30, conv_resi=1e-9, symmetrize=True, diag=d, max_it=500,
                        graph=g) for g in (False, True)]
    assert runs[0][3] == runs[1][3]                      # iterations
    assert np.array_equal(runs[0][0], runs[1][0])        # eigenvalues
    assert torch.equal(runs[0][1], runs[1][1])           # Ritz vectors
    assert np.array_equal(runs[0][2], runs[1][2])        # residual norms


def test_termwise_diagonal_matches_unit_vector_diagonal():
    """evr_sg4_diagonal (each term's diagonal as a grid->basis transform of its
    fields with per-mode pattern matrices) against H applied to blocks of
    unit vectors, to 1e-12 of the largest entry: type 10 with Q-dependent G,
    type 10 without G, type 1 with off-diagonal F2 and F1 terms, type 0."""
    need_cuda()
    from elvibrot_gb300 import ParamOp
    from elvibrot_gb300.configs import make_dipole
    m10 = make_model(5, 6, 10, 91)
    ops = [m10.operator()]
    b = ops[0].basis
    ops.append(ParamOp(b, 10, V_poly=m10.V))                        # G = identity
    rng = np.random.default_rng(92)
    F2 = np.triu(rng.normal(0.0, 0.3, size=(5, 5)))
    F1 = rng.normal(0.0, 0.2, size=5)
    ops.append(ParamOp(b, 1, V_poly=m10.V, F2=F2, F1=F1))
    ops.append(ParamOp(b, 0, V_poly=make_dipole(m10, 93)))
    for k, op in enumerate(ops):
        d_fast = op.diagonal()
        d_ref = op.diagonal(by_apply=True)
        torch.cuda.synchronize()
        err = float((d_fast - d_ref).abs().max() / d_ref.abs().max())
        print(f"operator {k}: term-wise vs unit-vector diagonal {err:.2e}")
        assert err <= 1e-12, (k, err)
