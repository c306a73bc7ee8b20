"""Device Chebyshev propagation (march_cheby) against the exact propagator.

exp(-i H t) psi0 from a dense diagonalisation of the oracle's H (type 1,
symmetric) is the yardstick; the Chebyshev expansion with enough terms is
exact to rounding, so the bar is 1e-11 on psi and on the autocorrelation.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elvibrot_gb300.configs import make_model
from oracle.oracle import OracleSG4

pytestmark = pytest.mark.gpu


def need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_chebyshev_matches_exact_propagator():
    need_cuda()
    m = make_model(3, 5, 1, 20261205)
    op = m.operator()
    O = OracleSG4(m.D, m.L, m.L, 1, 1, 2, 1, scaleQ=m.scaleQ)
    Q = O.grid_points()
    H = O.hpsi(np.eye(O.N), type_op=1, V=m.V(Q), F2=m.F2.ravel())
    w, U = np.linalg.eigh(0.5 * (H + H.T))
    rng = np.random.default_rng(3)
    # a packet made of the lowest 8 levels with random complex amplitudes, 2 RHS
    amp = (rng.normal(size=(8, 2)) + 1j * rng.normal(size=(8, 2)))
    psi0 = U[:, :8] @ amp
    psi0 /= np.linalg.norm(psi0, axis=0)
    dt, nsteps = 10.0, 12
    margin = 0.05 * (w[-1] - w[0])
    P = torch.from_numpy(np.ascontiguousarray(psi0.T)).cuda()
    ac, used = op.cheby_propagate(P, w[0] - margin, w[-1] + margin, dt, npoly=200, nsteps=nsteps, poly_tol=1e-20)
    got = P.cpu().numpy().T
    t = dt * nsteps
    exact = U @ (np.exp(-1j * w * t)[:, None] * (U.T @ psi0))
    assert np.max(np.abs(got - exact)) / np.max(np.abs(exact)) < 1e-11
    for k in range(nsteps + 1):
        ex = np.sum(np.conj(psi0) * (U @ (np.exp(-1j * w * dt * k)[:, None] * (U.T @ psi0))), axis=0)
        assert np.max(np.abs(ac[k] - ex)) < 1e-11
    assert used < 200


def test_chebyshev_retries_with_larger_hmax():
    need_cuda()
    m = make_model(3, 4, 1, 9)
    op = m.operator()
    O = OracleSG4(m.D, m.L, m.L, 1, 1, 2, 1, scaleQ=m.scaleQ)
    H = O.hpsi(np.eye(O.N), type_op=1, V=m.V(O.grid_points()), F2=m.F2.ravel())
    w, U = np.linalg.eigh(0.5 * (H + H.T))
    psi0 = U[:, :4].sum(axis=1)[:, None] / 2.0 + 0j
    P = torch.from_numpy(np.ascontiguousarray(psi0.T)).cuda()
    # Hmax far below the top of the spectrum: the expansion diverges and the step
    # is redone with Hmax raised (march_cheby :4320-4362)
    ac, used = op.cheby_propagate(P, w[0] - 0.01, w[0] + 0.3 * (w[-1] - w[0]), 5.0, npoly=120, nsteps=2,
                                  poly_tol=1e-18)
    exact = U @ (np.exp(-1j * w * 10.0)[:, None] * (U.T @ psi0))
    assert np.max(np.abs(P.cpu().numpy().T - exact)) < 1e-9


def test_chebyshev_graph_replay_is_bit_identical():
    """Fixed-order steps replayed from a recorded CUDA graph give the same bits
    as eager launches (same kernels, same order)."""
    need_cuda()
    m = make_model(4, 5, 1, 20261207)
    op = m.operator()
    O = OracleSG4(m.D, m.L, m.L, 1, 1, 2, 1, scaleQ=m.scaleQ)
    H = O.hpsi(np.eye(O.N), type_op=1, V=m.V(O.grid_points()), F2=m.F2.ravel())
    w, U = np.linalg.eigh(0.5 * (H + H.T))
    rng = np.random.default_rng(8)
    psi0 = (rng.normal(size=(O.N, 3)) + 1j * rng.normal(size=(O.N, 3)))
    psi0 /= np.linalg.norm(psi0, axis=0)
    margin = 0.05 * (w[-1] - w[0])
    outs = []
    for graph in (False, True):
        P = torch.from_numpy(np.ascontiguousarray(psi0.T)).cuda()
        ac, used = op.cheby_propagate(P, w[0] - margin, w[-1] + margin, 10.0, npoly=30, nsteps=6, graph=graph)
        outs.append((P.cpu(), ac))
    assert torch.equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
    # and the replayed propagation is the exact one
    exact = U @ (np.exp(-1j * w * 60.0)[:, None] * (U.T @ psi0))
    assert np.max(np.abs(outs[1][0].numpy().T - exact)) < 1e-10


def _oc_setup(nsteps, seed=20261206):
    from elvibrot_gb300 import ParamOp
    from elvibrot_gb300.configs import make_dipole
    m = make_model(4, 7, 1, seed)            # the 4-D L=7 optimal-control system
    H0 = m.operator()
    mu_poly = make_dipole(m, seed)
    mu = ParamOp(H0.basis, 0, V_poly=mu_poly)
    O = OracleSG4(m.D, m.L, m.L, 1, 1, 2, 1, scaleQ=m.scaleQ)
    Q = O.grid_points()
    H = O.hpsi(np.eye(O.N), type_op=1, V=m.V(Q), F2=m.F2.ravel())
    Mu = O.hpsi(np.eye(O.N), type_op=0, V=mu_poly(Q))
    w, U = np.linalg.eigh(0.5 * (H + H.T))
    E = np.random.default_rng(seed).normal(0.0, 1e-3, size=nsteps)
    E0 = 0.5 * (w[0] + w[-1])            # RK4 on H0 - E0 (fcn_field's para_H%E0)
    return H0, mu, H, Mu, U, E, E0


def test_rk4_field_matches_dense_rk4():
    need_cuda()
    H0, mu, H, Mu, U, E, E0 = _oc_setup(60)
    dt, nsub = 5.0, 20                       # field intervals of 5 a.u., RK4 steps of 0.25 a.u.
    h = dt / nsub
    psi0 = U[:, 0].astype(np.complex128)
    y = psi0.copy()
    I = np.eye(H.shape[0])
    for k in range(len(E)):                  # dense restatement of march_RK4_field
        A = -1j * (H - E0 * I - E[k] * Mu)
        for _ in range(nsub):
            k1 = A @ y
            k2 = A @ (y + 0.5 * h * k1)
            k3 = A @ (y + 0.5 * h * k2)
            k4 = A @ (y + h * k3)
            y = (y + h / 6.0 * (k1 + 2 * k2 + 2 * k3 + k4)) * np.exp(-1j * E0 * h)
    assert np.abs(np.linalg.norm(y) - 1.0) < 1e-4   # accurate, norm-preserving steps
    P = torch.from_numpy(psi0.copy()).cuda()
    H0.rk4_field(mu, E, P, dt, E0=E0, nsub=nsub)
    assert np.max(np.abs(P.cpu().numpy() - y)) < 1e-12


def test_oc_gradient_matches_central_differences():
    """Adjoint gradient of |<psi_3|psi(T)>|^2 vs central differences (h = 1e-6)
    on 20 random field samples, psi checkpointed every 45 steps."""
    need_cuda()
    nsteps, dt, h, nsub = 120, 5.0, 1e-6, 10
    H0, mu, H, Mu, U, E, E0 = _oc_setup(nsteps)
    psi0 = torch.from_numpy(U[:, 0].astype(np.complex128)).cuda()
    target = torch.from_numpy(U[:, 2].astype(np.complex128)).cuda()
    E = E * 50.0                              # a field strong enough to populate the target
    J, g = H0.oc_gradient(mu, E, psi0, target, dt, checkpoint=45, E0=E0, nsub=nsub)

    def objective(Ek):
        P = psi0.clone()
        H0.rk4_field(mu, Ek, P, dt, E0=E0, nsub=nsub)
        return abs(complex(torch.vdot(target, P).item())) ** 2

    assert abs(objective(E) - J) <= 1e-14 + 1e-12 * J
    ks = np.random.default_rng(1).choice(nsteps, size=20, replace=False)
    fd = []
    for k in ks:
        Ep, Em = E.copy(), E.copy()
        Ep[k] += h
        Em[k] -= h
        fd.append((objective(Ep) - objective(Em)) / (2 * h))
    fd = np.array(fd)
    scale = np.max(np.abs(g))
    print(f"OC gradient: J={J:.6e} max|g|={scale:.3e} max|g-fd|={np.max(np.abs(g[ks]-fd)):.3e}")
    assert np.max(np.abs(g[ks] - fd)) <= 1e-7 * scale
    # the checkpoint spacing does not change the gradient
    J1, g1 = H0.oc_gradient(mu, E, psi0, target, dt, checkpoint=1, E0=E0, nsub=nsub)
    assert np.max(np.abs(g1 - g)) <= 1e-12 * scale


def test_oc_gradient_as_autograd_function():
    """The adjoint gradient exposed to torch autograd inside the test harness
    (the product's C ABI stays torch-free): J(E) as a torch.autograd.Function
    whose backward calls evr_sg4_oc_gradient; torch.autograd.gradcheck compares
    it with central differences on a short field."""
    need_cuda()
    nsteps, dt, nsub = 12, 5.0, 10
    H0, mu, H, Mu, U, E, E0 = _oc_setup(nsteps)
    psi0 = torch.from_numpy(U[:, 0].astype(np.complex128)).cuda()
    target = torch.from_numpy(U[:, 2].astype(np.complex128)).cuda()

    class Yield(torch.autograd.Function):
        @staticmethod
        def forward(ctx, field):
            Ek = field.detach().cpu().numpy().astype(np.float64)
            J, g = H0.oc_gradient(mu, Ek, psi0, target, dt, checkpoint=4, E0=E0, nsub=nsub)
            ctx.save_for_backward(torch.from_numpy(g))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            (g,) = ctx.saved_tensors
            return gJ * g

    field = torch.tensor(E * 200.0, dtype=torch.float64, requires_grad=True)
    J = Yield.apply(field)
    J.backward()
    scale = float(field.grad.abs().max())
    assert scale > 0.0
    assert torch.autograd.gradcheck(Yield.apply, (field,), eps=1e-6, atol=1e-7 * scale, rtol=0.0)


def test_oc_gradient_converges_to_the_build_field_formula():
    """The reference's control update (build_field, sub_control.f90:907-1007)
    is the continuous-time derivative -2 Im(<psi|chi><chi|mu|psi>) (times
    1/(2 alpha)); integrated over each field interval with psi and chi
    propagated exactly (oracle/control.py), it is the limit of the exact
    discrete RK4 adjoint gradient as the RK4 step shrinks.  40 field samples
    of 5 a.u.: with 20 and 40 RK4 steps per sample the gradient approaches
    the formula at fourth order (error ratio near 16), and with 40 steps it
    agrees to 2e-5 of max|g|."""
    from oracle.control import field_gradient
    need_cuda()
    nsteps, dt = 40, 5.0
    H0, mu, H, Mu, U, E, E0 = _oc_setup(nsteps)
    E = E * 50.0
    psi0n, tgtn = U[:, 0].astype(np.complex128), U[:, 2].astype(np.complex128)
    Jref, gref = field_gradient(H, Mu, E, psi0n, tgtn, dt, m=64)
    psi0 = torch.from_numpy(psi0n).cuda()
    target = torch.from_numpy(tgtn).cuda()
    scale = np.max(np.abs(gref))
    errs = {}
    for nsub in (20, 40):
        J, g = H0.oc_gradient(mu, E, psi0, target, dt, checkpoint=7, E0=E0, nsub=nsub)
        errs[nsub] = np.max(np.abs(g - gref)) / scale
        print(f"nsub={nsub}: J={J:.10e} (formula {Jref:.10e}), max|g-g_formula|/max|g| = {errs[nsub]:.3e}")
    assert errs[40] <= 2e-5
    assert errs[20] / errs[40] >= 10.0


def test_rk4_and_gradient_graph_replay_is_bit_identical():
    """Each field interval replayed from its recorded CUDA graph gives the same
    bits as the same kernels launched one by one (forward sweep, and the
    gradient's forward, recompute and adjoint sweeps)."""
    need_cuda()
    H0, mu, H, Mu, U, E, E0 = _oc_setup(30)
    E = E * 50.0
    psi0 = torch.from_numpy(U[:, 0].astype(np.complex128)).cuda()
    target = torch.from_numpy(U[:, 2].astype(np.complex128)).cuda()
    outs = []
    for graph in (False, True):
        P = psi0.clone()
        H0.rk4_field(mu, E, P, 5.0, E0=E0, nsub=4, graph=graph)
        J, g = H0.oc_gradient(mu, E, psi0, target, 5.0, checkpoint=7, E0=E0, nsub=4, graph=graph)
        outs.append((P.cpu(), J, g))
    assert torch.equal(outs[0][0], outs[1][0])
    assert outs[0][1] == outs[1][1]
    assert np.array_equal(outs[0][2], outs[1][2])


def test_rk4_batch_packets_match_single_packet_runs():
    """Three packets, each under its own field, propagated together: every
    packet gets the bits of its own single-packet propagation."""
    need_cuda()
    H0, mu, H, Mu, U, E, E0 = _oc_setup(25)
    rng = np.random.default_rng(77)
    Eb = np.stack([E * 50.0, -E * 20.0, rng.normal(0.0, 0.05, size=len(E))], axis=1)   # (nsteps, 3)
    psi0 = np.stack([U[:, 0], U[:, 1] + 1j * U[:, 2], U[:, 3]]).astype(np.complex128)  # (3, N)
    P = torch.from_numpy(psi0.copy()).cuda()
    H0.rk4_field_batch(mu, Eb, P, 5.0, E0=E0, nsub=3)
    for b in range(3):
        Q = torch.from_numpy(psi0[b].copy()).cuda()
        H0.rk4_field(mu, Eb[:, b], Q, 5.0, E0=E0, nsub=3)
        assert torch.equal(P[b], Q), b


def test_oc_gradient_full_size_matches_central_differences():
    """The optimal-control workload at full size: 4-D L=7, 2000 field samples
    of 5 a.u. (10 RK4 steps each), psi checkpointed every 45 samples; the
    adjoint gradient against central differences (h = 1e-6) on 20 random
    samples, the 40 perturbed fields propagated together as one batch."""
    need_cuda()
    from elvibrot_gb300.configs import config
    cfg = config(3)
    nsteps, dt, h, nsub = 2000, 5.0, 1e-6, 10
    H0, mu, H, Mu, U, _, E0 = _oc_setup(8, seed=cfg["seed"])
    E = np.random.Generator(np.random.PCG64(cfg["seed"])).normal(0.0, 1e-3, size=nsteps)
    psi0 = torch.from_numpy(U[:, 0].astype(np.complex128)).cuda()
    target = torch.from_numpy(U[:, 2].astype(np.complex128)).cuda()
    J, g = H0.oc_gradient(mu, E, psi0, target, dt, checkpoint=45, E0=E0, nsub=nsub)
    ks = np.random.default_rng(2000).choice(nsteps, size=20, replace=False)
    Eb = np.repeat(E[:, None], 2 * len(ks) + 1, axis=1)
    for i, k in enumerate(ks):
        Eb[k, 2 * i] += h
        Eb[k, 2 * i + 1] -= h
    P = psi0[None, :].repeat(Eb.shape[1], 1).contiguous()
    H0.rk4_field_batch(mu, Eb, P, dt, E0=E0, nsub=nsub)
    Js = np.abs((target.conj()[None, :] * P).sum(dim=1).cpu().numpy()) ** 2
    assert abs(Js[-1] - J) <= 1e-12 * J                  # the unperturbed field: the gradient's own J
    fd = (Js[0:-1:2] - Js[1:-1:2]) / (2 * h)
    scale = np.max(np.abs(g))
    err = np.max(np.abs(g[ks] - fd))
    print(f"OC gradient, 2000 samples: J={J:.6e} max|g|={scale:.3e} max|g-fd|={err:.3e} ({err / scale:.2e})")
    assert err <= 1e-7 * scale
