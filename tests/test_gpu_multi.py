"""Several independent Hamiltonians in one persistent launch (evr_sg4_multi_*).

The merged work list runs every (context, term, rhs block) item with the same
kernel code and block sizes as the single-context launch, and each context's
contributions go through the same ordered accumulation, so the results must be
bit-identical to one evr_sg4_hpsi call per context.  The lock-step Chebyshev
propagator is checked the same way against evr_sg4_cheby_propagate at fixed
order, and against the exact propagator of the oracle's dense H.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elvibrot_gb300 import EVRError, MultiOp, ParamOp, hpsi_multi
from elvibrot_gb300.configs import make_dipole, make_model
from oracle.oracle import OracleSG4

pytestmark = pytest.mark.gpu


def need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _uneven_ops():
    """Contexts of different D, L and operator type; the 7-D L=9 type-10
    operator has terms that only fit in the global-scratch slabs."""
    out = []
    for D, L, t, seed in ((3, 6, 1, 11), (4, 5, 10, 12), (7, 9, 10, 13), (5, 4, 1, 14)):
        out.append(make_model(D, L, t, seed).operator())
    m = make_model(2, 9, 1, 15)
    b = m.operator().basis
    out.append(ParamOp(b, 0, V_poly=make_dipole(m, 15)))      # a type-0 (multiplicative) operator
    return out


def _rand(op, nrhs, cplx, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    a = torch.randn((nrhs, op.basis.N), generator=g, dtype=torch.float64)
    if cplx:
        a = a + 1j * torch.randn((nrhs, op.basis.N), generator=g, dtype=torch.float64)
    return a.cuda().contiguous()


@pytest.mark.parametrize("cplx,transpose", [(False, False), (True, False), (False, True)])
def test_multi_matches_one_launch_per_context(cplx, transpose):
    need_cuda()
    ops = _uneven_ops()
    nrhs = [3, 5, 2, 4, 1]
    psis = [_rand(op, r, cplx, 100 + k) for k, (op, r) in enumerate(zip(ops, nrhs))]
    E0 = [0.0, 0.3, -0.1, 0.0, 2.0]
    Esc = [1.0, 2.5, 1.0, 0.5, 1.0]
    ref = []
    for op, P, e0, es in zip(ops, psis, E0, Esc):
        O = torch.empty_like(P)
        op.hpsi_dev(P, O, E0=e0, Esc=es, transpose=transpose)
        ref.append(O)
    plan = MultiOp(ops, nrhs, complex_=cplx, transpose=transpose)
    outs = [torch.full_like(P, float("nan")) for P in psis]
    plan.hpsi(psis, outs, E0=E0, Esc=Esc)
    torch.cuda.synchronize()
    assert plan.last_launches() == 1 + 2 * len(ops)
    for k, (a, b) in enumerate(zip(outs, ref)):
        assert torch.equal(a, b), f"context {k}: max diff {(a - b).abs().max().item():.3e}"
    # the plan is reusable, and the one-shot form gives the same numbers
    plan.hpsi(psis, outs, E0=E0, Esc=Esc)
    outs2 = [torch.empty_like(P) for P in psis]
    hpsi_multi(ops, psis, outs2, E0=E0, Esc=Esc, transpose=transpose)
    torch.cuda.synchronize()
    for a, b, c in zip(outs, outs2, ref):
        assert torch.equal(a, c) and torch.equal(b, c)


def test_multi_two_launch_groups():
    """Contexts with D <= 6 whose items fill a narrow launch run in a launch
    of their own (eight CTAs per SM), the others in a second one; every
    context's values are the bits of its own single launch."""
    need_cuda()
    ops = [make_model(6, 7, 10, 51).operator(), make_model(7, 4, 1, 52).operator(),
           make_model(3, 5, 1, 53).operator()]
    nrhs = [20, 3, 2]
    psis = [_rand(op, r, False, 60 + k) for k, (op, r) in enumerate(zip(ops, nrhs))]
    ref = []
    for op, P in zip(ops, psis):
        O = torch.empty_like(P)
        op.hpsi_dev(P, O)
        ref.append(O)
    plan = MultiOp(ops, nrhs)
    outs = [torch.full_like(P, float("nan")) for P in psis]
    plan.hpsi(psis, outs)
    torch.cuda.synchronize()
    assert plan.last_launches() == 2 + 2 * 3
    for k in range(3):
        assert torch.equal(outs[k], ref[k]), f"context {k}"
    # with the 7-D context skipped only the narrow launch runs
    outs2 = [torch.full_like(P, 7.0) for P in psis]
    plan.hpsi([psis[0], None, psis[2]], outs2)
    torch.cuda.synchronize()
    assert plan.last_launches() == 1 + 2 * 2
    assert torch.equal(outs2[0], ref[0]) and torch.equal(outs2[2], ref[2]) and torch.all(outs2[1] == 7.0)
    groups = plan.groups()
    assert len(groups) == 2 and groups[0][0] == 1 and all(n > 0 for _, n in groups)
    # a geometry named on every context of a group is the group's; same bits in each
    for geo in (0, 2):
        ops[1].set_plan(geo)
        p2 = MultiOp(ops, nrhs)
        assert p2.groups()[1][0] == geo and p2.groups()[0][0] == 1
        outs3 = [torch.full_like(P, float("nan")) for P in psis]
        p2.hpsi(psis, outs3)
        torch.cuda.synchronize()
        for k in range(3):
            assert torch.equal(outs3[k], ref[k]), (geo, k)
    ops[1].set_plan(-1)


def test_multi_more_contexts_than_one_parameter_block():
    """70 contexts: more than one launch's parameter block holds (64), so the
    plan runs them in two launches; every context gets the bits of its own
    launch, also with contexts of both launches skipped."""
    need_cuda()
    ops = [make_model(2 + k % 3, 3 + k % 4, 1 if k % 2 else 10, 200 + k).operator() for k in range(70)]
    nrhs = [1 + k % 3 for k in range(70)]
    psis = [_rand(op, r, False, 300 + k) for k, (op, r) in enumerate(zip(ops, nrhs))]
    ref = []
    for op, P in zip(ops, psis):
        O = torch.empty_like(P)
        op.hpsi_dev(P, O)
        ref.append(O)
    plan = MultiOp(ops, nrhs)
    groups = plan.groups()
    assert len(groups) == 2 and all(n > 0 for _, n in groups)
    outs = [torch.full_like(P, float("nan")) for P in psis]
    plan.hpsi(psis, outs)
    torch.cuda.synchronize()
    assert plan.last_launches() == 2 + 2 * 70
    for k in range(70):
        assert torch.equal(outs[k], ref[k]), f"context {k}"
    skip = {3, 40, 65, 69}
    outs2 = [torch.full_like(P, 7.0) for P in psis]
    plan.hpsi([None if k in skip else P for k, P in enumerate(psis)], outs2)
    torch.cuda.synchronize()
    for k in range(70):
        assert torch.all(outs2[k] == 7.0) if k in skip else torch.equal(outs2[k], ref[k]), f"context {k}"


def test_multi_skips_null_contexts_and_leaves_contexts_usable():
    need_cuda()
    ops = _uneven_ops()[:4]
    nrhs = [2, 2, 1, 3]
    psis = [_rand(op, r, False, 200 + k) for k, (op, r) in enumerate(zip(ops, nrhs))]
    plan = MultiOp(ops, nrhs)
    sentinel = [torch.full_like(P, 7.0) for P in psis]
    plan.hpsi([psis[0], None, psis[2], None], sentinel)
    torch.cuda.synchronize()
    assert plan.last_launches() == 1 + 2 * 2
    for k in (1, 3):
        assert torch.all(sentinel[k] == 7.0)
    for k in (0, 2):
        O = torch.empty_like(psis[k])
        ops[k].hpsi_dev(psis[k], O)
        assert torch.equal(sentinel[k], O)
    # a single-context call with another nrhs in between leaves the plan intact
    P7 = _rand(ops[1], 7, False, 5)
    ops[1].hpsi_dev(P7, torch.empty_like(P7))
    outs = [torch.empty_like(P) for P in psis]
    plan.hpsi(psis, outs)
    for k in range(4):
        O = torch.empty_like(psis[k])
        ops[k].hpsi_dev(psis[k], O)
        assert torch.equal(outs[k], O)


def test_multi_rejects_a_changed_operator_and_bad_lists():
    need_cuda()
    m = make_model(3, 4, 1, 21)
    op = m.operator()
    op2 = make_model(3, 5, 10, 22).operator()
    plan = MultiOp([op, op2], [1, 1])
    P = [_rand(op, 1, False, 1), _rand(op2, 1, False, 2)]
    with pytest.raises(EVRError):
        plan.hpsi(P, [torch.empty_like(x) for x in P[:1]])
    with pytest.raises(EVRError):
        plan.hpsi([None, None], [torch.empty_like(x) for x in P])
    with pytest.raises(EVRError):
        plan.hpsi([P[0], P[1][:, :-1].contiguous()], [torch.empty_like(x) for x in P])
    # another operator type on a context invalidates the plan (its work split
    # depends on the type's buffer count)
    op.type_op = 10
    op.set_operator(V=m.V(op.basis.grid_points()), G0=np.eye(3), G1=np.zeros((3, 3, 3)))
    with pytest.raises(EVRError, match="changed"):
        plan.hpsi(P, [torch.empty_like(x) for x in P])
    with pytest.raises(EVRError):
        MultiOp([op, op2], [1, 0])
    with pytest.raises(EVRError):
        MultiOp([op], [2]).cheby_propagate([_rand(op, 2, True, 3)], [0.0], [1.0], 1.0, 10, 1)


def _dense(m):
    O = OracleSG4(m.D, m.L, m.L, 1, 1, 2, 1, scaleQ=m.scaleQ)
    H = O.hpsi(np.eye(O.N), type_op=1, V=m.V(O.grid_points()), F2=m.F2.ravel())
    return np.linalg.eigh(0.5 * (H + H.T))


def test_multi_chebyshev_matches_single_context_and_exact():
    need_cuda()
    models = [make_model(3, 5, 1, 31), make_model(4, 4, 1, 32), make_model(2, 7, 1, 33)]
    ops = [m.operator() for m in models]
    nrhs = [2, 1, 3]
    spec = [_dense(m) for m in models]
    Hmin = [w[0] - 0.05 * (w[-1] - w[0]) for w, _ in spec]
    Hmax = [w[-1] + 0.05 * (w[-1] - w[0]) for w, _ in spec]
    dt, npoly, nsteps = 10.0, 30, 4       # the order of the uneven-instance workload
    psis = []
    for k, (op, r) in enumerate(zip(ops, nrhs)):
        P = _rand(op, r, True, 300 + k)
        psis.append(P / torch.linalg.vector_norm(P, dim=1, keepdim=True))
    start = [P.cpu().numpy() for P in psis]
    single = [P.clone() for P in psis]
    ac_single = []
    for op, P, a, b in zip(ops, single, Hmin, Hmax):
        ac, used = op.cheby_propagate(P, a, b, dt, npoly=npoly, nsteps=nsteps, poly_tol=0.0, graph=False)
        ac_single.append(ac)
    plan = MultiOp(ops, nrhs, complex_=True)
    ac_multi = plan.cheby_propagate(psis, Hmin, Hmax, dt, npoly, nsteps)
    torch.cuda.synchronize()
    for k in range(3):
        d = (psis[k] - single[k]).abs().max().item()
        assert d <= 1e-14, f"context {k}: multi vs single {d:.3e}"
        assert np.max(np.abs(ac_multi[k] - ac_single[k])) <= 1e-14
        w, U = spec[k]
        ex = U @ (np.exp(-1j * w * dt * nsteps)[:, None] * (U.T @ start[k].T))
        assert np.max(np.abs(psis[k].cpu().numpy().T - ex)) < 1e-10
        for j in range(nsteps + 1):
            e = np.sum(np.conj(start[k].T) * (U @ (np.exp(-1j * w * dt * j)[:, None] * (U.T @ start[k].T))), axis=0)
            assert np.max(np.abs(ac_multi[k][j] - e)) < 1e-10


def test_multi_chebyshev_redoes_diverging_contexts_alone():
    need_cuda()
    models = [make_model(3, 4, 1, 41), make_model(3, 5, 1, 42)]
    ops = [m.operator() for m in models]
    spec = [_dense(m) for m in models]
    # context 1's Hmax is far too low: its steps diverge and are redone with a
    # larger Hmax, context 0 goes through in one attempt
    Hmin = [w[0] - 0.01 for w, _ in spec]
    Hmax = [spec[0][0][-1] + 0.01, spec[1][0][0] + 0.3 * (spec[1][0][-1] - spec[1][0][0])]
    psis, start = [], []
    for k, (w, U) in enumerate(spec):
        p0 = U[:, :4].sum(axis=1)[:, None] / 2.0 + 0j
        start.append(p0)
        psis.append(torch.from_numpy(np.ascontiguousarray(p0.T)).cuda())
    plan = MultiOp(ops, [1, 1], complex_=True)
    plan.cheby_propagate(psis, Hmin, Hmax, 5.0, 120, 2)
    for k, (w, U) in enumerate(spec):
        ex = U @ (np.exp(-1j * w * 10.0)[:, None] * (U.T @ start[k]))
        assert np.max(np.abs(psis[k].cpu().numpy().T - ex)) < 1e-9


def test_uneven_64_instances_lock_step_chebyshev():
    """The uneven-instance workload itself: 64 seeded Hamiltonians (D 3..9,
    L 4..10, type 1) with 8 complex packets each, propagated 5 steps of an
    order-30 Chebyshev expansion (dt = 10 a.u.) in lock-step, one merged
    H.psi launch per expansion order.  Each instance's packets keep their
    norm to 1e-11, and the 56 smallest instances (the per-instance reruns of
    the 8 largest would double the test's minutes) agree with their own
    single-context evr_sg4_cheby_propagate at the same fixed order to 1e-14
    (the bar of the small lock-step test above)."""
    need_cuda()
    from elvibrot_gb300.configs import uneven_instances
    models = uneven_instances(64)
    ops = [m.operator() for m in models]
    n, nrhs, dt, npoly, nsteps = len(ops), 8, 10.0, 30, 5
    # spectral bounds: power iteration on H and on Hmax - H, one real vector per instance
    p1 = MultiOp(ops, [1] * n)
    g = torch.Generator(device="cpu").manual_seed(5)
    v = [torch.randn((1, op.basis.N), generator=g, dtype=torch.float64).cuda() for op in ops]
    hv = [torch.empty_like(x) for x in v]
    for _ in range(40):
        v = [x / torch.linalg.vector_norm(x) for x in v]
        p1.hpsi(v, hv)
        top = np.array([float((a * b).sum()) for a, b in zip(v, hv)])
        v, hv = hv, v
    Hmax = top * 1.1
    v = [torch.randn((1, op.basis.N), generator=g, dtype=torch.float64).cuda() for op in ops]
    for _ in range(40):
        v = [x / torch.linalg.vector_norm(x) for x in v]
        p1.hpsi(v, hv, E0=list(Hmax), Esc=[-1.0] * n)
        low = Hmax - np.array([float((a * b).sum()) for a, b in zip(v, hv)])
        v, hv = hv, v
    Hmin = low - 0.1 * (Hmax - low)
    psis = []
    for k, op in enumerate(ops):
        P = _rand(op, nrhs, True, 500 + k)
        psis.append(P / torch.linalg.vector_norm(P, dim=1, keepdim=True))
    start = [P.clone() for P in psis]
    plan = MultiOp(ops, [nrhs] * n, complex_=True)
    ac = plan.cheby_propagate(psis, list(Hmin), list(Hmax), dt, npoly, nsteps)
    torch.cuda.synchronize()
    drift = max(float(torch.linalg.vector_norm(P, dim=1).sub(1.0).abs().max()) for P in psis)
    print(f"64 instances x 8 packets, {nsteps} lock-step order-{npoly} steps: max norm drift {drift:.2e}")
    assert drift <= 1e-11
    sizes = [op.basis.sum_nq for op in ops]
    small = sorted(range(n), key=lambda k: sizes[k])[:56]
    for k in small:
        P = start[k].clone()
        a1, used = ops[k].cheby_propagate(P, Hmin[k], Hmax[k], dt, npoly=npoly, nsteps=nsteps, poly_tol=0.0,
                                          graph=False)
        d = (P - psis[k]).abs().max().item()
        assert d <= 1e-14, (k, d)
        assert np.max(np.abs(a1 - ac[k])) <= 1e-14, k


def test_multi_chebyshev_graph_replay_is_bit_identical():
    """Lock-step steps replayed from the recorded CUDA graph of a whole step
    give the same bits as the same kernels launched one by one, also when a
    diverging context is redone eagerly between replays."""
    need_cuda()
    models = [make_model(3, 5, 1, 61), make_model(4, 4, 1, 62), make_model(2, 7, 1, 63)]
    ops = [m.operator() for m in models]
    nrhs = [2, 1, 3]
    spec = [_dense(m) for m in models]
    Hmin = [w[0] - 0.05 * (w[-1] - w[0]) for w, _ in spec]
    Hmax = [w[-1] + 0.05 * (w[-1] - w[0]) for w, _ in spec]
    Hmax[1] = spec[1][0][0] + 0.4 * (spec[1][0][-1] - spec[1][0][0])   # context 1 diverges and is redone
    start = []
    for k, (op, r) in enumerate(zip(ops, nrhs)):
        P = _rand(op, r, True, 600 + k)
        start.append(P / torch.linalg.vector_norm(P, dim=1, keepdim=True))
    outs = []
    for graph in (False, True):
        psis = [P.clone() for P in start]
        plan = MultiOp(ops, nrhs, complex_=True)
        ac = plan.cheby_propagate(psis, Hmin, Hmax, 10.0, 30, 4, graph=graph)
        torch.cuda.synchronize()
        outs.append((psis, ac))
    for k in range(3):
        assert torch.equal(outs[0][0][k], outs[1][0][k]), k
        assert np.array_equal(outs[0][1][k], outs[1][1][k]), k
