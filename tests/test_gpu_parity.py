"""GPU parity of the SG4 H.psi kernels (through the C ABI) against the CPU oracle.

Tolerance: the benchmark's bar of 1e-12 maximum relative error, measured
block-wise as max|H_gpu - H_oracle| / max|H_oracle| (FP64 throughout; the
GPU reorders sums and uses FMA, so results are not bitwise identical).
"""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elvibrot_gb300 import EVRError, ParamOp, Polynomial, SG4Basis, SG4Tables, sub_scaledOpPsi, sub_TabOpPsi
from elvibrot_gb300.configs import make_model, random_psi
from oracle.oracle import OracleSG4, oracle_tables

pytestmark = pytest.mark.gpu
TOL = 1e-12
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def gpu_apply(op, psi, **kw):
    P = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    H = sub_TabOpPsi(P, op, **kw)
    torch.cuda.synchronize()
    return H.cpu().numpy().T


def oracle_for(model):
    O = OracleSG4(model.D, model.L, model.L, 1, 1, 2, 1, scaleQ=model.scaleQ)
    Q = O.grid_points()
    V = model.V(Q)
    kw = dict(V=V)
    if model.type_op == 1:
        kw.update(type_op=1, F2=model.F2.ravel())
    else:
        tab_l = O.tables()[0]
        nq = np.prod(tab_l + 2, axis=1)
        kw.update(type_op=10, G=model.G_grid(Q, nq))
    return O, kw


def same_inputs_op(O, kw):
    """GPU operator built from the oracle's own tables and operator grids
    (the drop-in descriptor path: bit-identical inputs on both sides)."""
    T = SG4Tables(**oracle_tables(O))
    if kw["type_op"] == 1:
        return ParamOp(T, 1, V=kw.get("V"), F2=kw.get("F2"), F1=kw.get("F1"))
    if kw["type_op"] == 0:
        return ParamOp(T, 0, V=kw.get("V"))
    return ParamOp(T, 10, V=kw.get("V"), G=kw.get("G"), Jac=kw.get("Jac"), sqRho=kw.get("sqRho"))


def check_against_oracle(op, O, kw, psi, label):
    """GPU vs the oracle in double and in extended precision (the yardstick)."""
    got = gpu_apply(op, psi)
    ref = O.hpsi(psi, **kw)
    # extended precision is software binary128 on aarch64: two columns suffice
    ext = O.hpsi(psi[:, :2], extended=True, **kw)
    e_ext, e_ref, e_orc = rel_err(got[:, :2], ext), rel_err(got, ref), rel_err(ref[:, :2], ext)
    print(f"{label}: gpu-vs-extended {e_ext:.2e}  gpu-vs-double {e_ref:.2e}  double-vs-extended {e_orc:.2e}")
    assert e_ext <= TOL and e_ref <= TOL
    return got


def test_launch_geometries_match_oracle_and_each_other():
    """A 7-D type-10 operator: 24 right-hand sides make a plan of more than
    four waves of items (the mid geometry, six CTAs per SM), 2 a small one
    (wide, four per SM); a 6-D operator with 20 takes the narrow geometry.
    Each geometry runs the same arithmetic, so the values agree bit for bit."""
    need_cuda()
    m = make_model(7, 5, 10, 4242)
    O, kw = oracle_for(m)
    op = m.operator()
    psi = random_psi(O.N, 24, 7)
    got = gpu_apply(op, psi)
    assert op.last_geometry() == (2, 6)
    e = rel_err(got, O.hpsi(psi, **kw))
    print(f"7-D L=5 type 10, 24 RHS (mid geometry): gpu-vs-double {e:.2e}")
    assert e <= TOL
    got2 = gpu_apply(op, psi[:, :2])
    assert op.last_geometry() == (0, 4)
    assert np.array_equal(got2, got[:, :2])
    m6 = make_model(6, 7, 10, 4243)
    op6 = m6.operator()
    psi6 = random_psi(op6.basis.N, 20, 8)
    big = gpu_apply(op6, psi6)
    assert op6.last_geometry() == (1, 8)
    small = gpu_apply(op6, psi6[:, :1])
    assert op6.last_geometry() == (0, 4)
    assert np.array_equal(small, big[:, :1])


@pytest.mark.parametrize("D,L,type_op,nrhs", [(3, 6, 1, 1), (3, 6, 1, 5), (4, 5, 10, 7), (6, 4, 10, 3),
                                              (5, 5, 1, 4), (2, 9, 10, 2)])
def test_hpsi_matches_oracle(D, L, type_op, nrhs):
    need_cuda()
    m = make_model(D, L, type_op, 1234 + D * 10 + L)
    O, kw = oracle_for(m)
    psi = random_psi(O.N, nrhs, 99)
    check_against_oracle(same_inputs_op(O, kw), O, kw, psi, f"{D}-D L={L} type {type_op} (oracle tables)")
    op = m.operator()   # product tables + device-evaluated fields
    check_against_oracle(op, O, kw, psi, f"{D}-D L={L} type {type_op} (product tables)")
    assert op.last_launches == 3   # the item kernel + the two ordered-accumulation kernels


def test_type0_and_fields_from_grids():
    need_cuda()
    D, L = 4, 5
    b = SG4Basis(D, L, scaleQ=np.full(D, 0.4))
    O = OracleSG4(D, L, L, 1, 1, 2, 1, scaleQ=np.full(D, 0.4))
    rng = np.random.default_rng(5)
    V = rng.normal(size=b.sum_nq)
    psi = random_psi(b.N, 3, 5)
    op0 = ParamOp(b, 0, V=V)
    assert rel_err(gpu_apply(op0, psi), O.hpsi(psi, type_op=0, V=V)) <= TOL
    # type 10 with explicit G, Jac and sqRho grids (GGiq layout)
    G = rng.normal(size=b.sum_nq * D * D) * 0.1
    Jac = rng.uniform(0.5, 2.0, size=b.sum_nq)
    sq = rng.uniform(0.5, 2.0, size=b.sum_nq)
    op10 = ParamOp(b, 10, V=V, G=G, Jac=Jac, sqRho=sq)
    ref = O.hpsi(psi, type_op=10, V=V, G=G, Jac=Jac, sqRho=sq)
    assert rel_err(gpu_apply(op10, psi), ref) <= TOL
    # type 1 with off-diagonal and first-derivative terms
    F2 = np.triu(rng.normal(size=(D, D)))
    F1 = rng.normal(size=D)
    op1 = ParamOp(b, 1, V=V, F2=F2, F1=F1)
    ref = O.hpsi(psi, type_op=1, V=V, F2=F2.ravel(), F1=F1)
    assert rel_err(gpu_apply(op1, psi), ref) <= TOL


def test_plain_equals_batched_and_scaled_and_complex():
    need_cuda()
    m = make_model(4, 6, 10, 77)
    op = m.operator()
    N = op.basis.N
    psi = random_psi(N, 4, 3)
    P = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    hb = torch.empty_like(P)
    hp = torch.empty_like(P)
    op.hpsi_dev(P, hb)
    op.hpsi_dev(P, hp, plain=True)
    assert op.last_launches == 2 + op.basis.nb_SG
    torch.cuda.synchronize()
    assert rel_err(hp.cpu().numpy(), hb.cpu().numpy()) <= TOL
    # (H - E0)/Esc fused
    E0, Esc = 0.37, 2.5
    hs = sub_scaledOpPsi(P, op, E0, Esc)
    want = (hb - E0 * P) / Esc
    assert rel_err(hs.cpu().numpy(), want.cpu().numpy()) <= TOL
    # complex psi = real operator on Re and Im
    pc = random_psi(N, 3, 4, complex_=True)
    Pc = torch.from_numpy(np.ascontiguousarray(pc.T)).cuda()
    hc = sub_TabOpPsi(Pc, op).cpu().numpy().T
    hr = gpu_apply(op, np.ascontiguousarray(pc.real))
    hi = gpu_apply(op, np.ascontiguousarray(pc.imag))
    assert rel_err(hc, hr + 1j * hi) <= TOL
    # host-pointer path
    hh = op.hpsi_host(psi)
    assert rel_err(hh, hb.cpu().numpy().T) <= TOL


def test_large_terms_use_global_scratch():
    need_cuda()
    # a 7-D L=9 type-10 basis has terms whose D+4 work arrays exceed shared memory
    m = make_model(7, 9, 10, 4242)
    O, kw = oracle_for(m)
    psi = random_psi(O.N, 2, 8)
    op = same_inputs_op(O, kw)
    assert op.basis.max_nq * (7 + 4) > 110 * 1024 // 8
    check_against_oracle(op, O, kw, psi, "7-D L=9 type 10 (oracle tables, global scratch)")
    del op
    check_against_oracle(m.operator(), O, kw, psi, "7-D L=9 type 10 (product tables, global scratch)")


def test_benchmark_6d_workload_full_size():
    need_cuda()
    # 6-D L=8, Q-dependent G, 20 right-hand sides (the benchmark workload)
    m = make_model(6, 8, 10, 20261204)
    O, kw = oracle_for(m)
    psi = random_psi(O.N, 20, 20261204)
    check_against_oracle(same_inputs_op(O, kw), O, kw, psi, "6-D L=8 type 10 x20 (oracle tables)")
    op = m.operator()
    assert (op.basis.N, op.basis.nb_SG, op.basis.sum_nq) == (3003, 2975, 1953127)
    got = check_against_oracle(op, O, kw, psi, "6-D L=8 type 10 x20 (product tables)")
    # linearity: H(a x + b y) = a Hx + b Hy
    comb = gpu_apply(op, 0.3 * psi[:, :1] - 1.7 * psi[:, 1:2])
    assert rel_err(comb, 0.3 * got[:, :1] - 1.7 * got[:, 1:2]) <= TOL


def test_henon_heiles_golden_levels_on_gpu():
    need_cuda()
    c = json.load(open(os.path.join(GOLD, "hh_levels.json")))["cases"]["6D_Davidson_S0"]
    D, L, B = c["D"], c["L"], c["L_TO_nq_B"]
    b = SG4Basis(D, L, L, 1, B, 1, B)
    Q = b.grid_points()
    lam = c["lambda"]
    V = 0.5 * np.sum(Q ** 2, axis=1)
    for i in range(D - 1):
        V += lam * (Q[:, i] ** 2 * Q[:, i + 1] - Q[:, i + 1] ** 3 / 3.0)
    op = ParamOp(b, 1, V=V, F2=-0.5 * np.eye(D))
    H = gpu_apply(op, np.eye(b.N))
    ev = np.sort(np.linalg.eigvalsh(0.5 * (H + H.T)))
    ref = np.array(c["levels_au"])
    assert np.max(np.abs(ev[: len(ref)] - ref)) < 2e-7


def test_errors_are_status_codes():
    need_cuda()
    m = make_model(3, 4, 1, 1)
    op = m.operator()
    N = op.basis.N
    with pytest.raises(EVRError):
        sub_TabOpPsi(torch.zeros((0, N), dtype=torch.float64, device="cuda"), op)
    with pytest.raises(EVRError):
        op.hpsi_dev(torch.zeros((2, N + 1), dtype=torch.float64, device="cuda"),
                    torch.zeros((2, N + 1), dtype=torch.float64, device="cuda"))
    with pytest.raises(EVRError):
        ParamOp(op.basis, 10, V=np.full(op.basis.sum_nq, np.nan))
    # the context stays usable after rejected calls
    psi = random_psi(N, 1, 1)
    O, kw = oracle_for(m)
    assert rel_err(gpu_apply(op, psi), O.hpsi(psi, **kw)) <= TOL


@pytest.mark.parametrize("type_op", [0, 1, 10])
def test_transposed_operator_matches_dense_transpose(type_op):
    """evr_sg4_apply(EVR_APPLY_TRANSPOSE) = (dense oracle H)^T, with non-symmetric
    G and general Jac/rho so every swapped index and scaling is exercised."""
    need_cuda()
    D, L = 4, 4
    b = SG4Basis(D, L, scaleQ=np.full(D, 0.5))
    O = OracleSG4(D, L, L, 1, 1, 2, 1, scaleQ=np.full(D, 0.5))
    rng = np.random.default_rng(11 + type_op)
    kw = dict(type_op=type_op, V=rng.normal(size=b.sum_nq))
    if type_op == 1:
        kw.update(F2=np.triu(rng.normal(size=(D, D))).ravel(), F1=rng.normal(size=D))
        op = ParamOp(b, 1, V=kw["V"], F2=kw["F2"], F1=kw["F1"])
    elif type_op == 10:
        kw.update(G=rng.normal(size=b.sum_nq * D * D), Jac=rng.uniform(0.5, 2, b.sum_nq),
                  sqRho=rng.uniform(0.5, 2, b.sum_nq))
        op = ParamOp(b, 10, V=kw["V"], G=kw["G"], Jac=kw["Jac"], sqRho=kw["sqRho"])
    else:
        op = ParamOp(b, 0, V=kw["V"])
    H = O.hpsi(np.eye(O.N), **kw)
    psi = random_psi(O.N, 3, 2)
    P = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    out = torch.empty_like(P)
    op.hpsi_dev(P, out, transpose=True)
    torch.cuda.synchronize()
    assert rel_err(out.cpu().numpy().T, H.T @ psi) <= TOL
    # and H itself (for type 1 the fused passes with every mixed and first-derivative term)
    op.hpsi_dev(P, out)
    torch.cuda.synchronize()
    assert rel_err(out.cpu().numpy().T, H @ psi) <= TOL
    # complex psi through the transposed operator
    pc = random_psi(O.N, 2, 3, complex_=True)
    Pc = torch.from_numpy(np.ascontiguousarray(pc.T)).cuda()
    oc = torch.empty_like(Pc)
    op.hpsi_dev(Pc, oc, transpose=True)
    torch.cuda.synchronize()
    assert rel_err(oc.cpu().numpy().T, H.T @ pc) <= TOL


def test_autotuner_keeps_results_bitwise():
    """evr_sg4_tune picks the right-hand-side block cap by timing; results do not
    depend on the cap (per-vector arithmetic is the same in every block)."""
    need_cuda()
    m = make_model(5, 6, 10, 20261214)
    op = m.operator()
    P = torch.from_numpy(np.ascontiguousarray(random_psi(op.basis.N, 12, 3).T)).cuda()
    before = torch.empty_like(P)
    op.hpsi_dev(P, before)
    cap, ms = op.tune(12)
    assert cap in (1, 2, 4, 8, 16, 32) and ms > 0.0
    after = torch.empty_like(P)
    op.hpsi_dev(P, after)
    torch.cuda.synchronize()
    assert torch.equal(before, after)


def _time_hpsi(op, P, reps=5):
    out = torch.empty_like(P)
    op.hpsi_dev(P, out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for _ in range(reps):
        e0.record()
        op.hpsi_dev(P, out)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best, out


def test_plan_tuner_every_plan_same_bits_and_cached(tmp_path):
    """The autotuner's search space (geometry x RHS cap x mode-pass mapping)
    never changes the bits; the tuned plan is not slower than the automatic
    one beyond timing noise; its JSON cache gives the same plan without
    timing."""
    need_cuda()
    m = make_model(6, 6, 10, 20261215)
    op = m.operator()
    P = torch.from_numpy(np.ascontiguousarray(random_psi(op.basis.N, 20, 4).T)).cuda()
    t_auto, ref = _time_hpsi(op, P)
    for geo in (0, 1, 2):
        for rmax, split in ((32, 0), (4, 1), (8, 2)):
            op.set_plan(geo, rmax, split)
            out = torch.empty_like(P)
            op.hpsi_dev(P, out)
            torch.cuda.synchronize()
            assert torch.equal(out, ref), (geo, rmax, split)
    op.set_plan()
    cache = str(tmp_path / "tune.json")
    r = op.tune_plan(20, cache_path=cache)
    assert not r["from_cache"] and r["ms"] <= r["default_ms"]
    assert op.get_plan() == (r["geo"], r["rmax"], r["split"])
    t_tuned, out = _time_hpsi(op, P)
    assert torch.equal(out, ref)
    print(f"tuned plan {r}: {t_tuned:.3f} ms vs automatic {t_auto:.3f} ms")
    assert t_tuned <= 1.05 * t_auto
    op2 = m.operator()
    r2 = op2.tune_plan(20, cache_path=cache)
    assert r2["from_cache"] and (r2["geo"], r2["rmax"], r2["split"]) == (r["geo"], r["rmax"], r["split"])
    import json
    assert len(json.load(open(cache))) == 1


def _type1_grids(Q, D, rng, nonzero_pairs=None):
    """Q-dependent type-1 coefficients on the grid points Q[sum_nq, D]:
    F2_ij(Q) = a_ij (1 + 0.2 sin(Q_i + Q_j)), F1_i(Q) = b_i (1 + 0.1 Q_i^2),
    i <= j; one pair left zero everywhere (a grid_zero term)."""
    snq = Q.shape[0]
    F2g = np.zeros((D, D, snq))
    for i in range(D):
        for j in range(i, D):
            if nonzero_pairs is None or (i, j) in nonzero_pairs:
                F2g[i, j] = rng.normal() * (1.0 + 0.2 * np.sin(Q[:, i] + Q[:, j]))
    F2g[0, D - 1] = 0.0
    F1g = rng.normal(size=(D, 1)) * (1.0 + 0.1 * Q.T ** 2)
    return F2g, F1g


@pytest.mark.parametrize("D,L,nrhs", [(3, 5, 2), (5, 7, 20), (7, 5, 20)])
def test_type1_coefficient_grids_match_oracle(D, L, nrhs):
    """CASE 1 with Q-dependent coefficient grids (OpGrid(iterm)%Grid that is
    not grid_cte): GPU term by term vs the oracle, in the wide, narrow
    (5-D, 20 RHS) and mid (7-D, 20 RHS) launch geometries; H^T against the
    dense transpose; a grid that is constant gives the constant-coefficient
    operator."""
    need_cuda()
    sq = np.full(D, 0.45)
    b = SG4Basis(D, L, scaleQ=sq)
    O = OracleSG4(D, L, L, 1, 1, 2, 1, scaleQ=sq)
    rng = np.random.default_rng(40 + D)
    Q = O.grid_points()
    V = rng.normal(size=b.sum_nq)
    F2g, F1g = _type1_grids(Q, D, rng)
    op = ParamOp(b, 1, V=V, F2_grid=F2g, F1_grid=F1g)
    psi = random_psi(b.N, nrhs, 7 + D)
    ref = O.hpsi(psi, type_op=1, V=V, F2_grid=F2g, F1_grid=F1g)
    assert rel_err(gpu_apply(op, psi), ref) <= TOL
    lng = O.hpsi(psi, type_op=1, V=V, F2_grid=F2g, F1_grid=F1g, extended=True)
    assert rel_err(gpu_apply(op, psi), lng) <= TOL
    if D == 3:
        H = O.hpsi(np.eye(O.N), type_op=1, V=V, F2_grid=F2g, F1_grid=F1g)
        P = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
        out = torch.empty_like(P)
        op.hpsi_dev(P, out, transpose=True)
        torch.cuda.synchronize()
        assert rel_err(out.cpu().numpy().T, H.T @ psi) <= TOL
        pc = random_psi(O.N, 2, 3, complex_=True)
        Pc = torch.from_numpy(np.ascontiguousarray(pc.T)).cuda()
        oc = torch.empty_like(Pc)
        op.hpsi_dev(Pc, oc, transpose=True)
        torch.cuda.synchronize()
        assert rel_err(oc.cpu().numpy().T, H.T @ pc) <= TOL
        op.hpsi_dev(Pc, oc)
        torch.cuda.synchronize()
        assert rel_err(oc.cpu().numpy().T, H @ pc) <= TOL
    # constant grids: the constant-coefficient operator (other passes, same operator)
    F2 = np.triu(rng.normal(size=(D, D)))
    F1 = rng.normal(size=D)
    opg = ParamOp(b, 1, V=V, F2_grid=np.repeat(F2[:, :, None], b.sum_nq, axis=2),
                  F1_grid=np.repeat(F1[:, None], b.sum_nq, axis=1))
    opc = ParamOp(b, 1, V=V, F2=F2, F1=F1)
    assert rel_err(gpu_apply(opg, psi), gpu_apply(opc, psi)) <= TOL


def test_type1_coefficient_grids_in_a_multi_context_plan():
    """A context with coefficient grids merged with others: the bits of its own launch."""
    need_cuda()
    from elvibrot_gb300 import MultiOp
    D, L = 4, 6
    b = SG4Basis(D, L, scaleQ=np.full(D, 0.5))
    rng = np.random.default_rng(3)
    F2g, F1g = _type1_grids(b.grid_points(), D, rng)
    opg = ParamOp(b, 1, V=rng.normal(size=b.sum_nq), F2_grid=F2g, F1_grid=F1g)
    ops = [opg, make_model(5, 5, 10, 9).operator(), make_model(3, 6, 1, 8).operator()]
    nrhs = [4, 3, 2]
    psis = [torch.from_numpy(np.ascontiguousarray(random_psi(op.basis.N, r, 20 + k).T)).cuda()
            for k, (op, r) in enumerate(zip(ops, nrhs))]
    ref = []
    for op, P in zip(ops, psis):
        O = torch.empty_like(P)
        op.hpsi_dev(P, O)
        ref.append(O)
    outs = [torch.empty_like(P) for P in psis]
    MultiOp(ops, nrhs).hpsi(psis, outs)
    torch.cuda.synchronize()
    for k in range(3):
        assert torch.equal(outs[k], ref[k]), k
