"""Operator fields streamed per slice of Smolyak terms (evr_sg4_set_field_budget).

With a budget below the size of the analytic fields (V polynomial, affine G),
the context keeps only their coefficients and each H.psi evaluates them slice
by slice.  The per-term contributions and their ordered accumulation are the
same, so streamed and resident operators must agree bit for bit; the 12-D
case is also checked against the oracle.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elvibrot_gb300 import EVRError, MultiOp
from elvibrot_gb300.configs import make_model

from oracle.oracle import OracleSG4
from test_gpu_parity import check_against_oracle, oracle_for

pytestmark = pytest.mark.gpu


def need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def field_bytes(m, op):
    return op.basis.sum_nq * 8 * (1 + (m.D * m.D if m.type_op == 10 else 0))


def _rand(N, nrhs, cplx, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    a = torch.randn((nrhs, N), generator=g, dtype=torch.float64)
    if cplx:
        a = a + 1j * torch.randn((nrhs, N), generator=g, dtype=torch.float64)
    return a.cuda().contiguous()


@pytest.mark.parametrize("D,L,type_op,parts", [(4, 6, 10, 5), (5, 5, 1, 3), (3, 8, 10, 40)])
def test_streamed_fields_are_bit_identical_to_resident(D, L, type_op, parts):
    need_cuda()
    m = make_model(D, L, type_op, 20261210 + D)
    res = m.operator()
    st = m.operator(field_budget=field_bytes(m, res) // parts)
    assert res.field_slices == 0 and st.field_slices >= parts
    N = res.basis.N
    for cplx, transpose, nrhs in ((False, False, 7), (True, False, 3), (False, True, 4)):
        P = _rand(N, nrhs, cplx, 5 + nrhs)
        a, b = torch.empty_like(P), torch.empty_like(P)
        res.hpsi_dev(P, a, E0=0.1, Esc=2.0, transpose=transpose)
        st.hpsi_dev(P, b, E0=0.1, Esc=2.0, transpose=transpose)
        torch.cuda.synchronize()
        assert torch.equal(a, b), f"cplx={cplx} transpose={transpose}: {(a - b).abs().max().item():.3e}"
    # the diagonal (and so Davidson) runs on the streamed operator: from H on
    # unit vectors, the same bits as on the resident operator, and within
    # rounding of the resident operator's term-wise diagonal
    d_st = st.diagonal()
    assert torch.equal(res.diagonal(by_apply=True), d_st)
    d_res = res.diagonal()
    assert float((d_res - d_st).abs().max() / d_st.abs().max()) <= 1e-12


def test_streamed_12d_matches_oracle():
    need_cuda()
    m = make_model(12, 2, 10, 20261212)
    O, kw = oracle_for(m)
    op = m.operator(field_budget=200 * 1024 * 1024)          # ~1/4 of its 0.9 GB of fields
    assert op.field_slices >= 4
    psi = np.random.default_rng(12).normal(size=(O.N, 2))
    check_against_oracle(op, O, kw, psi, "12-D L=2 type 10, streamed fields")


def test_streamed_12d_l4_matches_oracle():
    """The 12-D type-10 construction (Q-dependent G) at L=4: 1820 Smolyak
    terms, 31 million grid points, 36 GB of V and G fields streamed through a
    4 GB budget (9+ slices).  The oracle evaluates the same polynomial V and
    affine G term by term (no stored grids) in double precision."""
    need_cuda()
    m = make_model(12, 4, 10, 20261216)
    op = m.operator(field_budget=4 * 1024 ** 3)
    assert op.field_slices >= 9
    O = OracleSG4(m.D, m.L, m.L, 1, 1, 2, 1, scaleQ=m.scaleQ)
    assert O.N == op.basis.N
    psi = np.random.default_rng(124).normal(size=(O.N, 2))
    P = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    out = torch.empty_like(P)
    op.hpsi_dev(P, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().T
    ref = O.hpsi(psi, type_op=10, V_poly=(m.V.coef, m.V.expo), G0=m.G0, G1=m.G1)
    err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    print(f"12-D L=4 streamed type 10: gpu-vs-oracle {err:.2e}")
    assert err <= 1e-12


def test_streamed_rejections():
    need_cuda()
    m = make_model(4, 5, 10, 3)
    res = m.operator()
    biggest = max(int(np.prod(np.asarray(l) + 2)) for l in res.basis.tables()[0])
    with pytest.raises(EVRError, match="budget"):
        m.operator(field_budget=8 * (1 + 16) * biggest - 8)  # below the fields of the largest term
    st = m.operator(field_budget=field_bytes(m, res) // 3)
    P = _rand(res.basis.N, 2, False, 1)
    with pytest.raises(EVRError):
        st.hpsi_dev(P, torch.empty_like(P), plain=True)
    with pytest.raises(EVRError):
        MultiOp([st], [2])
