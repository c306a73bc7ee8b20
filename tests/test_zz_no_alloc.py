"""The allocation-free H.psi entry point, checked against the allocating one.

evr_sg4_hpsi_noalloc is for callers that cannot call cudaMalloc (a host
program whose own allocator owns the device memory, a real-time loop that
must stay out of the driver's allocator).  It runs the same batched kernel
with its scratch taken from one fixed device array inside the library.  This
file is collected last on purpose: it runs after every other GPU test, and
also alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elvibrot_gb300 import EVRError, lib
from elvibrot_gb300.configs import make_model, random_psi

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the parity tolerance used for every H.psi comparison


def _noalloc(op, P, H, E0=0.0, Esc=1.0):
    L = lib()
    f = L.evr_sg4_hpsi_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                  ctypes.c_longlong, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    f.restype = ctypes.c_int
    N = op.basis.N
    rc = f(op._h, P.shape[0], P.data_ptr(), N, H.data_ptr(), N, E0, Esc, None)
    if rc != 0:
        raise EVRError(rc, L.evr_sg4_last_error().decode())


@pytest.mark.parametrize("D,L,type_op,nrhs", [(6, 6, 10, 8), (7, 9, 10, 2), (3, 6, 1, 5)])
def test_noalloc_matches_allocating_path_twice(D, L, type_op, nrhs):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    m = make_model(D, L, type_op, 31 + D)
    op = m.operator()
    N = op.basis.N
    P = torch.from_numpy(np.ascontiguousarray(random_psi(N, nrhs, 5).T)).cuda()
    ref = torch.empty_like(P)
    op.hpsi_dev(P, ref)
    for call in range(2):  # two calls in a row: the shared array keeps the last call's contents
        out = torch.full_like(P, np.nan)
        _noalloc(op, P, out)
        torch.cuda.synchronize()
        err = float((out - ref).abs().max() / ref.abs().max())
        assert err <= TOL, (call, err)
    # scaled form through the same entry point
    out = torch.empty_like(P)
    _noalloc(op, P, out, E0=0.25, Esc=3.0)
    torch.cuda.synchronize()
    want = (ref - 0.25 * P) / 3.0
    assert float((out - want).abs().max() / want.abs().max()) <= TOL


def test_noalloc_rejects_sizes_beyond_its_array():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    m = make_model(6, 8, 10, 7)      # 125,879 DP entries per right-hand side
    op = m.operator()
    N = op.basis.N
    nrhs = 64                          # 64 x 125,879 x 8 B > 32 MiB of contributions
    P = torch.zeros((nrhs, N), dtype=torch.float64, device="cuda")
    H = torch.zeros_like(P)
    with pytest.raises(EVRError) as e:
        _noalloc(op, P, H)
    assert e.value.code == 1 and "scratch" in str(e.value)
