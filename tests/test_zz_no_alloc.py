"""The allocation-free H.psi entry point, checked against the allocating one.

evr_sg4_hpsi_noalloc is for callers that cannot call cudaMalloc: a host
program whose own allocator owns every device byte, or a real-time loop that
must stay out of the driver's allocator.  It runs the same batched and
reduce kernels as evr_sg4_hpsi, with all of its scratch taken from one fixed
device array inside the library, so its results must be the same bits.  This
file is collected last on purpose (a run that stops at the first failure has
run every other test first); test_noalloc_in_a_fresh_process repeats the
check in a new Python process, where the first call on the device also does
the array's one-time set-up.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elvibrot_gb300 import EVRError, lib
from elvibrot_gb300.configs import make_model, random_psi

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the parity tolerance used for every H.psi comparison
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


def _device_free_bytes():
    # cudaMemGetInfo: device-wide free bytes (this process has the GPU to itself)
    return torch.cuda.mem_get_info()[0]


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
        # same kernels, same per-item arithmetic, same accumulation order: the same bits
        assert torch.equal(out, ref), (call, float((out - ref).abs().max() / ref.abs().max()))
    # the allocating path's own cached plan is untouched by the calls above
    again = torch.empty_like(P)
    op.hpsi_dev(P, again)
    torch.cuda.synchronize()
    assert torch.equal(again, ref)
    # scaled form through the same entry point
    out = torch.empty_like(P)
    _noalloc(op, P, out, E0=0.25, Esc=3.0)
    torch.cuda.synchronize()
    want = (ref - 0.25 * P) / 3.0
    assert float((out - want).abs().max() / want.abs().max()) <= TOL


def test_noalloc_allocates_no_device_memory():
    """After a first call per block size (the one-time set-up and the lazy
    loading of the kernels), further calls with several block sizes leave
    the device's free memory unchanged."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    m = make_model(5, 7, 10, 17)
    op = m.operator()
    N = op.basis.N
    blocks = {}
    for nrhs in (1, 3, 12):
        P = torch.from_numpy(np.ascontiguousarray(random_psi(N, nrhs, nrhs).T)).cuda()
        blocks[nrhs] = (P, torch.empty_like(P), torch.empty_like(P))
        op.hpsi_dev(P, blocks[nrhs][2])
        _noalloc(op, P, blocks[nrhs][1])
    torch.cuda.synchronize()
    free0 = _device_free_bytes()
    for rep in range(3):
        for nrhs, (P, H, ref) in blocks.items():
            _noalloc(op, P, H)
            torch.cuda.synchronize()
            assert torch.equal(H, ref), (rep, nrhs)
    assert _device_free_bytes() == free0


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


_FRESH = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
from tests.test_zz_no_alloc import _noalloc
from elvibrot_gb300.configs import make_model, random_psi
m = make_model(6, 6, 10, 37)
op = m.operator()
P = torch.from_numpy(np.ascontiguousarray(random_psi(op.basis.N, 8, 5).T)).cuda()
out = torch.empty_like(P)
_noalloc(op, P, out)          # the first call in this process: it also looks up the array
torch.cuda.synchronize()
ref = torch.empty_like(P)
op.hpsi_dev(P, ref)
torch.cuda.synchronize()
assert torch.equal(out, ref)
_noalloc(op, P, out)
torch.cuda.synchronize()
assert torch.equal(out, ref)
print("fresh ok")
"""


def test_noalloc_in_a_fresh_process():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    r = subprocess.run([sys.executable, "-c", _FRESH, ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "fresh ok" in r.stdout, r.stdout + r.stderr
