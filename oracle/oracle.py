"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline /
reference arm import this module; the product package never does.  The
oracle restates ElVibRot's SG4 H.psi (SRC/sub_Operator/sub_OpPsi_SG4.f90) in
plain C; see sg4_oracle.c for the routine-by-routine citations.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libsg4oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compiles the oracle with its Makefile (gcc + OpenMP)."""
    src = os.path.join(_HERE, "sg4_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int] * 7 + [dp, dp]
        L.orc_create_modes.restype = ctypes.c_void_p
        L.orc_create_modes.argtypes = [ctypes.c_int] * 3 + [ip] * 4 + [dp, dp]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_sizes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]
        L.orc_tables.argtypes = [ctypes.c_void_p, ip, dp, ip, ip]
        L.orc_basis1d.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [dp] * 8
        L.orc_grid_points.argtypes = [ctypes.c_void_p, dp]
        for fn in (L.orc_hpsi, L.orc_hpsi_ld):
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, dp, dp, ctypes.c_int]
        L.orc_gauss_hermite.argtypes = [ctypes.c_int, dp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctypes.c_double))
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctypes.c_int))
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class _OrcOp(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("V", ctypes.POINTER(ctypes.c_double)),
                ("G", ctypes.POINTER(ctypes.c_double)), ("Jac", ctypes.POINTER(ctypes.c_double)),
                ("sqRho", ctypes.POINTER(ctypes.c_double)), ("F2", ctypes.POINTER(ctypes.c_double)),
                ("F1", ctypes.POINTER(ctypes.c_double)), ("V_nterms", ctypes.c_int),
                ("V_coef", ctypes.POINTER(ctypes.c_double)), ("V_expo", ctypes.POINTER(ctypes.c_int)),
                ("G0", ctypes.POINTER(ctypes.c_double)), ("G1", ctypes.POINTER(ctypes.c_double)),
                ("F2_grid", ctypes.POINTER(ctypes.c_double)), ("F1_grid", ctypes.POINTER(ctypes.c_double))]


def gauss_hermite(nq: int):
    x = np.zeros(nq)
    w = np.zeros(nq)
    wr = np.zeros(nq)
    lib().orc_gauss_hermite(nq, _dp(x), _dp(w), _dp(wr))
    return x, w, wr


class OracleSG4:
    """The oracle's SG4 basis + operator action (one HO basis per mode).

    A_nb, B_nb, A_nq, B_nq: one rule for every mode, or a sequence of D rules."""

    def __init__(self, D, L, LB=None, A_nb=1, B_nb=1, A_nq=2, B_nq=1, Q0=None, scaleQ=None):
        self.D, self.L = D, L
        self.LB = L if LB is None else LB
        self.Q0 = np.zeros(D) if Q0 is None else np.ascontiguousarray(Q0, dtype=np.float64)
        self.scaleQ = np.ones(D) if scaleQ is None else np.ascontiguousarray(scaleQ, dtype=np.float64)
        rule = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.int32), (D,)))
        self.A_nb, self.B_nb, self.A_nq, self.B_nq = rule(A_nb), rule(B_nb), rule(A_nq), rule(B_nq)
        self.h = lib().orc_create_modes(D, L, self.LB, _ip(self.A_nb), _ip(self.B_nb), _ip(self.A_nq),
                                        _ip(self.B_nq), _dp(self.Q0), _dp(self.scaleQ))
        if not self.h:
            raise ValueError("orc_create failed")
        z = (ctypes.c_longlong * 8)()
        lib().orc_sizes(self.h, z)
        self.N, self.nb_SG, self.sum_nb, self.sum_nq, self.max_nb, self.max_nq = [int(v) for v in z[:6]]

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def tables(self):
        tab_l = np.zeros(self.nb_SG * self.D, dtype=np.int32)
        w = np.zeros(self.nb_SG)
        m = np.zeros(self.sum_nb, dtype=np.int32)
        p = np.zeros(self.N * self.D, dtype=np.int32)
        lib().orc_tables(self.h, _ip(tab_l), _dp(w), _ip(m), _ip(p))
        return tab_l.reshape(self.nb_SG, self.D), w, m, p.reshape(self.N, self.D)

    def nb_nq(self, l, mode=0):
        return (int(self.A_nb[mode] + self.B_nb[mode] * l), int(self.A_nq[mode] + self.B_nq[mode] * l))

    def basis1d(self, mode, l):
        nb, nq = self.nb_nq(l, mode)
        out = dict(x=np.zeros(nq), w=np.zeros(nq), d0=np.zeros(nq * nb), d1=np.zeros(nq * nb),
                   d2=np.zeros(nq * nb), bgw=np.zeros(nq * nb), d1gg=np.zeros(nq * nq), d2gg=np.zeros(nq * nq))
        lib().orc_basis1d(self.h, mode, l, *[_dp(out[k]) for k in ("x", "w", "d0", "d1", "d2", "bgw", "d1gg", "d2gg")])
        for k in ("d0", "d1", "d2"):
            out[k] = out[k].reshape(nb, nq).T
        out["bgw"] = out["bgw"].reshape(nq, nb).T
        out["d1gg"] = out["d1gg"].reshape(nq, nq).T
        out["d2gg"] = out["d2gg"].reshape(nq, nq).T
        return out

    def grid_points(self):
        Q = np.zeros(self.sum_nq * self.D)
        lib().orc_grid_points(self.h, _dp(Q))
        return Q.reshape(self.sum_nq, self.D)

    def hpsi(self, psi, type_op=10, V=None, G=None, Jac=None, sqRho=None, F2=None, F1=None, nthreads=0,
             extended=False, V_poly=None, G0=None, G1=None, F2_grid=None, F1_grid=None):
        """psi: (N,) or (N, nrhs) float64, column-major per RHS.

        V / G are grids; alternatively V_poly = (coef[nt], expo[nt, D]) and the
        affine G0[D, D], G1[D, D, D] are evaluated term by term at the grid
        points.  Type 1: F2[D, D] / F1[D] constant, or the grids
        F2_grid[D, D, sum_nq] / F1_grid[D, sum_nq] (Q-dependent coefficients).  extended=True runs the same algorithm with long-double
        intermediates (the accuracy yardstick); the result is rounded to double."""
        psi = np.asarray(psi, dtype=np.float64)
        one = psi.ndim == 1
        P = psi.reshape(self.N, -1)
        nrhs = P.shape[1]
        Pc = np.ascontiguousarray(P.T)  # rhs-major = column-major N x nrhs
        H = np.zeros_like(Pc)
        keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (V, G, Jac, sqRho, F2, F1)]
        coef = expo = None
        if V_poly is not None:
            coef = np.ascontiguousarray(V_poly[0], dtype=np.float64)
            expo = np.ascontiguousarray(V_poly[1], dtype=np.int32).reshape(len(coef), self.D)
        g0 = None if G0 is None else np.ascontiguousarray(G0, dtype=np.float64)
        g1 = None if G1 is None else np.ascontiguousarray(G1, dtype=np.float64)
        fg = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (F2_grid, F1_grid)]
        op = _OrcOp(type_op, *[_dp(a) for a in keep], 0 if coef is None else len(coef), _dp(coef), _ip(expo),
                    _dp(g0), _dp(g1), _dp(fg[0]), _dp(fg[1]))
        fn = lib().orc_hpsi_ld if extended else lib().orc_hpsi
        rc = fn(self.h, ctypes.byref(op), nrhs, _dp(Pc), _dp(H), int(nthreads))
        if rc != 0:
            raise RuntimeError(f"orc_hpsi failed rc={rc}")
        H = H.T
        return H[:, 0] if one else H


def oracle_tables(O: "OracleSG4"):
    """The oracle's SG4 tables in the evr_sg4_desc layout (a dict of arrays)."""
    D, L = O.D, O.L
    nb_of_l, nq_of_l, xs, rgb, bgw, d1, d2 = [], [], [], [], [], [], []
    for i in range(D):
        for l in range(L + 1):
            b = O.basis1d(i, l)
            nb, nq = O.nb_nq(l, i)
            nb_of_l.append(nb)
            nq_of_l.append(nq)
            xs.append(b["x"])
            rgb.append(b["d0"].ravel(order="F"))
            bgw.append(b["bgw"].ravel(order="F"))
            d1.append(b["d1gg"].ravel(order="F"))
            d2.append(b["d2gg"].ravel(order="F"))
    tab_l, w, m, _ = O.tables()
    return dict(D=D, L=L, LB=O.LB, nb_of_l=np.array(nb_of_l), nq_of_l=np.array(nq_of_l),
                x=np.concatenate(xs), RGB=np.concatenate(rgb), RBGwrho=np.concatenate(bgw),
                d1GG=np.concatenate(d1), d2GG=np.concatenate(d2), tab_l=tab_l, weight=w, map_=m, N=O.N)
