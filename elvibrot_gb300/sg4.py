"""Host-side mirror of ElVibRot's SG4 operator interface over libevrsg4.so.

The names follow the reference:

* :class:`SG4Basis` -- ``para_Op%BasisnD`` after ``RecSparseGrid_ForDP_type4``
  (SRC/sub_Basis/sub_quadra_SparseBasis.f90:922) for HO/Hermite modes.
* :class:`ParamOp` -- ``TYPE(param_Op)`` (SRC/sub_Operator/sub_module_SetOp.f90:59)
  restricted to what the SG4 action reads: ``type_Op`` (0, 1 or 10) and the
  cached operator grids (``OpGrid``).
* :func:`sub_TabOpPsi`, :func:`sub_OpPsi`, :func:`sub_scaledOpPsi` -- the
  reference's entry points (SRC/sub_Operator/sub_OpPsi.f90:705, :180, :2821)
  for SG4 bases: they return ``OpPsi`` with the packed layout of ``RvecB``
  (column-major N x nrhs), complex vectors going through the real operator on
  their real and imaginary parts like ``CplxPsi_TO_RCpsi``.

Vectors are torch tensors: CUDA tensors run on the device in place; host
(numpy or CPU torch) vectors go through ``evr_sg4_hpsi_host`` (copies in and
out).  There is no CPU fallback: without the CUDA library every call raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _build

EVR_OK = 0
_ERRORS = {1: "EVR_ERR_ARG", 2: "EVR_ERR_CUDA", 3: "EVR_ERR_ALLOC", 4: "EVR_ERR_STATE",
           5: "EVR_ERR_TIMEOUT", 6: "EVR_ERR_NUMERIC"}


class EVRError(RuntimeError):
    """A C-ABI call returned a non-zero status (the reference would STOP)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib():
    """Loads (building if needed) the in-tree libevrsg4.so."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path) or not _build.up_to_date():
            _build.build()
        L = ctypes.CDLL(path)
        _declare(L)
        _lib = L
    return _lib


class Desc(ctypes.Structure):
    _fields_ = [("D", ctypes.c_int), ("L", ctypes.c_int), ("LB", ctypes.c_int), ("nb0", ctypes.c_int),
                ("nb_of_l", ctypes.POINTER(ctypes.c_int)), ("nq_of_l", ctypes.POINTER(ctypes.c_int)),
                ("x", ctypes.POINTER(ctypes.c_double)), ("RGB", ctypes.POINTER(ctypes.c_double)),
                ("RBGwrho", ctypes.POINTER(ctypes.c_double)), ("d1GG", ctypes.POINTER(ctypes.c_double)),
                ("d2GG", ctypes.POINTER(ctypes.c_double)), ("nb_SG", ctypes.c_longlong),
                ("tab_l", ctypes.POINTER(ctypes.c_int)), ("weight", ctypes.POINTER(ctypes.c_double)),
                ("map", ctypes.POINTER(ctypes.c_int)), ("N", ctypes.c_longlong)]


class DavidsonOpts(ctypes.Structure):
    _fields_ = [("nev", ctypes.c_int), ("block", ctypes.c_int), ("max_subspace", ctypes.c_int),
                ("max_it", ctypes.c_int), ("conv_resi", ctypes.c_double), ("symmetrize", ctypes.c_int),
                ("no_graph", ctypes.c_int)]


class ChebyOpts(ctypes.Structure):
    _fields_ = [("Hmin", ctypes.c_double), ("Hmax", ctypes.c_double), ("dt", ctypes.c_double),
                ("npoly", ctypes.c_int), ("nsteps", ctypes.c_int), ("poly_tol", ctypes.c_double),
                ("no_graph", ctypes.c_int)]


class TuneResult(ctypes.Structure):
    _fields_ = [("geo", ctypes.c_int), ("rmax", ctypes.c_int), ("split", ctypes.c_int), ("ms", ctypes.c_double),
                ("default_ms", ctypes.c_double), ("from_cache", ctypes.c_int)]


class RK4Opts(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("nsteps", ctypes.c_int), ("checkpoint", ctypes.c_int),
                ("E0", ctypes.c_double), ("nsub", ctypes.c_int), ("no_graph", ctypes.c_int)]


class OpDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("V_grid", ctypes.POINTER(ctypes.c_double)),
                ("V_nterms", ctypes.c_int), ("V_coef", ctypes.POINTER(ctypes.c_double)),
                ("V_expo", ctypes.POINTER(ctypes.c_int)), ("G_grid", ctypes.POINTER(ctypes.c_double)),
                ("G0", ctypes.POINTER(ctypes.c_double)), ("G1", ctypes.POINTER(ctypes.c_double)),
                ("Jac_grid", ctypes.POINTER(ctypes.c_double)), ("sqRho_grid", ctypes.POINTER(ctypes.c_double)),
                ("F2", ctypes.POINTER(ctypes.c_double)), ("F1", ctypes.POINTER(ctypes.c_double)),
                ("F2_grid", ctypes.POINTER(ctypes.c_double)), ("F1_grid", ctypes.POINTER(ctypes.c_double))]


def _declare(L):
    vp, ip, dp, ll = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_longlong
    L.evr_sg4_last_error.restype = ctypes.c_char_p
    sig = {
        "evr_sg4_desc_sizes": [ctypes.POINTER(Desc), ctypes.POINTER(ll)],
        "evr_sg4_basis_build_ho": [ctypes.c_int] * 7 + [dp, dp, ctypes.POINTER(vp)],
        "evr_sg4_basis_build_ho_modes": [ctypes.c_int] * 3 + [ip] * 4 + [dp, dp, ctypes.POINTER(vp)],
        "evr_sg4_basis_desc": [vp, ctypes.POINTER(Desc)],
        "evr_sg4_basis_grid_points": [vp, dp],
        "evr_sg4_create": [ctypes.POINTER(Desc), ctypes.POINTER(vp)],
        "evr_sg4_destroy": [vp],
        "evr_sg4_set_operator": [vp, ctypes.POINTER(OpDesc)],
        "evr_sg4_hpsi": [vp, ctypes.c_int, vp, ll, vp, ll, ctypes.c_double, ctypes.c_double, vp],
        "evr_sg4_hpsi_plain": [vp, ctypes.c_int, vp, ll, vp, ll, vp],
        "evr_sg4_hpsi_cplx": [vp, ctypes.c_int, vp, ll, vp, ll, ctypes.c_double, ctypes.c_double, vp],
        "evr_sg4_hpsi_host": [vp, ctypes.c_int, vp, ll, vp, ll, ctypes.c_double, ctypes.c_double],
        "evr_sg4_apply": [vp, ctypes.c_int, ctypes.c_int, vp, ll, vp, ll, ctypes.c_double, ctypes.c_double, vp],
        "evr_sg4_flops_per_rhs": [vp, dp],
        "evr_sg4_last_launches": [vp, ctypes.POINTER(ll)],
        "evr_sg4_last_geometry": [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
        "evr_probe_fp64_peak": [dp],
        "evr_probe_fp64_pipes": [dp, dp, dp],
        "evr_sg4_set_plan": [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int],
        "evr_sg4_get_plan": [vp, ip, ip, ip],
        "evr_sg4_tune_plan": [vp, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.POINTER(TuneResult)],
        "evr_sg4_ctx_sizes": [vp, ctypes.POINTER(ll)],
        "evr_sg4_rk4_field": [vp, vp, ctypes.POINTER(RK4Opts), dp, vp, vp],
        "evr_sg4_rk4_field_batch": [vp, vp, ctypes.POINTER(RK4Opts), ctypes.c_int, dp, vp, vp],
        "evr_sg4_oc_gradient": [vp, vp, ctypes.POINTER(RK4Opts), dp, vp, vp, dp, dp, vp],
        "evr_sg4_cheby_propagate": [vp, ctypes.POINTER(ChebyOpts), ctypes.c_int, vp, vp, dp,
                                    ctypes.POINTER(ctypes.c_int), vp],
        "evr_sg4_diagonal": [vp, vp, vp],
        "evr_sg4_diagonal_by_apply": [vp, vp, vp],
        "evr_sg4_set_field_budget": [vp, ll],
        "evr_sg4_field_slices": [vp, ctypes.POINTER(ll)],
        "evr_sg4_tune": [vp, ctypes.c_int, ctypes.c_int, ip, dp],
        "evr_sg4_hpsi_multi": [ctypes.c_int, ctypes.POINTER(vp), ip, ctypes.POINTER(vp), ctypes.POINTER(ll),
                               ctypes.POINTER(vp), ctypes.POINTER(ll), dp, dp, ctypes.c_int, vp],
        "evr_sg4_multi_create": [ctypes.c_int, ctypes.POINTER(vp), ip, ctypes.c_int, ctypes.POINTER(vp)],
        "evr_sg4_multi_hpsi": [vp, ctypes.POINTER(vp), ctypes.POINTER(ll), ctypes.POINTER(vp), ctypes.POINTER(ll),
                               dp, dp, vp],
        "evr_sg4_multi_last_launches": [vp, ctypes.POINTER(ll)],
        "evr_sg4_multi_groups": [vp, ctypes.c_int, ip, ip, ctypes.POINTER(ll)],
        "evr_sg4_multi_destroy": [vp],
        "evr_sg4_multi_cheby_propagate": [vp, ctypes.POINTER(ChebyOpts), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                          ctypes.POINTER(ctypes.c_int), vp],
        "evr_sg4_davidson": [vp, ctypes.POINTER(DavidsonOpts), vp, ctypes.c_int, vp, dp, vp, dp,
                             ctypes.POINTER(ctypes.c_int), vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.evr_sg4_basis_free.argtypes = [vp]
    L.evr_sg4_basis_free.restype = None


def check(rc: int):
    if rc != EVR_OK:
        raise EVRError(rc, lib().evr_sg4_last_error().decode())


def _dp(a):
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctypes.c_double))
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctypes.c_int))
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class SG4Basis:
    """SG4 basis of D harmonic-oscillator modes (nb(l) = A_nb + B_nb l, nq(l) = A_nq + B_nq l)."""

    def __init__(self, D: int, L: int, LB: Optional[int] = None, A_nb=1, B_nb=1, A_nq=2, B_nq=1,
                 Q0: Optional[Sequence[float]] = None, scaleQ: Optional[Sequence[float]] = None, nb0: int = 1):
        """A_nb, B_nb, A_nq, B_nq: one rule for every mode or a sequence of D rules;
        nb0: channels (electronic states) of the vectors."""
        self.D, self.L = int(D), int(L)
        self.LB = self.L if LB is None else int(LB)
        self.A_nb, self.B_nb, self.A_nq, self.B_nq = A_nb, B_nb, A_nq, B_nq
        self.Q0 = np.zeros(D) if Q0 is None else np.ascontiguousarray(Q0, dtype=np.float64)
        self.scaleQ = np.ones(D) if scaleQ is None else np.ascontiguousarray(scaleQ, dtype=np.float64)
        h = ctypes.c_void_p()
        if all(np.ndim(v) == 0 for v in (A_nb, B_nb, A_nq, B_nq)):
            check(lib().evr_sg4_basis_build_ho(self.D, self.L, self.LB, int(A_nb), int(B_nb), int(A_nq), int(B_nq),
                                               _dp(self.Q0), _dp(self.scaleQ), ctypes.byref(h)))
        else:
            rule = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.int32), (self.D,)))
            self._rules = [rule(v) for v in (A_nb, B_nb, A_nq, B_nq)]
            check(lib().evr_sg4_basis_build_ho_modes(self.D, self.L, self.LB, *[_ip(r) for r in self._rules],
                                                     _dp(self.Q0), _dp(self.scaleQ), ctypes.byref(h)))
        self._h = h
        self.desc = Desc()
        check(lib().evr_sg4_basis_desc(self._h, ctypes.byref(self.desc)))
        self.desc.nb0 = int(nb0)
        z = (ctypes.c_longlong * 8)()
        check(lib().evr_sg4_desc_sizes(ctypes.byref(self.desc), z))
        self.N, self.nb_SG, self.sum_nb, self.sum_nq, self.max_nb, self.max_nq = [int(v) for v in z[:6]]
        self.nb0 = int(nb0)
        self.nvec = self.nb0 * self.N      # length of a vector (nb0 channel blocks of N)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.evr_sg4_basis_free(self._h)
            self._h = None

    def grid_points(self) -> np.ndarray:
        Q = np.zeros(self.sum_nq * self.D)
        check(lib().evr_sg4_basis_grid_points(self._h, _dp(Q)))
        return Q.reshape(self.sum_nq, self.D)

    def tables(self):
        """(tab_l[nb_SG,D], WeightSG[nb_SG], tab_iB_OF_SRep_TO_iB[sum_nb]) as numpy copies."""
        d = self.desc
        tab_l = np.ctypeslib.as_array(d.tab_l, shape=(self.nb_SG * self.D,)).reshape(self.nb_SG, self.D).copy()
        w = np.ctypeslib.as_array(d.weight, shape=(self.nb_SG,)).copy()
        m = np.ctypeslib.as_array(d.map, shape=(self.sum_nb,)).copy()
        return tab_l, w, m

    def basis1d(self, mode: int, l: int):
        """1-D matrices of (mode, level): dict x, RGB (nq x nb), RBGwrho (nb x nq), d1GG, d2GG."""
        d = self.desc
        nbl = np.ctypeslib.as_array(d.nb_of_l, shape=(self.D * (self.L + 1),))
        nql = np.ctypeslib.as_array(d.nq_of_l, shape=(self.D * (self.L + 1),))
        k = mode * (self.L + 1) + l
        ox = int(nql[:k].sum())
        om = int((nql[:k] * nbl[:k]).sum())
        og = int((nql[:k] ** 2).sum())
        nb, nq = int(nbl[k]), int(nql[k])
        arr = lambda p, o, n: np.ctypeslib.as_array(p, shape=(o + n,))[o:o + n].copy()
        return dict(x=arr(d.x, ox, nq), RGB=arr(d.RGB, om, nq * nb).reshape(nb, nq).T,
                    RBGwrho=arr(d.RBGwrho, om, nq * nb).reshape(nq, nb).T,
                    d1GG=arr(d.d1GG, og, nq * nq).reshape(nq, nq).T,
                    d2GG=arr(d.d2GG, og, nq * nq).reshape(nq, nq).T)


class SG4Tables:
    """SG4 tables supplied by the caller (what a Fortran host copies out of
    para_Op%BasisnD; see evr_sg4_desc in include/evr_sg4.h).

    Per-(mode, level) arrays are concatenated mode-major, level-minor;
    matrices are column-major: RGB nq x nb, RBGwrho nb x nq, d1GG/d2GG nq x nq.
    """

    def __init__(self, D, L, LB, nb_of_l, nq_of_l, x, RGB, RBGwrho, d1GG, d2GG, tab_l, weight, map_, N, nb0=1):
        self.D, self.L, self.LB = int(D), int(L), int(LB)
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32).ravel()
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64).ravel()
        self._keep = dict(nb_of_l=i32(nb_of_l), nq_of_l=i32(nq_of_l), x=f64(x), RGB=f64(RGB),
                          RBGwrho=f64(RBGwrho), d1GG=f64(d1GG), d2GG=f64(d2GG), tab_l=i32(tab_l),
                          weight=f64(weight), map=i32(map_))
        k = self._keep
        self.desc = Desc(self.D, self.L, self.LB, int(nb0), _ip(k["nb_of_l"]), _ip(k["nq_of_l"]), _dp(k["x"]),
                         _dp(k["RGB"]), _dp(k["RBGwrho"]), _dp(k["d1GG"]), _dp(k["d2GG"]),
                         len(k["weight"]), _ip(k["tab_l"]), _dp(k["weight"]), _ip(k["map"]), int(N))
        z = (ctypes.c_longlong * 8)()
        check(lib().evr_sg4_desc_sizes(ctypes.byref(self.desc), z))
        self.N, self.nb_SG, self.sum_nb, self.sum_nq, self.max_nb, self.max_nq = [int(v) for v in z[:6]]
        self.nb0 = int(nb0)
        self.nvec = self.nb0 * self.N


@dataclass
class Polynomial:
    """sum_t coef[t] prod_i Q_i**expo[t, i] (raw coordinates Q)."""
    coef: np.ndarray
    expo: np.ndarray

    def __call__(self, Q: np.ndarray) -> np.ndarray:
        kmax = int(self.expo.max()) if len(self.expo) else 0
        pw = [np.ones_like(Q)]
        for _ in range(kmax):
            pw.append(pw[-1] * Q)
        out = np.zeros(Q.shape[0])
        for c, e in zip(self.coef, self.expo):
            t = np.full(Q.shape[0], c)
            for i in np.nonzero(e)[0]:
                t *= pw[e[i]][:, i]
            out += t
        return out


class ParamOp:
    """SG4 operator on the GPU (param_Op with its Save_MemGrid grids).

    type_op 0 : V;  1 : V + sum F2_ij d_i d_j + sum F1_i d_i (F constant, or
    Q-dependent grids F2_grid [D, D, nb0*nb0, sum_nq] / F1_grid [D, nb0*nb0,
    sum_nq], channel pair (a, b) at a*nb0 + b);
    10 : -1/2 sum d_i Jac G_ji d_j s / (Jac s) + V with G grid or affine G(Q).
    """

    def __init__(self, basis: SG4Basis, type_op: int, V: Optional[np.ndarray] = None,
                 V_poly: Optional[Polynomial] = None, G: Optional[np.ndarray] = None,
                 G0: Optional[np.ndarray] = None, G1: Optional[np.ndarray] = None,
                 Jac: Optional[np.ndarray] = None, sqRho: Optional[np.ndarray] = None,
                 F2: Optional[np.ndarray] = None, F1: Optional[np.ndarray] = None, field_budget: int = 0,
                 F2_grid: Optional[np.ndarray] = None, F1_grid: Optional[np.ndarray] = None):
        self.basis = basis
        self.type_op = int(type_op)
        h = ctypes.c_void_p()
        check(lib().evr_sg4_create(ctypes.byref(basis.desc), ctypes.byref(h)))
        self._h = h
        if field_budget:
            check(lib().evr_sg4_set_field_budget(h, int(field_budget)))
        self.set_operator(V=V, V_poly=V_poly, G=G, G0=G0, G1=G1, Jac=Jac, sqRho=sqRho, F2=F2, F1=F1,
                          F2_grid=F2_grid, F1_grid=F1_grid)

    def set_operator(self, V=None, V_poly=None, G=None, G0=None, G1=None, Jac=None, sqRho=None, F2=None, F1=None,
                     F2_grid=None, F1_grid=None):
        D = self.basis.D
        c = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel()
        keep = dict(V=c(V), G=c(G), G0=c(G0), G1=c(G1), Jac=c(Jac), sqRho=c(sqRho), F2=c(F2), F1=c(F1),
                    F2_grid=c(F2_grid), F1_grid=c(F1_grid))
        snq = self.basis.sum_nq
        nc = self.basis.nb0 ** 2
        for name, n in (("F2_grid", D * D * nc * snq), ("F1_grid", D * nc * snq)):
            if keep[name] is not None and keep[name].size != n:
                raise EVRError(1, f"{name}: {keep[name].size} values, expected {n}")
        coef = expo = None
        nterms = 0
        if V_poly is not None and V is None:
            # one channel: coef (nterms,); nb0 channels: coef (nb0*nb0, nterms), element (a, b) in row a*nb0 + b
            coef = np.ascontiguousarray(V_poly.coef, dtype=np.float64)
            expo = np.ascontiguousarray(V_poly.expo, dtype=np.int32).reshape(-1, D)
            nterms = expo.shape[0]
            if coef.size != nterms * self.basis.nb0 ** 2:
                raise EVRError(1, f"V_poly: {coef.size} coefficients for {nterms} terms and nb0={self.basis.nb0}")
            coef = coef.ravel()
        op = OpDesc(self.type_op, _dp(keep["V"]), nterms, _dp(coef), _ip(expo), _dp(keep["G"]),
                    _dp(keep["G0"]), _dp(keep["G1"]), _dp(keep["Jac"]), _dp(keep["sqRho"]),
                    _dp(keep["F2"]), _dp(keep["F1"]), _dp(keep["F2_grid"]), _dp(keep["F1_grid"]))
        check(lib().evr_sg4_set_operator(self._h, ctypes.byref(op)))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.evr_sg4_destroy(self._h)
            self._h = None

    def tune(self, nrhs: int, complex_: bool = False):
        """Times H.psi for each cap on the right-hand sides per work item and keeps
        the fastest (evr_sg4_tune); returns (cap, ms)."""
        r, t = ctypes.c_int(), ctypes.c_double()
        check(lib().evr_sg4_tune(self._h, int(nrhs), 2 if complex_ else 0, ctypes.byref(r), ctypes.byref(t)))
        return r.value, t.value

    def tune_plan(self, nrhs: int, complex_: bool = False, cache_path: Optional[str] = None) -> dict:
        """Times the plan candidates on nrhs vectors and applies the fastest
        (evr_sg4_tune_plan); with cache_path the winner is recorded / reused."""
        r = TuneResult()
        path = cache_path.encode() if cache_path else None
        check(lib().evr_sg4_tune_plan(self._h, int(nrhs), 2 if complex_ else 0, path, ctypes.byref(r)))
        return {"geo": r.geo, "rmax": r.rmax, "split": r.split, "ms": r.ms, "default_ms": r.default_ms,
                "from_cache": bool(r.from_cache)}

    def set_plan(self, geo: int = -1, rmax: int = 0, split: int = -1):
        """Plan knobs (evr_sg4_set_plan); no arguments: the automatic plan."""
        check(lib().evr_sg4_set_plan(self._h, int(geo), int(rmax), int(split)))

    def get_plan(self):
        g, r, sp = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().evr_sg4_get_plan(self._h, ctypes.byref(g), ctypes.byref(r), ctypes.byref(sp)))
        return g.value, r.value, sp.value

    @property
    def field_slices(self) -> int:
        """Slices the analytic operator fields are evaluated in per H.psi (0: resident)."""
        n = ctypes.c_longlong()
        check(lib().evr_sg4_field_slices(self._h, ctypes.byref(n)))
        return n.value

    @property
    def flops_per_rhs(self) -> float:
        f = ctypes.c_double()
        check(lib().evr_sg4_flops_per_rhs(self._h, ctypes.byref(f)))
        return f.value

    @property
    def last_launches(self) -> int:
        n = ctypes.c_longlong()
        check(lib().evr_sg4_last_launches(self._h, ctypes.byref(n)))
        return n.value

    def last_geometry(self):
        """(geometry, CTAs per SM) of the current work plan: 0 wide, 1 narrow, 2 mid."""
        g, c = ctypes.c_int(), ctypes.c_int()
        check(lib().evr_sg4_last_geometry(self._h, ctypes.byref(g), ctypes.byref(c)))
        return g.value, c.value

    # -- device-pointer calls (torch CUDA tensors, column-major N x nrhs) --
    def hpsi_dev(self, psi, out, E0: float = 0.0, Esc: float = 1.0, stream: int = 0, plain: bool = False,
                 transpose: bool = False):
        import torch
        N = self.basis.nvec
        if psi.dtype not in (torch.float64, torch.complex128) or not psi.is_cuda:
            raise EVRError(1, "psi must be a CUDA float64/complex128 tensor")
        cplx = psi.dtype == torch.complex128
        P = psi if psi.dim() == 2 else psi.unsqueeze(0)   # (nrhs, N) rows = columns of RvecB
        O = out if out.dim() == 2 else out.unsqueeze(0)
        if P.shape[-1] != N or O.shape != P.shape or not P.is_contiguous() or not O.is_contiguous():
            raise EVRError(1, f"psi/out must be contiguous (nrhs, {N}) tensors of equal shape")
        nrhs = P.shape[0]
        if transpose:
            flags = 1 | (2 if cplx else 0) | (4 if plain else 0)
            check(lib().evr_sg4_apply(self._h, flags, nrhs, P.data_ptr(), N, O.data_ptr(), N, E0, Esc, stream))
            return out
        if plain:
            if cplx or E0 != 0.0 or Esc != 1.0:
                raise EVRError(1, "the plain per-term path takes real psi with E0=0, Esc=1")
            check(lib().evr_sg4_hpsi_plain(self._h, nrhs, P.data_ptr(), N, O.data_ptr(), N, stream))
        elif cplx:
            check(lib().evr_sg4_hpsi_cplx(self._h, nrhs, P.data_ptr(), N, O.data_ptr(), N, E0, Esc, stream))
        else:
            check(lib().evr_sg4_hpsi(self._h, nrhs, P.data_ptr(), N, O.data_ptr(), N, E0, Esc, stream))
        return out

    def diagonal(self, by_apply: bool = False):
        """Exact diag(H) as a CUDA tensor (the Davidson preconditioner): term by
        term (evr_sg4_diagonal), or from H on blocks of unit vectors (by_apply)."""
        import torch
        d = torch.empty(self.basis.nvec, dtype=torch.float64, device="cuda")
        fn = lib().evr_sg4_diagonal_by_apply if by_apply else lib().evr_sg4_diagonal
        check(fn(self._h, d.data_ptr(), 0))
        return d

    def davidson(self, nev: int, block: int = 0, max_subspace: int = 0, max_it: int = 500,
                 conv_resi: float = 1e-8, symmetrize: bool = False, guess=None, diag=None, graph: bool = True):
        """Lowest nev levels (sub_propagation_Davidson).  Returns (evals, evecs
        (CUDA tensor nev x N), residual norms, iterations); raises EVRError
        when max_it is reached."""
        import torch
        N = self.basis.nvec
        o = DavidsonOpts(nev, block, max_subspace, max_it, conv_resi, 1 if symmetrize else 0, 0 if graph else 1)
        ev = np.zeros(nev)
        rs = np.zeros(nev)
        vec = torch.empty((nev, N), dtype=torch.float64, device="cuda")
        its = ctypes.c_int()
        gptr, ng = (guess.data_ptr(), guess.shape[0]) if guess is not None else (None, 0)
        check(lib().evr_sg4_davidson(self._h, ctypes.byref(o), gptr, ng,
                                     diag.data_ptr() if diag is not None else None, _dp(ev), vec.data_ptr(),
                                     _dp(rs), ctypes.byref(its), 0))
        return ev, vec, rs, its.value

    def cheby_propagate(self, psi, Hmin: float, Hmax: float, dt: float, npoly: int, nsteps: int,
                        poly_tol: float = 0.0, psi0=None, graph: bool = True):
        """Propagates the CUDA complex128 tensor psi (nrhs, N) in place
        (march_cheby); returns (autocorrelation [(nsteps+1), nrhs], npoly used)."""
        import torch
        if psi.dtype != torch.complex128 or not psi.is_cuda or not psi.is_contiguous():
            raise EVRError(1, "psi must be a contiguous CUDA complex128 tensor (nrhs, N)")
        P = psi if psi.dim() == 2 else psi.unsqueeze(0)
        nrhs = P.shape[0]
        ac = np.zeros((nsteps + 1) * nrhs * 2)
        used = ctypes.c_int()
        o = ChebyOpts(Hmin, Hmax, dt, npoly, nsteps, poly_tol, 0 if graph else 1)
        check(lib().evr_sg4_cheby_propagate(self._h, ctypes.byref(o), nrhs, P.data_ptr(),
                                            psi0.data_ptr() if psi0 is not None else None, _dp(ac),
                                            ctypes.byref(used), 0))
        a = ac.reshape(nsteps + 1, nrhs, 2)
        return a[..., 0] + 1j * a[..., 1], used.value

    def rk4_field(self, mu: "ParamOp", E: np.ndarray, psi, dt: float, E0: float = 0.0, nsub: int = 1,
                  graph: bool = True):
        """march_RK4_field: propagates the CUDA complex128 vector psi (N,) in place
        under H0 - E(t) mu, E held at E[k] over step k."""
        E = np.ascontiguousarray(E, dtype=np.float64)
        o = RK4Opts(dt, len(E), 1, E0, nsub, 0 if graph else 1)
        check(lib().evr_sg4_rk4_field(self._h, mu._h, ctypes.byref(o), _dp(E), psi.data_ptr(), 0))
        return psi

    def rk4_field_batch(self, mu: "ParamOp", E: np.ndarray, psi, dt: float, E0: float = 0.0, nsub: int = 1,
                        graph: bool = True):
        """Several packets at once, each with its own field: E is (nsteps, nb),
        psi a contiguous CUDA complex128 (nb, N) tensor (row b = packet b),
        propagated in place."""
        E = np.ascontiguousarray(E, dtype=np.float64)
        if E.ndim != 2 or psi.dim() != 2 or psi.shape[0] != E.shape[1] or not psi.is_contiguous():
            raise EVRError(1, "rk4_field_batch: E (nsteps, nb) and a contiguous psi (nb, N)")
        o = RK4Opts(dt, E.shape[0], 1, E0, nsub, 0 if graph else 1)
        check(lib().evr_sg4_rk4_field_batch(self._h, mu._h, ctypes.byref(o), E.shape[1], _dp(E), psi.data_ptr(), 0))
        return psi

    def oc_gradient(self, mu: "ParamOp", E: np.ndarray, psi0, target, dt: float, checkpoint: int = 45,
                    E0: float = 0.0, nsub: int = 1, graph: bool = True):
        """(J, dJ/dE) for J = |<target|psi(T)>|^2 by the adjoint of the RK4 steps."""
        E = np.ascontiguousarray(E, dtype=np.float64)
        o = RK4Opts(dt, len(E), checkpoint, E0, nsub, 0 if graph else 1)
        J = ctypes.c_double()
        g = np.zeros(len(E))
        check(lib().evr_sg4_oc_gradient(self._h, mu._h, ctypes.byref(o), _dp(E), psi0.data_ptr(), target.data_ptr(),
                                        ctypes.byref(J), _dp(g), 0))
        return J.value, g

    def hpsi_host(self, psi: np.ndarray, E0: float = 0.0, Esc: float = 1.0) -> np.ndarray:
        """psi (N,) or (N, nrhs) host float64; returns the same shape (copies in/out)."""
        N = self.basis.nvec
        a = np.asarray(psi, dtype=np.float64)
        one = a.ndim == 1
        P = np.asfortranarray(a.reshape(N, -1))
        H = np.zeros_like(P, order="F")
        check(lib().evr_sg4_hpsi_host(self._h, P.shape[1], P.ctypes.data, N, H.ctypes.data, N, E0, Esc))
        return H[:, 0] if one else H


def sub_TabOpPsi(Psi, para_Op: ParamOp, E0: float = 0.0, Esc: float = 1.0):
    """OpPsi(:) for a block of vectors (sub_OpPsi.f90:705 -> sub_OpPsi_SG4.f90:681).

    ``Psi``: CUDA tensor (nrhs, N) float64/complex128 -> CUDA tensor; or a host
    array (N,) / (N, nrhs) float64 -> host array.  Raises EVRError (the
    reference STOPs) on empty input or inconsistent sizes.
    """
    try:
        import torch
        is_t = isinstance(Psi, torch.Tensor)
    except ImportError:
        is_t = False
    if is_t and Psi.is_cuda:
        if Psi.numel() == 0:
            raise EVRError(1, "size(Psi) = 0")
        out = torch.empty_like(Psi)
        return para_Op.hpsi_dev(Psi.contiguous(), out, E0=E0, Esc=Esc)
    a = Psi.cpu().numpy() if is_t else np.asarray(Psi)
    if a.size == 0:
        raise EVRError(1, "size(Psi) = 0")
    if np.iscomplexobj(a):
        return para_Op.hpsi_host(a.real, E0, Esc) + 1j * para_Op.hpsi_host(a.imag, E0, Esc)
    return para_Op.hpsi_host(a, E0, Esc)


def sub_OpPsi(Psi, para_Op: ParamOp):
    """OpPsi for one vector (sub_OpPsi.f90:180)."""
    return sub_TabOpPsi(Psi, para_Op)


def sub_scaledOpPsi(Psi, para_Op: ParamOp, E0: float, Esc: float):
    """(H Psi - E0 Psi) / Esc (sub_OpPsi.f90:2821-2864), fused into the H.psi launch."""
    return sub_TabOpPsi(Psi, para_Op, E0=E0, Esc=Esc)


def _check_blocks(ops, psis, outs, dtype):
    n = len(ops)
    if n == 0 or len(psis) != n or len(outs) != n:
        raise EVRError(1, "ops, psis and outs must be non-empty lists of equal length")
    rows = []
    for op, P, O in zip(ops, psis, outs):
        P2 = P if P.dim() == 2 else P.unsqueeze(0)
        O2 = O if O.dim() == 2 else O.unsqueeze(0)
        if (not P2.is_cuda or P2.dtype != dtype or P2.shape[-1] != op.basis.nvec or O2.shape != P2.shape
                or O2.dtype != dtype or not P2.is_contiguous() or not O2.is_contiguous()):
            raise EVRError(1, f"every psi/out must be a contiguous CUDA (nrhs, N) {dtype} tensor")
        rows.append(P2.shape[0])
    return rows


class MultiOp:
    """Several independent ParamOps applied in one persistent launch per call
    (evr_sg4_multi_*).  ``nrhs[k]`` vectors per operator, real or complex.
    No reference counterpart: ElVibRot applies one para_Op per sub_TabOpPsi
    call (sub_OpPsi.f90:705)."""

    def __init__(self, ops, nrhs, complex_: bool = False, transpose: bool = False):
        self.ops = list(ops)
        self.nrhs = [int(r) for r in nrhs]
        self.complex_ = complex_
        n = len(self.ops)
        self._h = ctypes.c_void_p()
        flags = (1 if transpose else 0) | (2 if complex_ else 0)
        check(lib().evr_sg4_multi_create(n, (ctypes.c_void_p * n)(*[op._h for op in self.ops]),
                                         (ctypes.c_int * n)(*self.nrhs), flags, ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.evr_sg4_multi_destroy(h)
            self._h = None

    def _dtype(self):
        import torch
        return torch.complex128 if self.complex_ else torch.float64

    def hpsi(self, psis, outs, E0=None, Esc=None, stream: int = 0):
        """outs[k] = (H_k psis[k] - E0[k] psis[k]) / Esc[k]; a None psi skips operator k."""
        n = len(self.ops)
        if len(psis) != n or len(outs) != n:
            raise EVRError(1, f"hpsi: {len(psis)} psis and {len(outs)} outs for {n} operators")
        act = [k for k in range(n) if psis[k] is not None]
        rows = _check_blocks([self.ops[k] for k in act], [psis[k] for k in act], [outs[k] for k in act],
                             self._dtype())
        for k, r in zip(act, rows):
            if r != self.nrhs[k]:
                raise EVRError(1, f"operator {k}: {r} vectors, the plan has {self.nrhs[k]}")
        VP, LL = ctypes.c_void_p * n, ctypes.c_longlong * n
        pp = VP(*[psis[k].data_ptr() if psis[k] is not None else None for k in range(n)])
        hp = VP(*[outs[k].data_ptr() if psis[k] is not None else None for k in range(n)])
        ld = LL(*[op.basis.nvec for op in self.ops])
        e0 = (ctypes.c_double * n)(*([0.0] * n if E0 is None else E0))
        es = (ctypes.c_double * n)(*([1.0] * n if Esc is None else Esc))
        check(lib().evr_sg4_multi_hpsi(self._h, pp, ld, hp, ld, e0, es, stream))
        return outs

    def last_launches(self) -> int:
        v = ctypes.c_longlong()
        check(lib().evr_sg4_multi_last_launches(self._h, ctypes.byref(v)))
        return v.value

    def groups(self):
        """[(geometry, work items)] per launch group (0 wide, 1 narrow, 2 mid)."""
        n = ctypes.c_int()
        check(lib().evr_sg4_multi_groups(self._h, 0, ctypes.byref(n), None, None))
        geo = (ctypes.c_int * max(1, n.value))()
        items = (ctypes.c_longlong * max(1, n.value))()
        check(lib().evr_sg4_multi_groups(self._h, n.value, ctypes.byref(n), geo, items))
        return [(geo[g], items[g]) for g in range(n.value)]

    def cheby_propagate(self, psis, Hmin, Hmax, dt: float, npoly: int, nsteps: int, stream: int = 0,
                        graph: bool = True):
        """Fixed-order Chebyshev propagation of every operator's complex packets
        in lock-step (each step replayed from a recorded CUDA graph unless
        graph=False); returns the autocorrelations [(nsteps+1) x nrhs_k] per operator."""
        import torch
        if not self.complex_:
            raise EVRError(1, "cheby_propagate needs a complex plan")
        n = len(self.ops)
        rows = _check_blocks(self.ops, psis, psis, torch.complex128)
        if rows != self.nrhs:
            raise EVRError(1, "psis do not match the plan's nrhs")
        opts = (ChebyOpts * n)(*[ChebyOpts(float(Hmin[k]), float(Hmax[k]), dt, npoly, nsteps, 0.0, 0 if graph else 1)
                                 for k in range(n)])
        ac = [np.zeros((nsteps + 1, r), dtype=np.complex128) for r in rows]
        used = ctypes.c_int()
        VP = ctypes.c_void_p * n
        check(lib().evr_sg4_multi_cheby_propagate(self._h, opts, VP(*[P.data_ptr() for P in psis]),
                                                  VP(*[a.ctypes.data for a in ac]), ctypes.byref(used), stream))
        return ac


def hpsi_multi(ops, psis, outs, E0=None, Esc=None, transpose: bool = False, stream: int = 0):
    """One-shot H_k psi_k for several independent operators in one persistent
    launch (evr_sg4_hpsi_multi); all psis float64 or all complex128."""
    import torch
    n = len(ops)
    dtype = psis[0].dtype if n else None
    if dtype not in (torch.float64, torch.complex128):
        raise EVRError(1, "hpsi_multi: psis must be float64 or complex128 CUDA tensors")
    nrhs = _check_blocks(ops, psis, outs, dtype)
    VP, LL = ctypes.c_void_p * n, ctypes.c_longlong * n
    ld = LL(*[op.basis.nvec for op in ops])
    e0 = (ctypes.c_double * n)(*([0.0] * n if E0 is None else E0))
    es = (ctypes.c_double * n)(*([1.0] * n if Esc is None else Esc))
    flags = (1 if transpose else 0) | (2 if dtype == torch.complex128 else 0)
    check(lib().evr_sg4_hpsi_multi(n, VP(*[op._h for op in ops]), (ctypes.c_int * n)(*nrhs),
                                   VP(*[P.data_ptr() for P in psis]), ld, VP(*[O.data_ptr() for O in outs]), ld,
                                   e0, es, flags, stream))
    return outs


def fp64_peak_tflops() -> float:
    t = ctypes.c_double()
    check(lib().evr_probe_fp64_peak(ctypes.byref(t)))
    return t.value


def fp64_pipes_tflops() -> dict:
    """DFMA, FP64 tensor-core MMA and both interleaved, in TFLOP/s."""
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    check(lib().evr_probe_fp64_pipes(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
    return {"dfma": a.value, "dmma": b.value, "dmma_plus_dfma": c.value}
