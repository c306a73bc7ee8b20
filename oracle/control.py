"""Dense restatement of ElVibRot's optimal-control field derivative
(TEST INFRASTRUCTURE ONLY: only tests/ import this module).

The reference updates the control field from the forward wave packet psi(t)
and the backward-propagated target chi(t) (build_field,
SRC/sub_propagation/sub_control.f90:907-1007): for one packet pair and one
polarisation (Turinici off, no envelope, alpha_j = alpha)

    S      = <psi(t)|chi(t)>                 (Overlap_psi1_psi2(S, WP(j), WP(jt)))
    avMu   = <chi(t)|mu psi(t)>              (sub_OpPsi(WP(j), w2, para_Dip) then
                                              Overlap_psi1_psi2(avMu, WP(jt), w2))
    E_new  = -Im(S avMu) / alpha                                   (:962-971)

which is 1/(2 alpha) times the functional derivative dJ/dE(t) of
J = |<target|psi(T)>|^2 for dpsi/dt = -i (H0 - E(t) mu) psi, with chi(t) the
target propagated back from T (chi(t) = U(T,t)^dagger target).  The field of
march_RK4_field's 'grid' mode is held at E_k over interval k
(SRC/sub_propagation/sub_module_propa_march.f90:397-548), so the derivative
with respect to the sample E_k is the integral of dJ/dE(t) over that interval.

Here psi and chi are propagated exactly (matrix exponential of the dense
H0 - E_k mu, which need not be symmetric: chi uses the adjoint propagator),
and the interval integral is the composite Simpson rule on `m` sub-steps.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg


def build_field_E_new(psi_t: np.ndarray, chi_t: np.ndarray, Mu: np.ndarray, alpha: float = 1.0) -> float:
    """E_new of build_field (sub_control.f90:962-971) for one packet pair."""
    S = np.vdot(psi_t, chi_t)                 # <psi|chi>
    avMu = np.vdot(chi_t, Mu @ psi_t)         # <chi|mu psi>
    return float(-np.imag(S * avMu) / alpha)


def field_gradient(H0: np.ndarray, Mu: np.ndarray, E: np.ndarray, psi0: np.ndarray, target: np.ndarray,
                   dt: float, m: int = 64):
    """J = |<target|psi(T)>|^2 and dJ/dE_k = int_{interval k} 2 E_new(t) dt
    (alpha = 1), with psi, chi exact and Simpson's rule on m sub-steps."""
    if m % 2:
        raise ValueError("Simpson's rule needs an even number of sub-steps")
    E = np.asarray(E, dtype=np.float64)
    nk = len(E)
    h = dt / m
    P = [scipy.linalg.expm(-1j * (H0 - Ek * Mu) * h) for Ek in E]   # one sub-step of interval k
    psi = [np.asarray(psi0, dtype=np.complex128)]
    for k in range(nk):                        # psi at the interval starts
        y = psi[-1]
        for _ in range(m):
            y = P[k] @ y
        psi.append(y)
    S = np.vdot(target, psi[-1])
    J = float(abs(S) ** 2)
    g = np.zeros(nk)
    chi_end = np.asarray(target, dtype=np.complex128)   # chi(T) = target
    w = np.ones(m + 1)
    w[1:-1:2] = 4.0
    w[2:-1:2] = 2.0
    w *= h / 3.0
    for k in range(nk - 1, -1, -1):
        ys = [psi[k]]
        for _ in range(m):
            ys.append(P[k] @ ys[-1])
        chis = [chi_end]
        Pd = P[k].conj().T                     # chi(t - h) = P^dagger chi(t)
        for _ in range(m):
            chis.append(Pd @ chis[-1])
        chis = chis[::-1]                      # chi at the same sub-points as ys
        f = np.array([2.0 * build_field_E_new(ys[j], chis[j], Mu) for j in range(m + 1)])
        g[k] = float(np.dot(w, f))
        chi_end = chis[0]
    return J, g


def rk4_field_dense(H0: np.ndarray, Mu: np.ndarray, E: np.ndarray, psi0: np.ndarray, dt: float, nsub: int,
                    E0: float = 0.0) -> np.ndarray:
    """march_RK4_field (sub_module_propa_march.f90:397-548) on dense matrices:
    nsub classic RK4 steps of dt/nsub per field sample on H0 - E0 - E_k mu,
    each followed by the phase exp(-i E0 h)."""
    h = dt / nsub
    y = np.asarray(psi0, dtype=np.complex128).copy()
    I = np.eye(H0.shape[0])
    ph = np.exp(-1j * E0 * h)
    for Ek in E:
        A = -1j * (H0 - E0 * I - Ek * Mu)
        for _ in range(nsub):
            k1 = A @ y
            k2 = A @ (y + 0.5 * h * k1)
            k3 = A @ (y + 0.5 * h * k2)
            k4 = A @ (y + h * k3)
            y = (y + h / 6.0 * (k1 + 2 * k2 + 2 * k3 + k4)) * ph
    return y
