"""Seeded synthetic SG4 workloads (the benchmark configurations).

No public dataset exists for this path: every workload is generated from a
numpy PCG64 seed ``20261203 + config_index`` with the shapes and value
distributions of the benchmark description.  Builder decisions recorded here:

* Modes are harmonic-oscillator ("HO"/"Hm") bases with nb(l) = l+1,
  nq(l) = l+2 (L_TO_nb_A=1, B=1; L_TO_nq_A=2, B=1), LB = L.
* V(Q) = sum_i 1/2 w_i Q_i^2 (mass 1, so mode i has frequency sqrt(w_i)),
  w_i ~ U[0.005, 0.02] hartree.  Couplings are written in the dimensionless
  coordinates y_i = s_i Q_i with the matched scaling s_i = w_i^(1/4) (also
  the basis scaleQ, Q0 = 0): all cubic terms c_ijk y_i y_j y_k (i<=j<=k) and
  quartic terms q_ij y_i^2 y_j^2 (i<=j), coefficients ~ N(0, 0.01 * mean(w)).
* Constant-G kinetic energy (type 1): -1/2 sum_i d^2/dQ_i^2 (F2 = -1/2 I).
* Q-dependent G (type 10): G_ij(Q) = delta_ij + 0.05 sum_k g_ijk y_k with
  g_ijk ~ N(0, 1/D) symmetrised in (i, j); Jac = rho = 1 (Euclidean volume
  element, sqRhoOVERJac = 1).
* psi: N(0, 1) entries, each column normalised.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from .sg4 import ParamOp, Polynomial, SG4Basis

SEED0 = 20261203


@dataclass
class SG4Model:
    D: int
    L: int
    omega: np.ndarray
    scaleQ: np.ndarray
    V: Polynomial
    type_op: int
    F2: Optional[np.ndarray] = None
    G0: Optional[np.ndarray] = None
    G1: Optional[np.ndarray] = None
    extras: dict = field(default_factory=dict)

    def basis(self) -> SG4Basis:
        return SG4Basis(self.D, self.L, self.L, 1, 1, 2, 1, Q0=np.zeros(self.D), scaleQ=self.scaleQ)

    def operator(self, basis: Optional[SG4Basis] = None, field_budget: int = 0) -> ParamOp:
        b = basis if basis is not None else self.basis()
        if self.type_op == 1:
            return ParamOp(b, 1, V_poly=self.V, F2=self.F2, field_budget=field_budget)
        return ParamOp(b, 10, V_poly=self.V, G0=self.G0, G1=self.G1, field_budget=field_budget)

    def G_grid(self, Q: np.ndarray, nq_per_term: np.ndarray) -> np.ndarray:
        """GGiq(iq, j, i) per term, concatenated (what the oracle consumes)."""
        D = self.D
        nq_per_term = np.asarray(nq_per_term, dtype=np.int64)
        off = np.concatenate([[0], np.cumsum(nq_per_term)[:-1]])
        g = self.G0[None, :, :] + np.einsum("ijk,pk->pij", self.G1, Q)   # [p, i, j]
        offp = np.repeat(off, nq_per_term)
        nqp = np.repeat(nq_per_term, nq_per_term)
        local = np.arange(Q.shape[0], dtype=np.int64) - offp
        ij = (D * np.arange(D)[:, None] + np.arange(D)[None, :]).ravel()      # D*i + j
        dest = (offp * D * D + local)[:, None] + nqp[:, None] * ij[None, :]
        out = np.empty(Q.shape[0] * D * D)
        out[dest.ravel()] = g.reshape(Q.shape[0], D * D).ravel()
        return out


def _potential(rng, D, omega, s):
    wbar = float(np.mean(omega))
    coef, expo = [], []
    for i in range(D):
        e = np.zeros(D, dtype=np.int32)
        e[i] = 2
        coef.append(0.5 * omega[i])
        expo.append(e)
    for i in range(D):
        for j in range(i, D):
            for k in range(j, D):
                c = rng.normal(0.0, 0.01 * wbar)
                e = np.zeros(D, dtype=np.int32)
                e[i] += 1
                e[j] += 1
                e[k] += 1
                coef.append(c * s[i] * s[j] * s[k])
                expo.append(e)
    for i in range(D):
        for j in range(i, D):
            c = rng.normal(0.0, 0.01 * wbar)
            e = np.zeros(D, dtype=np.int32)
            e[i] += 2
            e[j] += 2
            coef.append(c * s[i] ** 2 * s[j] ** 2)
            expo.append(e)
    return Polynomial(np.array(coef), np.array(expo, dtype=np.int32))


def make_model(D: int, L: int, type_op: int, seed: int) -> SG4Model:
    rng = np.random.Generator(np.random.PCG64(seed))
    omega = rng.uniform(0.005, 0.02, size=D)
    s = omega ** 0.25
    V = _potential(rng, D, omega, s)
    if type_op == 1:
        return SG4Model(D, L, omega, s, V, 1, F2=-0.5 * np.eye(D))
    g = rng.normal(0.0, 1.0 / np.sqrt(D), size=(D, D, D))
    g = 0.5 * (g + g.transpose(1, 0, 2))
    G1 = 0.05 * g * s[None, None, :]
    return SG4Model(D, L, omega, s, V, 10, G0=np.eye(D), G1=G1)


def make_dipole(model: SG4Model, seed: int) -> Polynomial:
    """mu(Q) = sum_i a_i y_i + sum_{i<=j} b_ij y_i y_j, a ~ N(0,1), b ~ N(0,0.1),
    in the dimensionless coordinates y = scaleQ Q (the optimal-control workload)."""
    rng = np.random.Generator(np.random.PCG64(seed + 11))
    D, s = model.D, model.scaleQ
    coef, expo = [], []
    for i in range(D):
        e = np.zeros(D, dtype=np.int32)
        e[i] = 1
        coef.append(rng.normal(0.0, 1.0) * s[i])
        expo.append(e)
    for i in range(D):
        for j in range(i, D):
            e = np.zeros(D, dtype=np.int32)
            e[i] += 1
            e[j] += 1
            coef.append(rng.normal(0.0, 0.1) * s[i] * s[j])
            expo.append(e)
    return Polynomial(np.array(coef), np.array(expo, dtype=np.int32))


def random_psi(N: int, nrhs: int, seed: int, complex_: bool = False) -> np.ndarray:
    """(N, nrhs) column-normalised N(0,1) vectors."""
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    a = rng.normal(size=(N, nrhs))
    if complex_:
        a = a + 1j * rng.normal(size=(N, nrhs))
    return a / np.linalg.norm(a, axis=0, keepdims=True)


def config(index: int) -> dict:
    """The benchmark configurations by index (sizes only; see module docstring)."""
    seed = SEED0 + index
    if index == 0:
        return dict(name="3-D L=6 HO SG4, type 1, 1 RHS", model=make_model(3, 6, 1, seed), nrhs=1, seed=seed)
    if index == 1:
        return dict(name="6-D L=8 HO SG4, type 10 (Q-dependent G), 20 RHS", model=make_model(6, 8, 10, seed),
                    nrhs=20, seed=seed)
    if index == 3:
        return dict(name="4-D L=7 HO SG4, type 1, complex", model=make_model(4, 7, 1, seed), nrhs=1, seed=seed)
    raise ValueError(f"config {index} is not a single-operator workload")


def uneven_instances(n: int = 64, seed: int = SEED0 + 2):
    """Config 2's 64 independent Hamiltonians: d ~ U{3..9}, L ~ U{4..10}."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n):
        d = int(rng.integers(3, 10))
        L = int(rng.integers(4, 11))
        out.append(make_model(d, L, 1, seed * 1000 + k))
    return out
