"""Oracle for the C-ABI problem model (``pgx_problem_desc`` in include/pgx.h).

TEST INFRASTRUCTURE ONLY -- the checker for the CUDA path, never part of it.

The library evaluates an *ensemble of members*.  Member m is the reference's
``QuantumSystem`` (or MR (drift, pwr) pair) with

    generator  G_m(u_k) = drift[drift_m] + offset_m * O + scale_m * sum_j u_jk C_j
    propagator U_mk     = exp(c * dt_k * G_m(u_k)),  c = -i (Hermitian H) or 1 (Liouvillian)

and the objective is  F = sum_m w_m sum_s f(z_ms)  with

    gate target : z_m  = Tr(T' U_m,total) / D          (Objectives.jl:239-246)
    state pairs : z_ms = <psi_t,s | U_m,total psi_i,s>  (Objectives.jl:221, GRAPEState.jl:208-211)
    f = |z|^2 (square) | Re z (real) | |z| (modulus).

Gradient modes:

* "ref_grape" restates the first-order formula of the GRAPE path
  (Gradients.jl:254-291 gate, :357-399 states): dU_k/du_jk is replaced by
  U_k (c dt_k scale_m C_j), because the backward chain Q[k] there contains
  U_k (Propagators.jl:399-404).
* "ref_mr" restates the MR kernels (GRAPEState.jl:220-230,
  GRAPELindblad.jl:183-195): dU_k/du_jk is replaced by (c dt_k scale_m C_j)
  alone, between the state before slice k and the costate after it; the
  Liouvillian case uses the Re prefactor of Lindblad.jl:220-232.
  In both first-order modes the chain-rule coefficient kappa is 2 conj(z)
  (square), 1 (real) and -- as in Objectives.jl:356-361 -- 1/|z| (modulus).
* EXACT uses the Frechet derivative dU_k = L_exp(A_k, c dt_k scale_m C_j)
  and the true chain rule (modulus: conj(z)/|z|).

With unit weights-per-member and one member this reduces exactly to the
reference's single-system functions; ``tests/test_oracle_kats.py`` checks
those identities against ``ref_semantics``.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import scipy.linalg as sla

from . import ref_semantics as rs

C128 = np.complex128


@dataclass
class Problem:
    """numpy mirror of pgx_problem_desc (matrices indexed [row, col])."""
    drifts: np.ndarray                 # [n_drift, D, D]
    controls: np.ndarray               # [n_c, D, D]
    dt: np.ndarray                     # [n_t]
    generator: str = "hermitian"       # "hermitian" | "liouvillian"
    offset_op: Optional[np.ndarray] = None
    member_drift: Optional[np.ndarray] = None
    member_scale: Optional[np.ndarray] = None
    member_offset: Optional[np.ndarray] = None
    member_weight: Optional[np.ndarray] = None
    target: str = "gate"               # "gate" | "states"
    fidelity: str = "square"           # "square" | "real" | "modulus"
    target_op: Optional[np.ndarray] = None
    states_init: Optional[np.ndarray] = None    # [n_pairs, D]
    states_target: Optional[np.ndarray] = None  # [n_pairs, D]
    n_members: int = 1
    # per-slice drift ramp: member m adds tau[k] ramp_ops[member_ramp[m]] at slice k
    ramp_ops: Optional[np.ndarray] = None       # [n_ops, D, D]
    member_ramp: Optional[np.ndarray] = None    # [n_members], -1 = none
    tau: Optional[np.ndarray] = None            # [n_t]

    @property
    def D(self) -> int:
        return self.drifts.shape[1]

    @property
    def n_c(self) -> int:
        return self.controls.shape[0]

    @property
    def n_t(self) -> int:
        return len(self.dt)

    @property
    def n_pairs(self) -> int:
        return 0 if self.target == "gate" else self.states_init.shape[0]

    def members(self):
        n = self.n_members
        di = np.zeros(n, int) if self.member_drift is None else np.asarray(self.member_drift)
        sc = np.ones(n) if self.member_scale is None else np.asarray(self.member_scale, float)
        of = np.zeros(n) if self.member_offset is None else np.asarray(self.member_offset, float)
        if self.member_weight is None:
            w = np.full(n, 1.0 / (n * max(self.n_pairs, 1)))
        else:
            w = np.asarray(self.member_weight, float)
        return di, sc, of, w

    def generator_of(self, m: int, uk: np.ndarray, k: Optional[int] = None) -> np.ndarray:
        di, sc, of, _ = self.members()
        G = self.drifts[di[m]].astype(C128).copy()
        if self.offset_op is not None and of[m] != 0.0:
            G = G + of[m] * self.offset_op
        if self.ramp_ops is not None and k is not None and self.member_ramp[m] >= 0:
            G = G + self.tau[k] * self.ramp_ops[self.member_ramp[m]]
        for j in range(self.n_c):
            G = G + (sc[m] * uk[j]) * self.controls[j]
        return G

    @property
    def c(self) -> complex:
        return -1j if self.generator == "hermitian" else 1.0

    def member_problem(self, m: int) -> "Problem":
        """Member m alone, with its own weight: its evaluation is member m's
        contribution to F and G."""
        di, sc, of, w = self.members()
        return dataclasses.replace(
            self, member_drift=di[m:m + 1], member_scale=sc[m:m + 1], member_offset=of[m:m + 1],
            member_weight=w[m:m + 1], n_members=1,
            member_ramp=None if self.member_ramp is None else np.array(self.member_ramp[m:m + 1]))

    def subproblem(self, n_members: int, n_t: int) -> "Problem":
        """The first n_members members over the first n_t slices (weights kept)."""
        di, sc, of, w = self.members()
        nm = min(n_members, self.n_members)
        return dataclasses.replace(
            self, dt=np.array(self.dt[:n_t]), member_drift=di[:nm], member_scale=sc[:nm],
            member_offset=of[:nm], member_weight=w[:nm], n_members=nm,
            member_ramp=None if self.member_ramp is None else np.array(self.member_ramp[:nm]),
            tau=None if self.tau is None else np.array(self.tau[:n_t]))

    @classmethod
    def from_spec(cls, spec) -> "Problem":
        """Copy of any object with the pgx_problem_desc fields (the package's
        seeded workload specs): the oracle keeps its own reading of them."""
        names = ("drifts", "controls", "dt", "generator", "offset_op", "member_drift", "member_scale",
                 "member_offset", "member_weight", "target", "fidelity", "target_op", "states_init",
                 "states_target", "n_members")
        kw = {}
        for n in names:
            v = getattr(spec, n)
            kw[n] = np.array(v) if isinstance(v, np.ndarray) else v
        return cls(**kw)


def _propagator(prob: Problem, G: np.ndarray, dt: float) -> np.ndarray:
    if prob.generator == "hermitian":
        return rs.expm_neg_i(G, dt)               # Propagators.jl:659-674
    return rs.expm_general(G * dt)                 # GRAPELindblad.jl:146-153


def frechet_exp(A: np.ndarray, E: np.ndarray, hermitian_generator_dt=None) -> np.ndarray:
    """L_exp(A, E).  For A = -i H dt (H Hermitian) the spectral form
    V (Gamma o (V' E V)) V' with exact divided differences is used; otherwise
    scipy's Al-Mohy-Higham Frechet algorithm."""
    if hermitian_generator_dt is not None:
        H, dt = hermitian_generator_dt
        lam, V = np.linalg.eigh(H)
        th = lam * dt                          # A = V diag(-i th) V'
        tp, tq = th[:, None], th[None, :]
        y = (tp - tq) / 2.0
        Gam = np.exp(-1j * (tp + tq) / 2.0) * np.sinc(y / np.pi)
        return V @ (Gam * (V.conj().T @ E @ V)) @ V.conj().T
    return sla.expm_frechet(A, E, compute_expm=False)


def _f_and_kappa(z: complex, fid: str, mode: str):
    if fid == "square":
        return abs(z) ** 2, 2.0 * np.conj(z)
    if fid == "real":
        return z.real, 1.0 + 0j
    if fid == "modulus":
        az = abs(z)
        if mode != "exact":
            return az, (0j if az < 1e-14 else 1.0 / az + 0j)
        return az, (0j if az < 1e-14 else np.conj(z) / az)
    raise ValueError(fid)


GRAD_MODES = ("ref_grape", "ref_mr", "exact")


def eval_problem(prob: Problem, u: np.ndarray, grad_mode: str = "exact", want_grad: bool = True,
                 per_member: bool = False):
    """(F, G[n_c, n_t]) exactly as pgx_eval defines them.

    Backward arrays from ``rs.backward_propagators``: Q[k] includes U_k, so the
    costate after slice k is Q[k+1] and the one before it is Q[k]."""
    if grad_mode not in GRAD_MODES:
        raise ValueError(grad_mode)
    u = np.asarray(u, float)
    n_c, n_t, D = prob.n_c, prob.n_t, prob.D
    di, sc, of, w = prob.members()
    F = 0.0
    G = np.zeros((n_c, n_t))
    Fm_list = []
    for m in range(prob.n_members):
        Gens = [prob.generator_of(m, u[:, k], k) for k in range(n_t)]
        U = np.stack([_propagator(prob, Gens[k], float(prob.dt[k])) for k in range(n_t)]) \
            if n_t else np.zeros((0, D, D), C128)
        P = rs.forward_propagators(U)
        Q = rs.backward_propagators(U)
        Utot = P[-1]
        Fm = 0.0
        if prob.target == "gate":
            T = np.asarray(prob.target_op, C128)
            z = np.trace(T.conj().T @ Utot) / D
            f, kap = _f_and_kappa(z, prob.fidelity, grad_mode)
            Fm += f
            if want_grad:
                for k in range(n_t):
                    if grad_mode != "exact":
                        Qk = Q[k] if grad_mode == "ref_grape" else Q[k + 1]
                        Mk = P[k] @ T.conj().T @ Qk.conj().T / D     # Gradients.jl:278-279
                        for j in range(n_c):
                            dz = np.sum(Mk * (prob.c * prob.dt[k] * sc[m] * prob.controls[j]).T)
                            G[j, k] += w[m] * (kap * dz).real
                    else:
                        A = prob.c * prob.dt[k] * Gens[k]
                        for j in range(n_c):
                            E = prob.c * prob.dt[k] * sc[m] * prob.controls[j]
                            L = frechet_exp(A, E, (Gens[k], prob.dt[k])
                                            if prob.generator == "hermitian" else None)
                            dz = np.trace(T.conj().T @ Q[k + 1].conj().T @ L @ P[k]) / D
                            G[j, k] += w[m] * (kap * dz).real
        else:
            for s in range(prob.n_pairs):
                psi_i = np.asarray(prob.states_init[s], C128)
                psi_t = np.asarray(prob.states_target[s], C128)
                z = np.vdot(psi_t, Utot @ psi_i)
                f, kap = _f_and_kappa(z, prob.fidelity, grad_mode)
                Fm += f
                if want_grad:
                    for k in range(n_t):
                        phi = P[k] @ psi_i                 # state before slice k
                        lam = Q[k + 1] @ psi_t             # costate after slice k
                        lam_before = Q[k] @ psi_t          # costate before slice k
                        for j in range(n_c):
                            E = prob.c * prob.dt[k] * sc[m] * prob.controls[j]
                            if grad_mode == "ref_grape":
                                dz = np.vdot(lam_before, E @ phi)
                            elif grad_mode == "ref_mr":
                                dz = np.vdot(lam, E @ phi)
                            else:
                                A = prob.c * prob.dt[k] * Gens[k]
                                L = frechet_exp(A, E, (Gens[k], prob.dt[k])
                                                if prob.generator == "hermitian" else None)
                                dz = np.vdot(lam, L @ phi)
                            G[j, k] += w[m] * (kap * dz).real
        Fm_list.append(Fm)
        F += w[m] * Fm
    if per_member:
        return F, G, np.array(Fm_list)
    return F, G



def eval_gate_exact_adjoint(prob: Problem, u: np.ndarray):
    """(F, G) of a gate-target problem with the exact gradient, evaluated with
    one Frechet derivative per slice instead of one per control.

    The exact gradient is dz_jk = Tr(T' Q_{k+1}' L(A_k, E_jk) P_k) / D
    = Tr(M_k L(A_k, E_jk)) with M_k = P_k T' Q_{k+1}' / D, and for the
    exponential (a power series with scalar coefficients)
    Tr(M L(A, E)) = Tr(L(A, M) E).  So X_k = L(A_k, M_k) is formed once per
    slice (spectral form for Hermitian generators, scipy's Al-Mohy-Higham
    Frechet algorithm for Liouvillians) and contracted with every control.
    Same result as eval_problem(prob, u, "exact") up to rounding."""
    if prob.target != "gate":
        raise ValueError("gate targets only")
    u = np.asarray(u, float)
    n_c, n_t, D = prob.n_c, prob.n_t, prob.D
    di, sc, of, w = prob.members()
    T = np.asarray(prob.target_op, C128)
    F, G = 0.0, np.zeros((n_c, n_t))
    for m in range(prob.n_members):
        Gens = [prob.generator_of(m, u[:, k], k) for k in range(n_t)]
        U = np.stack([_propagator(prob, Gens[k], float(prob.dt[k])) for k in range(n_t)])
        P = rs.forward_propagators(U)
        Q = rs.backward_propagators(U)
        z = np.trace(T.conj().T @ P[-1]) / D
        f, kap = _f_and_kappa(z, prob.fidelity, "exact")
        F += w[m] * f
        for k in range(n_t):
            M = P[k] @ T.conj().T @ Q[k + 1].conj().T / D
            A = prob.c * prob.dt[k] * Gens[k]
            X = frechet_exp(A, M, (Gens[k], prob.dt[k]) if prob.generator == "hermitian" else None)
            for j in range(n_c):
                E = prob.c * prob.dt[k] * sc[m] * prob.controls[j]
                G[j, k] += w[m] * (kap * np.sum(X * E.T)).real
    return F, G
