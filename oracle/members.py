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

    def generator_of(self, m: int, uk: np.ndarray) -> np.ndarray:
        di, sc, of, _ = self.members()
        G = self.drifts[di[m]].astype(C128).copy()
        if self.offset_op is not None and of[m] != 0.0:
            G = G + of[m] * self.offset_op
        for j in range(self.n_c):
            G = G + (sc[m] * uk[j]) * self.controls[j]
        return G

    @property
    def c(self) -> complex:
        return -1j if self.generator == "hermitian" else 1.0


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
        Gens = [prob.generator_of(m, u[:, k]) for k in range(n_t)]
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


# ----------------------------------------------------------------------------
# Builders for the benchmark workloads (seeded synthetic inputs)
# ----------------------------------------------------------------------------

SX = np.array([[0, 1], [1, 0]], C128)
SY = np.array([[0, -1j], [1j, 0]], C128)
SZ = np.array([[1, 0], [0, -1]], C128)
I2 = np.eye(2, dtype=C128)


def embed(op: np.ndarray, n: int, q: int) -> np.ndarray:
    out = np.array([[1.0 + 0j]])
    for i in range(n):
        out = np.kron(out, op if i == q else I2)
    return out


def haar_unitary(rng: np.random.Generator, d: int) -> np.ndarray:
    """QR of a complex Gaussian with the phase fix diag(sign(diag R))
    (test/fixtures/ProblemLibrary.jl:742-746)."""
    Z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2)
    Qm, R = np.linalg.qr(Z)
    ph = np.diag(R) / np.abs(np.diag(R))
    return Qm * ph[None, :]


def single_qubit_transfer(seed: int = 42, explicit_init: bool = False):
    """Quickstart problem: H_d = (2 pi 10 / 2) sz, H_c = [0.5 sx, 0.5 sy],
    100 slices over T = pi, |1> fixed-point target (legacy semantics) or the
    explicit |0> -> |1> transfer.  Amplitudes U[-0.5, 0.5] from this repo's
    seeded generator (the Julia MersenneTwister stream is not reproducible)."""
    rng = np.random.default_rng(seed)
    n_t = 100
    dt = np.pi / n_t
    u0 = 0.5 * (2 * rng.random((2, n_t)) - 1)
    psi_t = np.array([0, 1], C128)
    psi_i = np.array([1, 0], C128) if explicit_init else psi_t
    prob = Problem(drifts=(2 * np.pi * 10 / 2 * SZ)[None], controls=np.stack([0.5 * SX, 0.5 * SY]),
                   dt=np.full(n_t, dt), target="states", fidelity="square",
                   states_init=psi_i[None], states_target=psi_t[None])
    return prob, u0


def spin4_ensemble(seed: int = 7, n_t: int = 1000, n_off: int = 21, n_b1: int = 11):
    """Four coupled spin-1/2 (d=16): shifts U[-2,2] kHz, isotropic J U[5,200] Hz
    on all 6 pairs (QuantumSystem.jl:425-433), controls 2 pi sum Ix / sum Iy,
    Haar target (seed 7), dt = 1 us, amplitudes U[-10,10] kHz; ensemble of
    n_off offsets over +-1 kHz (2 pi off sum Iz) x n_b1 B1 scales 0.9..1.1."""
    rng = np.random.default_rng(seed)
    n = 4
    Ix = [embed(SX / 2, n, q) for q in range(n)]
    Iy = [embed(SY / 2, n, q) for q in range(n)]
    Iz = [embed(SZ / 2, n, q) for q in range(n)]
    shifts = rng.uniform(-2e3, 2e3, n)
    H = sum(2 * np.pi * shifts[q] * Iz[q] for q in range(n))
    for a in range(n):
        for b in range(a + 1, n):
            J = rng.uniform(5.0, 200.0)
            H = H + 2 * np.pi * J * (Ix[a] @ Ix[b] + Iy[a] @ Iy[b] + Iz[a] @ Iz[b])
    Hc = np.stack([2 * np.pi * sum(Ix), 2 * np.pi * sum(Iy)])
    T = haar_unitary(rng, 16)
    u0 = rng.uniform(-1e4, 1e4, (2, n_t))
    offs = np.linspace(-1e3, 1e3, n_off) if n_off > 1 else np.zeros(1)
    b1 = np.linspace(0.9, 1.1, n_b1) if n_b1 > 1 else np.ones(1)
    mo = np.repeat(2 * np.pi * offs, n_b1)
    ms = np.tile(b1, n_off)
    prob = Problem(drifts=H[None], controls=Hc, dt=np.full(n_t, 1e-6), offset_op=sum(Iz),
                   member_offset=mo, member_scale=ms, target="gate", fidelity="square",
                   target_op=T, n_members=n_off * n_b1)
    return prob, u0


def _rand_herm(rng, d, sigma):
    A = rng.normal(0.0, sigma, (d, d)) + 1j * rng.normal(0.0, sigma, (d, d))
    return (A + A.conj().T) / 2


def uneven_problem(rng: np.random.Generator, d: int = None, n_t: int = None, n_members: int = None):
    """One problem of the uneven batch: d uniform in {2,4,8,16,32}, n_t
    log-uniform in [50, 2000], ensemble size log-uniform in [1, 128]; drift a
    random Hermitian with Gaussian entries (sigma = 2 pi 1 MHz), 2-6 random
    Hermitian controls of the same scale, members spread by a B1 scale
    U[0.9, 1.1] and a detuning U[-0.1, 0.1] sigma along a random diagonal;
    Haar-random gate target; dt = 0.2 / (2 sigma sqrt(d)) so ||H dt|| ~ 0.2."""
    sigma = 2 * np.pi * 1e6
    d = int(rng.choice([2, 4, 8, 16, 32])) if d is None else d
    n_t = int(np.round(np.exp(rng.uniform(np.log(50), np.log(2000))))) if n_t is None else n_t
    nm = int(np.round(np.exp(rng.uniform(0.0, np.log(128))))) if n_members is None else n_members
    n_c = int(rng.integers(2, 7))
    H = _rand_herm(rng, d, sigma)
    C = np.stack([_rand_herm(rng, d, sigma) for _ in range(n_c)])
    O = np.diag(rng.uniform(-1, 1, d)).astype(C128)
    dt = 0.2 / (2 * sigma * np.sqrt(d))
    prob = Problem(drifts=H[None], controls=C, dt=np.full(n_t, dt), offset_op=O,
                   member_scale=rng.uniform(0.9, 1.1, nm), member_offset=rng.uniform(-0.1, 0.1, nm) * sigma,
                   target="gate", fidelity="square", target_op=haar_unitary(rng, d), n_members=nm)
    return prob, rng.uniform(-1, 1, (n_c, n_t))


def uneven_batch(n_problems: int = 512, seed: int = 4):
    rng = np.random.default_rng(seed)
    return [uneven_problem(rng) for _ in range(n_problems)]


def lindblad_3q(seed: int = 11, n_t: int = 500, n_draws: int = 32):
    """Three qubits, ZZ U[0.1,1] MHz on 3 pairs, detuning U[-0.5,0.5] MHz per
    qubit (redrawn per ensemble member), T1 U[20,100] us, T2 = T1 U(0.5,1);
    jumps sqrt(1/T1) s-  and sqrt(g_phi/2) sz with g_phi = 1/T2 - 1/(2 T1);
    controls sx_q, sy_q (x 2 pi 1 MHz); CCZ gate target as the superoperator
    conj(U) (x) U; 500 slices over 2 us."""
    rng = np.random.default_rng(seed)
    n = 3
    sm = np.array([[0, 1], [0, 0]], C128)
    ZZ = sum(2 * np.pi * rng.uniform(0.1e6, 1e6) * embed(SZ, n, a) @ embed(SZ, n, b)
             for a in range(n) for b in range(a + 1, n))
    T1 = rng.uniform(20e-6, 100e-6, n)
    T2 = T1 * rng.uniform(0.5, 1.0, n)
    jumps, rates = [], []
    for q in range(n):
        jumps.append(embed(sm, n, q))
        rates.append(1.0 / T1[q])
        gphi = 1.0 / T2[q] - 1.0 / (2 * T1[q])
        jumps.append(embed(SZ, n, q))
        rates.append(max(gphi, 0.0) / 2.0)
    drifts = []
    for _ in range(n_draws):
        det = rng.uniform(-0.5e6, 0.5e6, n)
        Hd = ZZ + sum(2 * np.pi * det[q] * embed(SZ, n, q) / 2 for q in range(n))
        drifts.append(rs.build_drift_liouvillian(Hd, jumps, rates))
    ctrls = []
    for q in range(n):
        ctrls.append(rs.build_control_liouvillian(2 * np.pi * 1e6 * embed(SX, n, q) / 2))
        ctrls.append(rs.build_control_liouvillian(2 * np.pi * 1e6 * embed(SY, n, q) / 2))
    ccz = np.diag([1, 1, 1, 1, 1, 1, 1, -1]).astype(C128)
    S = np.kron(ccz.conj(), ccz)
    u0 = rng.uniform(-0.5, 0.5, (2 * n, n_t))
    prob = Problem(drifts=np.stack(drifts), controls=np.stack(ctrls), dt=np.full(n_t, 2e-6 / n_t),
                   generator="liouvillian", member_drift=np.arange(n_draws), target="gate",
                   fidelity="square", target_op=S, n_members=n_draws)
    return prob, u0
