"""FP64 CPU restatement of Pulsar.jl's GRAPE fidelity-and-gradient path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: the parity tests, the
graft entry's smoke check and the CPU-baseline leg of ``bench.py`` use it as
the checker.  Nothing in the product path (``pulsar.jl_gb300``) imports it.

Every function restates one reference function in numpy/scipy and cites the
reference file and lines it follows (paths inside the Pulsar.jl project).
Conventions kept from the reference:

* matrices are indexed ``A[row, col]``; the C-ABI buffers are column-major,
  interleaved (re, im) -- ``to_colmajor`` / ``from_colmajor`` convert;
* ``ControlSequence.amplitudes`` is ``[n_t, n_c]`` and ``.controls`` its
  transpose ``[n_c, n_t]`` (src/Types/ControlSequence.jl:37-41,99-110);
* propagator stacks are ``[n_t(+1), d, d]`` (src/Computation/Propagators.jl:510-513).

Parity anchor: Julia is not installed here, so the reference cannot be run.
The restatement is pinned by the reference's own known-answer tests and
invariants (test/Physics/MathematicalCorrectness.jl, PhysicsValidation.jl,
test/Algorithms/EnsembleTests.jl, GRAPETests.jl), re-implemented in
``tests/test_oracle_kats.py``, and by the committed fixtures in
``tests/golden/`` made by ``tests/golden/make_fixtures.py``.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np
import scipy.linalg as sla

C128 = np.complex128


# ----------------------------------------------------------------------------
# Layout helpers (C-ABI buffers <-> numpy)
# ----------------------------------------------------------------------------

def to_colmajor(A: np.ndarray) -> np.ndarray:
    """Square complex matrix (or stack [..., D, D]) -> column-major buffer."""
    A = np.asarray(A, dtype=C128)
    return np.ascontiguousarray(np.swapaxes(A, -1, -2))


def from_colmajor(buf: np.ndarray, D: int) -> np.ndarray:
    b = np.asarray(buf, dtype=C128).reshape(-1, D, D)
    out = np.swapaxes(b, -1, -2).copy()
    return out[0] if out.shape[0] == 1 and np.asarray(buf).size == D * D else out


# ----------------------------------------------------------------------------
# Types (src/Types/QuantumSystem.jl:60-66, ControlSequence.jl:37-59,
# Targets.jl:37-43)
# ----------------------------------------------------------------------------

@dataclass
class QuantumSystem:
    H_drift: np.ndarray
    H_controls: list

    @property
    def dim(self) -> int:
        return self.H_drift.shape[0]

    @property
    def n_controls(self) -> int:
        return len(self.H_controls)


@dataclass
class ControlSequence:
    """amplitudes is [n_steps, n_controls] (ControlSequence.jl:37-41)."""
    amplitudes: np.ndarray
    dt: float

    @property
    def controls(self) -> np.ndarray:  # [n_c, n_t] view (ControlSequence.jl:99-103)
        return self.amplitudes.T

    @property
    def n_timesteps(self) -> int:
        return self.amplitudes.shape[0]

    @classmethod
    def from_controls(cls, controls: np.ndarray, dt: float) -> "ControlSequence":
        """4-argument outer constructor: [n_c, n_t] -> transposed storage
        (ControlSequence.jl:77-89)."""
        return cls(np.ascontiguousarray(np.asarray(controls, float).T), float(dt))


@dataclass
class QuantumTarget:
    type: str                       # "unitary" | "state"
    target_state: Optional[np.ndarray] = None
    target_unitary: Optional[np.ndarray] = None
    initial_state: Optional[np.ndarray] = None

    @property
    def dim(self) -> int:
        if self.type == "unitary":
            return self.target_unitary.shape[0]
        return self.target_state.shape[0]


def state_target(state, psi_init=None) -> QuantumTarget:
    """src/Types/Targets.jl:77-107 (validation: non-empty, finite, non-zero)."""
    psi = np.asarray(state, dtype=C128)
    if psi.size == 0:
        raise ValueError("Target state vector must be non-empty")
    if not np.all(np.isfinite(psi)):
        raise ValueError("Target state contains NaN or Inf values")
    if np.linalg.norm(psi) < np.finfo(float).eps:
        raise ValueError("Target state has zero norm")
    pi = None
    if psi_init is not None:
        pi = np.asarray(psi_init, dtype=C128)
        if pi.size != psi.size:
            raise ValueError("psi_init has wrong length")
        if np.linalg.norm(pi) < np.finfo(float).eps:
            raise ValueError("psi_init has zero norm")
    return QuantumTarget("state", target_state=psi, initial_state=pi)


def unitary_target(U) -> QuantumTarget:
    """src/Types/Targets.jl:131-144: ||U'U - I|| / d <= 1e-8."""
    U = np.asarray(U, dtype=C128)
    m, n = U.shape
    if m != n:
        raise ValueError("Target unitary must be square")
    if np.linalg.norm(U.conj().T @ U - np.eye(m)) / m > 1e-8:
        raise ValueError("Target matrix is not unitary")
    return QuantumTarget("unitary", target_unitary=U)


# ----------------------------------------------------------------------------
# Computation layer (src/Computation/Propagators.jl)
# ----------------------------------------------------------------------------

def build_total_hamiltonian(system: QuantumSystem, controls: ControlSequence) -> np.ndarray:
    """H_k = H_drift + sum_j amplitudes[k, j] H_j  (Propagators.jl:485-544)."""
    amps = controls.amplitudes
    n_t, n_c = amps.shape
    if n_c != system.n_controls:
        raise ValueError("controls/system n_controls mismatch")
    Hc = np.stack([np.asarray(h, C128) for h in system.H_controls]) if n_c else \
        np.zeros((0,) + system.H_drift.shape, C128)
    return system.H_drift[None, :, :] + np.einsum("kj,jab->kab", amps, Hc)


def expm_neg_i(H: np.ndarray, dt: float) -> np.ndarray:
    """exp(-i H dt) = V diag(cis(-lambda dt)) V'  (Propagators.jl:659-674, :64-90)."""
    if dt == 0.0:
        return np.eye(H.shape[0], dtype=C128)
    lam, V = np.linalg.eigh(H)
    return (V * np.exp(-1j * lam * dt)[None, :]) @ V.conj().T


def compute_propagators(H_total: np.ndarray, dt) -> np.ndarray:
    """Per-slice propagators (Propagators.jl:127-184).  ``dt`` may be a scalar
    or a per-slice array (MR ``pulse_dt``, GRAPEState.jl:187-193)."""
    n_t = H_total.shape[0]
    dts = np.broadcast_to(np.asarray(dt, float), (n_t,))
    return np.stack([expm_neg_i(H_total[k], float(dts[k])) for k in range(n_t)]) \
        if n_t else np.zeros_like(H_total)


def compute_total_propagator(props: np.ndarray) -> np.ndarray:
    """U_total = U_n ... U_1, identity for n=0 (Propagators.jl:212-238)."""
    d = props.shape[1]
    U = np.eye(d, dtype=C128)
    for k in range(props.shape[0]):
        U = props[k] @ U
    return U


def forward_propagators(props: np.ndarray) -> np.ndarray:
    """P[0] = I, P[k+1] = U_k P[k]  (Propagators.jl:309-325)."""
    n_t, d, _ = props.shape
    P = np.empty((n_t + 1, d, d), C128)
    P[0] = np.eye(d)
    for k in range(n_t):
        P[k + 1] = props[k] @ P[k]
    return P


def backward_propagators(props: np.ndarray, seed=None) -> np.ndarray:
    """Q[n] = I (or seed), Q[k] = U_k' Q[k+1]  (Propagators.jl:390-440).

    The reference's code multiplies by the slice's OWN propagator
    (``mul!(Q_out, U_k', Q_nxt)`` with ``U_k = propagators[k]``,
    Propagators.jl:399-404), so Q[k] = (U_{n-1} ... U_k)' includes U_k, even
    though its docstring (:335-345) describes U_{k+1}' ... U_n'.  The code is
    what the gradients consume, so it is restated here (0-based slices)."""
    n_t, d, _ = props.shape
    Q = np.empty((n_t + 1, d, d), C128)
    Q[n_t] = np.eye(d) if seed is None else seed
    for k in range(n_t - 1, -1, -1):
        Q[k] = props[k].conj().T @ Q[k + 1]
    return Q


# ----------------------------------------------------------------------------
# Physics layer: objectives (src/Physics/Objectives.jl)
# ----------------------------------------------------------------------------

def gate_fidelity(U: np.ndarray, U_target: np.ndarray) -> float:
    """:normalized -> |Tr(U_t' U)/d|^2  (Objectives.jl:239-246)."""
    d = U.shape[0]
    return float(abs(np.trace(U_target.conj().T @ U) / d) ** 2)


def state_fidelity(psi_t, psi_f, type: str = "real") -> float:
    """Objectives.jl:221-225 (:real, :square, :modulus)."""
    z = np.vdot(psi_t, psi_f)
    if type == "real":
        return float(z.real)
    if type == "square":
        return float(abs(z) ** 2)
    if type == "modulus":
        return float(abs(z))
    raise ValueError(f"unsupported state fidelity type {type}")


def fidelity_grad_prefactor(z: complex, inner: complex, dt_pwr: float, type: str) -> float:
    """Hilbert-space chain-rule coefficient (Objectives.jl:352-361).
    Note the reference's :modulus form is dt_pwr*Im(inner/|z|), kept verbatim."""
    if type == "real":
        return dt_pwr * inner.imag
    if type == "square":
        return 2.0 * dt_pwr * (np.conj(z) * inner).imag
    if type == "modulus":
        az = abs(z)
        return 0.0 if az < 1e-14 else dt_pwr * (inner / az).imag
    raise ValueError(type)


def lindblad_grad_prefactor(z: complex, inner: complex, dt_pwr: float, type: str) -> float:
    """Liouville-space coefficient, Re instead of Im (src/Physics/Lindblad.jl:220-232)."""
    if type == "square":
        return 2.0 * dt_pwr * (np.conj(z) * inner).real
    if type == "real":
        return dt_pwr * inner.real
    raise ValueError(type)


def compute_fidelity_U(U_total: np.ndarray, target: QuantumTarget) -> float:
    """Legacy dispatcher (Objectives.jl:609-630): gate -> :normalized; state ->
    :square with psi_init = initial_state, or target_state when unset."""
    if target.type == "unitary":
        return gate_fidelity(U_total, target.target_unitary)
    if target.type == "state":
        psi_init = target.target_state if target.initial_state is None else target.initial_state
        return state_fidelity(target.target_state, U_total @ psi_init, "square")
    raise ValueError(target.type)


def compute_fidelity(system: QuantumSystem, controls: ControlSequence,
                     target: QuantumTarget) -> float:
    """Objectives.jl:632-639."""
    H = build_total_hamiltonian(system, controls)
    return compute_fidelity_U(compute_total_propagator(compute_propagators(H, controls.dt)), target)


# ----------------------------------------------------------------------------
# Physics layer: first-order GRAPE gradients (src/Physics/Gradients.jl)
# ----------------------------------------------------------------------------

def gate_gradient(U_total, P, Q, H_controls, U_target, dt) -> np.ndarray:
    """_gate_gradient_into! (Gradients.jl:254-291):
    A_k = P_k U_t' Q_k';  G[j,k] = 2 Re(conj(Phi) (-i dt/d) sum_pq A_k[p,q] H_j[q,p])."""
    n_t = P.shape[0] - 1
    d = U_total.shape[0]
    dts = np.broadcast_to(np.asarray(dt, float), (n_t,))
    Phi = np.trace(U_target.conj().T @ U_total) / d
    Utd = U_target.conj().T
    G = np.zeros((len(H_controls), n_t))
    for k in range(n_t):
        A = P[k] @ Utd @ Q[k].conj().T
        for j, Hj in enumerate(H_controls):
            s = np.sum(A * Hj.T)
            inner = -1j * dts[k] * s / d
            G[j, k] = 2.0 * (np.conj(Phi) * inner).real
    return G


def state_gradient(U_total, P, Q, H_controls, psi_init, psi_target, dt) -> np.ndarray:
    """_state_gradient_into! (Gradients.jl:357-399): states are normalised;
    phi_k = P_k psi_i, lambda_k = Q_k psi_t,
    G[j,k] = 2 Re(conj(chi) (-i dt) <lambda_k|H_j|phi_k>)."""
    n_t = P.shape[0] - 1
    dts = np.broadcast_to(np.asarray(dt, float), (n_t,))
    ni, nt = np.linalg.norm(psi_init), np.linalg.norm(psi_target)
    if ni < np.finfo(float).eps or nt < np.finfo(float).eps:
        raise ValueError("zero-norm state")
    psi_i, psi_t = psi_init / ni, psi_target / nt
    chi = np.vdot(psi_t, U_total @ psi_i)
    G = np.zeros((len(H_controls), n_t))
    for k in range(n_t):
        phi = P[k] @ psi_i
        lam = Q[k] @ psi_t
        for j, Hj in enumerate(H_controls):
            inner = -1j * dts[k] * np.vdot(lam, Hj @ phi)
            G[j, k] = 2.0 * (np.conj(chi) * inner).real
    return G


def compute_grape_gradient(system: QuantumSystem, controls: ControlSequence,
                           target: QuantumTarget) -> np.ndarray:
    """Gradients.jl:80-127; honours target.initial_state for state targets."""
    H = build_total_hamiltonian(system, controls)
    U = compute_propagators(H, controls.dt)
    P, Q = forward_propagators(U), backward_propagators(U)
    U_total = P[-1]
    if target.type == "unitary":
        return gate_gradient(U_total, P, Q, system.H_controls, target.target_unitary, controls.dt)
    psi_init = target.target_state if target.initial_state is None else target.initial_state
    return state_gradient(U_total, P, Q, system.H_controls, psi_init, target.target_state,
                          controls.dt)


def compute_grape_gradient_with(system, target, P, Q, U_total, dt) -> np.ndarray:
    """Gradients.jl:141-163 -- the form grape_optimize calls.  For state
    targets it uses target_state on BOTH sides, even when initial_state is set
    (Gradients.jl:153-157)."""
    if target.type == "unitary":
        return gate_gradient(U_total, P, Q, system.H_controls, target.target_unitary, dt)
    return state_gradient(U_total, P, Q, system.H_controls, target.target_state,
                          target.target_state, dt)


def aggregate(fv, gv, aggregator: str, alpha: float = 0.2):
    """_agg_value / _agg_grad! of EnsembleObjective.jl:169-217: mean, the first
    argmin, or the mean over the max(1, round(alpha n)) smallest (stable
    sort; round half to even as Julia's round)."""
    fv = np.asarray(fv, float)
    n = len(fv)
    if aggregator == "mean":
        return float(np.mean(fv)), sum(gv) / n
    if aggregator == "worst_case":
        w = int(np.argmin(fv))
        return float(fv[w]), gv[w]
    if aggregator == "cvar":
        n_tail = max(1, int(round(alpha * n)))
        order = np.argsort(fv, kind="stable")[:n_tail]
        return float(np.mean(fv[order])), sum(gv[i] for i in order) / n_tail
    raise ValueError(aggregator)


def penalty_value_and_gradient(w, type, weight=1.0, l_bound=-1.0, u_bound=1.0, dt=None):
    """(weight P, weight dP/dw) of Penalties.jl:273-330 for w [n_ctrl, n_t]."""
    w = np.asarray(w, float)
    n_c, n_t = w.shape
    G = np.zeros_like(w)
    F = 0.0
    if type == "NS":
        F = float(np.sum(w ** 2))
        G = 2 * w
    elif type == "SNS":
        e = np.where(w > u_bound, w - u_bound, np.where(w < l_bound, w - l_bound, 0.0))
        F = float(np.sum(e ** 2))
        G = 2 * e
    elif type == "SNSA":
        for n in range(n_t):
            A = np.sqrt(np.sum(w[:, n] ** 2))
            sp = max(0.0, A - u_bound)
            F += sp ** 2
            if sp > 0.0 and A > 1e-14:
                G[:, n] += 2.0 * sp / A * w[:, n]
    elif type == "DNS":
        for k in range(n_c):
            for n in range(n_t - 1):
                d = w[k, n + 1] - w[k, n]
                F += d ** 2
                G[k, n] -= 2 * d
                G[k, n + 1] += 2 * d
    elif type == "energy":
        t = np.ones(n_t) if dt is None else np.broadcast_to(np.asarray(dt, float), (n_t,))
        F = float(np.sum(w ** 2 * t[None, :]))
        G = 2 * w * t[None, :]
    else:
        raise ValueError(type)
    return weight * F, weight * G


def gradient_cuda_formula(H_drift, H_ctrl, controls, target, dt) -> np.ndarray:
    """The reference's CUDA-backend gradient as written (its CPU form,
    src/Backend/Hardware/CUDABackend.jl:283-305): P[0] = I, P[k+1] = U_k P[k];
    Q[n] = T', Q[k] = Q[k+1] U_k; Phi = Tr(T' P[n]) / d;
    G[j, k] = (2 / d^2) Re(conj(Phi) Tr(Q[k+1]' (-i dt H_j) P[k])).
    Q[k+1]' (not Q[k+1]) and the extra 1/d are kept as the reference has them."""
    H_drift = np.asarray(H_drift, C128)
    d = H_drift.shape[0]
    u = np.asarray(controls, float)
    n_c, n = u.shape
    T = np.asarray(target, C128)
    Hk = [H_drift + sum(u[j, k] * np.asarray(H_ctrl[j], C128) for j in range(n_c)) for k in range(n)]
    Uk = [expm_neg_i(H, dt) for H in Hk]
    P = [np.eye(d, dtype=C128)]
    for k in range(n):
        P.append(Uk[k] @ P[k])
    Q = [None] * (n + 1)
    Q[n] = T.conj().T
    for k in range(n - 1, -1, -1):
        Q[k] = Q[k + 1] @ Uk[k]
    Phi = np.trace(T.conj().T @ P[n]) / d
    G = np.zeros((n_c, n))
    for k in range(n):
        for j in range(n_c):
            M = Q[k + 1].conj().T @ (-1j * dt * np.asarray(H_ctrl[j], C128)) @ P[k]
            G[j, k] = (2.0 / d ** 2) * np.real(np.conj(Phi) * np.trace(M))
    return G


def finite_difference_gradient(system, controls, target, eps=1e-6) -> np.ndarray:
    """Central differences (Gradients.jl:442-479)."""
    u = np.array(controls.controls, float)
    G = np.zeros_like(u)
    for j in range(u.shape[0]):
        for k in range(u.shape[1]):
            up, um = u.copy(), u.copy()
            up[j, k] += eps
            um[j, k] -= eps
            Fp = compute_fidelity(system, ControlSequence.from_controls(up, controls.dt), target)
            Fm = compute_fidelity(system, ControlSequence.from_controls(um, controls.dt), target)
            G[j, k] = (Fp - Fm) / (2 * eps)
    return G


# ----------------------------------------------------------------------------
# Optimization layer (src/Optimization/GRAPE.jl)
# ----------------------------------------------------------------------------

@dataclass
class GRAPEConfig:
    """Defaults from GRAPE.jl:94-127."""
    max_iter: int = 1000
    convergence_tol: float = 1e-8
    step_size: float = 0.01
    adapt_step_size: bool = True
    min_step_size: float = 1e-10
    max_step_size: float = 10.0
    gradient_norm_tol: float = 1e-6
    verbose: bool = False
    print_interval: int = 100
    callback: Optional[Callable] = None


@dataclass
class OptimizationResult:
    """GRAPE.jl:158-170."""
    controls: np.ndarray
    fidelity: float
    fidelity_history: list
    gradient_norm_history: list
    n_iterations: int
    converged: bool
    termination_reason: str
    total_time: float
    n_fidelity_evaluations: int
    n_gradient_evaluations: int
    metadata: dict = field(default_factory=dict)


def adapt_grape_step_size(history, step, min_step=1e-10, max_step=10.0,
                          growth=1.05, shrink=0.5) -> float:
    """GRAPE.jl:309-334."""
    if len(history) < 2:
        return step
    delta = history[-1] - history[-2]
    if delta > 0.0:
        new = step * growth
    elif delta < -1e-14:
        new = step * shrink
    else:
        new = step
    return min(max(new, min_step), max_step)


def check_grape_convergence(history, gnorm, config: GRAPEConfig):
    """GRAPE.jl:371-402."""
    n = len(history)
    if n == 0:
        return False, ""
    if history[-1] >= 1.0 - 1e-12:
        return True, "perfect fidelity (F >= 1 - 1e-12)"
    if gnorm < config.gradient_norm_tol:
        return True, "gradient norm below tolerance"
    if n >= 3 and abs(history[-1] - history[-2]) < config.convergence_tol:
        return True, "fidelity change below tolerance"
    return False, ""


def grape_optimize(system: QuantumSystem, target: QuantumTarget,
                   controls_init: ControlSequence, config: GRAPEConfig = GRAPEConfig(),
                   eval_fn=None) -> OptimizationResult:
    """Plain GRAPE ascent loop (GRAPE.jl:469-643).  ``eval_fn(u) -> (F, G)``
    may replace the in-loop physics (fidelity + compute_grape_gradient_with!)."""
    t0 = time.time()
    dt = controls_init.dt
    u = np.array(controls_init.controls, float)
    best = u.copy()
    fh, gh = [], []
    nf = ng = 0
    step = config.step_size
    converged, reason, n_iter = False, "maximum iterations reached", 0

    def _phys(uu):
        cs = ControlSequence.from_controls(uu, dt)
        H = build_total_hamiltonian(system, cs)
        U = compute_propagators(H, dt)
        P, Q = forward_propagators(U), backward_propagators(U)
        F = compute_fidelity_U(P[-1], target)
        G = compute_grape_gradient_with(system, target, P, Q, P[-1], dt)
        return F, G

    def _fid(uu):
        return compute_fidelity(system, ControlSequence.from_controls(uu, dt), target)

    phys = eval_fn if eval_fn is not None else _phys
    F = _fid(u)
    nf += 1
    fh.append(F)
    best_F = F
    for it in range(1, config.max_iter + 1):
        n_iter = it
        F, G = phys(u)
        nf += 1
        ng += 1
        gnorm = float(np.linalg.norm(G))
        fh.append(F)
        gh.append(gnorm)
        if F > best_F:
            best_F = F
            best = u.copy()
        if config.adapt_step_size and len(fh) >= 2:
            step = adapt_grape_step_size(fh, step, config.min_step_size, config.max_step_size)
        u = u + step * G
        if config.callback is not None:
            config.callback(it, F, gnorm, u)
        conv, why = check_grape_convergence(fh, gnorm, config)
        if conv:
            converged, reason = True, why
            Fp = _fid(u)
            fh.append(Fp)
            nf += 1
            if Fp > best_F:
                best_F = Fp
                best = u.copy()
            break
    F_final = _fid(best)
    nf += 1
    return OptimizationResult(best, F_final, fh, gh, n_iter, converged, reason,
                              time.time() - t0, nf, ng,
                              {"step_size_final": step, "algorithm": "GRAPE"})


def lbfgs_direction_ensemble(g, s_list, y_list) -> np.ndarray:
    """Two-loop recursion of grape_optimize_ensemble (GRAPE.jl:1064-1084):
    rho = 1/max(y.s, 1e-14), gamma = s.y / max(y.y, 1e-14)."""
    k = len(s_list)
    if k == 0:
        return g.copy()
    q = g.copy()
    al = np.zeros(k)
    for i in range(k - 1, -1, -1):
        rho = 1.0 / max(float(y_list[i] @ s_list[i]), 1e-14)
        al[i] = rho * float(s_list[i] @ q)
        q -= al[i] * y_list[i]
    gam = float(s_list[-1] @ y_list[-1]) / max(float(y_list[-1] @ y_list[-1]), 1e-14)
    q *= gam
    for i in range(k):
        rho = 1.0 / max(float(y_list[i] @ s_list[i]), 1e-14)
        b = rho * float(y_list[i] @ q)
        q += (al[i] - b) * s_list[i]
    return q


def grape_optimize_ensemble(ens_F, ens_G, controls_init: ControlSequence,
                            config: GRAPEConfig = GRAPEConfig(), lbfgs_memory: int = 10,
                            amplitude_limit: float = math.inf) -> OptimizationResult:
    """Ensemble L-BFGS-GRAPE (GRAPE.jl:1012-1230).  ``ens_F(u)`` and
    ``ens_G(u)`` are the ensemble-mean fidelity / gradient on [n_c, n_t]."""
    t0 = time.time()
    u = np.array(controls_init.controls, float)
    fh, gh = [], []
    nf = ng = 0
    s_list, y_list = [], []

    def _ls(uu, d_mat, F0, a0, max_bt=20):
        a, nls = a0, 0
        for _ in range(max_bt):
            un = uu + a * d_mat
            if math.isfinite(amplitude_limit):
                un = np.clip(un, -amplitude_limit, amplitude_limit)
            Fn = ens_F(un)
            nls += 1
            if Fn >= F0:
                return a, un, Fn, nls
            a *= 0.5
        uf = uu + a * d_mat
        if math.isfinite(amplitude_limit):
            uf = np.clip(uf, -amplitude_limit, amplitude_limit)
        return a, uf, ens_F(uf), max_bt + 1

    F = ens_F(u)
    nf += 1
    fh.append(F)
    best_F, best = F, u.copy()
    converged, reason = False, "maximum iterations reached"
    for it in range(1, config.max_iter + 1):
        G = ens_G(u)
        ng += 1
        g = G.reshape(-1, order="F")
        gnorm = float(np.linalg.norm(g))
        gh.append(gnorm)
        d = lbfgs_direction_ensemble(g, s_list, y_list)
        dmax = float(np.max(np.abs(d)))
        if dmax < 1e-14:
            converged, reason = True, "zero gradient direction"
            break
        d = d / dmax
        d_mat = d.reshape(u.shape, order="F")
        a0 = config.step_size * amplitude_limit if math.isfinite(amplitude_limit) else config.step_size
        a, un, Fn, nls = _ls(u, d_mat, F, a0)
        nf += nls
        Gn = ens_G(un)
        ng += 1
        s = a * d
        y = Gn.reshape(-1, order="F") - g
        if float(y @ s) > 1e-14 * float(np.linalg.norm(s)) ** 2:
            s_list.append(s)
            y_list.append(y)
            if len(s_list) > lbfgs_memory:
                s_list.pop(0)
                y_list.pop(0)
        u, F = un, Fn
        fh.append(F)
        if F > best_F:
            best_F, best = F, u.copy()
        if config.callback is not None:
            config.callback(it, F, gnorm, u)
        if gnorm < config.gradient_norm_tol:
            converged, reason = True, "gradient norm below tolerance"
            break
        if F >= 1.0 - 1e-8:
            converged, reason = True, "near-perfect fidelity"
            break
        if len(fh) >= 2 and abs(fh[-1] - fh[-2]) < config.convergence_tol:
            converged, reason = True, "fidelity change below tolerance"
            break
    return OptimizationResult(best, best_F, fh, gh, len(fh), converged, reason,
                              time.time() - t0, nf, ng,
                              {"algorithm": "Ensemble L-BFGS-GRAPE", "lbfgs_memory": lbfgs_memory})


def build_ensemble_from_systems(systems, target, controls: ControlSequence):
    """Mean aggregator closures (src/Optimization/Ensemble/SystemBuilder.jl:49-87,
    EnsembleObjective.jl:169-217,272-307): per-system compute_fidelity and
    compute_grape_gradient, averaged in system order."""
    dt = controls.dt

    def F(u):
        cs = ControlSequence.from_controls(u, dt)
        return float(sum(compute_fidelity(s, cs, target) for s in systems) / len(systems))

    def G(u):
        cs = ControlSequence.from_controls(u, dt)
        acc = np.zeros_like(np.asarray(u, float))
        for s in systems:
            acc += compute_grape_gradient(s, cs, target)
        return acc / len(systems)

    return F, G


# ----------------------------------------------------------------------------
# Lindblad builders (src/Physics/Lindblad.jl)
# ----------------------------------------------------------------------------

def vec_rho(rho: np.ndarray) -> np.ndarray:
    """Column stacking: vec(rho)[i + N j] = rho[i, j]  (Lindblad.jl:57-58)."""
    return np.asarray(rho, C128).reshape(-1, order="F")


def mat_rho(v: np.ndarray, N: int) -> np.ndarray:
    return np.asarray(v, C128).reshape((N, N), order="F")


def pure_state_to_vec_rho(psi) -> np.ndarray:
    """Lindblad.jl:89-92."""
    c = np.asarray(psi, C128)
    return vec_rho(np.outer(c, c.conj()))


def build_drift_liouvillian(H, jump_ops, rates) -> np.ndarray:
    """-i(I (x) H - H^T (x) I) + sum_k g_k [conj(L)(x)L - 1/2 I(x)L'L - 1/2 conj(L'L)(x)I]
    (Lindblad.jl:126-160).  Zero or non-finite rates are skipped; negative rates raise."""
    H = np.asarray(H, C128)
    N = H.shape[0]
    IN = np.eye(N, dtype=C128)
    L = -1j * np.kron(IN, H) + 1j * np.kron(H.T, IN)
    for Lk, g in zip(jump_ops, rates):
        if g == 0.0 or not math.isfinite(g):
            continue
        if g < 0.0:
            raise ValueError("Lindblad decay rate must be non-negative")
        Lk = np.asarray(Lk, C128)
        A = Lk.conj().T @ Lk
        L = L + g * (np.kron(Lk.conj(), Lk) - 0.5 * np.kron(IN, A) - 0.5 * np.kron(A.conj(), IN))
    return L


def build_control_liouvillian(Hc) -> np.ndarray:
    """-i(I (x) Hc - Hc^T (x) I)  (Lindblad.jl:189-197)."""
    Hc = np.asarray(Hc, C128)
    IN = np.eye(Hc.shape[0], dtype=C128)
    return -1j * np.kron(IN, Hc) + 1j * np.kron(Hc.T, IN)


# ----------------------------------------------------------------------------
# MR kernels (src/Application/MR/GRAPEState.jl, GRAPELindblad.jl)
# ----------------------------------------------------------------------------

@dataclass
class MRControl:
    """Fields used by the kernels (src/Application/MR/OptControl.jl:137-259)."""
    drifts: list
    operators: list
    rho_init: list
    rho_targ: list
    pwr_levels: list
    pulse_dt: np.ndarray
    fidelity: str = "real"
    l_bound: float = -1.0
    u_bound: float = 1.0
    max_iter: int = 500
    grad_tol: float = 1e-7
    lbfgs_memory: int = 10


def grape_state_kernel(waveform: np.ndarray, ctrl: MRControl):
    """_grape_cpu (GRAPEState.jl:136-250): ensemble over (drift, pwr) pairs x
    state pairs; H = H_drift + pwr sum_k w[k,n] Op_k; forward/backward
    matvec chains; grad[k,n] += prefactor(z, <lambda[n+1]|Op_k|psi[n]>, dt_n pwr).
    Penalties are not applied (no penalty terms configured)."""
    n_ctrl, n_t = waveform.shape
    pairs = [(H, p) for H in ctrl.drifts for p in ctrl.pwr_levels]
    N_ens = len(pairs) * len(ctrl.rho_init)
    fid = 0.0
    grad = np.zeros((n_ctrl, n_t))
    ops = [np.asarray(o, C128) for o in ctrl.operators]
    for H_d, pwr in pairs:
        Ps = []
        for n in range(n_t):
            H = np.asarray(H_d, C128) + sum(pwr * waveform[k, n] * ops[k] for k in range(n_ctrl))
            Ps.append(expm_neg_i(H, float(ctrl.pulse_dt[n])))
        for psi0, psit in zip(ctrl.rho_init, ctrl.rho_targ):
            psi0 = np.asarray(psi0, C128)
            psit = np.asarray(psit, C128)
            fwd = [psi0]
            for n in range(n_t):
                fwd.append(Ps[n] @ fwd[-1])
            z = np.vdot(psit, fwd[-1])
            fid += state_fidelity(psit, fwd[-1], ctrl.fidelity)
            lam = [None] * (n_t + 1)
            lam[n_t] = psit
            for n in range(n_t - 1, -1, -1):
                lam[n] = Ps[n].conj().T @ lam[n + 1]
            for n in range(n_t):
                for k in range(n_ctrl):
                    inner = np.vdot(lam[n + 1], ops[k] @ fwd[n])
                    grad[k, n] += fidelity_grad_prefactor(z, inner, ctrl.pulse_dt[n] * pwr,
                                                          ctrl.fidelity)
    return fid / N_ens, grad / N_ens


def sample_drift_trajectories(dH_finals, n_timesteps: int) -> list:
    """sample_drift_trajectories (RobustOpt.jl:168-182): trajectory s is the
    linear ramp (k-1)/max(1, n_t-1) dH_final_s, k = 1..n_t, with dH_final_s
    drawn as sample_parametric_perturbations draws them (given here)."""
    out = []
    for dH in dH_finals:
        out.append([((k - 1) / max(1, n_timesteps - 1)) * np.asarray(dH, C128) for k in range(1, n_timesteps + 1)])
    return out


def fidelity_with_perturbation(H0, H_ctrls, controls: np.ndarray, dt: float, U_tgt, perturbation) -> float:
    """_fidelity_with_perturbation (RobustOpt.jl:739-761): H_k = H0 + dH_k +
    sum_j u_jk H_j (dH_k = perturbation[k] for a trajectory, the matrix
    itself otherwise), U = prod exp(-i dt H_k), F = clamp(|Tr(U_t' U)|^2 /
    d^2, 0, 1)."""
    H0 = np.asarray(H0, C128)
    d = H0.shape[0]
    U = np.eye(d, dtype=C128)
    for k in range(controls.shape[1]):
        dHk = perturbation[k] if isinstance(perturbation, list) else perturbation
        H = H0 + dHk + sum(controls[j, k] * np.asarray(H_ctrls[j], C128) for j in range(len(H_ctrls)))
        U = expm_neg_i(H, dt) @ U
    F = abs(np.trace(np.asarray(U_tgt, C128).conj().T @ U)) ** 2 / d ** 2
    return float(min(max(F, 0.0), 1.0))


@dataclass
class TrackingPoint:
    """GRAPETracking.jl:82-91: the density matrix after propagating through
    ``step`` (1-based, 1..n_t) is compared with ``target_dm``, weight w."""
    step: int
    target_dm: np.ndarray
    weight: float


def grape_tracking_kernel(waveform: np.ndarray, ctrl: MRControl, tracking):
    """_grape_tracking_cpu_threaded (GRAPETracking.jl:166-277), density-matrix
    form as the reference computes it: rho[1] = psi0 psi0', rho[n+1] = U_n
    rho[n] U_n'; Phi += w Re Tr(rho_tar rho[step+1]); co-state Lambda = 0,
    at a checkpoint step Lambda += 2 w (rho_tar - rho[n+1]), grad[k,n] +=
    -dt_n Re(i Tr(Lambda' [pwr Op_k, rho[n+1]])), Lambda <- U_n' Lambda U_n;
    ensemble and pairs averaged.  Penalties are not applied here."""
    n_ctrl, n_t = waveform.shape
    pairs = [(H, p) for H in ctrl.drifts for p in ctrl.pwr_levels]
    N_ens = len(pairs) * len(ctrl.rho_init)
    ckpt = {}
    for tp in tracking:
        if tp.step < 1 or tp.step > n_t:
            raise ValueError(f"TrackingPoint.step={tp.step} out of range [1, {n_t}]")
        ckpt.setdefault(tp.step, []).append((float(tp.weight), np.asarray(tp.target_dm, C128)))
    steps = sorted(ckpt)
    ops = [np.asarray(o, C128) for o in ctrl.operators]
    fid = 0.0
    grad = np.zeros((n_ctrl, n_t))
    for H_d, pwr in pairs:
        Ps = []
        for n in range(n_t):
            H = np.asarray(H_d, C128) + sum(pwr * waveform[k, n] * ops[k] for k in range(n_ctrl))
            Ps.append(expm_neg_i(H, float(ctrl.pulse_dt[n])))
        for psi0 in ctrl.rho_init:
            psi0 = np.asarray(psi0, C128)
            rho = [np.outer(psi0, psi0.conj())]          # rho[0] here = rho_traj[1]
            for n in range(n_t):
                rho.append(Ps[n] @ rho[-1] @ Ps[n].conj().T)
            for n_ck in steps:
                for w_k, rt in ckpt[n_ck]:
                    fid += w_k * float(np.real(np.trace(rt @ rho[n_ck])))
            Lam = np.zeros_like(rho[0])
            for n in range(n_t, 0, -1):                 # 1-based step n, slice n-1
                for w_k, rt in ckpt.get(n, ()):
                    Lam = Lam + 2.0 * w_k * (rt - rho[n])
                r1 = rho[n]
                dt_n = float(ctrl.pulse_dt[n - 1])
                for k in range(n_ctrl):
                    Hk = pwr * ops[k]
                    comm = Hk @ r1 - r1 @ Hk
                    grad[k, n - 1] += -dt_n * float(np.real(1j * np.trace(Lam.conj().T @ comm)))
                Lam = Ps[n - 1].conj().T @ Lam @ Ps[n - 1]
    return fid / N_ens, grad / N_ens


def grape_phase_kernel(phi: np.ndarray, ctrl: MRControl, amplitudes=None):
    """grape_phase_kernel (GRAPEPhase.jl:52-93): w[2ch-1] = a cos(phi),
    w[2ch] = a sin(phi); dF/dphi = -G_x sin(phi) + G_y cos(phi)."""
    phi = np.asarray(phi, float)
    n_ch, n_t = phi.shape
    a = np.ones_like(phi) if amplitudes is None else np.asarray(amplitudes, float)
    if len(ctrl.operators) != 2 * n_ch:
        raise ValueError("length(operators) must be 2 x n_channels")
    if a.shape != phi.shape:
        raise ValueError("amplitudes must match phi_profile")
    if np.any(a < 0):
        raise ValueError("all amplitudes must be >= 0")
    w = np.zeros((2 * n_ch, n_t))
    w[0::2] = a * np.cos(phi)
    w[1::2] = a * np.sin(phi)
    F, G = grape_state_kernel(w, ctrl)
    return F, -G[0::2] * np.sin(phi) + G[1::2] * np.cos(phi)


def expm_general(A: np.ndarray) -> np.ndarray:
    """Julia LinearAlgebra.exp (Higham 2005 scaling-and-squaring Pade-13) is
    restated by scipy.linalg.expm (Al-Mohy-Higham 2009, same family)."""
    return sla.expm(A)


def grape_lindblad_kernel(waveform: np.ndarray, L_drifts, L_controls, sigma_init, sigma_targ,
                          pwr_levels, pulse_dt, fidelity: str = "square"):
    """_grape_lindblad_cpu (GRAPELindblad.jl:96-215): Phi_n = exp((L_d + pwr
    sum_k w[k,n] L_k) dt_n); z = <sigma_targ|sigma(T)>; Re prefactor."""
    n_ctrl, n_t = waveform.shape
    pairs = [(L, p) for L in L_drifts for p in pwr_levels]
    N_ens = len(pairs) * len(sigma_init)
    fid = 0.0
    grad = np.zeros((n_ctrl, n_t))
    for L_d, pwr in pairs:
        Phi = []
        for n in range(n_t):
            L = np.asarray(L_d, C128) + sum(pwr * waveform[k, n] * L_controls[k] for k in range(n_ctrl))
            Phi.append(expm_general(L * pulse_dt[n]))
        for s0, st in zip(sigma_init, sigma_targ):
            fwd = [np.asarray(s0, C128)]
            for n in range(n_t):
                fwd.append(Phi[n] @ fwd[-1])
            z = np.vdot(st, fwd[-1])
            fid += float((np.conj(z) * z).real) if fidelity == "square" else float(z.real)
            lam = [None] * (n_t + 1)
            lam[n_t] = np.asarray(st, C128)
            for n in range(n_t - 1, -1, -1):
                lam[n] = Phi[n].conj().T @ lam[n + 1]
            for n in range(n_t):
                for k in range(n_ctrl):
                    inner = np.vdot(lam[n + 1], L_controls[k] @ fwd[n])
                    grad[k, n] += lindblad_grad_prefactor(z, inner, pulse_dt[n] * pwr, fidelity)
    return fid / N_ens, grad / N_ens


def lbfgs_direction_mr(g, s_list, y_list) -> np.ndarray:
    """_lbfgs_direction (OptControl.jl:565-590): no 1e-14 guards."""
    k = len(s_list)
    if k == 0:
        return g.copy()
    q = g.copy()
    al = np.zeros(k)
    rho = [1.0 / float(y_list[i] @ s_list[i]) for i in range(k)]
    for i in range(k - 1, -1, -1):
        al[i] = rho[i] * float(s_list[i] @ q)
        q -= al[i] * y_list[i]
    gam = float(s_list[-1] @ y_list[-1]) / float(y_list[-1] @ y_list[-1])
    r = gam * q
    for i in range(k):
        b = rho[i] * float(y_list[i] @ r)
        r += (al[i] - b) * s_list[i]
    return r


def optimcon_lbfgs(kernel, guess: np.ndarray, l_bound=-1.0, u_bound=1.0, max_iter=500,
                   grad_tol=1e-7, lbfgs_memory=10) -> OptimizationResult:
    """_optimcon_lbfgs (OptControl.jl:380-482) with _line_search (:594-611):
    clamp to bounds, max-abs normalised direction, alpha0 = 0.05 (u-l),
    Armijo-like acceptance F_new >= F0 - 1e-4 |alpha|, stall |dF| < 1e-9."""
    t0 = time.time()
    w = np.clip(np.array(guess, float), l_bound, u_bound)
    F, G = kernel(w)
    best_w, best_F = w.copy(), F
    nf = ng = 1
    fh, gh = [F], [float(np.linalg.norm(G))]
    s_list, y_list = [], []
    converged, reason = False, "max iterations reached"

    def _ls(ww, d, F0, a0):
        a = a0
        for h in range(1, 21):
            wn = np.clip(ww + a * d, l_bound, u_bound)
            Fn, _ = kernel(wn)
            if Fn >= F0 - 1e-4 * abs(a):
                return a, wn, Fn, h + 1
            a *= 0.5
        wn = np.clip(ww + a * d, l_bound, u_bound)
        Fn, _ = kernel(wn)
        return a, (wn if Fn > F0 else ww.copy()), max(Fn, F0), 21

    for it in range(1, max_iter + 1):
        g = G.reshape(-1, order="F")
        d = lbfgs_direction_mr(g, s_list, y_list)
        dmax = float(np.max(np.abs(d)))
        if dmax < 1e-14:
            converged, reason = True, "zero gradient direction"
            break
        d = d / dmax
        d_mat = d.reshape(w.shape, order="F")
        a, wn, Fn, nls = _ls(w, d_mat, F, 0.05 * (u_bound - l_bound))
        nf += nls
        F2, Gn = kernel(wn)
        nf += 1
        ng += 1
        s = (wn - w).reshape(-1, order="F")
        y = Gn.reshape(-1, order="F") - g
        if float(y @ s) > 1e-14 * float(np.linalg.norm(s)) ** 2:
            s_list.append(s)
            y_list.append(y)
            if len(s_list) > lbfgs_memory:
                s_list.pop(0)
                y_list.pop(0)
        w, G = wn, Gn
        F_prev, F = F, F2
        fh.append(F)
        gn = float(np.linalg.norm(G))
        gh.append(gn)
        if F > best_F:
            best_F, best_w = F, w.copy()
        if F >= 1.0 - 1e-8:
            converged, reason = True, "near-perfect fidelity"
            break
        if gn < grad_tol:
            converged, reason = True, "gradient norm below tolerance"
            break
        if len(fh) >= 2 and abs(F - F_prev) < 1e-9:
            converged, reason = True, "fidelity stalled"
            break
    return OptimizationResult(best_w, best_F, fh, gh, len(fh) - 1, converged, reason,
                              time.time() - t0, nf, ng, {"algorithm": "L-BFGS"})


def optimcon_grape(kernel, guess: np.ndarray, l_bound=-1.0, u_bound=1.0, max_iter=500,
                   grad_tol=1e-7) -> OptimizationResult:
    """_optimcon_grape (OptControl.jl:486-561): step 0.05 (u-l) / max|G| along
    G, clamp, stop at F >= 1 - 1e-8 or ||G|| below grad_tol."""
    t0 = time.time()
    w = np.clip(np.array(guess, float), l_bound, u_bound)
    F, G = kernel(w)
    best_w, best_F = w.copy(), F
    nf = ng = 1
    fh, gh = [F], [float(np.linalg.norm(G))]
    converged, reason = False, "max iterations reached"
    for it in range(1, max_iter + 1):
        g_max = float(np.max(np.abs(G)))
        if g_max > 1e-14:
            w = np.clip(w + (0.05 * (u_bound - l_bound) / g_max) * G, l_bound, u_bound)
        F, G = kernel(w)
        nf += 1
        ng += 1
        fh.append(F)
        gn = float(np.linalg.norm(G))
        gh.append(gn)
        if F > best_F:
            best_F, best_w = F, w.copy()
        if F >= 1.0 - 1e-8:
            converged, reason = True, "near-perfect fidelity"
            break
        if gn < grad_tol:
            converged, reason = True, "gradient norm below tolerance"
            break
    return OptimizationResult(best_w, best_F, fh, gh, len(fh) - 1, converged, reason,
                              time.time() - t0, nf, ng, {"algorithm": "GRAPE"})
