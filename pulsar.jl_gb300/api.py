"""Pulsar.jl's GRAPE API surface, served by libpulsar_gb300.so.

Names, argument meanings, defaults and error behaviour follow the reference
(paths inside the Pulsar.jl project):

  QuantumSystem / quantum_system      src/Types/QuantumSystem.jl:60-66,318-341
  ControlSequence / random_controls   src/Types/ControlSequence.jl:37-158
  QuantumTarget / state_target /
  unitary_target                      src/Types/Targets.jl:37-144
  compute_propagator                  src/Computation/Propagators.jl:64-90
  compute_fidelity                    src/Physics/Objectives.jl:609-639
  compute_grape_gradient              src/Physics/Gradients.jl:80-127
  GRAPEConfig / OptimizationResult    src/Optimization/GRAPE.jl:60-211
  grape_optimize                      src/Optimization/GRAPE.jl:469-643
  grape_optimize_ensemble             src/Optimization/GRAPE.jl:1012-1230
  build_ensemble_from_systems         src/Optimization/Ensemble/SystemBuilder.jl:49-87
  MRControl / LindbladMRControl       src/Application/MR/OptControl.jl:137-259,733-885
  grape_state_kernel                  src/Application/MR/GRAPEState.jl:73-250
  grape_lindblad_kernel               src/Application/MR/GRAPELindblad.jl:83-215
  fidelity_forward                    src/Application/MR/GRAPEState.jl:434-566
  optimcon                            src/Application/MR/OptControl.jl:310-370,913-948
  build_drift_liouvillian, build_control_liouvillian, vec_rho, mat_rho,
  pure_state_to_vec_rho               src/Physics/Lindblad.jl:57-197

Every physics evaluation runs on the GPU through the C ABI.  Argument errors
raise ValueError (the reference's ArgumentError / DimensionMismatch).  There
is no CPU fallback: without the library every call raises.

Gradient modes: the reference's own first-order formulas are the defaults of
the reference entry points (``grad_mode="ref_grape"`` for the GRAPE path,
``"ref_mr"`` for the MR kernels); ``grad_mode="exact"`` gives the exact
Frechet-derivative gradient of the same objective.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

from . import _abi as _A
from .engine import Context, Problem, default_context

C128 = np.complex128


# ---------------------------------------------------------------------------
# Types
# ---------------------------------------------------------------------------

def _check_hermitian(H: np.ndarray, name: str, tol: float = 1e-10):
    dev = float(np.max(np.abs(H - H.conj().T))) if H.size else 0.0
    if dev > tol:
        raise ValueError(f"{name} is not Hermitian: max|H - H'| = {dev} > tol = {tol}")


@dataclass
class QuantumSystem:
    H_drift: np.ndarray
    H_controls: list
    metadata: dict = field(default_factory=dict)

    @property
    def dim(self) -> int:
        return int(self.H_drift.shape[0])

    @property
    def n_controls(self) -> int:
        return len(self.H_controls)


def quantum_system(H_drift, H_controls, metadata=None) -> QuantumSystem:
    """Validates Hermiticity (1e-10) and shapes (QuantumSystem.jl:318-341)."""
    Hd = np.asarray(H_drift, C128)
    if Hd.ndim != 2 or Hd.shape[0] != Hd.shape[1]:
        raise ValueError("H_drift must be square")
    _check_hermitian(Hd, "H_drift")
    Hcs = []
    for j, Hc in enumerate(H_controls):
        Hc = np.asarray(Hc, C128)
        if Hc.shape != Hd.shape:
            raise ValueError(f"H_controls[{j}] has size {Hc.shape} but expected {Hd.shape}")
        _check_hermitian(Hc, f"H_controls[{j}]")
        Hcs.append(Hc)
    return QuantumSystem(Hd, Hcs, dict(metadata or {}))


class ControlSequence:
    """amplitudes: [n_steps, n_controls]; .controls is the [n_c, n_t] view."""

    def __init__(self, amplitudes, dt: float, n_steps: Optional[int] = None):
        a = np.asarray(amplitudes, np.float64)
        if dt < 0:
            raise ValueError(f"dt must be non-negative, got {dt}")
        if n_steps is not None and a.shape[0] != n_steps:
            raise ValueError(f"amplitudes has {a.shape[0]} rows but n_steps = {n_steps}")
        self.amplitudes = a
        self.dt = float(dt)

    @classmethod
    def from_controls(cls, controls, dt: float, total_time: Optional[float] = None,
                      n_timesteps: Optional[int] = None) -> "ControlSequence":
        """The 4-argument constructor of ControlSequence.jl:77-89."""
        c = np.asarray(controls, np.float64)
        if n_timesteps is not None and c.shape[1] != n_timesteps:
            raise ValueError(f"controls has {c.shape[1]} columns but n_timesteps = {n_timesteps}")
        return cls(np.ascontiguousarray(c.T), dt)

    @property
    def controls(self) -> np.ndarray:
        return self.amplitudes.T

    @property
    def n_steps(self) -> int:
        return self.amplitudes.shape[0]

    n_timesteps = n_steps

    @property
    def total_time(self) -> float:
        return self.dt * self.n_steps


def random_controls(system: QuantumSystem, total_time: float, n_timesteps: int, amplitude=1.0,
                    rng: Optional[np.random.Generator] = None) -> ControlSequence:
    """U(-amplitude, amplitude) amplitudes (ControlSequence.jl:142-158); the
    stream is numpy's, not Julia's MersenneTwister."""
    if total_time <= 0:
        raise ValueError(f"total_time must be positive, got {total_time}")
    if n_timesteps <= 0:
        raise ValueError(f"n_timesteps must be positive, got {n_timesteps}")
    rng = rng or np.random.default_rng()
    a = amplitude * (2 * rng.random((n_timesteps, system.n_controls)) - 1)
    return ControlSequence(a, total_time / n_timesteps)


@dataclass
class QuantumTarget:
    type: str
    target_state: Optional[np.ndarray] = None
    target_unitary: Optional[np.ndarray] = None
    initial_state: Optional[np.ndarray] = None

    @property
    def dim(self) -> int:
        return int((self.target_unitary if self.type == "unitary" else self.target_state).shape[0])


def state_target(state, psi_init=None) -> QuantumTarget:
    """Targets.jl:77-107.  Without psi_init the objective is the fixed-point
    overlap |<t|U|t>|^2 (Objectives.jl:620-623)."""
    psi = np.asarray(state, C128).ravel()
    if psi.size == 0:
        raise ValueError("Target state vector must be non-empty")
    if not np.all(np.isfinite(psi)):
        raise ValueError("Target state contains NaN or Inf values")
    if np.linalg.norm(psi) < np.finfo(float).eps:
        raise ValueError("Target state has zero norm")
    pi = None
    if psi_init is not None:
        pi = np.asarray(psi_init, C128).ravel()
        if pi.size != psi.size:
            raise ValueError(f"psi_init has length {pi.size}; expected {psi.size}")
        if not np.all(np.isfinite(pi)):
            raise ValueError("psi_init contains NaN or Inf values")
        if np.linalg.norm(pi) < np.finfo(float).eps:
            raise ValueError("psi_init has zero norm")
    return QuantumTarget("state", target_state=psi, initial_state=pi)


def unitary_target(U) -> QuantumTarget:
    """Targets.jl:131-144: square and ||U'U - I|| / d <= 1e-8."""
    U = np.asarray(U, C128)
    if U.ndim != 2 or U.shape[0] != U.shape[1]:
        raise ValueError(f"Target unitary must be square, got {U.shape}")
    dev = np.linalg.norm(U.conj().T @ U - np.eye(U.shape[0])) / U.shape[0]
    if dev > 1e-8:
        raise ValueError(f"Target matrix is not unitary: ||U'U - I|| / dim = {dev} > 1e-8")
    return QuantumTarget("unitary", target_unitary=U)


@dataclass
class GRAPEConfig:
    """GRAPE.jl:60-127 (defaults and validation kept)."""
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
    use_threads: bool = True
    backend: str = "gpu"
    grad_mode: str = "ref_grape"
    precision: str = "fp64"

    def __post_init__(self):
        if self.max_iter <= 0:
            raise ValueError("max_iter must be positive")
        if self.convergence_tol <= 0:
            raise ValueError("convergence_tol must be positive")
        if self.step_size <= 0:
            raise ValueError("step_size must be positive")
        if self.min_step_size <= 0:
            raise ValueError("min_step_size must be positive")
        if self.max_step_size < self.step_size:
            raise ValueError("max_step_size must be >= step_size")
        if self.min_step_size > self.step_size:
            raise ValueError("min_step_size must be <= step_size")
        if self.gradient_norm_tol <= 0:
            raise ValueError("gradient_norm_tol must be positive")
        if self.print_interval <= 0:
            raise ValueError("print_interval must be positive")
        if self.backend not in ("auto", "cpu", "gpu", "hybrid"):
            raise ValueError("backend must be :auto, :cpu, :gpu, or :hybrid")


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


# ---------------------------------------------------------------------------
# Problem construction from reference objects
# ---------------------------------------------------------------------------

def _dt_vec(dt, n_t: int) -> np.ndarray:
    return np.broadcast_to(np.asarray(dt, np.float64), (n_t,)).copy()


def _normalise(v):
    v = np.asarray(v, C128)
    n = np.linalg.norm(v)
    if n < np.finfo(float).eps:
        raise ValueError("state has zero norm")
    return v / n


def _system_problem(system: QuantumSystem, target: QuantumTarget, n_t: int, dt, *,
                    grad_mode: str, precision: str = "fp64", legacy_state_gradient: bool = False,
                    normalise_states: bool = False, ctx: Optional[Context] = None) -> Problem:
    kw = dict(ctx=ctx, grad_mode=grad_mode, precision=precision)
    if target.type == "unitary":
        return Problem(system.H_drift, np.stack(system.H_controls), _dt_vec(dt, n_t),
                       target="gate", fidelity="square", target_op=target.target_unitary, **kw)
    if target.type != "state":
        raise ValueError(f'Unknown target type "{target.type}"; expected "unitary" or "state"')
    psi_t = target.target_state
    psi_i = psi_t if target.initial_state is None else target.initial_state
    grad_init = psi_t if legacy_state_gradient else psi_i
    if normalise_states:
        psi_t, psi_i, grad_init = _normalise(psi_t), _normalise(psi_i), _normalise(grad_init)
    return Problem(system.H_drift, np.stack(system.H_controls), _dt_vec(dt, n_t), target="states",
                   fidelity="square", states_init=psi_i, states_target=psi_t,
                   grad_states_init=grad_init, **kw)


# ---------------------------------------------------------------------------
# Computation / physics entry points
# ---------------------------------------------------------------------------

def compute_propagator(H, dt: float, ctx: Optional[Context] = None) -> np.ndarray:
    """exp(-i H dt) on the device; identity for dt = 0 (Propagators.jl:64-90)."""
    H = np.asarray(H, C128)
    if H.ndim != 2 or H.shape[0] != H.shape[1]:
        raise ValueError(f"H must be square, got {H.shape}")
    if dt == 0.0:
        return np.eye(H.shape[0], dtype=C128)
    _check_hermitian(H, "H")
    return (ctx or default_context()).propagator(H, dt, "hermitian")


def propagate(system: QuantumSystem, controls: ControlSequence) -> np.ndarray:
    """U_total (Propagators.jl:566-571)."""
    prob = Problem(system.H_drift, np.stack(system.H_controls),
                   _dt_vec(controls.dt, controls.n_steps), target="gate",
                   target_op=np.eye(system.dim), grad_mode="ref_grape")
    try:
        return prob.total_propagator(controls.controls, 0)
    finally:
        prob.close()


def compute_fidelity(system: QuantumSystem, controls: ControlSequence, target: QuantumTarget) -> float:
    """Objectives.jl:632-639: gate |Tr(U_t'U)/d|^2, state |<t|U i>|^2 with
    i = initial_state or target_state."""
    if controls.amplitudes.shape[1] != system.n_controls:
        raise ValueError("controls and system disagree on the number of control fields")
    prob = _system_problem(system, target, controls.n_steps, controls.dt, grad_mode="ref_grape")
    try:
        return prob.eval(controls.controls, want_grad=False)[0]
    finally:
        prob.close()


def compute_grape_gradient(system: QuantumSystem, controls: ControlSequence, target: QuantumTarget,
                           grad_mode: str = "ref_grape") -> np.ndarray:
    """G[n_c, n_t] (Gradients.jl:80-127): honours initial_state; state vectors
    are normalised as in Gradients.jl:377-381."""
    prob = _system_problem(system, target, controls.n_steps, controls.dt, grad_mode=grad_mode,
                           normalise_states=True)
    try:
        return prob.eval(controls.controls)[1]
    finally:
        prob.close()


# ---------------------------------------------------------------------------
# Propagator stacks, chains and metrics (Propagators.jl, Objectives.jl,
# Gradients.jl building blocks) -- each a device call
# ---------------------------------------------------------------------------

def _ctx_handle(ctx: Optional[Context]):
    return (ctx or default_context()).handle


def _cbuf(stack: np.ndarray) -> np.ndarray:
    """[n, d, d] complex -> n column-major interleaved matrices (doubles)."""
    return _A.cmat_buf(np.asarray(stack, C128))


def _cstack(buf: np.ndarray, n: int, d: int) -> np.ndarray:
    m = buf.reshape(n, d, d, 2)
    return (m[..., 0] + 1j * m[..., 1]).transpose(0, 2, 1).copy()


def build_total_hamiltonian(system: QuantumSystem, controls: ControlSequence,
                            ctx: Optional[Context] = None) -> np.ndarray:
    """H_total[k] = H_drift + sum_j amplitudes[k, j] H_j, [n_steps, d, d]
    (Propagators.jl:485-544)."""
    n_t, n_c = controls.amplitudes.shape
    if n_c != system.n_controls:
        raise ValueError(f"controls has {n_c} control channels but system has {system.n_controls} "
                         "control fields")
    d = system.dim
    Hd = _cbuf(system.H_drift[None])
    Hc = _cbuf(np.stack(system.H_controls)) if n_c else np.zeros(2)
    u = np.ascontiguousarray(np.asarray(controls.controls, float).T).ravel()
    out = np.zeros(2 * d * d * max(n_t, 1))
    _A.check(_A.lib().pgx_total_hamiltonian(_ctx_handle(ctx), d, n_c, n_t, _A.as_dptr(Hd), _A.as_dptr(Hc),
                                            _A.as_dptr(u if u.size else np.zeros(1)), _A.as_dptr(out)),
             _ctx_handle(ctx))
    return _cstack(out, n_t, d) if n_t else np.zeros((0, d, d), C128)


def compute_propagators(H_total, dt, ctx: Optional[Context] = None, generator: str = "hermitian") -> np.ndarray:
    """U[k] = exp(-i H[k] dt) for H_total [n_steps, d, d] (Propagators.jl:127-184);
    dt a scalar or one value per slice."""
    H = np.asarray(H_total, C128)
    if H.ndim != 3:
        raise ValueError(f"H_total must be a 3-D array [n_timesteps x dim x dim], got {H.ndim}-D")
    n, d1, d2 = H.shape
    if d1 != d2:
        raise ValueError(f"H_total last two dimensions must be equal (square matrices), got {d1} x {d2}")
    dts = np.atleast_1d(np.asarray(dt, float))
    if np.any(dts <= 0):
        raise ValueError(f"dt must be positive, got {dt}")
    if n == 0:
        return np.zeros((0, d1, d1), C128)
    out = np.zeros(2 * d1 * d1 * n)
    _A.check(_A.lib().pgx_propagator_stack(_ctx_handle(ctx), d1, _A.GEN[generator], n, _A.as_dptr(_cbuf(H)),
                                           _A.as_dptr(np.ascontiguousarray(dts)), dts.size, _A.as_dptr(out)),
             _ctx_handle(ctx))
    return _cstack(out, n, d1)


def _chains(props, seed=None, want=("P",), ctx: Optional[Context] = None):
    U = np.asarray(props, C128)
    if U.ndim != 3 or U.shape[1] != U.shape[2]:
        raise ValueError(f"propagators must be a 3-D array [n x dim x dim], got shape {U.shape}")
    n, d, _ = U.shape
    if seed is not None:
        seed = np.asarray(seed, C128)
        if seed.shape != (d, d):
            raise ValueError(f"seed must be {d} x {d}, got {seed.shape}")
    P = np.zeros(2 * d * d * (n + 1)) if "P" in want else None
    Q = np.zeros(2 * d * d * (n + 1)) if "Q" in want else None
    T = np.zeros(2 * d * d) if "T" in want else None
    ub = _cbuf(U) if n else np.zeros(2)
    _A.check(_A.lib().pgx_propagator_chains(
        _ctx_handle(ctx), d, n, _A.as_dptr(ub), _A.as_dptr(_cbuf(seed[None])) if seed is not None else None,
        _A.as_dptr(P) if P is not None else None, _A.as_dptr(Q) if Q is not None else None,
        _A.as_dptr(T) if T is not None else None), _ctx_handle(ctx))
    return (_cstack(P, n + 1, d) if P is not None else None, _cstack(Q, n + 1, d) if Q is not None else None,
            _cstack(T, 1, d)[0] if T is not None else None)


def compute_total_propagator(propagators, ctx: Optional[Context] = None) -> np.ndarray:
    """U_total = U[n-1] ... U[0]; identity for n = 0 (Propagators.jl:212-238)."""
    return _chains(propagators, want=("T",), ctx=ctx)[2]


def compute_forward_propagators(propagators, ctx: Optional[Context] = None) -> np.ndarray:
    """P[0] = I, P[k+1] = U[k] P[k]; [n+1, d, d] (Propagators.jl:291-325)."""
    return _chains(propagators, want=("P",), ctx=ctx)[0]


def compute_backward_propagators(propagators, seed=None, ctx: Optional[Context] = None) -> np.ndarray:
    """Q[n] = I (or seed), Q[k] = U[k]' Q[k+1]; [n+1, d, d].  As the reference's
    code (Propagators.jl:399-404) Q[k] includes the slice's own propagator."""
    return _chains(propagators, seed=seed, want=("Q",), ctx=ctx)[1]


def _overlap(a, b, ctx: Optional[Context] = None) -> complex:
    """sum conj(a) b over all entries, on the device (matrices: Tr(a'b))."""
    a = np.asarray(a, C128)
    b = np.asarray(b, C128)
    if a.shape != b.shape:
        raise ValueError(f"shape mismatch {a.shape} vs {b.shape}")
    fa = np.ascontiguousarray(np.stack([a.real, a.imag], -1).ravel())
    fb = np.ascontiguousarray(np.stack([b.real, b.imag], -1).ravel())
    z = np.zeros(2)
    _A.check(_A.lib().pgx_overlap(_ctx_handle(ctx), a.size, _A.as_dptr(fa), _A.as_dptr(fb), _A.as_dptr(z)),
             _ctx_handle(ctx))
    return complex(z[0], z[1])


def gate_fidelity(U, U_target, type: str = "normalized", ctx: Optional[Context] = None) -> float:
    """:normalized |Tr(U_t'U)|^2/d^2, :real Re Tr(U_t'U)/d, :average
    (d F_norm + 1)/(d + 1) (Objectives.jl:239-265)."""
    U = np.asarray(U, C128)
    d = U.shape[0]
    z = _overlap(U_target, U, ctx) / d
    if type == "normalized":
        return abs(z) ** 2
    if type == "real":
        return z.real
    if type == "average":
        return (d * abs(z) ** 2 + 1.0) / (d + 1.0)
    raise ValueError(f"unknown gate fidelity type :{type}")


def state_fidelity(psi_targ, psi_final, type: str = "real", ctx: Optional[Context] = None) -> float:
    """:real Re<t|f>, :square |<t|f>|^2, :modulus |<t|f>|, :dm_linear Re Tr(rho'sigma)
    (Objectives.jl:455-470).  :dm_uhlmann (matrix square roots of density
    matrices) is outside the GRAPE path and not served."""
    if type == "dm_uhlmann":
        raise ValueError("state_fidelity(:dm_uhlmann) is not served by the GPU library")
    z = _overlap(psi_targ, psi_final, ctx)
    if type in ("real", "dm_linear"):
        return z.real
    if type == "square":
        return abs(z) ** 2
    if type == "modulus":
        return abs(z)
    raise ValueError(f"unknown state fidelity type :{type}")


def fidelity_grad_prefactor(z: complex, inner: complex, dt_pwr: float, type: str) -> float:
    """GRAPE chain-rule prefactor (Objectives.jl:352-361); :modulus keeps the
    reference's dt_pwr Im(inner/|z|)."""
    if type == "real":
        return dt_pwr * inner.imag
    if type == "square":
        return 2.0 * dt_pwr * (np.conj(z) * inner).imag
    if type == "modulus":
        az = abs(z)
        return 0.0 if az < 1e-14 else dt_pwr * (inner / az).imag
    raise ValueError(f"unknown fidelity metric :{type}")


def lindblad_grad_prefactor(z: complex, inner: complex, dt_pwr: float, type: str) -> float:
    """Liouville-space prefactor with Re in place of Im (Lindblad.jl:220-232)."""
    if type == "square":
        return 2.0 * dt_pwr * (np.conj(z) * inner).real
    if type == "real":
        return dt_pwr * inner.real
    raise ValueError(f"lindblad_grad_prefactor: ':{type}' not supported. Use :square or :real.")


def finite_difference_gradient(system: QuantumSystem, controls: ControlSequence, target: QuantumTarget,
                               eps: float = 1e-6) -> np.ndarray:
    """Central differences (F(u + eps e_jk) - F(u - eps e_jk)) / 2 eps with F =
    compute_fidelity (Gradients.jl:442-479); every F is a device evaluation."""
    if eps <= 0:
        raise ValueError(f"eps must be positive, got {eps}")
    prob = _system_problem(system, target, controls.n_steps, controls.dt, grad_mode="ref_grape")
    try:
        u = np.array(controls.controls, float)
        G = np.zeros_like(u)
        for j in range(u.shape[0]):
            for k in range(u.shape[1]):
                up, um = u.copy(), u.copy()
                up[j, k] += eps
                um[j, k] -= eps
                G[j, k] = (prob.eval(up, want_grad=False)[0] - prob.eval(um, want_grad=False)[0]) / (2 * eps)
        return G
    finally:
        prob.close()


def grape_gradient_check(system: QuantumSystem, target: QuantumTarget, controls: ControlSequence,
                         eps: float = 1e-5) -> dict:
    """Analytical vs central-difference gradient (GRAPE.jl:911-951): the
    gradient grape_optimize uses against finite differences of its objective."""
    G_ana = compute_grape_gradient(system, controls, target)
    prob = _system_problem(system, target, controls.n_steps, controls.dt, grad_mode="ref_grape")
    try:
        u = np.array(controls.controls, float)
        G_num = np.zeros_like(u)
        for j in range(u.shape[0]):
            for k in range(u.shape[1]):
                up, um = u.copy(), u.copy()
                up[j, k] += eps
                um[j, k] -= eps
                G_num[j, k] = (prob.eval(up, want_grad=False)[0] - prob.eval(um, want_grad=False)[0]) / (2 * eps)
    finally:
        prob.close()
    diff = np.abs(G_ana - G_num)
    max_err = float(np.max(diff)) if diff.size else 0.0
    scale = max(1.0, float(np.max(np.abs(G_num))) if G_num.size else 0.0)
    return {"analytical_gradient": G_ana, "numerical_gradient": G_num, "max_error": max_err,
            "max_relative_error": max_err / scale, "passed": max_err < 1e-4}


def penalty_value_and_gradient(w, type: str, weight: float = 1.0, l_bound: float = -1.0, u_bound: float = 1.0,
                               dt=None, ctx: Optional[Context] = None):
    """(weight P(w), weight dP/dw) for the waveform w [n_ctrl, n_t]
    (Penalties.jl:260-271), on the device."""
    w = np.asarray(w, np.float64)
    if w.ndim != 2:
        raise ValueError("w must be [n_ctrl x n_t]")
    if type not in _A.PENALTY:
        raise ValueError(f"Unknown penalty ':{type}'. Valid: {', '.join(_A.PENALTY)}")
    if weight == 0.0:
        return 0.0, np.zeros_like(w)
    n_c, n_t = w.shape
    pen = _A.Penalty(_A.PENALTY[type], 0, float(weight), float(l_bound), float(u_bound))
    ub = np.ascontiguousarray(w.T).ravel()
    G = np.zeros(n_c * n_t)
    P = np.zeros(1)
    dtb = None if dt is None else np.ascontiguousarray(np.broadcast_to(np.asarray(dt, float), (n_t,)))
    _A.check(_A.lib().pgx_penalty_eval(_ctx_handle(ctx), n_c, n_t, _A.as_dptr(ub),
                                       _A.as_dptr(dtb) if dtb is not None else None, _A.C.byref(pen),
                                       _A.as_dptr(P), _A.as_dptr(G)), _ctx_handle(ctx))
    return float(P[0]), G.reshape(n_t, n_c).T.copy()


def penalty_value(w, type: str, weight: float = 1.0, l_bound: float = -1.0, u_bound: float = 1.0,
                  dt=None) -> float:
    """weight P(w) (Penalties.jl:226-241)."""
    return penalty_value_and_gradient(w, type, weight, l_bound, u_bound, dt)[0]


def penalty_gradient(w, type: str, weight: float = 1.0, l_bound: float = -1.0, u_bound: float = 1.0,
                     dt=None) -> np.ndarray:
    """weight dP/dw (Penalties.jl:243-258)."""
    return penalty_value_and_gradient(w, type, weight, l_bound, u_bound, dt)[1]


# ---- the reference's CUDA backend entry points (CUDABackend.jl) -------------

@dataclass(frozen=True)
class CUDABackend:
    """CUDABackend.jl:55-75 (fields kept; the library always runs on the GPU)."""
    device_id: int = 0
    memory_limit_gb: float = math.inf
    use_tensor_cores: bool = False
    use_async: bool = False


def cuda_backend(device_id: int = 0, memory_limit_gb: float = math.inf, use_tensor_cores: bool = False,
                 use_async: bool = False) -> CUDABackend:
    return CUDABackend(device_id, memory_limit_gb, use_tensor_cores, use_async)


def _backend_ctx(backend: CUDABackend) -> Context:
    return default_context() if backend.device_id == 0 else Context(backend.device_id)


def matrix_exponential_cuda(H, dt: float, backend: CUDABackend) -> np.ndarray:
    """exp(-i H dt) (CUDABackend.jl:126-150); no CPU fallback."""
    return compute_propagator(H, dt, ctx=_backend_ctx(backend))


def batch_propagators_cuda(H_array, dt: float, backend: CUDABackend) -> np.ndarray:
    """H_array [dim, dim, n_steps] -> exp(-i H_k dt) in the same layout
    (CUDABackend.jl:166-207)."""
    H = np.asarray(H_array, C128)
    U = compute_propagators(np.moveaxis(H, 2, 0), dt, ctx=_backend_ctx(backend))
    return np.moveaxis(U, 0, 2)


def fidelity_cuda(U_total, U_target, backend: CUDABackend) -> float:
    """|Tr(U_target' U_total)|^2 / dim^2 (CUDABackend.jl:222-245)."""
    d = np.asarray(U_total).shape[0]
    return abs(_overlap(U_target, U_total, _backend_ctx(backend))) ** 2 / d ** 2


def gradient_cuda(H_drift, H_ctrl, controls, target, dt: float, backend: CUDABackend) -> np.ndarray:
    """The reference's GPU gradient, restated as it computes
    (CUDABackend.jl:271-373): P[0] = I, P[k+1] = U_k P[k]; Q[n] = T',
    Q[k] = Q[k+1] U_k; G[j, k] = (2/d^2) Re(conj(Phi) Tr(Q[k+1]' (-i dt H_j) P[k]))
    with Phi = Tr(T'P[n])/d.  The Q[k+1]' there (the adjoint chain would use
    Q[k+1]) and the extra 1/d make this differ from compute_grape_gradient;
    it is kept as written.  Every product and trace runs on the device."""
    ctx = _backend_ctx(backend)
    Hd = np.asarray(H_drift, C128)
    Hc = [np.asarray(h, C128) for h in H_ctrl]
    u = np.asarray(controls, float)
    T = np.asarray(target, C128)
    d, n_c, n = Hd.shape[0], len(Hc), u.shape[1]
    sysq = QuantumSystem(Hd, Hc)
    H = build_total_hamiltonian(sysq, ControlSequence.from_controls(u, dt), ctx=ctx)
    U = compute_propagators(H, dt, ctx=ctx)
    # the reference's Q[k] = T' U_{n-1} ... U_k is the adjoint of the
    # backward chain seeded with T: Q_ref[k+1]' = Q[k+1]
    P, Q, Utot = _chains(U, seed=T, want=("P", "Q", "T"), ctx=ctx)
    Phi = _overlap(T, Utot, ctx) / d
    X = np.ascontiguousarray(Q[1:])                     # Q_ref[k+1]'
    Y = np.ascontiguousarray(P[:n])                     # P[k]
    out = np.zeros(2 * n_c * n)
    _A.check(_A.lib().pgx_trace_products(ctx.handle, d, n, n_c, _A.as_dptr(_cbuf(X)), _A.as_dptr(_cbuf(np.stack(Hc))),
                                         _A.as_dptr(_cbuf(Y)), _A.as_dptr(out)), ctx.handle)
    tr = (out[0::2] + 1j * out[1::2]).reshape(n, n_c).T      # tr[j, k] = Tr(Q[k+1] H_j P[k])
    return (2.0 / d ** 2) * np.real(np.conj(Phi) * (-1j * dt) * tr)


# ---------------------------------------------------------------------------
# Optimisation
# ---------------------------------------------------------------------------

def _result(o, algorithm: str, extra: Optional[dict] = None) -> OptimizationResult:
    md = {"algorithm": algorithm, "step_size_final": o.step_size_final}
    md.update(extra or {})
    return OptimizationResult(o.controls, o.fidelity, o.fidelity_history, o.gradient_norm_history,
                              o.n_iterations, o.converged, o.termination_reason, o.total_time,
                              o.n_fidelity_evaluations, o.n_gradient_evaluations, md)


def grape_optimize(system: QuantumSystem, target: QuantumTarget, controls_init: ControlSequence,
                   config: GRAPEConfig = GRAPEConfig()) -> OptimizationResult:
    """GRAPE ascent (GRAPE.jl:469-643) on the device-resident problem.  As in
    the reference, F uses initial_state while the in-loop gradient
    (compute_grape_gradient_with!, Gradients.jl:153-157) uses target_state on
    both sides."""
    n_c, n_t = controls_init.controls.shape
    if n_c != system.n_controls:
        raise ValueError(f"controls_init.controls size {(n_c, n_t)} does not match system")
    prob = _system_problem(system, target, n_t, controls_init.dt, grad_mode=config.grad_mode,
                           precision=config.precision, legacy_state_gradient=True)
    try:
        o = prob.optimize(controls_init.controls, "grape", max_iter=config.max_iter,
                          convergence_tol=config.convergence_tol, step_size=config.step_size,
                          adapt_step_size=config.adapt_step_size, min_step_size=config.min_step_size,
                          max_step_size=config.max_step_size,
                          gradient_norm_tol=config.gradient_norm_tol)
    finally:
        prob.close()
    return _result(o, "GRAPE", {"n_controls": n_c, "n_timesteps": n_t, "dt": controls_init.dt,
                                "total_time": controls_init.total_time})


def _systems_as_members(systems: Sequence[QuantumSystem]):
    """Ensemble of systems -> (drifts, controls, member_scale).  Members must
    share their control Hamiltonians up to one real scale per member (B1)."""
    ref = np.stack(systems[0].H_controls)
    scales = []
    for i, s in enumerate(systems):
        Hc = np.stack(s.H_controls)
        if Hc.shape != ref.shape:
            raise ValueError(f"system {i} has a different control set")
        den = np.vdot(ref.ravel(), ref.ravel()).real
        sc = np.vdot(ref.ravel(), Hc.ravel()).real / den if den > 0 else 1.0
        if np.max(np.abs(Hc - sc * ref)) > 1e-12 * max(1.0, np.max(np.abs(Hc))):
            raise ValueError("systems must share control Hamiltonians up to a common real scale")
        scales.append(sc)
    drifts = np.stack([s.H_drift for s in systems])
    return drifts, ref, np.asarray(scales)


class EnsembleObjective:
    """Ensemble objective served by one batched GPU evaluation over all
    samples: the ``batched_eval`` plug of EnsembleObjective.jl:145-163 for
    :mean, and the :worst_case / :cvar aggregators of :169-217 with each
    ensemble member a sample."""

    def __init__(self, problem: Problem, n_samples: int, n_c: int, n_t: int, aggregator: str = "mean",
                 cvar_alpha: float = 0.2):
        if aggregator not in ("mean", "worst_case", "cvar"):
            raise ValueError(f"Unknown aggregator {aggregator}")
        self.problem = problem
        self.n_samples = n_samples
        self.aggregator = aggregator
        self.cvar_alpha = float(cvar_alpha)
        self._shape = (n_c, n_t)

    def _u(self, theta):
        return np.asarray(theta, np.float64).reshape(self._shape, order="F")

    def batched_eval(self, theta):
        if self.aggregator == "mean":
            F, G = self.problem.eval(self._u(theta))
        else:
            F, G = self.problem.eval_aggregate(self._u(theta), self.aggregator, self.cvar_alpha)
        return F, G.reshape(-1, order="F")

    def value(self, theta) -> float:
        if self.aggregator == "mean":
            return self.problem.eval(self._u(theta), want_grad=False)[0]
        return self.problem.eval_aggregate(self._u(theta), self.aggregator, self.cvar_alpha, want_grad=False)[0]

    value_and_grad = batched_eval


def build_ensemble_from_systems(systems, target: QuantumTarget, controls: ControlSequence,
                                aggregator: str = "mean", grad_mode: str = "ref_grape",
                                precision: str = "fp64", cvar_alpha: float = 0.2) -> EnsembleObjective:
    """SystemBuilder.jl:49-87: per-system compute_fidelity +
    compute_grape_gradient, aggregated by :mean, :worst_case or :cvar."""
    if not systems:
        raise ValueError("systems must be non-empty")
    drifts, ctrls, scales = _systems_as_members(systems)
    n = len(systems)
    n_t = controls.n_steps
    kw = dict(member_drift=np.arange(n), member_scale=scales, member_weight=np.full(n, 1.0 / n),
              grad_mode=grad_mode, precision=precision)
    if target.type == "unitary":
        prob = Problem(drifts, ctrls, _dt_vec(controls.dt, n_t), target="gate",
                       target_op=target.target_unitary, **kw)
    else:
        psi_t = target.target_state
        psi_i = psi_t if target.initial_state is None else target.initial_state
        # compute_fidelity uses raw states; compute_grape_gradient normalises
        prob = Problem(drifts, ctrls, _dt_vec(controls.dt, n_t), target="states",
                       states_init=psi_i, states_target=psi_t, **kw)
    return EnsembleObjective(prob, n, ctrls.shape[0], n_t, aggregator, cvar_alpha)


def sample_parametric_perturbations(system: QuantumSystem, n_samples: int, magnitude: float,
                                    rng: Optional[np.random.Generator] = None) -> list:
    """Random Hermitian dH with ||dH||_F = magnitude ||H_drift||_F
    (RobustOpt.jl:137-158): X complex Gaussian / sqrt 2, dH = (X + X')/2,
    rescaled.  numpy's generator stands in for Julia's MersenneTwister."""
    rng = rng or np.random.default_rng()
    H0 = system.H_drift
    d = H0.shape[0]
    n0 = np.linalg.norm(H0)
    n0 = 1.0 if n0 < 1e-14 else n0
    out = []
    for _ in range(n_samples):
        X = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2.0)
        dH = (X + X.conj().T) / 2.0
        out.append(dH * (magnitude * n0 / max(np.linalg.norm(dH), 1e-14)))
    return out


def drift_ramp_schedule(n_timesteps: int) -> np.ndarray:
    """(k - 1) / max(1, n_t - 1), k = 1..n_t: the linear drift ramp of
    sample_drift_trajectories (RobustOpt.jl:173-177)."""
    return np.arange(n_timesteps, dtype=np.float64) / max(1, n_timesteps - 1)


def sample_drift_trajectories(system: QuantumSystem, n_samples: int, magnitude: float, n_timesteps: int,
                              rng: Optional[np.random.Generator] = None) -> list:
    """RobustOpt.jl:168-182: trajectory s is the ramp tau_k dH_final_s over the
    n_t slices, dH_final drawn as sample_parametric_perturbations draws."""
    tau = drift_ramp_schedule(n_timesteps)
    return [[t * dH for t in tau] for dH in sample_parametric_perturbations(system, n_samples, magnitude, rng)]


class PerturbationEnsemble(EnsembleObjective):
    """build_ensemble_from_perturbations (PerturbationBuilder.jl:52-133).
    :parametric -- sample i evolves under H_drift + dH_i; :drift -- under
    H_drift + tau_k dH_i, the linear ramp of sample_drift_trajectories, as a
    per-slice drift ramp of the device problem.  All samples are members of
    one device problem; with resample=True the perturbations are redrawn
    (seed + call count) before every value_and_grad.  The gradient is the
    exact gradient of each sample's fidelity (the reference differentiates by
    central differences, eps 1e-5)."""

    def __init__(self, system: QuantumSystem, target: QuantumTarget, controls: ControlSequence, magnitude: float,
                 n_samples: int, aggregator: str, cvar_alpha: float, resample: bool, seed: int,
                 grad_mode: str = "exact", precision: str = "fp64", uncertainty_type: str = "parametric"):
        if target.type != "unitary":
            raise ValueError("perturbation ensembles score gate fidelities (RobustOpt.jl:739-761)")
        self.system, self.magnitude, self.resample, self.seed = system, float(magnitude), resample, int(seed)
        self.kind = uncertainty_type
        self._calls = 0
        n_t = controls.n_steps
        self._tau = drift_ramp_schedule(n_t)
        pert = sample_parametric_perturbations(system, n_samples, magnitude, np.random.default_rng(seed))
        drift_kind = self.kind == "drift"
        drifts = system.H_drift[None] if drift_kind else np.stack([system.H_drift + dH for dH in pert])
        prob = Problem(drifts, np.stack(system.H_controls), _dt_vec(controls.dt, n_t),
                       member_drift=np.zeros(n_samples, int) if drift_kind else np.arange(n_samples),
                       member_weight=np.full(n_samples, 1.0 / n_samples), n_members=n_samples,
                       target="gate", fidelity="square", target_op=target.target_unitary, grad_mode=grad_mode,
                       precision=precision)
        if drift_kind:
            prob.set_drift_ramp(np.stack(pert), np.arange(n_samples), self._tau)
        super().__init__(prob, n_samples, system.n_controls, n_t, aggregator, cvar_alpha)

    def _redraw(self):
        self._calls += 1
        rng = np.random.default_rng(self.seed + self._calls)
        pert = sample_parametric_perturbations(self.system, self.n_samples, self.magnitude, rng)
        if self.kind == "drift":
            self.problem.set_drift_ramp(np.stack(pert), np.arange(self.n_samples), self._tau)
        else:
            self.problem.set_drifts(np.stack([self.system.H_drift + dH for dH in pert]))

    def batched_eval(self, theta):
        if self.resample:
            self._redraw()
        return super().batched_eval(theta)

    value_and_grad = batched_eval


def build_ensemble_from_perturbations(system: QuantumSystem, target: QuantumTarget, controls: ControlSequence,
                                      uncertainty_type: str = "parametric", magnitude: float = 0.05,
                                      n_samples: int = 20, aggregator: str = "mean", cvar_alpha: float = 0.2,
                                      resample: bool = True, seed: int = 42, precision: str = "fp64"):
    """PerturbationBuilder.jl:52-133 (:parametric and :drift)."""
    if uncertainty_type not in ("parametric", "drift"):
        raise ValueError("uncertainty_type must be :parametric or :drift for this builder; use robust_optimize "
                         "for :noise")
    if n_samples <= 0:
        raise ValueError("n_samples must be positive")
    return PerturbationEnsemble(system, target, controls, magnitude, n_samples, aggregator, cvar_alpha, resample,
                                seed, precision=precision, uncertainty_type=uncertainty_type)


def grape_optimize_ensemble(systems, target: QuantumTarget, controls_init: ControlSequence,
                            config: GRAPEConfig = GRAPEConfig(), lbfgs_memory: int = 10,
                            amplitude_limit: float = math.inf) -> OptimizationResult:
    """Ensemble L-BFGS-GRAPE (GRAPE.jl:1012-1230) on the device."""
    if len(systems) == 0:
        raise ValueError("systems must be non-empty")
    if lbfgs_memory <= 0:
        raise ValueError("lbfgs_memory must be positive")
    obj = build_ensemble_from_systems(systems, target, controls_init, grad_mode=config.grad_mode,
                                      precision=config.precision)
    try:
        o = obj.problem.optimize(controls_init.controls, "ensemble_lbfgs", max_iter=config.max_iter,
                                 convergence_tol=config.convergence_tol, step_size=config.step_size,
                                 min_step_size=config.min_step_size,
                                 max_step_size=config.max_step_size,
                                 gradient_norm_tol=config.gradient_norm_tol,
                                 lbfgs_memory=lbfgs_memory, amplitude_limit=amplitude_limit)
    finally:
        obj.problem.close()
    return _result(o, "Ensemble L-BFGS-GRAPE", {"n_systems": len(systems), "lbfgs_memory": lbfgs_memory})


# ---------------------------------------------------------------------------
# Lindblad builders (src/Physics/Lindblad.jl) -- problem set-up, host side
# ---------------------------------------------------------------------------

def vec_rho(rho) -> np.ndarray:
    return np.asarray(rho, C128).reshape(-1, order="F")


def mat_rho(v, N: int) -> np.ndarray:
    return np.asarray(v, C128).reshape((N, N), order="F")


def pure_state_to_vec_rho(psi) -> np.ndarray:
    c = np.asarray(psi, C128)
    return vec_rho(np.outer(c, c.conj()))


def build_drift_liouvillian(H_drift, jump_ops, decay_rates) -> np.ndarray:
    """-i(I(x)H - H^T(x)I) + sum_k g_k [conj(L)(x)L - 1/2 I(x)L'L - 1/2 conj(L'L)(x)I]."""
    H = np.asarray(H_drift, C128)
    N = H.shape[0]
    IN = np.eye(N, dtype=C128)
    L = -1j * np.kron(IN, H) + 1j * np.kron(H.T, IN)
    for Lk, g in zip(jump_ops, decay_rates):
        if g == 0.0 or not math.isfinite(g):
            continue
        if g < 0.0:
            raise ValueError(f"Lindblad decay rate must be non-negative; got {g}")
        Lk = np.asarray(Lk, C128)
        Ak = Lk.conj().T @ Lk
        L = L + g * (np.kron(Lk.conj(), Lk) - 0.5 * np.kron(IN, Ak) - 0.5 * np.kron(Ak.conj(), IN))
    return L


def build_control_liouvillian(H_ctrl) -> np.ndarray:
    Hc = np.asarray(H_ctrl, C128)
    IN = np.eye(Hc.shape[0], dtype=C128)
    return -1j * np.kron(IN, Hc) + 1j * np.kron(Hc.T, IN)


# ---------------------------------------------------------------------------
# MR contexts and kernels
# ---------------------------------------------------------------------------

def _wrap_states(x):
    a = np.asarray(x, C128)
    return [a] if a.ndim == 1 else [np.asarray(v, C128) for v in x]


@dataclass
class TrackingPoint:
    """GRAPETracking.jl:82-91: the density matrix after propagating through
    ``step`` (1-based) should match ``target_dm`` with weight ``weight``."""
    step: int
    target_dm: np.ndarray
    weight: float

    def __post_init__(self):
        self.step = int(self.step)
        self.target_dm = np.array(self.target_dm, C128)
        self.weight = float(self.weight)


@dataclass
class MRControl:
    """OptControl.jl:137-259 (fields the GRAPE path uses; defaults kept)."""
    drifts: list
    operators: list
    rho_init: list
    rho_targ: list
    pwr_levels: list
    pulse_dt: np.ndarray
    l_bound: float = -1.0
    u_bound: float = 1.0
    method: str = "lbfgs"
    max_iter: int = 500
    grad_tol: float = 1e-7
    fidelity: str = "real"
    lbfgs_memory: int = 10
    backend: str = "cuda"
    grad_mode: str = "ref_mr"
    precision: str = "fp64"
    penalties: list = field(default_factory=list)   # symbols, OptControl.jl (:none skipped)
    p_weights: list = field(default_factory=list)
    tracking: list = field(default_factory=list)    # TrackingPoint checkpoints (OptControl.jl:156,222)

    def __post_init__(self):
        self.rho_init = _wrap_states(self.rho_init)
        self.rho_targ = _wrap_states(self.rho_targ)
        if len(self.rho_init) != len(self.rho_targ):
            raise ValueError("rho_init and rho_targ must have the same length")
        self.pulse_dt = np.asarray(self.pulse_dt, np.float64)
        self.tracking = [tp if isinstance(tp, TrackingPoint) else TrackingPoint(tp.step, tp.target_dm, tp.weight)
                         for tp in self.tracking]
        self._prob = None
        self._track_prob = None

    def _make_problem(self) -> Problem:
        n_d, n_p = len(self.drifts), len(self.pwr_levels)
        md = np.repeat(np.arange(n_d), n_p)
        ms = np.tile(np.asarray(self.pwr_levels, np.float64), n_d)
        prob = Problem(np.stack(self.drifts), np.stack(self.operators), self.pulse_dt,
                       member_drift=md, member_scale=ms, target="states",
                       fidelity=self.fidelity, states_init=np.stack(self.rho_init),
                       states_target=np.stack(self.rho_targ), grad_mode=self.grad_mode,
                       precision=self.precision)
        _set_ctrl_penalties(self, prob)
        return prob

    def problem(self, tracking: bool = False) -> Problem:
        """The device problem of grape_state_kernel, or (tracking=True) of
        grape_tracking_kernel: the same ensemble with the checkpoints set."""
        if not tracking:
            if self._prob is None:
                self._prob = self._make_problem()
            return self._prob
        if not self.tracking:
            raise RuntimeError("grape_tracking_kernel: ctrl.tracking is empty. "
                               "Add TrackingPoint entries or call grape_state_kernel instead.")
        if self._track_prob is None:
            self._track_prob = self._make_problem()
            self._track_prob.set_tracking([tp.step for tp in self.tracking], [tp.weight for tp in self.tracking],
                                          np.stack([tp.target_dm for tp in self.tracking]))
        return self._track_prob


def _set_ctrl_penalties(ctrl, prob: Problem):
    """_apply_penalties! (GRAPEState.jl:571-584): every (pen, weight) with pen
    != :none and weight != 0, bounds l_bound / u_bound of the control."""
    pens = [(str(p), float(wt), ctrl.l_bound, ctrl.u_bound) for p, wt in zip(ctrl.penalties, ctrl.p_weights)
            if str(p) != "none" and float(wt) != 0.0]
    if pens:
        prob.set_penalties(pens)


@dataclass
class LindbladMRControl:
    """OptControl.jl:733-885: Liouvillians precomputed at construction."""
    drifts: list
    operators: list
    rho_init: list
    rho_targ: list
    pwr_levels: list
    pulse_dt: np.ndarray
    jump_ops: list = field(default_factory=list)
    decay_rates: list = field(default_factory=list)
    l_bound: float = -1.0
    u_bound: float = 1.0
    method: str = "lbfgs"
    max_iter: int = 500
    grad_tol: float = 1e-7
    fidelity: str = "square"
    lbfgs_memory: int = 10
    backend: str = "cuda"
    precision: str = "fp64"
    grad_mode: str = "ref_mr"
    penalties: list = field(default_factory=list)
    p_weights: list = field(default_factory=list)

    def __post_init__(self):
        if len(self.jump_ops) != len(self.decay_rates):
            raise ValueError("jump_ops and decay_rates must have the same length")
        if self.fidelity not in ("real", "square"):
            raise ValueError("LindbladMRControl fidelity must be :square or :real")
        if not self.l_bound < self.u_bound:
            raise ValueError("l_bound must be < u_bound")
        N = np.asarray(self.drifts[0]).shape[0]
        self._N = N
        self._L_drifts = [build_drift_liouvillian(H, self.jump_ops, self.decay_rates)
                          for H in self.drifts]
        self._L_controls = [build_control_liouvillian(op) for op in self.operators]

        def to_sigma(psi):
            psi = np.asarray(psi, C128)
            if psi.size == N:
                return pure_state_to_vec_rho(psi)
            if psi.size == N * N:
                return psi
            raise ValueError(f"State vector has length {psi.size}; expected N={N} or N^2={N * N}")

        self.rho_init = _wrap_states(self.rho_init)
        self.rho_targ = _wrap_states(self.rho_targ)
        if len(self.rho_init) != len(self.rho_targ):
            raise ValueError("rho_init and rho_targ must have the same length")
        self._sigma_init = [to_sigma(s) for s in self.rho_init]
        self._sigma_targ = [to_sigma(s) for s in self.rho_targ]
        self.pulse_dt = np.asarray(self.pulse_dt, np.float64)
        self._prob = None

    def problem(self) -> Problem:
        if self._prob is None:
            n_d, n_p = len(self._L_drifts), len(self.pwr_levels)
            self._prob = Problem(np.stack(self._L_drifts), np.stack(self._L_controls), self.pulse_dt,
                                 generator="liouvillian", member_drift=np.repeat(np.arange(n_d), n_p),
                                 member_scale=np.tile(np.asarray(self.pwr_levels, np.float64), n_d),
                                 target="states", fidelity=self.fidelity,
                                 states_init=np.stack(self._sigma_init),
                                 states_target=np.stack(self._sigma_targ), grad_mode=self.grad_mode,
                                 precision=self.precision)
            _set_ctrl_penalties(self, self._prob)
        return self._prob


def ensemble_value(obj: EnsembleObjective, theta) -> float:
    """Aggregated ensemble fidelity at the flat parameter vector theta
    (EnsembleObjective.jl:224-244, batched :mean path)."""
    return obj.value(theta)


def ensemble_value_and_grad(obj: EnsembleObjective, theta):
    """(F, grad F) at theta (EnsembleObjective.jl:265-307, batched :mean path)."""
    return obj.value_and_grad(theta)


def build_ensemble_from_mrcontrol(ctrl, aggregator: str = "mean", cvar_alpha: float = 0.2) -> EnsembleObjective:
    """EnsembleBuilder.jl:72-182: one batched device evaluation over drifts x
    pwr_levels x state pairs (n_samples = their product).  :worst_case and
    :cvar take each (drift, pwr) member, averaged over its state pairs, as a
    sample; the reference splits the pairs into separate samples as well."""
    if aggregator not in ("mean", "worst_case", "cvar"):
        raise ValueError(f"Unknown aggregator {aggregator}")
    n_pairs = len(ctrl.rho_init)
    n_drifts = len(ctrl.drifts)
    prob = ctrl.problem()
    return EnsembleObjective(prob, n_drifts * len(ctrl.pwr_levels) * n_pairs, len(ctrl.operators),
                             len(ctrl.pulse_dt), aggregator, cvar_alpha)


def grape_state_kernel(waveform, ctrl: MRControl):
    """(fidelity, grad) averaged over drifts x pwr_levels x state pairs."""
    return ctrl.problem().eval(np.asarray(waveform, np.float64))


def grape_lindblad_kernel(waveform, ctrl: LindbladMRControl):
    return ctrl.problem().eval(np.asarray(waveform, np.float64))


def grape_tracking_kernel(waveform, ctrl: MRControl):
    """(fidelity, grad) of trajectory tracking (GRAPETracking.jl:150-277):
    weighted checkpoint fidelities averaged over the ensemble and state
    pairs; the gradient of ctrl.grad_mode (the reference's co-state formula
    for "ref_mr")."""
    return ctrl.problem(tracking=True).eval(np.asarray(waveform, np.float64))


def grape_phase_kernel(phi_profile, ctrl: MRControl, amplitudes=None):
    """Phase-only kernel (GRAPEPhase.jl:52-93): (F, dF/dphi) with the
    amplitude profile held fixed (default 1)."""
    phi = np.asarray(phi_profile, np.float64)
    n_ch, n_t = phi.shape
    if len(ctrl.operators) != 2 * n_ch:
        raise ValueError(f"grape_phase_kernel: ctrl has {len(ctrl.operators)} operators but phi_profile has "
                         f"{n_ch} rows -- expected length(operators) == 2 x n_channels.")
    amp = np.ones_like(phi) if amplitudes is None else np.asarray(amplitudes, np.float64)
    if amp.shape != phi.shape:
        raise ValueError(f"grape_phase_kernel: amplitudes {amp.shape} must match phi_profile {phi.shape}.")
    if np.any(amp < 0):
        raise ValueError("grape_phase_kernel: all amplitudes must be >= 0.")
    return ctrl.problem().eval_phase(phi, amp)


def fidelity_forward(waveform, ctrl) -> float:
    """Forward-only ensemble fidelity (GRAPEState.jl:434-566)."""
    return ctrl.problem().eval(np.asarray(waveform, np.float64), want_grad=False)[0]


def optimcon(ctrl, guess) -> OptimizationResult:
    """optimcon(::MRControl | ::LindbladMRControl, guess) with :lbfgs or :grape."""
    guess = np.asarray(guess, np.float64)
    n_c, n_t = guess.shape
    if n_c != len(ctrl.operators):
        raise ValueError(f"guess rows {n_c} != length(ctrl.operators) {len(ctrl.operators)}")
    if n_t != len(ctrl.pulse_dt):
        raise ValueError(f"guess columns {n_t} != length(ctrl.pulse_dt) {len(ctrl.pulse_dt)}")
    if ctrl.method not in ("lbfgs", "grape"):
        raise ValueError(f"method :{ctrl.method} is not served on the device (:lbfgs, :grape)")
    # a non-empty ctrl.tracking selects _optimcon_*_tracking (OptControl.jl:328-345):
    # the same loops on the tracking kernel
    prob = ctrl.problem(tracking=True) if getattr(ctrl, "tracking", None) else ctrl.problem()
    o = prob.optimize(guess, "mr_lbfgs" if ctrl.method == "lbfgs" else "mr_grape", max_iter=ctrl.max_iter,
                      gradient_norm_tol=ctrl.grad_tol, lbfgs_memory=ctrl.lbfgs_memory, l_bound=ctrl.l_bound,
                      u_bound=ctrl.u_bound)
    return _result(o, "L-BFGS" if ctrl.method == "lbfgs" else "GRAPE")
