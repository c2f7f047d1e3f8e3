"""Seeded synthetic workloads (the benchmark configurations).

Each generator returns ``(Spec, u0)``: a plain description of an ensemble
problem in the member model of ``pgx_problem_desc`` (matrices indexed
[row, col]) and initial controls ``u0[n_c, n_t]``.  ``Spec.problem_kwargs()``
gives the keywords of ``engine.Problem`` / ``engine.Server.submit``.  No data
sets or checkpoints are involved: every workload is drawn from numpy's
seeded generator with the shapes and value distributions of the reference's
configurations.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

from .api import build_control_liouvillian, build_drift_liouvillian

C128 = np.complex128


@dataclass
class Spec:
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
        """(drift index, B1 scale, offset, weight) of every member; weights
        default to 1 / (n_members * max(n_pairs, 1)) as pgx_problem_desc does."""
        n = self.n_members
        di = np.zeros(n, int) if self.member_drift is None else np.asarray(self.member_drift)
        sc = np.ones(n) if self.member_scale is None else np.asarray(self.member_scale, float)
        of = np.zeros(n) if self.member_offset is None else np.asarray(self.member_offset, float)
        if self.member_weight is None:
            w = np.full(n, 1.0 / (n * max(self.n_pairs, 1)))
        else:
            w = np.asarray(self.member_weight, float)
        return di, sc, of, w

    def problem_kwargs(self, grad_mode: str = "exact", precision: str = "fp64") -> dict:
        di, sc, of, w = self.members()
        kw = dict(drifts=self.drifts, controls=self.controls, dt=self.dt, generator=self.generator,
                  offset_op=self.offset_op, member_drift=di, member_scale=sc, member_offset=of,
                  member_weight=w, target=self.target, fidelity=self.fidelity, grad_mode=grad_mode,
                  precision=precision)
        if self.target == "gate":
            kw["target_op"] = self.target_op
        else:
            kw["states_init"], kw["states_target"] = self.states_init, self.states_target
        return kw


SX = np.array([[0, 1], [1, 0]], C128)
SY = np.array([[0, -1j], [1j, 0]], C128)
SZ = np.array([[1, 0], [0, -1]], C128)
I2 = np.eye(2, dtype=C128)


def embed(op: np.ndarray, n: int, q: int) -> np.ndarray:
    """op on qubit q of n (qubit 0 is the most significant factor)."""
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
    explicit |0> -> |1> transfer.  Amplitudes U[-0.5, 0.5] from numpy's seeded
    generator (the Julia MersenneTwister stream is not reproducible here)."""
    rng = np.random.default_rng(seed)
    n_t = 100
    dt = np.pi / n_t
    u0 = 0.5 * (2 * rng.random((2, n_t)) - 1)
    psi_t = np.array([0, 1], C128)
    psi_i = np.array([1, 0], C128) if explicit_init else psi_t
    spec = Spec(drifts=(2 * np.pi * 10 / 2 * SZ)[None], controls=np.stack([0.5 * SX, 0.5 * SY]),
                dt=np.full(n_t, dt), target="states", fidelity="square",
                states_init=psi_i[None], states_target=psi_t[None])
    return spec, u0


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
    spec = Spec(drifts=H[None], controls=Hc, dt=np.full(n_t, 1e-6), offset_op=sum(Iz),
                member_offset=mo, member_scale=ms, target="gate", fidelity="square",
                target_op=T, n_members=n_off * n_b1)
    return spec, u0


def spin4_state_transfer(seed: int = 7, n_t: int = 1000, n_off: int = 21, n_b1: int = 11):
    """The spin-4 broadband system as an MR state-transfer ensemble
    (MRControl / grape_state_kernel, GRAPEState.jl:136-250): the same members,
    controls and amplitudes, two basis-state pairs |0000> -> |1111> and
    |0101> -> |1010>, square fidelity, weights 1 / (members x pairs)."""
    spec, u0 = spin4_ensemble(seed, n_t, n_off, n_b1)
    e = np.eye(16, dtype=C128)
    spec.target, spec.fidelity, spec.target_op = "states", "square", None
    spec.states_init, spec.states_target = np.stack([e[0], e[5]]), np.stack([e[15], e[10]])
    return spec, u0


def _rand_herm(rng, d, sigma):
    A = rng.normal(0.0, sigma, (d, d)) + 1j * rng.normal(0.0, sigma, (d, d))
    return (A + A.conj().T) / 2


def _log_uniform_int(rng, lo, hi):
    return int(np.round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))


def uneven_problem(rng: np.random.Generator, d: int = None, n_t: int = None, n_members: int = None):
    """One problem of the uneven batch: d uniform in {2,4,8,16,32}, n_t
    log-uniform in [50, 2000], ensemble size log-uniform in [1, 128]; drift a
    random Hermitian with Gaussian entries (sigma = 2 pi 1 MHz), 2-6 random
    Hermitian controls of the same scale, members spread by a B1 scale
    U[0.9, 1.1] and a detuning U[-0.1, 0.1] sigma along a random diagonal;
    Haar-random gate target; dt = 0.2 / (2 sigma sqrt(d)) so ||H dt|| ~ 0.2."""
    sigma = 2 * np.pi * 1e6
    d = int(rng.choice([2, 4, 8, 16, 32])) if d is None else d
    n_t = _log_uniform_int(rng, 50, 2000) if n_t is None else n_t
    nm = int(np.round(np.exp(rng.uniform(0.0, np.log(128))))) if n_members is None else n_members
    n_c = int(rng.integers(2, 7))
    H = _rand_herm(rng, d, sigma)
    C = np.stack([_rand_herm(rng, d, sigma) for _ in range(n_c)])
    O = np.diag(rng.uniform(-1, 1, d)).astype(C128)
    dt = 0.2 / (2 * sigma * np.sqrt(d))
    spec = Spec(drifts=H[None], controls=C, dt=np.full(n_t, dt), offset_op=O,
                member_scale=rng.uniform(0.9, 1.1, nm), member_offset=rng.uniform(-0.1, 0.1, nm) * sigma,
                target="gate", fidelity="square", target_op=haar_unitary(rng, d), n_members=nm)
    return spec, rng.uniform(-1, 1, (n_c, n_t))


def uneven_batch(n_problems: int = 512, seed: int = 4):
    rng = np.random.default_rng(seed)
    return [uneven_problem(rng) for _ in range(n_problems)]


def lindblad_gate(seed: int = 11, n_qubits: int = 3, n_t: int = 500, n_draws: int = 32,
                  duration: float = 2e-6):
    """n_qubits qubits (Hilbert d = 2^n, Liouville D = d^2): ZZ U[0.1,1] MHz on
    every pair, detuning U[-0.5,0.5] MHz per qubit (redrawn per ensemble
    member), T1 U[20,100] us, T2 = T1 U(0.5,1); jumps sqrt(1/T1) s- and
    sqrt(g_phi/2) sz with g_phi = 1/T2 - 1/(2 T1); controls sx_q, sy_q
    (x 2 pi 1 MHz); the C^(n-1)Z gate (CCZ for three qubits) as the
    superoperator conj(U) (x) U; n_t slices over `duration`."""
    rng = np.random.default_rng(seed)
    n = n_qubits
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
        drifts.append(build_drift_liouvillian(Hd, jumps, rates))
    ctrls = []
    for q in range(n):
        ctrls.append(build_control_liouvillian(2 * np.pi * 1e6 * embed(SX, n, q) / 2))
        ctrls.append(build_control_liouvillian(2 * np.pi * 1e6 * embed(SY, n, q) / 2))
    gate = np.ones(2 ** n, C128)
    gate[-1] = -1
    Ug = np.diag(gate)
    S = np.kron(Ug.conj(), Ug)
    u0 = rng.uniform(-0.5, 0.5, (2 * n, n_t))
    spec = Spec(drifts=np.stack(drifts), controls=np.stack(ctrls), dt=np.full(n_t, duration / n_t),
                generator="liouvillian", member_drift=np.arange(n_draws), target="gate",
                fidelity="square", target_op=S, n_members=n_draws)
    return spec, u0


def lindblad_3q(seed: int = 11, n_t: int = 500, n_draws: int = 32):
    """Three qubits (D = 64), CCZ target, 500 slices over 2 us, 32 detuning
    draws: ``lindblad_gate`` with n_qubits = 3."""
    return lindblad_gate(seed=seed, n_qubits=3, n_t=n_t, n_draws=n_draws)


@dataclass
class ServeJob:
    arrival_s: float
    spec: Spec
    u0: np.ndarray
    kind: str


def serve_stream(seed: int = 5, rate: float = 200.0, duration_s: float = 60.0, lindblad_frac: float = 0.2,
                 max_slices: int = 2000, max_members: int = 128, lindblad_slices: int = 500,
                 lindblad_draws: int = 32):
    """Poisson arrivals at `rate` jobs/s over `duration_s`: a fraction
    `lindblad_frac` are Lindblad gate jobs on 2 or 3 qubits (Hilbert d = 4 or
    8), the rest draws of the uneven-batch distribution.  `max_slices`,
    `max_members`, `lindblad_slices` and `lindblad_draws` bound the sizes (the
    full distribution uses n_t log-uniform in [50, 2000] and up to 128
    members; smaller bounds scale the stream to a shorter run)."""
    rng = np.random.default_rng(seed)
    jobs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration_s:
            break
        if rng.random() < lindblad_frac:
            nq = int(rng.choice([2, 3]))
            spec, u0 = lindblad_gate(seed=int(rng.integers(1 << 31)), n_qubits=nq, n_t=lindblad_slices,
                                     n_draws=lindblad_draws)
            jobs.append(ServeJob(t, spec, u0, f"lindblad{nq}q"))
        else:
            lo = min(50, max_slices)
            n_t = _log_uniform_int(rng, lo, max_slices)
            nm = int(np.round(np.exp(rng.uniform(0.0, np.log(max_members)))))
            spec, u0 = uneven_problem(rng, n_t=n_t, n_members=nm)
            jobs.append(ServeJob(t, spec, u0, f"uneven_d{spec.D}"))
    return jobs
