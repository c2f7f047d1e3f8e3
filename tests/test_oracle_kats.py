"""The oracle pinned against the reference's own known-answer tests.

Julia is not installed, so the reference cannot be executed here; the FP64
restatement in oracle/ is instead held to every invariant and known answer the
reference's test-suite states for this path.  Each test names the reference
test it re-implements.  Seeds are numpy's (the Julia MersenneTwister stream is
not reproducible); the sizes and scales are the reference tests' own.
"""
import numpy as np
import pytest

from oracle import members as mb
import fx
from oracle import ref_semantics as rs

SX = np.array([[0, 1], [1, 0]], complex)
SY = np.array([[0, -1j], [1j, 0]], complex)
SZ = np.array([[1, 0], [0, -1]], complex)
I2 = np.eye(2, dtype=complex)


def herm(rng, d):
    A = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    return A + A.conj().T


# --- test/Physics/MathematicalCorrectness.jl "Propagator correctness" -------

def test_zero_hamiltonian_identity():          # :34-37
    U = rs.expm_neg_i(np.zeros((2, 2), complex), 1e-6)
    assert np.linalg.norm(U - I2) < 1e-12


def test_random_hermitian_unitary():           # :40-46, :77-81
    rng = np.random.default_rng(42)
    U = rs.expm_neg_i(herm(rng, 2), 1e-7)
    assert np.linalg.norm(U.conj().T @ U - I2) < 1e-10
    assert np.linalg.norm(U @ U.conj().T - I2) < 1e-10
    U4 = rs.expm_neg_i(herm(rng, 4), 5e-8)
    assert np.linalg.norm(U4.conj().T @ U4 - np.eye(4)) < 1e-10


def test_sigma_z_known_rotation():             # :48-61
    U = rs.expm_neg_i(np.pi * SZ, 1.0)
    assert abs(U[0, 0] - np.exp(-1j * np.pi)) < 1e-10
    assert abs(U[1, 1] - np.exp(1j * np.pi)) < 1e-10
    assert abs(U[0, 1]) < 1e-10 and abs(U[1, 0]) < 1e-10


def test_product_and_piecewise_formula():      # :63-75
    t1, t2 = 1.5e-6, 2.3e-6
    H = 2 * np.pi * 1e5 * SX
    assert np.linalg.norm(rs.expm_neg_i(H, t1 + t2) - rs.expm_neg_i(H, t2) @ rs.expm_neg_i(H, t1)) < 1e-8
    steps = np.stack([rs.expm_neg_i(H, t1 / 50)] * 50)
    assert np.linalg.norm(rs.expm_neg_i(H, t1) - rs.compute_total_propagator(steps)) < 1e-8


def test_det_of_traceless_generator():         # :300-315 (Jacobi's formula)
    rng = np.random.default_rng(3)
    H = herm(rng, 4)
    H -= np.trace(H) / 4 * np.eye(4)
    assert abs(np.linalg.det(rs.expm_neg_i(H, 0.3)) - 1.0) < 1e-12


# --- "Fidelity bounds" --------------------------------------------------------

def test_fidelity_bounds():                    # :88-140
    assert abs(rs.gate_fidelity(I2, I2) - 1.0) < 1e-12
    rng = np.random.default_rng(7)
    for _ in range(20):
        Ua, Ub = fx.haar_unitary(rng, 2), fx.haar_unitary(rng, 2)
        assert -1e-12 <= rs.gate_fidelity(Ua, Ub) <= 1 + 1e-12
    assert abs(rs.state_fidelity([1, 0], [0, 1], "square")) < 1e-14
    p = np.array([1, 1]) / np.sqrt(2)
    assert abs(rs.state_fidelity(p, p, "square") - 1.0) < 1e-12
    for _ in range(10):
        v, w = rng.standard_normal(2) + 1j * rng.standard_normal(2), rng.standard_normal(2) + 0j
        v, w = v / np.linalg.norm(v), w / np.linalg.norm(w)
        assert abs(rs.state_fidelity(v, w, "square") - rs.state_fidelity(w, v, "square")) < 1e-12
    assert rs.gate_fidelity(SX, SZ) < 0.5
    assert abs(rs.gate_fidelity(I2, np.exp(0.7j) * I2) - 1.0) < 1e-12


# --- "Gradient correctness" (first-order at 1e-2, exact at 1e-6) -------------

def _fd_case(two_qubit: bool, seed=99):
    rng = np.random.default_rng(seed)
    n_ts, dt = 60, 1e-7
    if not two_qubit:
        Hd = 2 * np.pi * 5e3 * SZ
        Hc = [2 * np.pi * 1e4 * SX, 2 * np.pi * 1e4 * SY]
        u0 = 0.3 * rng.standard_normal((2, n_ts))
        T = SX
    else:
        k = np.kron
        Hd = 2 * np.pi * (8e3 * k(SZ, I2) + 6e3 * k(I2, SZ) + 2e2 * k(SZ, SZ))
        Hc = [2 * np.pi * 1e4 * k(SX, I2), 2 * np.pi * 1e4 * k(SY, I2),
              2 * np.pi * 1e4 * k(I2, SX), 2 * np.pi * 1e4 * k(I2, SY)]
        u0 = 0.2 * rng.standard_normal((4, n_ts))
        T = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], complex)
    sysq = rs.QuantumSystem(Hd, Hc)
    return sysq, rs.unitary_target(T), rs.ControlSequence.from_controls(u0, dt)


@pytest.mark.parametrize("two_qubit", [False, True])
def test_gradient_vs_finite_differences(two_qubit):   # :136-193
    sysq, tgt, cs = _fd_case(two_qubit)
    G_ref = rs.compute_grape_gradient(sysq, cs, tgt)
    G_fd = rs.finite_difference_gradient(sysq, cs, tgt, eps=1e-6)
    assert np.linalg.norm(G_ref - G_fd) / np.linalg.norm(G_fd) < 1e-2
    prob = mb.Problem(drifts=sysq.H_drift[None], controls=np.stack(sysq.H_controls),
                      dt=np.full(cs.n_timesteps, cs.dt), target="gate", target_op=tgt.target_unitary)
    _, G_ex = mb.eval_problem(prob, cs.controls, "exact")
    assert np.linalg.norm(G_ex - G_fd) / np.linalg.norm(G_fd) < 1e-6


# --- PhysicsValidation.jl "Closed-system vs Lindblad (zero rates)" -----------

def test_zero_rate_lindblad_equals_unitary():          # :312-350
    Om = 2 * np.pi * 1.5e6
    Hd = 2 * np.pi * 2.0e5 * SZ
    Hc = [Om / 2 * SX, Om / 2 * SY]
    amps, t = [0.3, 0.2], 1.2e-7
    Htot = Hd + amps[0] * Hc[0] + amps[1] * Hc[1]
    U = rs.expm_neg_i(Htot, t)
    rho0 = np.array([[0.7, 0.1 - 0.2j], [0.1 + 0.2j, 0.3]])
    Ld = rs.build_drift_liouvillian(Hd, [SX, SZ], [0.0, 0.0])
    Lc = [rs.build_control_liouvillian(h) for h in Hc]
    Lt = Ld + amps[0] * Lc[0] + amps[1] * Lc[1]
    rho_l = rs.mat_rho(rs.expm_general(Lt * t) @ rs.vec_rho(rho0), 2)
    assert np.linalg.norm(rho_l - U @ rho0 @ U.conj().T) < 1e-10
    assert abs(np.trace(rho_l) - 1.0) < 1e-10
    assert np.linalg.norm(rho_l - rho_l.conj().T) < 1e-10


def test_liouvillian_rejects_negative_rate():          # Lindblad.jl:145-148
    with pytest.raises(ValueError):
        rs.build_drift_liouvillian(SZ, [SX], [-1.0])


# --- EnsembleTests.jl -------------------------------------------------------

def _en_qubit(delta):
    return rs.QuantumSystem(0.5 * delta * SZ, [0.5 * SX, 0.5 * SY])


def test_ensemble_mean_equals_hand_average():          # :65-91
    rng = np.random.default_rng(31)
    systems = [_en_qubit(d) for d in (-0.3, 0.0, 0.3)]
    tgt = rs.state_target([0, 1])
    cs = rs.ControlSequence(0.05 * rng.standard_normal((18, 2)), 0.08)
    F, G = rs.build_ensemble_from_systems(systems, tgt, cs)
    Fh = np.mean([rs.compute_fidelity(s, cs, tgt) for s in systems])
    Gh = np.mean([rs.compute_grape_gradient(s, cs, tgt) for s in systems], axis=0)
    assert abs(F(cs.controls) - Fh) < 1e-10
    assert np.max(np.abs(G(cs.controls) - Gh)) <= 1e-10
    # the member model reproduces the same numbers (drift per member)
    prob = mb.Problem(drifts=np.stack([s.H_drift for s in systems]), controls=np.stack([0.5 * SX, 0.5 * SY]),
                      dt=np.full(18, 0.08), member_drift=np.arange(3), n_members=3, target="states",
                      states_init=np.array([[0, 1]], complex), states_target=np.array([[0, 1]], complex))
    Fm, Gm = mb.eval_problem(prob, cs.controls, "ref_grape")
    assert abs(Fm - Fh) < 1e-12 and np.max(np.abs(Gm - Gh)) < 1e-14


def test_mr_batched_equals_kernel():                   # :144-183
    Ix, Iy, Iz = SX / 2, SY / 2, SZ / 2
    drifts = [2 * np.pi * off * Iz for off in (-3000.0, 0.0, 3000.0)]
    ctrl = rs.MRControl(drifts=drifts, operators=[Ix, Iy], rho_init=[np.array([1, 0], complex)],
                        rho_targ=[np.array([1, -1j]) / np.sqrt(2)], pwr_levels=[2 * np.pi * 1e4],
                        pulse_dt=np.full(40, 5e-6), fidelity="square")
    w0 = 0.1 * np.random.default_rng(17).standard_normal((2, 40))
    F, G = rs.grape_state_kernel(w0, ctrl)
    prob = mb.Problem(drifts=np.stack(drifts), controls=np.stack([Ix, Iy]), dt=ctrl.pulse_dt,
                      member_drift=np.arange(3), member_scale=np.full(3, 2 * np.pi * 1e4), n_members=3,
                      target="states", fidelity="square", states_init=np.array([ctrl.rho_init[0]]),
                      states_target=np.array([ctrl.rho_targ[0]]))
    Fm, Gm = mb.eval_problem(prob, w0, "ref_mr")
    assert abs(F - Fm) <= 1e-12
    assert np.max(np.abs(G - Gm)) <= 1e-12


def test_lindblad_kernel_matches_member_model():
    rng = np.random.default_rng(5)
    N = 2
    Hs = [2 * np.pi * o * SZ / 2 for o in (-1e3, 1e3)]
    Ls = [rs.build_drift_liouvillian(H, [np.array([[0, 1], [0, 0]], complex)], [50.0]) for H in Hs]
    Lc = [rs.build_control_liouvillian(SX / 2), rs.build_control_liouvillian(SY / 2)]
    s0 = rs.pure_state_to_vec_rho([1, 0])
    st = rs.pure_state_to_vec_rho([0, 1])
    w = 0.2 * rng.standard_normal((2, 12))
    dt = np.full(12, 2e-5)
    F, G = rs.grape_lindblad_kernel(w, Ls, Lc, [s0], [st], [2 * np.pi * 5e3], dt, "square")
    prob = mb.Problem(drifts=np.stack(Ls), controls=np.stack(Lc), dt=dt, generator="liouvillian",
                      member_drift=np.arange(2), member_scale=np.full(2, 2 * np.pi * 5e3), n_members=2,
                      target="states", fidelity="square", states_init=s0[None], states_target=st[None])
    Fm, Gm = mb.eval_problem(prob, w, "ref_mr")
    assert abs(F - Fm) <= 1e-12 and np.max(np.abs(G - Gm)) <= 1e-12


# --- GRAPETests.jl ------------------------------------------------------------

def test_grape_optimize_reproducible_and_monotone_best():   # :141-161, :106-111
    prob, u0 = fx.single_qubit_transfer()
    sysq = rs.QuantumSystem(prob.drifts[0], list(prob.controls))
    tgt = rs.state_target([0, 1])
    cfg = rs.GRAPEConfig(max_iter=60, step_size=0.05, adapt_step_size=True)
    r1 = rs.grape_optimize(sysq, tgt, rs.ControlSequence.from_controls(u0, prob.dt[0]), cfg)
    r2 = rs.grape_optimize(sysq, tgt, rs.ControlSequence.from_controls(u0, prob.dt[0]), cfg)
    assert r1.fidelity == r2.fidelity and np.array_equal(r1.controls, r2.controls)
    assert r1.fidelity >= r1.fidelity_history[0]


def test_exact_gradient_of_modulus_and_real_metrics_vs_fd():
    rng = np.random.default_rng(2)
    H = herm(rng, 3) * 0.3
    C = [herm(rng, 3) * 0.2, herm(rng, 3) * 0.2]
    psi = np.array([1, 0, 0], complex)
    tgt = fx.haar_unitary(rng, 3)[:, 0]
    for fid in ("real", "modulus", "square"):
        prob = mb.Problem(drifts=H[None], controls=np.stack(C), dt=np.full(6, 0.4), target="states",
                          fidelity=fid, states_init=psi[None], states_target=tgt[None])
        u = rng.standard_normal((2, 6))
        _, G = mb.eval_problem(prob, u, "exact")
        h = 1e-6
        for (j, k) in ((0, 0), (1, 3), (0, 5)):
            up, um = u.copy(), u.copy()
            up[j, k] += h
            um[j, k] -= h
            fd = (mb.eval_problem(prob, up, want_grad=False)[0] - mb.eval_problem(prob, um, want_grad=False)[0]) / (2 * h)
            assert abs(fd - G[j, k]) < 1e-7 * max(1.0, abs(fd))


def test_frechet_spectral_matches_scipy():
    rng = np.random.default_rng(8)
    H = herm(rng, 5)
    E = rng.standard_normal((5, 5)) + 1j * rng.standard_normal((5, 5))
    dt = 0.37
    A = -1j * dt * H
    L1 = mb.frechet_exp(A, E, (H, dt))
    L2 = mb.frechet_exp(A, E)
    assert np.max(np.abs(L1 - L2)) < 1e-12 * max(1.0, np.max(np.abs(L2)))


# --- test/Physics/PhysicsValidation.jl (textbook results) -----------------------
# The pulse sequences below are the reference tests' own; PHYS_* build them
# once for these oracle checks and for the device checks in
# tests/test_physics_kats_gpu.py.

RABI_OMEGA = 2 * np.pi * 1e5                                   # :285
ECHO_T_FREE = 5e-6                                            # :55
ECHO_DOMEGA = (0.0, 1e3, 5e3, -3e3, 10e3)                     # :54


def phys_rabi(theta: float):
    """One slice of H = Omega sigma_x / 2 for the pulse area theta (:284-308):
    a state-transfer problem |0> -> |1>, square fidelity = P1."""
    prob = mb.Problem(drifts=np.zeros((1, 2, 2), complex), controls=(SX / 2)[None],
                      dt=np.array([theta / RABI_OMEGA]), target="states", fidelity="square",
                      states_init=np.array([[1, 0]], complex), states_target=np.array([[0, 1]], complex))
    return prob, np.array([[RABI_OMEGA]])


def phys_echo(domega: float):
    """pi/2 - free - pi - free - pi/2 about x, free precession domega sigma_z,
    each interval T_free (:50-73), as five slices with controls (sigma_x,
    sigma_z); square fidelity |<1|psi>|^2 = P1."""
    T = ECHO_T_FREE
    u = np.array([[np.pi / 4 / T, 0.0, np.pi / 2 / T, 0.0, np.pi / 4 / T],
                  [0.0, domega, 0.0, domega, 0.0]])
    prob = mb.Problem(drifts=np.zeros((1, 2, 2), complex), controls=np.stack([SX, SZ]), dt=np.full(5, T),
                      target="states", fidelity="square", states_init=np.array([[1, 0]], complex),
                      states_target=np.array([[0, 1]], complex))
    return prob, u


def test_pi_pulse_and_two_half_pi_pulses_flip_the_qubit():     # :24-48
    psi0 = np.array([1, 0], complex)
    out = rs.expm_neg_i(np.pi / 2 * SX, 1.0) @ psi0
    assert abs(out[0]) ** 2 < 1e-10 and abs(abs(out[1]) ** 2 - 1) < 1e-10
    Uh = rs.expm_neg_i(np.pi / 4 * SX, 1.0)
    out2 = Uh @ (Uh @ psi0)
    assert abs(out2[0]) ** 2 < 1e-10 and abs(abs(out2[1]) ** 2 - 1) < 1e-10


def test_x_rotation_is_the_not_gate():                         # :104-106
    U = rs.expm_neg_i(np.pi / 2 * SX, 1.0)
    assert abs(rs.gate_fidelity(U, SX) - 1.0) < 1e-10


@pytest.mark.parametrize("theta,p1", [(np.pi, 1.0), (2 * np.pi, 0.0), (np.pi / 2, 0.5)])
def test_rabi_populations(theta, p1):                          # :280-308
    prob, u = phys_rabi(theta)
    F, _ = mb.eval_problem(prob, u, want_grad=False)
    assert abs(F - p1) < 1e-10


def test_spin_echo_refocuses_every_offset():                   # :50-73
    F0 = mb.eval_problem(*phys_echo(0.0), want_grad=False)[0]
    assert abs(F0) < 1e-10  # a net 2 pi rotation about x: back in |0>
    for dw in ECHO_DOMEGA[1:]:
        F = mb.eval_problem(*phys_echo(dw), want_grad=False)[0]
        assert abs(F - F0) < 1e-6


# --- test/Algorithms/EnsembleTests.jl "aggregator correctness" (:33-62) ------

def test_ensemble_aggregators_on_synthetic_samples():
    offsets = [0.9, 0.8, 0.7, 0.6]
    grads = [np.array([1.0, 0.0]) for _ in offsets]
    F_m, G_m = rs.aggregate(offsets, grads, "mean")
    F_wc, G_wc = rs.aggregate(offsets, grads, "worst_case")
    F_cv, _ = rs.aggregate(offsets, grads, "cvar", 0.5)
    assert abs(F_m - sum(offsets) / 4) < 1e-15 and np.allclose(G_m, [1.0, 0.0])
    assert F_wc == min(offsets) and np.allclose(G_wc, [1.0, 0.0])
    assert abs(F_cv - (0.6 + 0.7) / 2) < 1e-15
    assert F_wc <= F_cv <= F_m + 1e-12


# --- PhysicsValidation.jl "State transfer" (:138-186) and INEPT (:191-276) ----

PHYS_STATE_SX, PHYS_STATE_SY = 2 * np.pi * SX, 2 * np.pi * SY


def phys_inept():
    """The INEPT sequence's analytic gate on a 1H-13C pair (J = 125 Hz,
    tau = 1 / 4J), its drift 2 pi J (2 Iz_H Iz_C) and controls
    (Ix_H, Iy_H, Ix_C, Iy_C)."""
    SzH, SzC = np.kron(SZ / 2, I2), np.kron(I2, SZ / 2)
    J = 125.0
    tau = 1.0 / (4 * J)
    Hd = 2 * np.pi * J * (2.0 * SzH @ SzC)
    Hc = [np.kron(SX / 2, I2), np.kron(SY / 2, I2), np.kron(I2, SX / 2), np.kron(I2, SY / 2)]
    ex = lambda H: rs.expm_neg_i(H, 1.0)  # noqa: E731
    U = (ex(np.pi / 4 * np.kron(I2, SY)) @ ex(np.pi / 4 * np.kron(SY, I2)) @ rs.expm_neg_i(Hd, tau)
         @ ex(np.pi / 2 * np.kron(I2, SX)) @ ex(np.pi / 2 * np.kron(SX, I2)) @ rs.expm_neg_i(Hd, tau)
         @ ex(np.pi / 4 * np.kron(SY, I2)))
    return Hd, Hc, U, tau, SzH, SzC


def test_state_transfer_with_the_target_as_initial_state():
    # A state target without an initial state starts from the target itself
    # (the reference's legacy convention), so near-zero controls already give
    # F ~ 1 and the loop stops on its perfect-fidelity rule.
    rng = np.random.default_rng(101)
    sys_ = rs.QuantumSystem(np.zeros((2, 2), complex), [PHYS_STATE_SX, PHYS_STATE_SY])
    cfg = rs.GRAPEConfig(max_iter=300, convergence_tol=1e-9)
    F = {}
    for name, tgt in (("one", np.array([0, 1], complex)), ("plus", np.array([1, 1], complex) / np.sqrt(2))):
        u = 0.1 * rng.standard_normal((2, 50))
        r = rs.grape_optimize(sys_, rs.state_target(tgt), rs.ControlSequence(np.ascontiguousarray(u.T), 1e-7), cfg)
        assert r.fidelity > 0.99
        F[name] = r.fidelity
    sys_off = rs.QuantumSystem(2 * np.pi * 5e6 * SZ, [PHYS_STATE_SX, PHYS_STATE_SY])
    u_short = 0.001 * rng.standard_normal((2, 3))
    r_off = rs.grape_optimize(sys_off, rs.state_target(np.array([1, 1], complex) / np.sqrt(2)),
                              rs.ControlSequence(np.ascontiguousarray(u_short.T), 1e-10),
                              rs.GRAPEConfig(max_iter=20))
    assert F["plus"] > r_off.fidelity


def test_inept_antiphase_and_grape_improvement():
    Hd, Hc, U, tau, SzH, SzC = phys_inept()
    psi = np.array([1, 0, 0, 0], complex)
    out = U @ psi
    anti = 2 * SzH @ SzC
    assert abs((out.conj() @ anti @ out).real - (psi.conj() @ anti @ psi).real) > 0.1
    assert (psi.conj() @ SzH @ psi).real > 0
    rng = np.random.default_rng(77)
    cs = rs.ControlSequence(np.ascontiguousarray((0.05 * rng.standard_normal((4, 40))).T), tau / 10)
    sys_ = rs.QuantumSystem(Hd, Hc)
    tgt = rs.unitary_target(U)
    F0 = rs.compute_fidelity(sys_, cs, tgt)
    r = rs.grape_optimize(sys_, tgt, cs, rs.GRAPEConfig(max_iter=200))
    assert r.fidelity > F0


# --- test/Algorithms/GRAPETests.jl (:20-288) -----------------------------------
# Resonant qubit with 1 MHz Rabi drives, and a ZZ-coupled qubit pair; the
# reference's seeds are MersenneTwister streams, these numpy's.  GRAPE_CASES
# feeds these oracle checks and the device runs in tests/test_optimize_gpu.py:
# name -> (system, target, u [n_c, n_t], dt, GRAPEConfig keywords).

def grape_qubit():                                             # :20-30
    return np.zeros((2, 2), complex), [2 * np.pi * 1e6 * SX, 2 * np.pi * 1e6 * SY]


def grape_two_qubit():                                         # :35-53
    ZI, IZ, ZZ = np.kron(SZ, I2), np.kron(I2, SZ), np.kron(SZ, SZ)
    H = 2 * np.pi * (80e3 * ZI + 60e3 * IZ + 50e3 * ZZ)
    Hc = [2 * np.pi * 1e6 * np.kron(SX, I2), 2 * np.pi * 1e6 * np.kron(SY, I2),
          2 * np.pi * 1e6 * np.kron(I2, SX), 2 * np.pi * 1e6 * np.kron(I2, SY)]
    return H, Hc


CNOT = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], complex)
KET1 = np.array([0, 1], complex)


def grape_cases():
    r = np.random.default_rng
    return {
        "convergence": (grape_qubit(), ("state", KET1), 0.1 * r(42).standard_normal((2, 100)), 1e-7,
                        dict(max_iter=500, convergence_tol=1e-9)),                        # :59-85
        "monotone": (grape_qubit(), ("state", KET1), 0.05 * r(7).standard_normal((2, 50)), 1e-7,
                     dict(max_iter=200)),                                                 # :88-113
        "gradient_vanishes": (grape_qubit(), ("state", KET1), 0.1 * r(11).standard_normal((2, 80)), 1e-7,
                              dict(max_iter=600, convergence_tol=1e-10)),                 # :116-138
        "x_gate": (grape_qubit(), ("gate", SX), 0.1 * r(55).standard_normal((2, 100)), 1e-7,
                   dict(max_iter=600, convergence_tol=1e-9)),                             # :181-195
        "cnot": (grape_two_qubit(), ("gate", CNOT), 0.02 * r(33).standard_normal((4, 120)), 5e-8,
                 dict(max_iter=1000, convergence_tol=1e-8)),                              # :198-224
        "improves": (grape_qubit(), ("state", KET1), 0.001 * r(999).standard_normal((2, 30)), 1e-7,
                     dict(max_iter=50)),                                                  # :227-243
        "long_pulse": (grape_qubit(), ("state", KET1), 0.05 * r(123).standard_normal((2, 500)), 2e-8,
                       dict(max_iter=200)),                                               # :271-290
    }


def grape_case_checks(name, r, F0):
    """The reference test's assertions on a result r (F0: the start's F)."""
    hist = np.asarray(r.fidelity_history)
    if name == "convergence":
        assert r.fidelity > 0.99 and (r.converged or r.n_iterations == 500)
        assert np.all(np.diff(hist) >= -1e-8)
    elif name == "monotone":
        assert np.all(np.diff(hist) >= -1e-8)
    elif name == "gradient_vanishes":
        assert r.gradient_norm_history[-1] < 1e-3
    elif name == "x_gate":
        assert r.fidelity > 0.99
    elif name == "cnot":
        assert r.fidelity > 0.95
    elif name == "improves":
        assert r.fidelity > F0
    elif name == "long_pulse":
        assert np.isfinite(r.fidelity) and 0.0 <= r.fidelity <= 1.0 + 1e-10


def _oracle_grape(name):
    (H, Hc), (kind, T), u, dt, kw = grape_cases()[name]
    sys_ = rs.QuantumSystem(H, Hc)
    tgt = rs.state_target(T) if kind == "state" else rs.unitary_target(T)
    cs = rs.ControlSequence(np.ascontiguousarray(u.T), dt)
    return rs.grape_optimize(sys_, tgt, cs, rs.GRAPEConfig(**kw)), rs.compute_fidelity(sys_, cs, tgt)


@pytest.mark.parametrize("name", ["convergence", "monotone", "gradient_vanishes", "x_gate", "cnot", "improves",
                                  "long_pulse"])
def test_grape_reference_cases(name):
    r, F0 = _oracle_grape(name)
    grape_case_checks(name, r, F0)
