"""Textbook known answers of the reference's test/Physics/PhysicsValidation.jl
on the device: the propagator entry points (FP64) and whole problem
evaluations through the C ABI in both precisions (the mixed one takes the
register-resident d = 2 expm and the df state chain).
"""
import numpy as np
import pytest

from oracle import ref_semantics as rs
from test_oracle_kats import ECHO_DOMEGA, ECHO_T_FREE, RABI_OMEGA, SX, SZ, phys_echo, phys_rabi
from test_parity_gpu import to_gpu

pytestmark = pytest.mark.gpu

PSI0 = np.array([1, 0], complex)


def test_pi_pulses_and_not_gate_propagators(pg):           # :24-48, :104-106
    U = pg.compute_propagator(np.pi / 2 * SX, 1.0)
    out = U @ PSI0
    assert abs(out[0]) ** 2 < 1e-10 and abs(abs(out[1]) ** 2 - 1) < 1e-10
    assert abs(pg.gate_fidelity(U, SX) - 1.0) < 1e-10
    Uh = pg.compute_propagator(np.pi / 4 * SX, 1.0)
    out2 = Uh @ (Uh @ PSI0)
    assert abs(out2[0]) ** 2 < 1e-10 and abs(abs(out2[1]) ** 2 - 1) < 1e-10


@pytest.mark.parametrize("theta,p1", [(np.pi, 1.0), (2 * np.pi, 0.0), (np.pi / 2, 0.5)])
def test_rabi_propagators(pg, theta, p1):                   # :280-308
    U = pg.compute_propagator(RABI_OMEGA * SX / 2, theta / RABI_OMEGA)
    assert abs(abs((U @ PSI0)[1]) ** 2 - p1) < 1e-10


def test_spin_echo_propagator_stack(pg):                    # :50-73
    T = ECHO_T_FREE
    ref = None
    for dw in ECHO_DOMEGA:
        H = np.stack([np.pi / 4 / T * SX, dw * SZ, np.pi / 2 / T * SX, dw * SZ, np.pi / 4 / T * SX])
        props = pg.compute_propagators(H, T)
        Uo = rs.compute_propagators(H, T)
        assert np.max(np.abs(props - Uo)) < 1e-12
        U = pg.compute_total_propagator(props)
        assert np.max(np.abs(U - rs.compute_total_propagator(Uo))) < 1e-12
        pops = np.abs(U @ PSI0) ** 2
        if ref is None:
            ref = pops
        assert np.max(np.abs(pops - ref)) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rabi_and_echo_problems(pg, precision):
    for theta, p1 in ((np.pi, 1.0), (2 * np.pi, 0.0), (np.pi / 2, 0.5)):
        prob, u = phys_rabi(theta)
        p = to_gpu(pg, prob, "exact", precision=precision)
        F, _ = p.eval(u)
        p.close()
        assert abs(F - p1) < 1e-10, (theta, F)
    F0 = None
    for dw in ECHO_DOMEGA:
        prob, u = phys_echo(dw)
        p = to_gpu(pg, prob, "exact", precision=precision)
        F, _ = p.eval(u)
        p.close()
        if F0 is None:
            F0 = F
            assert abs(F0) < 1e-10
        assert abs(F - F0) < 1e-6, (dw, F, F0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_state_transfer_optimisations(pg, precision):     # :138-186
    """The reference's state-transfer runs: a state target without an
    initial state starts from the target, so the loop stops at once on its
    perfect-fidelity rule with F ~ 1, as the oracle does."""
    from test_oracle_kats import PHYS_STATE_SX, PHYS_STATE_SY

    rng = np.random.default_rng(101)
    rng_o = np.random.default_rng(101)
    sys_g = pg.quantum_system(np.zeros((2, 2), complex), [PHYS_STATE_SX, PHYS_STATE_SY])
    sys_o = rs.QuantumSystem(np.zeros((2, 2), complex), [PHYS_STATE_SX, PHYS_STATE_SY])
    F = {}
    for name, tgt in (("one", np.array([0, 1], complex)), ("plus", np.array([1, 1], complex) / np.sqrt(2))):
        u = 0.1 * rng.standard_normal((2, 50))
        uo = 0.1 * rng_o.standard_normal((2, 50))
        r = pg.grape_optimize(sys_g, pg.state_target(tgt), pg.ControlSequence.from_controls(u, 1e-7),
                              pg.GRAPEConfig(max_iter=300, convergence_tol=1e-9, precision=precision))
        ro = rs.grape_optimize(sys_o, rs.state_target(tgt), rs.ControlSequence(np.ascontiguousarray(uo.T), 1e-7),
                               rs.GRAPEConfig(max_iter=300, convergence_tol=1e-9))
        assert r.fidelity > 0.99
        assert r.n_iterations == ro.n_iterations and abs(r.fidelity - ro.fidelity) < 1e-10
        F[name] = r.fidelity
    sys_off = pg.quantum_system(2 * np.pi * 5e6 * SZ, [PHYS_STATE_SX, PHYS_STATE_SY])
    r_off = pg.grape_optimize(sys_off, pg.state_target(np.array([1, 1], complex) / np.sqrt(2)),
                              pg.ControlSequence.from_controls(0.001 * rng.standard_normal((2, 3)), 1e-10),
                              pg.GRAPEConfig(max_iter=20, precision=precision))
    assert F["plus"] > r_off.fidelity


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_inept_gate_optimisation(pg, precision):         # :191-276
    from test_oracle_kats import phys_inept

    Hd, Hc, U, tau, _, _ = phys_inept()
    u = 0.05 * np.random.default_rng(77).standard_normal((4, 40))
    sys_g = pg.quantum_system(Hd, Hc)
    tgt = pg.unitary_target(U)
    cs = pg.ControlSequence.from_controls(u, tau / 10)
    F0 = pg.compute_fidelity(sys_g, cs, tgt)
    Fo0 = rs.compute_fidelity(rs.QuantumSystem(Hd, Hc), rs.ControlSequence(np.ascontiguousarray(u.T), tau / 10),
                              rs.unitary_target(U))
    assert abs(F0 - Fo0) < 1e-12
    r = pg.grape_optimize(sys_g, tgt, cs, pg.GRAPEConfig(max_iter=200, precision=precision))
    assert r.fidelity > F0
    if precision == "fp64":
        ro = rs.grape_optimize(rs.QuantumSystem(Hd, Hc), rs.unitary_target(U),
                               rs.ControlSequence(np.ascontiguousarray(u.T), tau / 10), rs.GRAPEConfig(max_iter=200))
        assert r.n_iterations == ro.n_iterations and abs(r.fidelity - ro.fidelity) < 1e-8
