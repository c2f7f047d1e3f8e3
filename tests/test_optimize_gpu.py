"""Optimiser loops on the device against the oracle's restatement of the
reference loops (GRAPE.jl:469-643, :1012-1230; OptControl.jl:380-611).

Both sides run the same deterministic control flow; the physics differs only
by method rounding (~1e-15 per evaluation), so the fidelity histories must
agree to tight tolerances until convergence.
"""
import numpy as np
import pytest

from oracle import members as mb
import fx
from oracle import ref_semantics as rs

pytestmark = pytest.mark.gpu

SX = np.array([[0, 1], [1, 0]], complex)
SY = np.array([[0, -1j], [1j, 0]], complex)
SZ = np.diag([1.0, -1.0]).astype(complex)


def _hist_close(a, b, tol):
    n = min(len(a), len(b))
    assert n > 0
    assert np.max(np.abs(np.asarray(a[:n]) - np.asarray(b[:n]))) <= tol


@pytest.mark.parametrize("explicit", [False, True])
def test_grape_optimize_quickstart(pg, explicit):
    """Config-1 quickstart: 1 qubit, 100 slices over pi, GRAPEConfig(max_iter=500,
    step_size=0.05, adapt_step_size=true); legacy gradient semantics."""
    prob, u0 = fx.single_qubit_transfer(explicit_init=explicit)
    dt = prob.dt[0]
    psi_i = prob.states_init[0] if explicit else None
    sys_o = rs.QuantumSystem(prob.drifts[0], list(prob.controls))
    tgt_o = rs.state_target([0, 1], psi_init=psi_i)
    cfg_o = rs.GRAPEConfig(max_iter=500, step_size=0.05, adapt_step_size=True)
    ro = rs.grape_optimize(sys_o, tgt_o, rs.ControlSequence.from_controls(u0, dt), cfg_o)

    sys_g = pg.quantum_system(prob.drifts[0], list(prob.controls))
    tgt_g = pg.state_target([0, 1], psi_init=psi_i)
    rg = pg.grape_optimize(sys_g, tgt_g, pg.ControlSequence.from_controls(u0, dt),
                           pg.GRAPEConfig(max_iter=500, step_size=0.05, adapt_step_size=True))
    assert rg.n_iterations == ro.n_iterations
    assert rg.converged == ro.converged
    _hist_close(rg.fidelity_history, ro.fidelity_history, 1e-9)
    _hist_close(rg.gradient_norm_history, ro.gradient_norm_history, 1e-9)
    assert abs(rg.fidelity - ro.fidelity) <= 1e-9
    assert np.max(np.abs(rg.controls - ro.controls)) <= 1e-7
    assert rg.fidelity >= rg.fidelity_history[0]          # GRAPETests.jl:83,110


def test_grape_optimize_ensemble_lbfgs(pg):
    """Ensemble L-BFGS over three offset qubits (EnsembleTests.jl systems)."""
    rng = np.random.default_rng(42)
    systems_o = [rs.QuantumSystem(0.5 * d * SZ, [0.5 * SX, 0.5 * SY]) for d in (-0.1, 0.0, 0.1)]
    u0 = 0.1 * rng.standard_normal((2, 12))
    T = np.array([[0, 1], [1, 0]], complex)
    tgt = rs.unitary_target(T)
    cs = rs.ControlSequence.from_controls(u0, 0.1)
    F, G = rs.build_ensemble_from_systems(systems_o, tgt, cs)
    cfg = rs.GRAPEConfig(max_iter=15, step_size=0.05)
    ro = rs.grape_optimize_ensemble(F, G, cs, cfg, lbfgs_memory=5, amplitude_limit=20.0)

    systems_g = [pg.quantum_system(s.H_drift, s.H_controls) for s in systems_o]
    rg = pg.grape_optimize_ensemble(systems_g, pg.unitary_target(T), pg.ControlSequence.from_controls(u0, 0.1),
                                    pg.GRAPEConfig(max_iter=15, step_size=0.05), lbfgs_memory=5,
                                    amplitude_limit=20.0)
    assert rg.n_iterations == ro.n_iterations
    _hist_close(rg.fidelity_history, ro.fidelity_history, 1e-9)
    assert abs(rg.fidelity - ro.fidelity) <= 1e-9


def test_optimcon_mr_lbfgs(pg):
    """MR state transfer over three offsets (EnsembleTests.jl:144-183 set-up)."""
    Ix, Iy, Iz = SX / 2, SY / 2, SZ / 2
    drifts = [2 * np.pi * off * Iz for off in (-3000.0, 0.0, 3000.0)]
    rho_i = np.array([1, 0], complex)
    rho_t = np.array([1, -1j]) / np.sqrt(2)
    w0 = 0.1 * np.random.default_rng(17).standard_normal((2, 40))
    ctrl_o = rs.MRControl(drifts=drifts, operators=[Ix, Iy], rho_init=[rho_i], rho_targ=[rho_t],
                          pwr_levels=[2 * np.pi * 1e4], pulse_dt=np.full(40, 5e-6), fidelity="square")
    ro = rs.optimcon_lbfgs(lambda w: rs.grape_state_kernel(w, ctrl_o), w0, max_iter=12)
    ctrl_g = pg.MRControl(drifts=drifts, operators=[Ix, Iy], rho_init=[rho_i], rho_targ=[rho_t],
                          pwr_levels=[2 * np.pi * 1e4], pulse_dt=np.full(40, 5e-6), fidelity="square",
                          max_iter=12)
    rg = pg.optimcon(ctrl_g, w0)
    assert rg.n_iterations == ro.n_iterations
    _hist_close(rg.fidelity_history, ro.fidelity_history, 1e-9)
    assert abs(rg.fidelity - ro.fidelity) <= 1e-9


def test_optimcon_lindblad(pg):
    """LindbladMRControl, 1-spin T1 relaxation (LindbladMRAlgorithmSweepTests.jl set-up)."""
    Ix, Iy, Iz = SX / 2, SY / 2, SZ / 2
    drifts = [2 * np.pi * off * Iz for off in (-500.0, 500.0)]
    sm = np.array([[0, 1], [0, 0]], complex)
    ctrl_g = pg.LindbladMRControl(drifts=drifts, operators=[Ix, Iy], jump_ops=[sm], decay_rates=[20.0],
                                  rho_init=[np.array([1, 0], complex)], rho_targ=[np.array([0, 1], complex)],
                                  pwr_levels=[2 * np.pi * 5e3], pulse_dt=np.full(30, 4e-6), max_iter=10)
    w0 = 0.2 * np.random.default_rng(3).standard_normal((2, 30))
    Ls = ctrl_g._L_drifts
    Lc = ctrl_g._L_controls

    def kern(w):
        return rs.grape_lindblad_kernel(w, Ls, Lc, ctrl_g._sigma_init, ctrl_g._sigma_targ,
                                        [2 * np.pi * 5e3], np.full(30, 4e-6), "square")

    ro = rs.optimcon_lbfgs(kern, w0, max_iter=10)
    rg = pg.optimcon(ctrl_g, w0)
    assert rg.n_iterations == ro.n_iterations
    _hist_close(rg.fidelity_history, ro.fidelity_history, 1e-9)
    assert rg.fidelity > rg.fidelity_history[0]


def test_compute_fidelity_and_gradient_api(pg):
    """The reference-named single-system entry points."""
    rng = np.random.default_rng(1)
    H = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    H = (H + H.conj().T) / 2
    Hc = [np.kron(SX, np.eye(2)), np.kron(np.eye(2), SY)]
    u0 = rng.uniform(-1, 1, (2, 20))
    T = fx.haar_unitary(rng, 4)
    for tgt_o, tgt_g in ((rs.unitary_target(T), pg.unitary_target(T)),
                         (rs.state_target(T[:, 0], psi_init=T[:, 1]), pg.state_target(T[:, 0], psi_init=T[:, 1]))):
        so, sg = rs.QuantumSystem(H, Hc), pg.quantum_system(H, Hc)
        cso, csg = rs.ControlSequence.from_controls(u0, 0.05), pg.ControlSequence.from_controls(u0, 0.05)
        assert abs(pg.compute_fidelity(sg, csg, tgt_g) - rs.compute_fidelity(so, cso, tgt_o)) <= 1e-12
        Go = rs.compute_grape_gradient(so, cso, tgt_o)
        Gg = pg.compute_grape_gradient(sg, csg, tgt_g)
        assert np.max(np.abs(Gg - Go)) <= 1e-10 * max(1.0, np.max(np.abs(Go)))
    Uo = rs.compute_total_propagator(rs.compute_propagators(
        rs.build_total_hamiltonian(rs.QuantumSystem(H, Hc), rs.ControlSequence.from_controls(u0, 0.05)), 0.05))
    assert np.max(np.abs(pg.propagate(pg.quantum_system(H, Hc), pg.ControlSequence.from_controls(u0, 0.05)) - Uo)) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["convergence", "monotone", "gradient_vanishes", "x_gate", "cnot", "improves",
                                  "long_pulse"])
def test_grape_reference_cases_on_device(pg, name, precision):
    """The runs of the reference's GRAPETests.jl through grape_optimize on the
    device: each passes the reference test's own assertions, and in FP64
    follows the oracle's loop (iteration count, F history)."""
    from test_oracle_kats import _oracle_grape, grape_case_checks, grape_cases

    (H, Hc), (kind, T), u, dt, kw = grape_cases()[name]
    sys_g = pg.quantum_system(H, Hc)
    tgt = pg.state_target(T) if kind == "state" else pg.unitary_target(T)
    cs = pg.ControlSequence.from_controls(u, dt)
    F0 = pg.compute_fidelity(sys_g, cs, tgt)
    r = pg.grape_optimize(sys_g, tgt, cs, pg.GRAPEConfig(precision=precision, **kw))
    grape_case_checks(name, r, F0)
    if precision == "fp64":
        ro, Fo0 = _oracle_grape(name)
        assert abs(F0 - Fo0) < 1e-12
        assert r.n_iterations == ro.n_iterations
        _hist_close(r.fidelity_history, ro.fidelity_history, 1e-9)
