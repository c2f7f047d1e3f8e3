"""Standalone building blocks of the path, each a device call, against the
oracle's restatements: build_total_hamiltonian, compute_propagators, the
forward / backward / total chains (Propagators.jl:127-544), gate and state
fidelities (Objectives.jl), finite differences and grape_gradient_check
(Gradients.jl:442-479, GRAPE.jl:911-951), the CUDA-backend entry points
(CUDABackend.jl:126-373) and the batched ensemble objective.
"""
import numpy as np
import pytest

import fx
from oracle import ref_semantics as rs

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _herm(rng, d, s=1.0):
    A = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    return s * (A + A.conj().T) / 2


def _unitary(rng, d):
    Z = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    Q, R = np.linalg.qr(Z)
    return Q * (np.diag(R) / np.abs(np.diag(R)))[None, :]


@pytest.mark.parametrize("d", [2, 3, 16, 40])
def test_total_hamiltonian_and_propagator_stack(pg, d):
    rng = np.random.default_rng(d)
    n_t, n_c = 6, 3
    sys_g = pg.quantum_system(_herm(rng, d), [_herm(rng, d) for _ in range(n_c)])
    cs = pg.ControlSequence(rng.uniform(-1, 1, (n_t, n_c)), 0.03)
    H = pg.build_total_hamiltonian(sys_g, cs)
    Ho = rs.build_total_hamiltonian(rs.QuantumSystem(sys_g.H_drift, sys_g.H_controls),
                                    rs.ControlSequence(cs.amplitudes, cs.dt))
    assert np.max(np.abs(H - Ho)) <= TOL * max(1.0, np.max(np.abs(Ho)))
    U = pg.compute_propagators(H, cs.dt)
    Uo = rs.compute_propagators(Ho, cs.dt)
    assert np.max(np.abs(U - Uo)) <= 1e-12
    dts = rng.uniform(0.01, 0.05, n_t)                   # one dt per slice (MR pulse_dt)
    assert np.max(np.abs(pg.compute_propagators(H, dts) - rs.compute_propagators(Ho, dts))) <= 1e-12


def test_liouvillian_stack(pg):
    rng = np.random.default_rng(5)
    L = np.stack([rs.build_drift_liouvillian(_herm(rng, 2), [np.array([[0, 1], [0, 0]], complex)], [0.3])
                  for _ in range(4)])
    U = pg.compute_propagators(L, 0.2, generator="liouvillian")
    Uo = np.stack([rs.expm_general(0.2 * L[k]) for k in range(4)])
    assert np.max(np.abs(U - Uo)) <= 1e-12


@pytest.mark.parametrize("d", [3, 16, 64])
def test_chains(pg, d):
    rng = np.random.default_rng(10 + d)
    n = 7
    U = np.stack([_unitary(rng, d) for _ in range(n)])
    seed = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    P = pg.compute_forward_propagators(U)
    assert np.max(np.abs(P - rs.forward_propagators(U))) <= 1e-12
    assert np.max(np.abs(pg.compute_backward_propagators(U) - rs.backward_propagators(U))) <= 1e-12
    Qs = pg.compute_backward_propagators(U, seed)
    assert np.max(np.abs(Qs - rs.backward_propagators(U, seed))) <= 1e-12 * np.max(np.abs(seed))
    assert np.max(np.abs(pg.compute_total_propagator(U) - rs.compute_total_propagator(U))) <= 1e-12
    assert np.array_equal(pg.compute_total_propagator(U[:0]), np.eye(d))     # empty product


def test_fidelities_and_prefactors(pg):
    rng = np.random.default_rng(3)
    d = 5
    U, T = _unitary(rng, d), _unitary(rng, d)
    z = np.trace(T.conj().T @ U) / d
    assert abs(pg.gate_fidelity(U, T) - rs.gate_fidelity(U, T)) <= TOL
    assert abs(pg.gate_fidelity(U, T, type="real") - z.real) <= TOL
    assert abs(pg.gate_fidelity(U, T, type="average") - (d * abs(z) ** 2 + 1) / (d + 1)) <= TOL
    a = rng.standard_normal(d) + 1j * rng.standard_normal(d)
    b = rng.standard_normal(d) + 1j * rng.standard_normal(d)
    for t in ("real", "square", "modulus"):
        assert abs(pg.state_fidelity(a, b, type=t) - rs.state_fidelity(a, b, t)) <= TOL
    with pytest.raises(ValueError):
        pg.state_fidelity(a, b, type="dm_uhlmann")
    zc, inner = 0.3 + 0.4j, -0.2 + 0.7j
    for t in ("real", "square", "modulus"):
        assert pg.fidelity_grad_prefactor(zc, inner, 0.1, t) == rs.fidelity_grad_prefactor(zc, inner, 0.1, t)
    for t in ("real", "square"):
        assert pg.lindblad_grad_prefactor(zc, inner, 0.1, t) == rs.lindblad_grad_prefactor(zc, inner, 0.1, t)


def test_finite_differences_and_gradient_check(pg):
    rng = np.random.default_rng(8)
    d, n_c, n_t = 3, 2, 5
    Hd, Hc = _herm(rng, d), [_herm(rng, d) for _ in range(n_c)]
    u = rng.uniform(-1, 1, (n_c, n_t))
    T = _unitary(rng, d)
    sys_g = pg.quantum_system(Hd, Hc)
    cs = pg.ControlSequence.from_controls(u, 0.1)
    G = pg.finite_difference_gradient(sys_g, cs, pg.unitary_target(T))
    Go = rs.finite_difference_gradient(rs.QuantumSystem(Hd, Hc), rs.ControlSequence.from_controls(u, 0.1),
                                       rs.unitary_target(T))
    assert np.max(np.abs(G - Go)) <= 1e-8
    chk = pg.grape_gradient_check(sys_g, pg.unitary_target(T), cs)
    assert set(chk) >= {"analytical_gradient", "numerical_gradient", "max_error", "max_relative_error", "passed"}
    assert np.max(np.abs(chk["numerical_gradient"] - Go)) <= 1e-6


def test_cuda_backend_entry_points(pg):
    rng = np.random.default_rng(21)
    d, n_c, n_t, dt = 4, 2, 6, 0.07
    be = pg.cuda_backend()
    Hd, Hc = _herm(rng, d), [_herm(rng, d) for _ in range(n_c)]
    u = rng.uniform(-1, 1, (n_c, n_t))
    T = _unitary(rng, d)
    assert np.max(np.abs(pg.matrix_exponential_cuda(Hd, dt, be) - rs.expm_neg_i(Hd, dt))) <= 1e-12
    Harr = np.stack([_herm(rng, d) for _ in range(3)], axis=2)           # (dim, dim, n_steps)
    Ub = pg.batch_propagators_cuda(Harr, dt, be)
    for k in range(3):
        assert np.max(np.abs(Ub[:, :, k] - rs.expm_neg_i(Harr[:, :, k], dt))) <= 1e-12
    U = _unitary(rng, d)
    assert abs(pg.fidelity_cuda(U, T, be) - abs(np.trace(T.conj().T @ U)) ** 2 / d ** 2) <= TOL
    G = pg.gradient_cuda(Hd, Hc, u, T, dt, be)
    Go = rs.gradient_cuda_formula(Hd, Hc, u, T, dt)
    assert np.max(np.abs(G - Go)) <= 1e-12 * max(1.0, np.max(np.abs(Go)))


def test_ensemble_value_functions_and_mr_builder(pg):
    rng = np.random.default_rng(4)
    d, n_t = 2, 8
    SX = np.array([[0, 1], [1, 0]], complex)
    SY = np.array([[0, -1j], [1j, 0]], complex)
    SZ = np.diag([1.0, -1.0]).astype(complex)
    ctrl = pg.MRControl(drifts=[0.5 * o * SZ for o in (-0.2, 0.0, 0.3)], operators=[0.5 * SX, 0.5 * SY],
                        rho_init=[np.array([1, 0], complex)], rho_targ=[np.array([0, 1], complex)],
                        pwr_levels=[0.9, 1.0, 1.1], pulse_dt=np.full(n_t, 0.2))
    obj = pg.build_ensemble_from_mrcontrol(ctrl)
    assert obj.n_samples == 9
    w = rng.uniform(-1, 1, (2, n_t))
    theta = w.reshape(-1, order="F")
    F, G = pg.grape_state_kernel(w, ctrl)
    assert pg.ensemble_value(obj, theta) == F
    Fv, g = pg.ensemble_value_and_grad(obj, theta)
    assert Fv == F and np.array_equal(g, G.reshape(-1, order="F"))
    with pytest.raises(ValueError):
        pg.build_ensemble_from_mrcontrol(ctrl, aggregator="median")


@pytest.mark.parametrize("ptype", ["NS", "SNS", "SNSA", "DNS", "energy"])
def test_penalty_value_and_gradient(pg, ptype):
    rng = np.random.default_rng(40)
    w = rng.uniform(-1.6, 1.6, (3, 11))
    dt = rng.uniform(0.5, 1.5, 11)
    P, G = pg.penalty_value_and_gradient(w, ptype, weight=0.3, l_bound=-0.8, u_bound=0.9, dt=dt)
    Po, Go = rs.penalty_value_and_gradient(w, ptype, 0.3, -0.8, 0.9, dt)
    assert abs(P - Po) <= 1e-12 * max(1.0, abs(Po))
    assert np.max(np.abs(G - Go)) <= 1e-12
    assert pg.penalty_value(w, ptype, 0.0) == 0.0


def test_penalties_fused_into_the_evaluation(pg):
    """MR kernels subtract the penalties (GRAPEState.jl:571-584)."""
    from oracle import members as mb
    import fx
    spec_prob, u0 = fx.spin4_ensemble(n_t=10, n_off=2, n_b1=1)
    pens = [("NS", 1e-9), ("DNS", 2e-9), ("SNS", 1e-8, -5e3, 5e3)]
    for precision, ftol, gtol in (("fp64", 1e-10, 1e-8), ("mixed", 1e-8, 1e-4)):
        di, sc, of, wgt = spec_prob.members()
        p = pg.Problem(spec_prob.drifts, spec_prob.controls, spec_prob.dt, offset_op=spec_prob.offset_op,
                       member_drift=di, member_scale=sc, member_offset=of, member_weight=wgt, target="gate",
                       target_op=spec_prob.target_op, grad_mode="exact", precision=precision)
        p.set_penalties(pens)
        F, G = p.eval(u0)
        p.close()
        Fo, Go = mb.eval_problem(spec_prob, u0, "exact")
        for pen in pens:
            lo, hi = (pen[2], pen[3]) if len(pen) > 2 else (-1.0, 1.0)
            Pv, Pg = rs.penalty_value_and_gradient(u0, pen[0], pen[1], lo, hi)
            Fo -= Pv
            Go = Go - Pg
        assert abs(F - Fo) <= ftol, (precision, F, Fo)
        assert np.max(np.abs(G - Go)) <= gtol * np.max(np.abs(Go)), precision


@pytest.mark.parametrize("aggregator", ["mean", "worst_case", "cvar"])
def test_ensemble_aggregators(pg, aggregator):
    """:mean / :worst_case / :cvar over per-system samples (EnsembleObjective.jl:169-217)."""
    rng = np.random.default_rng(12)
    SX = np.array([[0, 1], [1, 0]], complex)
    SY = np.array([[0, -1j], [1j, 0]], complex)
    SZ = np.diag([1.0, -1.0]).astype(complex)
    systems_o = [rs.QuantumSystem(0.5 * d * SZ, [0.5 * SX, 0.5 * SY]) for d in (-0.3, -0.1, 0.0, 0.15, 0.4)]
    systems_g = [pg.quantum_system(s.H_drift, s.H_controls) for s in systems_o]
    u = 0.3 * rng.standard_normal((2, 14))
    T = np.array([[0, 1], [1, 0]], complex)
    cs_o = rs.ControlSequence.from_controls(u, 0.1)
    Fi = np.array([rs.compute_fidelity(s, cs_o, rs.unitary_target(T)) for s in systems_o])
    Gi = [rs.compute_grape_gradient(s, cs_o, rs.unitary_target(T)) for s in systems_o]
    Fo, Go = rs.aggregate(Fi, Gi, aggregator, 0.4)
    obj = pg.build_ensemble_from_systems(systems_g, pg.unitary_target(T), pg.ControlSequence.from_controls(u, 0.1),
                                         aggregator=aggregator, cvar_alpha=0.4)
    theta = u.reshape(-1, order="F")
    F, g = obj.value_and_grad(theta)
    assert abs(F - Fo) <= 1e-12
    assert np.max(np.abs(g - Go.reshape(-1, order="F"))) <= 1e-10 * max(1.0, np.max(np.abs(Go)))
    assert abs(obj.value(theta) - Fo) <= 1e-12


@pytest.mark.parametrize("aggregator", ["mean", "worst_case", "cvar"])
def test_parametric_perturbation_ensemble(pg, aggregator):
    """build_ensemble_from_perturbations(:parametric) against the oracle on
    the same perturbations: per-sample exact F and G, then the aggregator."""
    from oracle import members as mb
    rng = np.random.default_rng(31)
    d, n_c, n_t = 3, 2, 9
    Hd, Hc = _herm(rng, d), [_herm(rng, d) for _ in range(n_c)]
    T = _unitary(rng, d)
    sys_g = pg.quantum_system(Hd, Hc)
    u = rng.uniform(-1, 1, (n_c, n_t))
    cs = pg.ControlSequence.from_controls(u, 0.1)
    obj = pg.build_ensemble_from_perturbations(sys_g, pg.unitary_target(T), cs, magnitude=0.1, n_samples=6,
                                               aggregator=aggregator, cvar_alpha=0.34, resample=False, seed=5)
    pert = pg.sample_parametric_perturbations(sys_g, 6, 0.1, np.random.default_rng(5))
    Fi, Gi = [], []
    for dH in pert:
        prob = mb.Problem(drifts=(Hd + dH)[None], controls=np.stack(Hc), dt=np.full(n_t, 0.1), target="gate",
                          fidelity="square", target_op=T)
        F1, G1 = mb.eval_problem(prob, u, "exact")
        Fi.append(F1)
        Gi.append(G1)
    Fo, Go = rs.aggregate(Fi, Gi, aggregator, 0.34)
    theta = u.reshape(-1, order="F")
    F, g = obj.value_and_grad(theta)
    assert abs(F - Fo) <= 1e-12
    assert np.max(np.abs(g - Go.reshape(-1, order="F"))) <= 1e-9 * max(1.0, np.max(np.abs(Go)))
    # resampling redraws (seed + call count): a different objective, same shape
    obj2 = pg.build_ensemble_from_perturbations(sys_g, pg.unitary_target(T), cs, magnitude=0.1, n_samples=6,
                                                aggregator=aggregator, resample=True, seed=5)
    F2, g2 = obj2.value_and_grad(theta)
    assert F2 != F and g2.shape == g.shape


@pytest.mark.parametrize("aggregator", ["mean", "worst_case", "cvar"])
def test_drift_trajectory_ensemble(pg, aggregator):
    """build_ensemble_from_perturbations(:drift): sample i evolves under
    H_drift + tau_k dH_i (sample_drift_trajectories' linear ramp,
    RobustOpt.jl:168-182).  Per-sample F against the reference's
    _fidelity_with_perturbation on the trajectory (RobustOpt.jl:739-761) and
    (F, exact G) against the oracle's member model, then the aggregator."""
    from oracle import members as mb
    rng = np.random.default_rng(41)
    d, n_c, n_t, dt = 3, 2, 11, 0.1
    Hd, Hc = _herm(rng, d), [_herm(rng, d) for _ in range(n_c)]
    T = _unitary(rng, d)
    sys_g = pg.quantum_system(Hd, Hc)
    u = rng.uniform(-1, 1, (n_c, n_t))
    cs = pg.ControlSequence.from_controls(u, dt)
    obj = pg.build_ensemble_from_perturbations(sys_g, pg.unitary_target(T), cs, uncertainty_type="drift",
                                               magnitude=0.3, n_samples=5, aggregator=aggregator, cvar_alpha=0.4,
                                               resample=False, seed=7)
    finals = pg.sample_parametric_perturbations(sys_g, 5, 0.3, np.random.default_rng(7))
    trajs = pg.sample_drift_trajectories(sys_g, 5, 0.3, n_t, np.random.default_rng(7))
    tau = pg.drift_ramp_schedule(n_t)
    Fi, Gi = [], []
    for dH, traj in zip(finals, trajs):
        prob = mb.Problem(drifts=Hd[None], controls=np.stack(Hc), dt=np.full(n_t, dt), target="gate",
                          fidelity="square", target_op=T, ramp_ops=dH[None], member_ramp=np.zeros(1, int), tau=tau)
        F1, G1 = mb.eval_problem(prob, u, "exact")
        assert abs(F1 - rs.fidelity_with_perturbation(Hd, Hc, u, dt, T, traj)) <= 1e-12
        Fi.append(F1)
        Gi.append(G1)
    Fo, Go = rs.aggregate(Fi, Gi, aggregator, 0.4)
    theta = u.reshape(-1, order="F")
    F, g = obj.value_and_grad(theta)
    assert abs(F - Fo) <= 1e-12
    assert np.max(np.abs(g - Go.reshape(-1, order="F"))) <= 1e-9 * max(1.0, np.max(np.abs(Go)))
    obj2 = pg.build_ensemble_from_perturbations(sys_g, pg.unitary_target(T), cs, uncertainty_type="drift",
                                                magnitude=0.3, n_samples=5, aggregator=aggregator, seed=7)
    F2, _ = obj2.value_and_grad(theta)       # resampled (seed + 1) before the evaluation
    assert F2 != F


def test_drift_ramp_mixed_and_validation(pg, ctx):
    """The ramp in the df32 / FP32 generator assembly (mixed precision), on a
    d = 16 ensemble, against the oracle; and the setter's validation."""
    from oracle import members as mb
    spec, u0 = fx.W.spin4_ensemble(n_t=12, n_off=3, n_b1=2)
    rng = np.random.default_rng(3)
    ops = np.stack([_herm(rng, 16) * 2e3 for _ in range(2)])
    mo = np.array([0, 1, -1, 0, 1, -1])
    tau = np.linspace(0.0, 1.0, 12)
    prob = mb.Problem.from_spec(spec)
    prob.ramp_ops, prob.member_ramp, prob.tau = ops, mo, tau
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    for precision, ftol, gtol in (("fp64", 1e-10, 1e-8), ("mixed", 1e-8, 1e-4)):
        p = pg.Problem(ctx=ctx, **spec.problem_kwargs("exact", precision))
        p.set_drift_ramp(ops, mo, tau)
        F, G = p.eval(u0)
        assert abs(F - Fo) <= ftol, (precision, F, Fo)
        assert np.max(np.abs(G - Go)) <= gtol * np.max(np.abs(Go)), precision
        p.set_drift_ramp([], [], [])                # removed: the plain problem again
        F0, _ = p.eval(u0)
        assert abs(F0 - mb.eval_problem(mb.Problem.from_spec(spec), u0, "exact")[0]) <= ftol
        E = pg._abi.PgxError
        with pytest.raises(E) as e:
            p.set_drift_ramp(ops, [0, 1, 2, 0, 1, 0], tau)      # index beyond the operators
        assert e.value.status == 1
        with pytest.raises(E) as e:
            p.set_drift_ramp(ops + 1j * np.eye(16), mo, tau)     # not Hermitian
        assert e.value.status == 1
        p.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ensemble_aggregators_reference_samples(pg, precision):
    """EnsembleTests.jl:33-62 on the device: four qubits whose gate fidelities
    to the identity are the reference test's samples 0.9, 0.8, 0.7, 0.6 (an x
    rotation by theta has F = cos^2(theta / 2)), aggregated by :mean,
    :worst_case and :cvar with alpha = 0.5."""
    samples = np.array([0.9, 0.8, 0.7, 0.6])
    theta = 2 * np.arccos(np.sqrt(samples))
    sx = np.array([[0, 1], [1, 0]], complex)
    systems = [pg.quantum_system(np.zeros((2, 2), complex), [t * sx / 2]) for t in theta]
    cs = pg.ControlSequence(np.ones((1, 1)), 1.0)
    tgt = pg.unitary_target(np.eye(2, dtype=complex))
    got = {}
    for agg in ("mean", "worst_case", "cvar"):
        obj = pg.build_ensemble_from_systems(systems, tgt, cs, aggregator=agg, precision=precision, cvar_alpha=0.5)
        got[agg] = obj.value(np.ones(1))
    assert abs(got["mean"] - samples.mean()) < 1e-12
    assert abs(got["worst_case"] - 0.6) < 1e-12
    assert abs(got["cvar"] - (0.6 + 0.7) / 2) < 1e-12
    assert got["worst_case"] <= got["cvar"] <= got["mean"] + 1e-12
