"""GPU parity: libpulsar_gb300.so against the FP64 oracle, through the C ABI.

Tolerances (FP64 path): |dF| <= 1e-10 and max|dG| / max|G_oracle| <= 1e-8.
The oracle's propagators come from Hermitian eigendecompositions (as the
reference) or scipy's Pade expm (Liouvillians); the GPU uses scaling-and-
squaring Taylor -- the difference is method rounding, ~1e-15 per slice.
"""
import numpy as np
import pytest

from oracle import members as mb
import fx

pytestmark = pytest.mark.gpu

F_TOL = 1e-10
G_RTOL = 1e-8


def to_gpu(pg, prob: mb.Problem, grad_mode: str, precision: str = "fp64", **extra):
    di, sc, of, w = prob.members()
    kw = dict(generator=prob.generator, member_drift=di, member_scale=sc, member_offset=of,
              member_weight=w, offset_op=prob.offset_op, target=prob.target, fidelity=prob.fidelity,
              grad_mode=grad_mode, precision=precision)
    if prob.target == "gate":
        kw["target_op"] = prob.target_op
    else:
        kw["states_init"] = prob.states_init
        kw["states_target"] = prob.states_target
    kw.update(extra)
    return pg.Problem(prob.drifts, prob.controls, prob.dt, **kw)


def assert_parity(F, G, Fo, Go, ftol=F_TOL, grtol=G_RTOL):
    assert abs(F - Fo) <= ftol, (F, Fo, abs(F - Fo))
    scale = max(np.max(np.abs(Go)), 1e-300)
    err = np.max(np.abs(G - Go)) / scale
    assert err <= grtol, err


def rand_herm(rng, d, s=1.0):
    A = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    return s * (A + A.conj().T) / 2


def random_gate_problem(rng, d, n_t, n_c=2, n_members=1, dt=0.05, scale=1.0):
    drifts = np.stack([rand_herm(rng, d, scale) for _ in range(n_members)])
    ctrls = np.stack([rand_herm(rng, d, scale) for _ in range(n_c)])
    prob = mb.Problem(drifts=drifts, controls=ctrls, dt=np.full(n_t, dt), member_drift=np.arange(n_members),
                      member_scale=rng.uniform(0.9, 1.1, n_members), n_members=n_members, target="gate",
                      target_op=fx.haar_unitary(rng, d))
    return prob, rng.uniform(-1, 1, (n_c, n_t))


MODES = ("ref_grape", "ref_mr", "exact")


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("explicit", [False, True])
def test_single_qubit_transfer(pg, mode, explicit):
    prob, u0 = fx.single_qubit_transfer(explicit_init=explicit)
    p = to_gpu(pg, prob, mode)
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    assert_parity(F, G, Fo, Go)
    p.close()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("d", [2, 3, 4, 5, 8, 12, 16, 20, 32])
def test_random_gate(pg, mode, d):
    rng = np.random.default_rng(100 + d)
    prob, u0 = random_gate_problem(rng, d, n_t=6, n_members=2, dt=0.3 / np.sqrt(d))
    p = to_gpu(pg, prob, mode)
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    assert_parity(F, G, Fo, Go)
    p.close()


@pytest.mark.parametrize("mode", MODES)
def test_large_norm_needs_squaring(pg, mode):
    rng = np.random.default_rng(5)
    prob, u0 = random_gate_problem(rng, 8, n_t=5, dt=0.9, scale=3.0)   # ||A||_1 >> 1
    p = to_gpu(pg, prob, mode)
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    assert_parity(F, G, Fo, Go, grtol=1e-8)
    p.close()


@pytest.mark.parametrize("mode", MODES)
def test_spin4_broadband_ensemble_small(pg, mode):
    prob, u0 = fx.spin4_ensemble(n_t=10, n_off=3, n_b1=2)
    p = to_gpu(pg, prob, mode)
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    assert_parity(F, G, Fo, Go)
    p.close()


@pytest.mark.parametrize("fid", ["square", "real", "modulus"])
@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("d", [2, 3, 6])
def test_state_pairs_mr(pg, fid, mode, d):
    rng = np.random.default_rng(7 * d)
    drifts = np.stack([rand_herm(rng, d, 0.5) for _ in range(3)])
    ctrls = np.stack([rand_herm(rng, d, 0.5) for _ in range(2)])
    si = np.stack([fx.haar_unitary(rng, d)[:, 0] for _ in range(2)])
    st = np.stack([fx.haar_unitary(rng, d)[:, 0] for _ in range(2)])
    prob = mb.Problem(drifts=drifts, controls=ctrls, dt=rng.uniform(0.05, 0.2, 9),
                      member_drift=np.repeat(np.arange(3), 2), member_scale=np.tile([0.8, 1.3], 3),
                      n_members=6, target="states", fidelity=fid, states_init=si, states_target=st)
    u0 = rng.uniform(-1, 1, (2, 9))
    p = to_gpu(pg, prob, mode)
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    assert_parity(F, G, Fo, Go)
    p.close()


@pytest.mark.parametrize("mode", MODES)
def test_lindblad_gate_superoperator(pg, mode):
    prob, u0 = fx.lindblad_3q(n_t=3, n_draws=2)
    p = to_gpu(pg, prob, mode)
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    assert_parity(F, G, Fo, Go)
    p.close()


@pytest.mark.parametrize("mode", MODES)
def test_lindblad_states_mr(pg, mode):
    from oracle import ref_semantics as rs
    rng = np.random.default_rng(9)
    SZ = np.diag([1.0, -1.0]).astype(complex)
    SX = np.array([[0, 1], [1, 0]], complex)
    SY = np.array([[0, -1j], [1j, 0]], complex)
    sm = np.array([[0, 1], [0, 0]], complex)
    Ls = np.stack([rs.build_drift_liouvillian(2 * np.pi * o * SZ / 2, [sm, SZ], [40.0, 15.0])
                   for o in (-500.0, 0.0, 500.0)])
    Lc = np.stack([rs.build_control_liouvillian(SX / 2), rs.build_control_liouvillian(SY / 2)])
    prob = mb.Problem(drifts=Ls, controls=Lc, dt=np.full(15, 1e-5), generator="liouvillian",
                      member_drift=np.arange(3), member_scale=np.full(3, 2 * np.pi * 1e4), n_members=3,
                      target="states", fidelity="square",
                      states_init=rs.pure_state_to_vec_rho([1, 0])[None],
                      states_target=rs.pure_state_to_vec_rho([0, 1])[None])
    u0 = rng.uniform(-1, 1, (2, 15))
    p = to_gpu(pg, prob, mode)
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    assert_parity(F, G, Fo, Go)
    p.close()


def test_forward_only_matches(pg):
    prob, u0 = fx.spin4_ensemble(n_t=7, n_off=2, n_b1=2)
    p = to_gpu(pg, prob, "exact")
    F1, _ = p.eval(u0, want_grad=False)
    F2, _ = p.eval(u0)
    assert F1 == F2
    p.close()


@pytest.mark.parametrize("d", [2, 4, 7, 16, 32, 64])
def test_single_propagator(pg, ctx, d):
    from oracle import ref_semantics as rs
    rng = np.random.default_rng(d)
    H = rand_herm(rng, d)
    for dt in (1e-3, 0.1, 2.0):
        U = ctx.propagator(H, dt)
        assert np.max(np.abs(U - rs.expm_neg_i(H, dt))) < 1e-12 * max(1.0, dt * np.abs(H).sum(0).max())


def test_propagator_kats(pg):
    SZ = np.diag([1.0, -1.0]).astype(complex)
    U = pg.compute_propagator(np.pi * SZ, 1.0)
    assert abs(U[0, 0] - np.exp(-1j * np.pi)) < 1e-10 and abs(U[1, 1] - np.exp(1j * np.pi)) < 1e-10
    assert abs(U[0, 1]) < 1e-10 and abs(U[1, 0]) < 1e-10
    assert np.linalg.norm(pg.compute_propagator(np.zeros((2, 2)), 1e-6) - np.eye(2)) < 1e-12
    with pytest.raises(ValueError):
        pg.compute_propagator(np.array([[0, 1], [0, 0]], complex), 1.0)


def test_total_propagator(pg):
    from oracle import ref_semantics as rs
    prob, u0 = fx.spin4_ensemble(n_t=9, n_off=2, n_b1=1)
    p = to_gpu(pg, prob, "exact")
    for m in range(2):
        Gs = np.stack([prob.generator_of(m, u0[:, k]) for k in range(9)])
        Uo = rs.compute_total_propagator(rs.compute_propagators(Gs, prob.dt))
        assert np.max(np.abs(p.total_propagator(u0, m) - Uo)) < 1e-12
    p.close()


def test_deterministic_and_member_independent(pg):
    prob, u0 = fx.spin4_ensemble(n_t=20, n_off=3, n_b1=3)
    p = to_gpu(pg, prob, "exact")
    F1, G1 = p.eval(u0)
    Fm1 = p.member_fidelities()
    F2, G2 = p.eval(u0)
    assert F1 == F2 and np.array_equal(G1, G2)
    # a member alone gives bit-identical per-member results
    sub = mb.Problem(drifts=prob.drifts, controls=prob.controls, dt=prob.dt, offset_op=prob.offset_op,
                     member_offset=prob.member_offset[4:5], member_scale=prob.member_scale[4:5],
                     n_members=1, target="gate", target_op=prob.target_op)
    q = to_gpu(pg, sub, "exact")
    q.eval(u0)
    assert q.member_fidelities()[0] == Fm1[4]
    p.close()
    q.close()


def test_validation_errors(pg):
    E = pg._abi.PgxError
    H = np.array([[0, 1], [0, 0]], complex)     # not Hermitian
    with pytest.raises(E):
        pg.Problem(H, np.eye(2)[None], [0.1], target="gate", target_op=np.eye(2))
    with pytest.raises(E):                       # not unitary
        pg.Problem(np.eye(2), np.eye(2)[None], [0.1], target="gate", target_op=2 * np.eye(2))
    p = pg.Problem(np.eye(2), np.diag([1.0, -1])[None], [0.1, 0.1], target="gate", target_op=np.eye(2))
    with pytest.raises(E):
        p.eval(np.array([[np.nan, 0.0]]))
    with pytest.raises(ValueError):
        p.eval(np.zeros((2, 2)))
    p.close()
    small = pg.Context(0, hbm_budget=64 * 1024)   # a 1000-slice stack needs more
    with pytest.raises(E) as ei:
        pg.Problem(np.eye(2), np.eye(2)[None], np.full(1000, 0.1), target="gate", target_op=np.eye(2),
                   ctx=small)
    assert ei.value.status == 4
    assert small.hbm_used() == 0
    ok = pg.Problem(np.eye(2), np.eye(2)[None], [0.1], target="gate", target_op=np.eye(2), ctx=small)
    assert 0 < small.hbm_used() <= 64 * 1024
    ok.close()
    assert small.hbm_used() == 0
    small.close()


def test_spin4_full_size_vs_c_oracle(pg):
    """The bench workload at full size (231 members x 1000 slices, d = 16,
    exact gradient) against the oracle's C restatement."""
    from oracle import cpu_port
    prob, u0 = fx.spin4_ensemble()
    p = to_gpu(pg, prob, "exact")
    F, G = p.eval(u0)
    Fo, Go = cpu_port.CpuProblem(prob, "exact").eval(u0)
    assert_parity(F, G, Fo, Go)
    assert 0.0 <= F <= 1.0
    p.close()
