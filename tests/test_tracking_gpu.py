"""Trajectory-tracking and phase-only MR kernels on the device
(pgx_problem_set_tracking, pgx_eval_phase) against the oracle's restatement
of GRAPETracking.jl / GRAPEPhase.jl: the checkpoint objective, the
reference's co-state gradient (PGX_GRAD_REF_MR), the exact gradient against
finite differences of the oracle objective, the phase chain rule, and
optimcon with tracking against the oracle's MR loops on the tracking kernel."""
import numpy as np
import pytest

from oracle import ref_semantics as rs

pytestmark = pytest.mark.gpu

SX = np.array([[0, 1], [1, 0]], complex)
SY = np.array([[0, -1j], [1j, 0]], complex)
SZ = np.diag([1.0, -1.0]).astype(complex)
I2 = np.eye(2, dtype=complex)


def _proj(v):
    v = np.asarray(v, complex)
    return np.outer(v, v.conj())


def _one_spin(n_t=40, dt=1e-5):
    up, dn = np.array([1, 0], complex), np.array([0, 1], complex)
    kw = dict(drifts=[2 * np.pi * off * SZ / 2 for off in (-300.0, 0.0, 450.0)], operators=[SX / 2, SY / 2],
              rho_init=[up, (up + 1j * dn) / np.sqrt(2)], rho_targ=[dn, dn],
              pwr_levels=[2 * np.pi * 0.9e3, 2 * np.pi * 1.1e3], pulse_dt=np.full(n_t, dt))
    mixed = 0.7 * _proj(dn) + 0.3 * _proj(up)
    track = [(8, _proj(dn), 0.2), (8, mixed, 0.1), (21, _proj(up), 0.3), (n_t, _proj(dn), 0.4)]
    return kw, track


def _two_spins(n_t=30):
    Ix = [np.kron(SX / 2, I2), np.kron(I2, SX / 2)]
    Iy = [np.kron(SY / 2, I2), np.kron(I2, SY / 2)]
    Iz = [np.kron(SZ / 2, I2), np.kron(I2, SZ / 2)]
    J = 2 * np.pi * 40.0 * (Ix[0] @ Ix[1] + Iy[0] @ Iy[1] + Iz[0] @ Iz[1])
    drifts = [2 * np.pi * (150 * Iz[0] - 220 * Iz[1]) + J, 2 * np.pi * (-80 * Iz[0] + 60 * Iz[1]) + J]
    e = np.eye(4, dtype=complex)
    kw = dict(drifts=drifts, operators=[Ix[0] + Ix[1], Iy[0] + Iy[1]], rho_init=[e[0], e[1]], rho_targ=[e[3], e[2]],
              pwr_levels=[2 * np.pi * 1e3], pulse_dt=np.full(n_t, 2e-5))
    rng = np.random.default_rng(4)
    A = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    rho = A @ A.conj().T
    track = [(10, _proj(e[3]), 0.5), (n_t, rho / np.trace(rho).real, 0.5)]
    return kw, track


def _pair(kw, track, grad_mode):
    import pulsar_gb300 as pg
    ctrl = pg.MRControl(**kw, grad_mode=grad_mode, tracking=[pg.TrackingPoint(s, t, w) for s, t, w in track])
    octrl = rs.MRControl(**kw)
    otrack = [rs.TrackingPoint(s, t, w) for s, t, w in track]
    return ctrl, octrl, otrack


@pytest.mark.parametrize("case", [_one_spin, _two_spins])
def test_tracking_matches_the_reference_formula(pg, case):
    kw, track = case()
    ctrl, octrl, otrack = _pair(kw, track, "ref_mr")
    n_t = len(kw["pulse_dt"])
    w = np.random.default_rng(7).uniform(-1, 1, (2, n_t))
    F, G = pg.grape_tracking_kernel(w, ctrl)
    Fo, Go = rs.grape_tracking_kernel(w, octrl, otrack)
    assert abs(F - Fo) <= 1e-10, (F, Fo)
    assert np.max(np.abs(G - Go)) <= 1e-8 * np.max(np.abs(Go)), np.max(np.abs(G - Go))
    # grape_state_kernel on the same ctrl keeps the terminal objective
    Fs, _ = pg.grape_state_kernel(w, ctrl)
    assert abs(Fs - rs.grape_state_kernel(w, octrl)[0]) <= 1e-10


@pytest.mark.parametrize("case", [_one_spin, _two_spins])
def test_tracking_exact_gradient_vs_finite_differences(pg, case):
    kw, track = case()
    ctrl, octrl, otrack = _pair(kw, track, "exact")
    n_t = len(kw["pulse_dt"])
    w = np.random.default_rng(8).uniform(-1, 1, (2, n_t))
    F, G = pg.grape_tracking_kernel(w, ctrl)
    assert abs(F - rs.grape_tracking_kernel(w, octrl, otrack)[0]) <= 1e-10
    eps = 1e-6
    Gfd = np.zeros_like(w)
    for idx in np.ndindex(*w.shape):
        wp, wm = w.copy(), w.copy()
        wp[idx] += eps
        wm[idx] -= eps
        Gfd[idx] = (rs.grape_tracking_kernel(wp, octrl, otrack)[0] -
                    rs.grape_tracking_kernel(wm, octrl, otrack)[0]) / (2 * eps)
    assert np.max(np.abs(G - Gfd)) <= 1e-6 * np.max(np.abs(Gfd)), np.max(np.abs(G - Gfd))


def test_tracking_residual_and_validation(pg, ctx):
    kw, track = _one_spin()
    ctrl, _, _ = _pair(kw, track, "ref_mr")
    prob = ctrl.problem(tracking=True)
    w = np.zeros((2, len(kw["pulse_dt"])))
    _, _, st = prob.eval(w, want_grad=False, stats=True)
    assert st["residual_kind"] == "norm" and st["residual"] <= 1e-13
    E = pg._abi.PgxError
    with pytest.raises(E) as e:                       # GRAPETracking.jl:190-191
        prob.set_tracking([0], [1.0], [np.eye(2)])
    assert e.value.status == 1
    with pytest.raises(E) as e:
        prob.set_tracking([len(kw["pulse_dt"]) + 1], [1.0], [np.eye(2)])
    assert e.value.status == 1
    with pytest.raises(E) as e:                       # not a density matrix
        prob.set_tracking([3], [1.0], [np.array([[0, 1], [0, 0]], complex)])
    assert e.value.status == 1
    p2 = pg.Problem(np.stack(kw["drifts"]), np.stack(kw["operators"]), kw["pulse_dt"], ctx=ctx,
                    target="gate", target_op=SX, member_drift=[0, 1, 2])
    with pytest.raises(E) as e:                       # tracking is a state-target objective
        p2.set_tracking([3], [1.0], [np.eye(2)])
    assert e.value.status == 6
    p2.close()
    plain = pg.MRControl(**kw)
    with pytest.raises(RuntimeError):
        pg.grape_tracking_kernel(w, plain)
    # clearing the checkpoints restores the terminal objective
    prob.set_tracking([], [], [])
    assert abs(prob.eval(w, want_grad=False)[0] - ctrl.problem().eval(w, want_grad=False)[0]) == 0.0


@pytest.mark.parametrize("method", ["lbfgs", "grape"])
def test_optimcon_tracking_follows_the_reference_loops(pg, method):
    """_optimcon_lbfgs_tracking / _optimcon_grape_tracking (OptControl.jl:1040-1236):
    the MR loops on the tracking kernel."""
    kw, track = _one_spin(n_t=30)
    ctrl, octrl, otrack = _pair(kw, track, "ref_mr")
    ctrl.method, ctrl.max_iter = method, 12
    w0 = 0.3 * np.random.default_rng(3).standard_normal((2, 30))
    kern = lambda w: rs.grape_tracking_kernel(w, octrl, otrack)
    ref = (rs.optimcon_lbfgs(kern, w0, max_iter=12) if method == "lbfgs" else rs.optimcon_grape(kern, w0, max_iter=12))
    r = pg.optimcon(ctrl, w0)
    assert r.n_iterations == ref.n_iterations
    assert np.allclose(r.fidelity_history, ref.fidelity_history, rtol=0, atol=1e-9)
    assert abs(r.fidelity - ref.fidelity) <= 1e-9
    assert r.fidelity > r.fidelity_history[0]


def test_phase_kernel_matches_the_oracle(pg):
    up, dn = np.array([1, 0], complex), np.array([0, 1], complex)
    kw = dict(drifts=[2 * np.pi * off * SZ / 2 for off in (-200.0, 250.0)], operators=[SX / 2, SY / 2],
              rho_init=[up], rho_targ=[dn], pwr_levels=[2 * np.pi * 1e3, 2 * np.pi * 1.2e3],
              pulse_dt=np.full(25, 2e-5), fidelity="square")
    ctrl, octrl = pg.MRControl(**kw, grad_mode="ref_mr"), rs.MRControl(**kw)
    rng = np.random.default_rng(5)
    phi, amp = rng.uniform(-np.pi, np.pi, (1, 25)), rng.uniform(0.3, 1.0, (1, 25))
    for a in (None, amp):
        F, Gp = pg.grape_phase_kernel(phi, ctrl, a)
        Fo, Gpo = rs.grape_phase_kernel(phi, octrl, a)
        assert abs(F - Fo) <= 1e-10
        assert np.max(np.abs(Gp - Gpo)) <= 1e-8 * np.max(np.abs(Gpo))
    with pytest.raises(ValueError):
        pg.grape_phase_kernel(np.zeros((2, 25)), ctrl)
    with pytest.raises(ValueError):
        pg.grape_phase_kernel(phi, ctrl, -amp)
