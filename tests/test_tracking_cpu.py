"""The oracle's restatement of trajectory-tracking GRAPE (GRAPETracking.jl)
and of the phase-only wrapper (GRAPEPhase.jl), pinned by what the reference
documents and tests for them: fidelity in [0, 1] for pure targets with
weights summing to one, the co-state gradient against finite differences
(first-order formula at the reference's 1e-2 bar; the reference's co-state
carries 2 w_c, so its gradient is twice the derivative), the state-vector
form of the density-matrix recursion, and the polar chain rule."""
import numpy as np
import pytest

from oracle import ref_semantics as rs

SX = np.array([[0, 1], [1, 0]], complex)
SY = np.array([[0, -1j], [1j, 0]], complex)
SZ = np.diag([1.0, -1.0]).astype(complex)
UP, DN = np.array([1, 0], complex), np.array([0, 1], complex)


def _ctrl(n_t=20):
    return rs.MRControl(drifts=[2 * np.pi * 100 * SZ / 2, -2 * np.pi * 50 * SZ / 2], operators=[SX / 2, SY / 2],
                        rho_init=[UP, (UP + DN) / np.sqrt(2)], rho_targ=[DN, DN],
                        pwr_levels=[2 * np.pi * 1e3, 2 * np.pi * 1.1e3], pulse_dt=np.full(n_t, 2e-5))


def _track():
    p = lambda v: np.outer(v, v.conj())
    return [rs.TrackingPoint(5, p(DN), 0.25), rs.TrackingPoint(12, p(UP), 0.25), rs.TrackingPoint(12, p(DN), 0.1),
            rs.TrackingPoint(20, p(DN), 0.4)]


def _fd(fun, w, eps=1e-6):
    g = np.zeros_like(w)
    for idx in np.ndindex(*w.shape):
        wp, wm = w.copy(), w.copy()
        wp[idx] += eps
        wm[idx] -= eps
        g[idx] = (fun(wp) - fun(wm)) / (2 * eps)
    return g


def test_tracking_fidelity_is_a_weighted_checkpoint_overlap():
    ctrl, tr = _ctrl(), _track()
    w = np.random.default_rng(0).uniform(-1, 1, (2, 20))
    F, _ = rs.grape_tracking_kernel(w, ctrl, tr)
    assert 0.0 <= F <= 1.0
    # the same objective from state vectors: rho[n] = psi[n] psi[n]'
    tot, n_ens = 0.0, 0
    for H_d in ctrl.drifts:
        for pwr in ctrl.pwr_levels:
            Us = [rs.expm_neg_i(H_d + pwr * (w[0, n] * SX / 2 + w[1, n] * SY / 2), 2e-5) for n in range(20)]
            for psi0 in ctrl.rho_init:
                psi = [psi0]
                for U in Us:
                    psi.append(U @ psi[-1])
                tot += sum(tp.weight * np.real(np.vdot(psi[tp.step], tp.target_dm @ psi[tp.step])) for tp in tr)
                n_ens += 1
    assert abs(F - tot / n_ens) < 1e-13


def test_tracking_gradient_is_twice_the_derivative():
    ctrl, tr = _ctrl(), _track()
    ctrl.pulse_dt = np.full(20, 5e-6)   # ~0.035 rad per slice: first-order error below 1e-2
    w = np.random.default_rng(1).uniform(-1, 1, (2, 20))
    _, G = rs.grape_tracking_kernel(w, ctrl, tr)
    Gfd = _fd(lambda x: rs.grape_tracking_kernel(x, ctrl, tr)[0], w)
    scale = np.max(np.abs(Gfd))
    assert np.max(np.abs(G - 2 * Gfd)) / scale < 1e-2       # first-order formula, reference bar
    assert np.max(np.abs(G - Gfd)) / scale > 0.5            # not the derivative itself


def test_tracking_step_out_of_range_and_weights_sum():
    ctrl = _ctrl()
    w = np.zeros((2, 20))
    with pytest.raises(ValueError, match="out of range"):
        rs.grape_tracking_kernel(w, ctrl, [rs.TrackingPoint(21, np.eye(2), 1.0)])
    with pytest.raises(ValueError, match="out of range"):
        rs.grape_tracking_kernel(w, ctrl, [rs.TrackingPoint(0, np.eye(2), 1.0)])
    # identity targets with unit total weight: every checkpoint reads Tr(rho) = |psi|^2 = 1
    F, G = rs.grape_tracking_kernel(w, ctrl, [rs.TrackingPoint(s, np.eye(2), 0.25) for s in (1, 7, 7, 20)])
    assert abs(F - 1.0) < 1e-13 and np.max(np.abs(G)) < 1e-12


def test_phase_kernel_chain_rule():
    ctrl = rs.MRControl(drifts=[2 * np.pi * 80 * SZ / 2], operators=[SX / 2, SY / 2], rho_init=[UP], rho_targ=[DN],
                        pwr_levels=[2 * np.pi * 1e3], pulse_dt=np.full(15, 3e-5), fidelity="square")
    rng = np.random.default_rng(2)
    phi, amp = rng.uniform(-np.pi, np.pi, (1, 15)), rng.uniform(0.2, 1.0, (1, 15))
    F, Gp = rs.grape_phase_kernel(phi, ctrl, amp)
    w = np.vstack([amp * np.cos(phi), amp * np.sin(phi)])
    assert F == rs.grape_state_kernel(w, ctrl)[0]
    _, G = rs.grape_state_kernel(w, ctrl)
    assert np.allclose(Gp, -G[0::2] * np.sin(phi) + G[1::2] * np.cos(phi), rtol=0, atol=1e-15)
    with pytest.raises(ValueError):
        rs.grape_phase_kernel(np.zeros((2, 15)), ctrl)
    with pytest.raises(ValueError):
        rs.grape_phase_kernel(phi, ctrl, -amp)
