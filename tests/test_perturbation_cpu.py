"""Drift trajectories in the oracle: the member model's per-slice ramp
(tau_k dH added to the drift) reproduces the reference's
_fidelity_with_perturbation on the trajectory that sample_drift_trajectories
builds (RobustOpt.jl:168-182, 739-761), and the ramp is linear from 0 to 1."""
import numpy as np

from oracle import members as mb
from oracle import ref_semantics as rs


def _herm(rng, d):
    A = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    return (A + A.conj().T) / 2


def test_ramp_member_model_equals_reference_trajectory_fidelity():
    rng = np.random.default_rng(41)
    d, n_c, n_t, dt = 3, 2, 11, 0.1
    Hd, Hc = _herm(rng, d), [_herm(rng, d) for _ in range(n_c)]
    T = np.linalg.qr(rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d)))[0]
    u = rng.uniform(-1, 1, (n_c, n_t))
    finals = [0.2 * _herm(rng, d) for _ in range(3)]
    trajs = rs.sample_drift_trajectories(finals, n_t)
    for dH, traj in zip(finals, trajs):
        assert np.allclose(traj[0], 0) and np.allclose(traj[-1], dH)
        tau = np.array([np.linalg.norm(t) / np.linalg.norm(dH) for t in traj])
        assert np.allclose(np.diff(tau), 1.0 / (n_t - 1))
        prob = mb.Problem(drifts=Hd[None], controls=np.stack(Hc), dt=np.full(n_t, dt), target="gate",
                          fidelity="square", target_op=T, ramp_ops=dH[None], member_ramp=np.zeros(1, int),
                          tau=np.arange(n_t) / (n_t - 1))
        F, _ = mb.eval_problem(prob, u, "exact", want_grad=False)
        assert abs(F - rs.fidelity_with_perturbation(Hd, Hc, u, dt, T, traj)) <= 1e-14
    # a constant perturbation is the :parametric case
    F_par = rs.fidelity_with_perturbation(Hd, Hc, u, dt, T, finals[0])
    prob = mb.Problem(drifts=(Hd + finals[0])[None], controls=np.stack(Hc), dt=np.full(n_t, dt), target="gate",
                      fidelity="square", target_op=T)
    assert abs(mb.eval_problem(prob, u, "exact", want_grad=False)[0] - F_par) <= 1e-14
