"""Every benchmark configuration at its full size against the FP64 oracle.

* lindblad3q: 3-qubit Lindblad gate (D = 64 superoperators), 32 detuning draws
  x 500 slices, exact gradient, FP64 and mixed precision, against the numpy
  oracle (scipy Pade propagators, scipy's Al-Mohy-Higham Frechet derivative)
  evaluated member-parallel in spawned processes.
* uneven512: all 512 uneven problems batched in one CUDA graph in mixed
  precision; the d = 32 and longest-chain extremes and 64 random others
  against the oracle's C restatement (exact gradient).
* spin4 ensemble L-BFGS: 20 iterations of grape_optimize_ensemble's L-BFGS
  (GRAPE.jl:1012-1230) at 231 members x 1000 slices on the device, mixed
  against the plain FP64 GPU trajectory.
* served jobs: a sample of the served stream's jobs (uneven Hermitian and
  Lindblad gate jobs) optimised by the server in mixed precision; each
  returned fidelity against the oracle at the returned controls.

Bars: FP64 |dF| <= 1e-10 and max|dG|/max|G| <= 1e-8; mixed |dF| <= 1e-8 and
max|dG|/max|G| <= 1e-4.
"""
import os

import numpy as np
import pytest

from oracle import members as mb
import fx
from test_parity_gpu import to_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

F_TOL = {"fp64": 1e-10, "mixed": 1e-8}
G_RTOL = {"fp64": 1e-8, "mixed": 1e-4}


def _check(prec, F, G, Fo, Go):
    assert abs(F - Fo) <= F_TOL[prec], (prec, F, Fo, abs(F - Fo))
    err = np.max(np.abs(G - Go)) / max(np.max(np.abs(Go)), 1e-300)
    assert err <= G_RTOL[prec], (prec, err)
    return abs(F - Fo), err


@pytest.fixture(scope="module")
def lindblad3q_oracle():
    from oracle import parallel
    prob, u0 = fx.lindblad_3q()
    assert (prob.n_members, prob.n_t, prob.D) == (32, 500, 64)
    Fo, Go = parallel.eval_problem_parallel(prob, u0, "exact")
    return prob, u0, Fo, Go


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_lindblad3q_full_size_vs_oracle(pg, lindblad3q_oracle, prec):
    prob, u0, Fo, Go = lindblad3q_oracle
    p = to_gpu(pg, prob, "exact", precision=prec)
    F, G = p.eval(u0)
    p.close()
    dF, dG = _check(prec, F, G, Fo, Go)
    print(f"lindblad3q 32 x 500 {prec}: |dF| = {dF:.2e}, grad rel = {dG:.2e}")


def test_uneven512_batched_mixed_vs_c_oracle(pg):
    """The whole 512-problem draw runs batched in mixed precision; the largest
    d = 32 problem, the longest chain, the largest problem and 64 random
    others are checked against the C restatement of the oracle."""
    from oracle import cpu_port
    cases = fx.uneven_batch(512)
    probs = [to_gpu(pg, pr, "exact", precision="mixed") for pr, _ in cases]
    b = pg.Batch(probs, n_streams=16)
    for i, (_, u0) in enumerate(cases):
        b.set_controls(i, u0)
    F = b.eval()
    units = np.array([pr.n_members * pr.n_t for pr, _ in cases])
    ds = np.array([pr.D for pr, _ in cases])
    d32 = [i for i in range(len(cases)) if ds[i] == 32]
    extremes = {int(np.argmax(units)), max(d32, key=lambda i: units[i]),
                int(np.argmax([pr.n_t for pr, _ in cases]))}
    rng = np.random.default_rng(2024)
    pick = sorted(extremes | set(rng.choice(len(cases), 64, replace=False).tolist()))
    G = {i: b.get_controls(i)[1] for i in pick}
    b.close()
    for p in probs:
        p.close()
    big = max(pick, key=lambda i: units[i])
    cpu_port.calibrate(cases[big][0], cases[big][1], "exact", os.cpu_count() or 1)
    worst_F, worst_G = 0.0, 0.0
    for i in pick:
        pr, u0 = cases[i]
        Fo, Go = cpu_port.CpuProblem(pr, "exact").eval(u0)
        dF, dG = _check("mixed", F[i], G[i], Fo, Go)
        worst_F, worst_G = max(worst_F, dF), max(worst_G, dG)
    print(f"uneven512: {len(pick)} problems checked, max |dF| = {worst_F:.2e}, max grad rel = {worst_G:.2e}")


def test_spin4_ensemble_lbfgs_20_iterations_mixed_vs_fp64(pg):
    """grape_optimize_ensemble's L-BFGS on the 231 x 1000 ensemble: the
    mixed-precision trajectory follows the plain FP64 one to 1e-8 in F.  The
    controls are in rad/s, so gradients are ~1e-6 per entry: the stall and
    gradient-norm rules are off and every run takes its 20 iterations."""
    prob, u0 = fx.spin4_ensemble()
    out = {}
    for prec in ("fp64", "mixed"):
        p = to_gpu(pg, prob, "exact", precision=prec)
        out[prec] = p.optimize(u0, "ensemble_lbfgs", max_iter=20, lbfgs_memory=10, step_size=0.01,
                               convergence_tol=1e-300, gradient_norm_tol=1e-300)
        p.close()
    a, m = out["fp64"], out["mixed"]
    assert a.n_iterations == m.n_iterations >= 20
    assert a.termination_reason == m.termination_reason
    assert len(a.fidelity_history) == len(m.fidelity_history)
    dF = np.max(np.abs(np.array(a.fidelity_history) - np.array(m.fidelity_history)))
    assert dF <= 1e-8, dF
    assert abs(a.fidelity - m.fidelity) <= 1e-8
    assert m.fidelity > m.fidelity_history[0]
    print(f"spin4 L-BFGS 20 iterations: F {m.fidelity_history[0]:.6f} -> {m.fidelity:.6f}, "
          f"max |dF| along the trajectory {dF:.2e}")


def test_served_jobs_vs_oracle(pg, ctx):
    """Jobs of the served stream's distribution (uneven Hermitian problems and
    2-3 qubit Lindblad gates) optimised by the server in mixed precision under
    the served stop rule; every returned F against the oracle at the returned
    controls."""
    from oracle import cpu_port
    from pulsar_gb300 import workloads as W
    jobs = W.serve_stream(seed=17, rate=1000.0, duration_s=0.03, lindblad_frac=0.25, max_slices=120,
                          max_members=8, lindblad_slices=30, lindblad_draws=2)
    assert len(jobs) >= 16
    srv = pg.Server(ctx, max_inflight=32, target_fidelity=0.999)
    ids = [srv.submit(u0=j.u0, opt=dict(max_iter=30, step_size=0.01, lbfgs_memory=10), method="ensemble_lbfgs",
                      **j.spec.problem_kwargs("exact", "mixed")) for j in jobs]
    srv.drain()
    res = [srv.fetch(i) for i in ids]
    srv.close()
    worst = 0.0
    kinds = set()
    for j, r in zip(jobs, res):
        assert r.state == "done", r.termination_reason
        prob = mb.Problem.from_spec(j.spec)
        if prob.generator == "hermitian":
            Fo = cpu_port.CpuProblem(prob, "exact").eval(r.controls, want_grad=False)[0]
        else:
            Fo = mb.eval_problem(prob, r.controls, "exact", want_grad=False)[0]
        kinds.add(prob.generator)
        worst = max(worst, abs(r.fidelity - Fo))
        assert abs(r.fidelity - Fo) <= F_TOL["mixed"], (j.kind, r.fidelity, Fo)
    assert kinds == {"hermitian", "liouvillian"}
    print(f"served: {len(jobs)} jobs, max |dF| vs oracle = {worst:.2e}")
