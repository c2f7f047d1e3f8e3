"""Continuous-batching server (pgx_server).

A served job runs the kernels of a solo run on its own stream, so its result
must be bit-identical whether it runs alone or among other jobs of other
sizes; its stop rules and best-controls bookkeeping must be those of
grape_optimize (GRAPE.jl:536-610, check_grape_convergence :371-402), which the
device-resident optimiser (itself checked against the oracle's restated loop)
implements on the host.
"""
import time

import numpy as np
import pytest

import fx

pytestmark = pytest.mark.gpu

W = fx.W
OPT = dict(max_iter=15, step_size=0.5, convergence_tol=1e-12, gradient_norm_tol=1e-12)


def _jobs(seed=13):
    rng = np.random.default_rng(seed)
    out = []
    for d, n_t, nm in [(4, 30, 3), (16, 20, 2), (2, 60, 5), (8, 25, 4), (32, 10, 2), (3, 17, 1)]:
        out.append(W.uneven_problem(rng, d=d, n_t=n_t, n_members=nm))
    out.append(W.lindblad_gate(seed=3, n_qubits=2, n_t=12, n_draws=2))
    return out


def _run(server, jobs, precision, opt=OPT, stagger_s=0.0):
    ids = []
    for i, (spec, u0) in enumerate(jobs):
        ids.append(server.submit(u0=u0, opt=opt, **spec.problem_kwargs("exact", precision)))
        if stagger_s and i == len(jobs) // 2:
            time.sleep(stagger_s)
    assert server.drain(timeout_s=300)
    return [server.fetch(j) for j in ids]


def _same(a, b):
    assert a.state == b.state == "done"
    assert a.n_iterations == b.n_iterations, (a.n_iterations, b.n_iterations)
    assert a.termination_reason == b.termination_reason
    assert a.fidelity == b.fidelity, (a.fidelity, b.fidelity)
    assert a.step_size_final == b.step_size_final
    assert np.array_equal(a.controls, b.controls)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_job_identical_alone_and_in_the_mix(pg, ctx, precision):
    jobs = _jobs()
    solo = []
    s = pg.Server(ctx, max_inflight=1, target_fidelity=2.0)
    for job in jobs:
        solo.extend(_run(s, [job], precision))
    s.close()
    mix = pg.Server(ctx, max_inflight=8, target_fidelity=2.0)
    mixed = _run(mix, jobs, precision, stagger_s=0.002)
    st = mix.stats()
    mix.close()
    for a, b in zip(solo, mixed):
        _same(a, b)
    assert st["completed"] == len(jobs) and st["failed"] == 0
    assert st["kernel_launches"] > 0
    assert st["units"] == sum(sp.n_members * sp.n_t * (r.n_iterations + 1) for (sp, _), r in zip(jobs, mixed))
    assert 0 < st["p50_latency_s"] <= st["p99_latency_s"]


def test_served_job_follows_grape_optimize(pg, ctx):
    """Stop rules, iteration count and best controls as grape_optimize."""
    rng = np.random.default_rng(5)
    cases = [W.uneven_problem(rng, d=4, n_t=40, n_members=2), W.single_qubit_transfer(explicit_init=True)]
    settings = [dict(max_iter=30, step_size=0.5, convergence_tol=1e-9),   # stops at max_iter
                dict(max_iter=500, step_size=0.05, convergence_tol=1e-8)]  # stops on a reference rule
    srv = pg.Server(ctx, max_inflight=4, target_fidelity=2.0)
    for (spec, u0), opt in zip(cases, settings):
        p = pg.Problem(ctx=ctx, **spec.problem_kwargs("exact", "fp64"))
        ref = p.optimize(u0, "grape", **opt)
        p.close()
        jid = srv.submit(u0=u0, opt=opt, **spec.problem_kwargs("exact", "fp64"))
        assert srv.drain(timeout_s=300)
        r = srv.fetch(jid)
        assert r.state == "done"
        assert r.n_iterations == ref.n_iterations
        assert r.converged == ref.converged
        assert r.termination_reason == ref.termination_reason
        assert abs(r.fidelity - ref.fidelity) <= 1e-12, (r.fidelity, ref.fidelity)
        scale = max(np.max(np.abs(ref.controls)), 1.0)
        assert np.max(np.abs(r.controls - ref.controls)) <= 1e-10 * scale
        assert abs(r.step_size_final - ref.step_size_final) <= 1e-12 * ref.step_size_final
    srv.close()


def test_target_fidelity_stops_a_job(pg, ctx):
    spec, u0 = W.single_qubit_transfer(explicit_init=True)
    srv = pg.Server(ctx, max_inflight=2, target_fidelity=0.99)
    jid = srv.submit(u0=u0, opt=dict(max_iter=500, step_size=0.05), **spec.problem_kwargs("exact", "fp64"))
    assert srv.drain(timeout_s=120)
    r = srv.fetch(jid)
    srv.close()
    assert r.state == "done" and r.converged
    assert r.termination_reason == "target fidelity reached"
    assert r.fidelity >= 0.99


def test_admission_by_hbm_budget(pg, ctx):
    jobs = _jobs()[:4]
    opt = dict(OPT, max_iter=6)
    footprints = []
    for sp, _ in jobs:
        d, _, _ = pg.problem_desc(**sp.problem_kwargs("exact", "fp64"))
        b = pg._abi.C.c_uint64()
        pg._abi.check(pg._abi.lib().pgx_problem_footprint(pg._abi.C.byref(d), pg._abi.C.byref(b)))
        footprints.append(int(b.value))
    budget = int(1.5 * max(footprints)) + (1 << 20)
    # a job larger than the whole budget is refused at submission
    small = pg.Server(ctx, max_inflight=4, hbm_budget_bytes=min(footprints) // 2)
    with pytest.raises(pg._abi.PgxError) as e:
        small.submit(u0=jobs[0][1], opt=opt, **jobs[0][0].problem_kwargs("exact", "fp64"))
    assert e.value.status == 4
    small.close()
    # jobs that fit only a few at a time still all complete, with the same results
    srv = pg.Server(ctx, max_inflight=4, hbm_budget_bytes=budget)
    got = _run(srv, jobs, "fp64", opt=opt)
    st = srv.stats()
    srv.close()
    assert st["hbm_peak"] <= budget
    ref = pg.Server(ctx, max_inflight=4)
    want = _run(ref, jobs, "fp64", opt=opt)
    ref.close()
    for a, b in zip(got, want):
        _same(a, b)


def test_cancel_queued_and_running(pg, ctx):
    spec, u0 = W.uneven_problem(np.random.default_rng(9), d=16, n_t=200, n_members=8)
    kw = spec.problem_kwargs("exact", "fp64")
    srv = pg.Server(ctx, max_inflight=1, target_fidelity=2.0)
    long_opt = dict(max_iter=100000, step_size=1e-3, convergence_tol=1e-300, gradient_norm_tol=0.0)
    a = srv.submit(u0=u0, opt=long_opt, **kw)
    b = srv.submit(u0=u0, opt=long_opt, **kw)
    assert srv.poll(b)["state"] == "queued"
    srv.cancel(b)
    assert srv.poll(b)["state"] == "cancelled"
    t0 = time.time()
    while srv.poll(a)["iterations"] < 2 and time.time() - t0 < 60:
        time.sleep(0.01)
    assert srv.poll(a)["state"] == "running"
    srv.cancel(a)
    assert srv.drain(timeout_s=60)
    ra, rb = srv.fetch(a), srv.fetch(b)
    assert ra.state == "cancelled" and rb.state == "cancelled"
    assert ra.n_iterations >= 2
    assert ra.controls.shape == u0.shape and np.all(np.isfinite(ra.controls))
    st = srv.stats()
    assert st["cancelled"] == 2 and st["completed"] == 0
    srv.close()


def test_submit_validation(pg, ctx):
    spec, u0 = W.uneven_problem(np.random.default_rng(2), d=4, n_t=10, n_members=1)
    srv = pg.Server(ctx, max_inflight=2)
    with pytest.raises(pg._abi.PgxError) as e:
        srv.submit(u0=u0, opt=dict(max_iter=0), **spec.problem_kwargs("exact", "fp64"))
    assert e.value.status == 1
    bad = u0.copy()
    bad[0, 0] = np.nan
    with pytest.raises(pg._abi.PgxError) as e:
        srv.submit(u0=bad, **spec.problem_kwargs("exact", "fp64"))
    assert e.value.status == 10
    assert srv.stats()["submitted"] == 0
    srv.close()


LB_OPT = dict(max_iter=12, step_size=0.3, lbfgs_memory=5, convergence_tol=1e-12, gradient_norm_tol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lbfgs_job_identical_alone_and_in_the_mix(pg, ctx, precision):
    jobs = _jobs()[:5]
    solo = []
    s = pg.Server(ctx, max_inflight=1, target_fidelity=2.0)
    for spec, u0 in jobs:
        jid = s.submit(u0=u0, opt=LB_OPT, method="ensemble_lbfgs", **spec.problem_kwargs("exact", precision))
        assert s.drain(timeout_s=300)
        solo.append(s.fetch(jid))
    s.close()
    mix = pg.Server(ctx, max_inflight=8, target_fidelity=2.0)
    ids = []
    for i, (spec, u0) in enumerate(jobs):  # L-BFGS and GRAPE jobs side by side
        ids.append(mix.submit(u0=u0, opt=LB_OPT, method="ensemble_lbfgs", **spec.problem_kwargs("exact", precision)))
        mix.submit(u0=u0, opt=OPT, **spec.problem_kwargs("exact", precision))
    assert mix.drain(timeout_s=300)
    mixed = [mix.fetch(j) for j in ids]
    mix.close()
    for a, b in zip(solo, mixed):
        _same(a, b)


def test_lbfgs_job_follows_grape_optimize_ensemble(pg, ctx):
    """Iteration count, stop rule and result of the device-resident L-BFGS
    against the host loop of grape_optimize_ensemble (GRAPE.jl:1012-1230); the
    two differ only in the summation order of the dot products."""
    rng = np.random.default_rng(17)
    cases = [W.uneven_problem(rng, d=4, n_t=30, n_members=3), W.uneven_problem(rng, d=8, n_t=20, n_members=2)]
    opts = [dict(max_iter=15, step_size=0.5, lbfgs_memory=4, convergence_tol=1e-12),
            dict(max_iter=40, step_size=0.2, lbfgs_memory=6, convergence_tol=1e-6, amplitude_limit=1.5)]
    srv = pg.Server(ctx, max_inflight=4, target_fidelity=2.0)
    for (spec, u0), opt in zip(cases, opts):
        p = pg.Problem(ctx=ctx, **spec.problem_kwargs("exact", "fp64"))
        ref = p.optimize(u0, "ensemble_lbfgs", **opt)
        p.close()
        jid = srv.submit(u0=u0, opt=opt, method="ensemble_lbfgs", **spec.problem_kwargs("exact", "fp64"))
        assert srv.drain(timeout_s=300)
        r = srv.fetch(jid)
        assert r.state == "done"
        assert r.n_iterations == ref.n_iterations, (r.n_iterations, ref.n_iterations)
        assert r.termination_reason == ref.termination_reason
        assert r.converged == ref.converged
        assert abs(r.fidelity - ref.fidelity) <= 1e-9, (r.fidelity, ref.fidelity)
        assert np.max(np.abs(r.controls - ref.controls)) <= 1e-6 * max(1.0, np.max(np.abs(ref.controls)))
    srv.close()


def test_lbfgs_submit_validation(pg, ctx):
    spec, u0 = W.uneven_problem(np.random.default_rng(2), d=4, n_t=10, n_members=1)
    srv = pg.Server(ctx, max_inflight=2)
    with pytest.raises(pg._abi.PgxError) as e:
        srv.submit(u0=u0, opt=dict(lbfgs_memory=0), method="ensemble_lbfgs", **spec.problem_kwargs("exact", "fp64"))
    assert e.value.status == 1
    for bad in (dict(l_bound=1.0, u_bound=-1.0), dict(l_bound=-np.inf), dict(lbfgs_memory=65)):
        with pytest.raises(pg._abi.PgxError) as e:   # MR methods need finite bounds l < u
            srv.submit(u0=u0, opt=bad, method="mr_lbfgs", **spec.problem_kwargs("exact", "fp64"))
        assert e.value.status == 1
    srv.close()


def _mr_problem(seed=2, n_t=40):
    """An MR state-transfer ensemble (drifts x pwr levels, two pairs), the
    kind optimcon serves (OptControl.jl:137-259)."""
    rng = np.random.default_rng(seed)
    sx = np.array([[0, 1], [1, 0]], complex) / 2
    sy = np.array([[0, -1j], [1j, 0]], complex) / 2
    sz = np.diag([0.5, -0.5]).astype(complex)
    drifts = np.stack([2 * np.pi * off * sz for off in (-400.0, 0.0, 300.0)])
    pwr = np.array([2 * np.pi * 0.9e3, 2 * np.pi * 1.1e3])
    kw = dict(drifts=drifts, controls=np.stack([sx, sy]), dt=np.full(n_t, 1.2e-5), target="states",
              fidelity="real", member_drift=np.repeat(np.arange(3), 2), member_scale=np.tile(pwr, 3),
              states_init=np.array([[1, 0], [0, 1]], complex), states_target=np.array([[0, 1], [1, 0]], complex),
              grad_mode="ref_mr")
    return kw, rng.uniform(-0.8, 0.8, (2, n_t))


@pytest.mark.parametrize("method", ["mr_lbfgs", "mr_grape"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mr_jobs_follow_optimcon(pg, ctx, method, precision):
    """Served MR L-BFGS / GRAPE against the solo optimiser's optimcon loops
    (OptControl.jl:380-561): iteration count, stop rule, result and histories;
    the two differ only in the order of the device's dot products."""
    kw, u0 = _mr_problem()
    kw["precision"] = precision
    opt = dict(max_iter=25, gradient_norm_tol=1e-9, lbfgs_memory=5, l_bound=-1.0, u_bound=1.0)
    p = pg.Problem(ctx=ctx, **kw)
    ref = p.optimize(u0 * 1.5, method, **opt)       # the guess is clamped to the bounds first
    p.close()
    srv = pg.Server(ctx, max_inflight=2, target_fidelity=2.0)
    jid = srv.submit(u0=u0 * 1.5, opt=opt, method=method, **kw)
    assert srv.drain(timeout_s=300)
    r = srv.fetch(jid)
    srv.close()
    assert r.state == "done"
    assert r.n_iterations == ref.n_iterations, (r.n_iterations, ref.n_iterations)
    assert r.termination_reason == ref.termination_reason, (r.termination_reason, ref.termination_reason)
    assert r.converged == ref.converged
    assert abs(r.fidelity - ref.fidelity) <= 1e-9, (r.fidelity, ref.fidelity)
    assert np.max(np.abs(r.controls - ref.controls)) <= 1e-6
    assert np.max(r.controls) <= 1.0 and np.min(r.controls) >= -1.0
    assert len(r.fidelity_history) == len(ref.fidelity_history)
    assert np.allclose(r.fidelity_history, ref.fidelity_history, rtol=0, atol=1e-9)
    assert len(r.gradient_norm_history) == len(ref.gradient_norm_history)
    assert np.allclose(r.gradient_norm_history, ref.gradient_norm_history, rtol=1e-7, atol=1e-12)


def test_mr_jobs_identical_alone_and_in_the_mix(pg, ctx):
    kw, u0 = _mr_problem(seed=5)
    opt = dict(max_iter=15, lbfgs_memory=4)
    solo = {}
    for method in ("mr_lbfgs", "mr_grape"):
        s = pg.Server(ctx, max_inflight=1, target_fidelity=2.0)
        solo[method] = _run_one(s, kw, u0, method, opt)
        s.close()
    mix = pg.Server(ctx, max_inflight=8, target_fidelity=2.0)
    ids = {m: mix.submit(u0=u0, opt=opt, method=m, **kw) for m in ("mr_lbfgs", "mr_grape")}
    for spec, ux in _jobs()[:3]:
        mix.submit(u0=ux, opt=OPT, **spec.problem_kwargs("exact", "mixed"))
    assert mix.drain(timeout_s=300)
    for m, jid in ids.items():
        r = mix.fetch(jid)
        a = solo[m]
        assert r.n_iterations == a.n_iterations and r.fidelity == a.fidelity
        assert np.array_equal(r.controls, a.controls)
        assert r.fidelity_history == a.fidelity_history
    mix.close()


def _run_one(srv, kw, u0, method, opt):
    jid = srv.submit(u0=u0, opt=opt, method=method, **kw)
    assert srv.drain(timeout_s=300)
    return srv.fetch(jid)


def _served_vs_solo(pg, ctx, kw, u0, method, opt, setup, extras, ftol=1e-9):
    p = pg.Problem(ctx=ctx, **kw)
    setup(p)
    ref = p.optimize(u0, method, **opt)
    p.close()
    srv = pg.Server(ctx, max_inflight=2, target_fidelity=2.0)
    jid = srv.submit(u0=u0, opt=opt, method=method, **extras, **kw)
    assert srv.drain(timeout_s=300)
    r = srv.fetch(jid)
    srv.close()
    assert r.state == "done", r.termination_reason
    assert r.n_iterations == ref.n_iterations, (r.n_iterations, ref.n_iterations)
    assert r.termination_reason == ref.termination_reason
    assert abs(r.fidelity - ref.fidelity) <= ftol, (r.fidelity, ref.fidelity)
    assert np.max(np.abs(r.controls - ref.controls)) <= 1e-6 * max(1.0, np.max(np.abs(ref.controls)))
    assert np.allclose(r.fidelity_history, ref.fidelity_history, rtol=0, atol=ftol)
    return r


def test_served_mr_job_with_penalties(pg, ctx):
    """An MR L-BFGS job with waveform penalties (GRAPEState.jl:571-584)."""
    kw, u0 = _mr_problem(seed=8)
    pens = [("SNS", 0.02, -0.6, 0.6), ("DNS", 0.01)]
    opt = dict(max_iter=20, lbfgs_memory=5)
    r = _served_vs_solo(pg, ctx, kw, u0, "mr_lbfgs", opt, lambda p: p.set_penalties(pens), dict(penalties=pens))
    assert r.n_iterations > 2


def test_served_tracking_job(pg, ctx):
    """An MR GRAPE job on a trajectory-tracking objective (optimcon with
    ctrl.tracking, OptControl.jl:328-345)."""
    kw, u0 = _mr_problem(seed=9)
    dn, up = np.array([0, 1], complex), np.array([1, 0], complex)
    steps, weights = [10, 25, 40], [0.3, 0.3, 0.4]
    targets = np.stack([np.outer(dn, dn), np.outer(up, up), np.outer(dn, dn)])
    opt = dict(max_iter=15)
    _served_vs_solo(pg, ctx, kw, u0, "mr_grape", opt, lambda p: p.set_tracking(steps, weights, targets),
                    dict(tracking=(steps, weights, targets)))


def test_served_drift_ramp_job_and_exact_resume(pg, ctx):
    """A grape_optimize job on a drift-ramp ensemble; its exact snapshot
    continues only with the same extras (they are part of the fingerprint)."""
    rng = np.random.default_rng(12)
    spec, u0 = W.uneven_problem(rng, d=8, n_t=60, n_members=3)
    kw = spec.problem_kwargs("exact", "fp64")
    A = rng.standard_normal((2, 8, 8)) + 1j * rng.standard_normal((2, 8, 8))
    ops = 2 * np.pi * 1e5 * (A + np.conj(np.transpose(A, (0, 2, 1)))) / 2
    ramp = (ops, [0, 1, -1], np.linspace(0.0, 1.0, 60))
    opt = dict(max_iter=30, step_size=0.3, convergence_tol=1e-14)
    r = _served_vs_solo(pg, ctx, kw, u0, "grape", opt, lambda p: p.set_drift_ramp(*ramp), dict(drift_ramp=ramp),
                        ftol=1e-12)
    srv = pg.Server(ctx, max_inflight=1, target_fidelity=2.0)
    jid = srv.submit(u0=u0, opt=dict(opt, max_iter=400), drift_ramp=ramp, **kw)
    import time
    t0 = time.time()
    while srv.poll(jid)["iterations"] < 3 and time.time() - t0 < 60:
        time.sleep(0.001)
    srv.cancel(jid)
    assert srv.drain(timeout_s=300)
    blob = srv.checkpoint(jid)
    ref = srv.fetch(jid)
    assert pg.checkpoint_parse(blob)["exact"]
    with pytest.raises(pg._abi.PgxError):              # without its ramp: another problem
        srv.submit_resume(checkpoint=blob, mode="continue", **kw)
    full = srv.submit(u0=u0, opt=dict(opt, max_iter=400), drift_ramp=ramp, **kw)
    cont = srv.submit_resume(checkpoint=blob, mode="continue", drift_ramp=ramp, **kw)
    assert srv.drain(timeout_s=300)
    a, b = srv.fetch(full), srv.fetch(cont)
    assert a.n_iterations == b.n_iterations and a.fidelity == b.fidelity
    assert np.array_equal(a.controls, b.controls) and a.fidelity_history == b.fidelity_history
    srv.close()
    assert ref.state == "cancelled" and r.n_iterations == 30
