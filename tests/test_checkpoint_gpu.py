"""Checkpoints of served jobs (pgx_job_checkpoint / pgx_submit_resume).

An exact snapshot holds a job's device state at an iteration boundary, so a
job resumed from it with PGX_RESUME_CONTINUE must produce the iterates,
histories and result of a run that was never interrupted -- bit for bit,
since both run the same kernels -- and taking a snapshot must not disturb
the running job.  PGX_RESUME_RESTART is resume_optimization
(IO/Checkpoint.jl:220-298): a fresh run from w_opt whose histories and
iteration count follow the checkpoint's.  Histories follow
OptimizationResult's conventions (GRAPE.jl:158-170), checked against the
solo optimiser.
"""
import time

import numpy as np
import pytest

import fx

pytestmark = pytest.mark.gpu

W = fx.W
GRAPE_OPT = dict(max_iter=400, step_size=0.2, convergence_tol=1e-15, gradient_norm_tol=1e-15)
# the ascent L-BFGS keeps a pair only where y.s > 0; with this step the first
# iterations of the workload below keep two (checked on the oracle)
LB_OPT = dict(max_iter=300, step_size=0.05, lbfgs_memory=4, convergence_tol=1e-15, gradient_norm_tol=1e-15)


def _job(seed=21):
    """Large enough that an iteration takes milliseconds: a snapshot lands mid-run."""
    rng = np.random.default_rng(seed)
    return W.uneven_problem(rng, d=16, n_t=300, n_members=8)


def _wait_iterations(srv, jid, k, timeout_s=60.0):
    t0 = time.time()
    while time.time() - t0 < timeout_s:
        p = srv.poll(jid)
        if p["state"] != "running" and p["state"] != "queued":
            raise AssertionError(f"job ended before iteration {k}: {p}")
        if p["iterations"] >= k:
            return p["iterations"]
        time.sleep(0.0005)
    raise AssertionError("job too slow")


def _identical(a, b):
    assert a.state == b.state == "done", (a.state, b.state)
    assert a.n_iterations == b.n_iterations, (a.n_iterations, b.n_iterations)
    assert a.termination_reason == b.termination_reason
    assert a.converged == b.converged
    assert a.fidelity == b.fidelity, (a.fidelity, b.fidelity)
    assert a.step_size_final == b.step_size_final
    assert np.array_equal(a.controls, b.controls)
    assert a.fidelity_history == b.fidelity_history
    assert a.gradient_norm_history == b.gradient_norm_history


def _submit(srv, spec, u0, method, opt, precision):
    return srv.submit(u0=u0, opt=opt, method=method, **spec.problem_kwargs("exact", precision))


MR_OPT = dict(max_iter=300, gradient_norm_tol=1e-15, lbfgs_memory=4)


@pytest.mark.parametrize("method,precision", [("grape", "fp64"), ("grape", "mixed"), ("ensemble_lbfgs", "fp64"),
                                              ("ensemble_lbfgs", "mixed"), ("mr_lbfgs", "mixed"),
                                              ("mr_grape", "fp64")])
def test_exact_continuation_is_bit_identical(pg, ctx, method, precision):
    spec, u0 = _job()
    opt = {"grape": GRAPE_OPT, "ensemble_lbfgs": LB_OPT}.get(method, MR_OPT)
    kw = spec.problem_kwargs("exact", precision)
    srv = pg.Server(ctx, max_inflight=4, target_fidelity=2.0)
    a = _submit(srv, spec, u0, method, opt, precision)          # never interrupted
    assert srv.drain(timeout_s=600)
    ref = srv.fetch(a)
    assert ref.n_iterations >= 10

    # B: snapshotted mid-run, then left alone -- the snapshot must not perturb it
    b = _submit(srv, spec, u0, method, opt, precision)
    _wait_iterations(srv, b, 4)
    blob_b = srv.checkpoint(b, timeout_s=60)
    info = pg.checkpoint_parse(blob_b)
    assert info["exact"] and 4 <= info["iteration"] < ref.n_iterations
    # C: cancelled mid-run; its final state is exact too
    c = _submit(srv, spec, u0, method, opt, precision)
    _wait_iterations(srv, c, 6)
    srv.cancel(c)
    assert srv.drain(timeout_s=600)
    blob_c = srv.checkpoint(c)
    info_c = pg.checkpoint_parse(blob_c)
    assert info_c["exact"] and info_c["iteration"] < ref.n_iterations
    rb, rc = srv.fetch(b), srv.fetch(c)
    _identical(ref, rb)
    assert rc.state == "cancelled"

    # continuing either snapshot reproduces the uninterrupted run
    ids = [srv.submit_resume(checkpoint=blob, mode="continue", **kw) for blob in (blob_b, blob_c)]
    assert srv.drain(timeout_s=600)
    for jid in ids:
        _identical(ref, srv.fetch(jid))
    if method == "ensemble_lbfgs":
        assert info["lbfgs_pairs"] > 0
    srv.close()


def test_exact_snapshot_survives_a_checkpoint_file(pg, ctx, tmp_path):
    """save_checkpoint / load_checkpoint keep the device state (metadata is
    re-wrapped around the same payload)."""
    spec, u0 = _job(seed=4)
    kw = spec.problem_kwargs("exact", "mixed")
    srv = pg.Server(ctx, max_inflight=2, target_fidelity=2.0)
    a = _submit(srv, spec, u0, "grape", GRAPE_OPT, "mixed")
    _wait_iterations(srv, a, 5)
    ck = pg.Checkpoint.from_bytes(srv.checkpoint(a, timeout_s=60))
    ck.metadata["dt"] = float(spec.dt[0])
    ck.domain = "qc"
    path = str(tmp_path / "job.ckpt")
    pg.save_checkpoint(path, ck)
    assert srv.drain(timeout_s=600)
    ref = srv.fetch(a)
    L = pg.load_checkpoint(path)
    assert L.exact and L.domain == "qc" and L.metadata["dt"] == float(spec.dt[0])
    r = srv.submit_resume(checkpoint=L.to_bytes(), mode="continue", **kw)
    assert srv.drain(timeout_s=600)
    _identical(ref, srv.fetch(r))
    srv.close()


@pytest.mark.parametrize("method", ["grape", "ensemble_lbfgs"])
def test_restart_follows_resume_optimization(pg, ctx, method):
    """A finished job's checkpoint resumed with RESTART equals a fresh job
    from its best controls, with the checkpoint's histories ahead and the
    iteration counts added (Checkpoint.jl:279-287)."""
    rng = np.random.default_rng(9)
    spec, u0 = W.uneven_problem(rng, d=4, n_t=40, n_members=3)
    kw = spec.problem_kwargs("exact", "fp64")
    base = dict(step_size=0.4, convergence_tol=1e-15, gradient_norm_tol=1e-15)
    if method == "ensemble_lbfgs":
        base["lbfgs_memory"] = 5
    srv = pg.Server(ctx, max_inflight=2, target_fidelity=2.0)
    first = srv.submit(u0=u0, opt=dict(base, max_iter=10), method=method, **kw)
    assert srv.drain(timeout_s=300)
    blob = srv.checkpoint(first)
    r1 = srv.fetch(first)
    info = pg.checkpoint_parse(blob)
    assert not info["exact"] and info["iteration"] == r1.n_iterations
    assert np.array_equal(info["w_opt"], r1.controls) and info["F_opt"] == r1.fidelity
    assert info["fidelity_history"] == r1.fidelity_history
    resumed = srv.submit_resume(checkpoint=blob, mode="restart", opt=dict(base, max_iter=15), method=method, **kw)
    fresh = srv.submit(u0=r1.controls, opt=dict(base, max_iter=15), method=method, **kw)
    assert srv.drain(timeout_s=300)
    R, F = srv.fetch(resumed), srv.fetch(fresh)
    assert R.state == F.state == "done"
    assert np.array_equal(R.controls, F.controls) and R.fidelity == F.fidelity
    assert R.n_iterations == r1.n_iterations + F.n_iterations
    assert R.fidelity_history == r1.fidelity_history + F.fidelity_history
    assert R.gradient_norm_history == r1.gradient_norm_history + F.gradient_norm_history
    assert R.termination_reason == F.termination_reason
    # the checkpoint's own settings (max_iter 10) are used when none are given
    again = srv.submit_resume(checkpoint=blob, mode="restart", **kw)
    fresh10 = srv.submit(u0=r1.controls, opt=dict(base, max_iter=10), method=method, **kw)
    assert srv.drain(timeout_s=300)
    A, F10 = srv.fetch(again), srv.fetch(fresh10)
    assert A.n_iterations == r1.n_iterations + F10.n_iterations and np.array_equal(A.controls, F10.controls)
    srv.close()


def test_server_histories_follow_the_solo_optimiser(pg, ctx):
    """Fidelity / gradient-norm histories of served jobs have the lengths and
    values of OptimizationResult's (pgx_optimize): grape_optimize's F(u0)
    twice, the post-step F of a converged run, ||G|| per iteration."""
    rng = np.random.default_rng(5)
    cases = [(W.uneven_problem(rng, d=4, n_t=40, n_members=2), "grape",
              dict(max_iter=30, step_size=0.5, convergence_tol=1e-9)),
             (W.single_qubit_transfer(explicit_init=True), "grape",
              dict(max_iter=500, step_size=0.05, convergence_tol=1e-8)),
             (W.uneven_problem(rng, d=4, n_t=30, n_members=3), "ensemble_lbfgs",
              dict(max_iter=15, step_size=0.5, lbfgs_memory=4, convergence_tol=1e-12))]
    srv = pg.Server(ctx, max_inflight=4, target_fidelity=2.0)
    for (spec, u0), method, opt in cases:
        p = pg.Problem(ctx=ctx, **spec.problem_kwargs("exact", "fp64"))
        ref = p.optimize(u0, method, **opt)
        p.close()
        jid = srv.submit(u0=u0, opt=opt, method=method, **spec.problem_kwargs("exact", "fp64"))
        assert srv.drain(timeout_s=300)
        r = srv.fetch(jid)
        assert len(r.fidelity_history) == len(ref.fidelity_history), (method, opt)
        assert len(r.gradient_norm_history) == len(ref.gradient_norm_history), (method, opt)
        tol = 1e-12 if method == "grape" else 1e-9
        assert np.allclose(r.fidelity_history, ref.fidelity_history, rtol=0, atol=tol)
        assert np.allclose(r.gradient_norm_history, ref.gradient_norm_history, rtol=1e-9, atol=1e-14)
    srv.close()


def test_resume_validation(pg, ctx):
    rng = np.random.default_rng(3)
    spec, u0 = W.uneven_problem(rng, d=4, n_t=20, n_members=2)
    kw = spec.problem_kwargs("exact", "fp64")
    srv = pg.Server(ctx, max_inflight=1, target_fidelity=2.0)
    jid = srv.submit(u0=u0, opt=dict(max_iter=5, step_size=0.3), **kw)
    assert srv.drain(timeout_s=120)
    blob = srv.checkpoint(jid)
    srv.fetch(jid)
    E = pg._abi.PgxError
    with pytest.raises(E) as e:        # a finished job's checkpoint cannot continue exactly
        srv.submit_resume(checkpoint=blob, mode="continue", **kw)
    assert e.value.status == 1
    n_c = u0.shape[0]
    g = np.random.default_rng(4)
    while True:                        # an 8-level problem with as many controls
        spec3, u3 = W.uneven_problem(g, d=8, n_t=20, n_members=2)
        if u3.shape[0] == n_c:
            break
    with pytest.raises(E) as e:        # system dimension (Checkpoint.jl:236-240)
        srv.submit_resume(checkpoint=blob, mode="restart", **spec3.problem_kwargs("exact", "fp64"))
    assert e.value.status == 1
    with pytest.raises(E) as e:        # n_controls (Checkpoint.jl:242-246)
        srv.submit_resume(checkpoint=blob, mode="restart", **dict(kw, controls=kw["controls"][:-1]))
    assert e.value.status == 1
    with pytest.raises(E) as e:        # a waveform of another length
        srv.submit_resume(checkpoint=blob, mode="restart", **dict(kw, dt=np.full(21, kw["dt"][0])))
    assert e.value.status == 2
    # a different problem of the same shape: RESTART is a warm start, allowed
    r = srv.submit_resume(checkpoint=blob, mode="restart", **dict(kw, dt=kw["dt"] * 1.01))
    assert srv.drain(timeout_s=120)
    assert srv.fetch(r).state == "done"
    with pytest.raises(E):
        srv.submit_resume(checkpoint=blob[:-1], mode="restart", **kw)
    # an exact snapshot continues only on its own problem and method
    big, ub = _job(seed=8)
    kb = big.problem_kwargs("exact", "fp64")
    j = srv.submit(u0=ub, opt=GRAPE_OPT, **kb)
    q = srv.submit(u0=ub, opt=GRAPE_OPT, **kb)        # queued behind j (one slot)
    with pytest.raises(E) as e:
        srv.checkpoint(q)
    assert e.value.status == 9
    srv.cancel(q)
    _wait_iterations(srv, j, 3)
    snap = srv.checkpoint(j, timeout_s=60)
    srv.cancel(j)
    assert srv.drain(timeout_s=300)
    other = dict(kb, dt=kb["dt"] * 1.001)
    with pytest.raises(E) as e:
        srv.submit_resume(checkpoint=snap, mode="continue", **other)
    assert e.value.status == 1
    with pytest.raises(E) as e:
        srv.submit_resume(checkpoint=snap, mode="continue", method="ensemble_lbfgs", **kb)
    assert e.value.status == 1
    srv.close()


def test_python_resume_optimization(pg, ctx):
    """resume_optimization on the solo optimiser: histories concatenated,
    iterations added, resumed_from_iter recorded (Checkpoint.jl:220-298)."""
    X = np.array([[0, 1], [1, 0]], complex)
    Y = np.array([[0, -1j], [1j, 0]], complex)
    Z = np.diag([1.0, -1.0]).astype(complex)
    system = pg.quantum_system(0.3 * Z, [X, Y])
    tgt = pg.unitary_target(X)
    cs = pg.ControlSequence.from_controls(np.full((2, 20), 0.1), 0.05)
    r1 = pg.grape_optimize(system, tgt, cs, pg.GRAPEConfig(max_iter=8, step_size=0.2))
    ck = pg.create_checkpoint(r1.n_iterations, r1.controls, r1.fidelity, r1.fidelity_history,
                              r1.gradient_norm_history, {}, system, {"dt": 0.05})
    r2 = pg.resume_optimization(ck, system, tgt, additional_iterations=6, verbose=False)
    fresh = pg.grape_optimize(system, tgt, pg.ControlSequence.from_controls(r1.controls, 0.05),
                              pg.GRAPEConfig(max_iter=6))
    assert r2.n_iterations == r1.n_iterations + fresh.n_iterations
    assert r2.fidelity_history == list(r1.fidelity_history) + list(fresh.fidelity_history)
    assert r2.gradient_norm_history == list(r1.gradient_norm_history) + list(fresh.gradient_norm_history)
    assert r2.fidelity == fresh.fidelity and np.array_equal(r2.controls, fresh.controls)
    assert r2.metadata["resumed_from_iter"] == r1.n_iterations
    r3 = pg.resume_optimization(ck, system, tgt, additional_iterations=4, optimizer="lbfgs", verbose=False)
    assert r3.n_iterations >= r1.n_iterations and r3.fidelity >= ck.F_opt - 1e-12
