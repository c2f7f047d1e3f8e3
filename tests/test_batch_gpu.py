"""Batched uneven problems (one CUDA graph per evaluation / iteration).

Each problem in a batch runs the kernels of its solo evaluation, so batched
objectives and gradients must be bit-identical to solo ones, and the batched
grape_optimize ascent must follow the reference step rule (GRAPE.jl:309-334,
:261-268) applied to the solo evaluations.
"""
import numpy as np
import pytest

from oracle import members as mb
import fx
from test_parity_gpu import to_gpu

pytestmark = pytest.mark.gpu


def _small_uneven(n=12, seed=21, precision="mixed"):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        d = [2, 3, 4, 8, 16, 32][i % 6]
        prob, u0 = fx.uneven_problem(rng, d=d, n_t=int(rng.integers(5, 40)), n_members=int(rng.integers(1, 6)))
        out.append((prob, u0))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_eval_bit_identical_to_solo(pg, precision):
    cases = _small_uneven(precision=precision)
    solo = []
    for prob, u0 in cases:
        p = to_gpu(pg, prob, "exact", precision=precision)
        solo.append(p.eval(u0))
        p.close()
    probs = [to_gpu(pg, prob, "exact", precision=precision) for prob, _ in cases]
    b = pg.Batch(probs, n_streams=4)
    for i, (_, u0) in enumerate(cases):
        b.set_controls(i, u0)
    F = b.eval()
    for i, (Fs, Gs) in enumerate(solo):
        assert F[i] == Fs
        _, G = b.get_controls(i)
        assert np.array_equal(G, Gs)
    F2 = b.eval()                       # graph relaunch gives the same numbers
    assert np.array_equal(F, F2)
    b.close()
    for p in probs:
        p.close()


def test_batch_recaptures_after_a_member_changes(pg):
    """A setter on a member problem (here a drift ramp) invalidates the batch's
    captured graphs: the next batch evaluation matches the changed problem
    evaluated alone."""
    cases = _small_uneven(n=6, seed=23)
    probs = [to_gpu(pg, prob, "exact", precision="mixed") for prob, _ in cases]
    b = pg.Batch(probs, n_streams=2)
    for i, (_, u0) in enumerate(cases):
        b.set_controls(i, u0)
    F1 = b.eval()
    prob, u0 = cases[4]
    rng = np.random.default_rng(9)
    R = rng.standard_normal((1, prob.D, prob.D)) * 0.3
    R = (R + R.transpose(0, 2, 1)) * np.abs(prob.drifts).max()
    probs[4].set_drift_ramp(R, np.zeros(prob.n_members, int), np.linspace(0, 1, prob.n_t))
    F2 = b.eval()
    Fs, _ = probs[4].eval(u0)
    assert F2[4] == Fs and F2[4] != F1[4]
    assert np.array_equal(np.delete(F2, 4), np.delete(F1, 4))
    b.close()
    for p in probs:
        p.close()


def test_batch_iterate_follows_grape_step_rule(pg):
    cases = _small_uneven(n=6, seed=5)
    probs = [to_gpu(pg, prob, "exact", precision="mixed") for prob, _ in cases]
    b = pg.Batch(probs, n_streams=3)
    for i, (_, u0) in enumerate(cases):
        b.set_controls(i, u0)
    n_iter, step0 = 6, 0.05
    trace = b.iterate(n_iter, step_size=step0, adapt_step_size=True)
    for i, (prob, u0) in enumerate(cases):
        p = to_gpu(pg, prob, "exact", precision="mixed")
        u = u0.copy()
        F_prev, _ = p.eval(u, want_grad=False)
        step, hist = step0, []
        for _ in range(n_iter):                   # grape_optimize without convergence exits
            F, G = p.eval(u)
            hist.append(F)
            d = F - F_prev
            step = min(max(step * (1.05 if d > 0 else (0.5 if d < -1e-14 else 1.0)), 1e-10), 10.0)
            u = u + step * G
            F_prev = F
        assert np.allclose(trace[:, i], hist, rtol=0, atol=1e-12)
        ub, _ = b.get_controls(i)
        assert np.allclose(ub, u, rtol=0, atol=1e-12 * max(1.0, np.abs(u).max()))
        p.close()
    b.close()
    for p in probs:
        p.close()


def test_batch_rejects_foreign_or_duplicate_problems(pg):
    cases = _small_uneven(n=2)
    p0 = to_gpu(pg, cases[0][0], "exact")
    with pytest.raises(pg._abi.PgxError):
        pg.Batch([p0, p0])
    other = pg.Context(0)
    p1 = to_gpu(pg, cases[1][0], "exact", ctx=other)
    with pytest.raises(pg._abi.PgxError):
        pg.Batch([p0, p1])
    p0.close()
    p1.close()
    other.close()
