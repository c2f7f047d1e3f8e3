"""The oracle-free error estimate pgx_eval reports (pgx_eval_stats.residual):
unitarity of U_total for Hermitian gate problems, trace preservation of the
Liouvillian propagator for Lindblad gate problems, and norm / trace drift of
the propagated states.  Each is checked against the same quantity computed
on the host from the oracle's propagators, and against the bar the
reference's own tests set for propagators (unitarity < 1e-10,
MathematicalCorrectness.jl:40-46,77-81)."""
import numpy as np
import pytest

import fx
from oracle import members as mb

pytestmark = pytest.mark.gpu

W = fx.W


def _unitarity(U):
    return np.max(np.abs(U.conj().T @ U - np.eye(U.shape[0])))


def _oracle_total(prob, u, m):
    U = np.eye(prob.D, dtype=complex)
    for k in range(prob.n_t):
        U = mb._propagator(prob, prob.generator_of(m, u[:, k]), prob.dt[k]) @ U
    return U


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gate_unitarity_residual(pg, ctx, precision):
    spec, u0 = W.spin4_ensemble(n_t=60, n_off=3, n_b1=2)
    p = pg.Problem(ctx=ctx, **spec.problem_kwargs("exact", precision))
    F, G, st = p.eval(u0, stats=True)
    F2, _, st2 = p.eval(u0, want_grad=False, stats=True)
    p.close()
    assert st["residual_kind"] == "unitarity" and st2["residual_kind"] == "unitarity"
    assert 0.0 <= st["residual"] <= (1e-12 if precision == "fp64" else 1e-11), st["residual"]
    assert st2["residual"] == st["residual"]          # same U_total either way
    # the oracle's own U_total has a residual of the same order
    prob = mb.Problem.from_spec(spec)
    ref = max(_unitarity(_oracle_total(prob, u0, m)) for m in range(prob.n_members))
    assert ref <= 1e-12
    assert st["n_launches"] > 0


def test_lindblad_gate_trace_residual(pg, ctx):
    spec, u0 = W.lindblad_gate(seed=3, n_qubits=2, n_t=30, n_draws=3)
    for precision in ("fp64", "mixed"):
        p = pg.Problem(ctx=ctx, **spec.problem_kwargs("exact", precision))
        _, _, st = p.eval(u0, stats=True)
        p.close()
        assert st["residual_kind"] == "trace"
        assert 0.0 <= st["residual"] <= 1e-11, (precision, st["residual"])


def test_state_norm_residual(pg, ctx):
    spec, u0 = W.single_qubit_transfer(explicit_init=True)
    p = pg.Problem(ctx=ctx, **spec.problem_kwargs("exact", "fp64"))
    _, _, st = p.eval(u0, stats=True)
    _, _, st_f = p.eval(u0, want_grad=False, stats=True)
    p.close()
    assert st["residual_kind"] == "norm" and 0.0 <= st["residual"] <= 1e-13
    assert st_f["residual_kind"] == "none" and st_f["residual"] == 0.0


def test_lindblad_state_trace_residual(pg, ctx):
    Ix, Iy, Iz = W.SX / 2, W.SY / 2, W.SZ / 2
    sm = np.array([[0, 1], [0, 0]], complex)
    drifts = np.stack([pg.build_drift_liouvillian(2 * np.pi * off * Iz, [sm], [20.0]) for off in (-300.0, 400.0)])
    ctrls = np.stack([pg.build_control_liouvillian(2 * np.pi * 5e3 * H) for H in (Ix, Iy)])
    r0 = pg.pure_state_to_vec_rho(np.array([1, 0], complex))
    r1 = pg.pure_state_to_vec_rho(np.array([0, 1], complex))
    u0 = 0.3 * np.random.default_rng(2).standard_normal((2, 25))
    p = pg.Problem(drifts, ctrls, np.full(25, 4e-6), ctx=ctx, generator="liouvillian", target="states",
                   fidelity="real", states_init=r0[None], states_target=r1[None], member_drift=[0, 1],
                   grad_mode="exact", precision="fp64")
    _, _, st = p.eval(u0, stats=True)
    p.close()
    assert st["residual_kind"] == "state_trace" and 0.0 <= st["residual"] <= 1e-12, st


def test_autotune_plan_is_reused_by_later_problems(pg, ctx):
    """pgx_autotune records its plan under the problem's key; problems created
    afterwards with the same key (on any context, the server's included)
    start from it, with results unchanged."""
    pg.plan_clear()
    spec, u0 = W.spin4_ensemble(n_t=40, n_off=3, n_b1=2)
    kw = spec.problem_kwargs("exact", "mixed")
    assert pg.plan_lookup(**kw) is None
    a = pg.Problem(ctx=ctx, **kw)
    default = a.teams
    F0, G0 = a.eval(u0)
    a.autotune(u0, reps=1)
    tuned = a.teams
    a.close()
    assert pg.plan_lookup(**kw) == tuned
    spec2, u2 = W.spin4_ensemble(seed=9, n_t=25, n_off=2, n_b1=2)       # same key, other sizes
    other = pg.Context(0)
    b = pg.Problem(ctx=other, **spec2.problem_kwargs("exact", "mixed"))
    assert b.teams == tuned
    b.close()
    other.close()
    c = pg.Problem(ctx=ctx, **kw)
    F1, G1 = c.eval(u0)
    c.close()
    assert F1 == F0 and np.array_equal(G1, G0)
    # another key (FP64 path, or another grad mode) is not affected
    assert pg.plan_lookup(**spec.problem_kwargs("ref_grape", "mixed")) is None
    pg.plan_clear()
    assert pg.plan_lookup(**kw) is None
    d = pg.Problem(ctx=ctx, **kw)
    assert d.teams == default
    d.close()
