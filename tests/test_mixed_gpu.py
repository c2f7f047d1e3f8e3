"""Mixed-precision path (PGX_PREC_MIXED) against the FP64 oracle.

Bars: |dF| <= 1e-8 (the objective runs through double-float propagators and
chain) and max|dG|/max|G| <= 1e-4 (the gradient is FP32 by design).
"""
import numpy as np
import pytest

from oracle import members as mb
import fx
from test_parity_gpu import random_gate_problem, to_gpu

pytestmark = pytest.mark.gpu

F_TOL_MIXED = 1e-8
G_RTOL_MIXED = 1e-4


def check(F, G, Fo, Go):
    assert abs(F - Fo) <= F_TOL_MIXED, (F, Fo, abs(F - Fo))
    err = np.max(np.abs(G - Go)) / max(np.max(np.abs(Go)), 1e-300)
    assert err <= G_RTOL_MIXED, err
    return abs(F - Fo), err


@pytest.mark.parametrize("mode", ["ref_grape", "ref_mr", "exact"])
@pytest.mark.parametrize("d", [2, 4, 7, 16, 32])
def test_mixed_random_gate(pg, mode, d):
    rng = np.random.default_rng(300 + d)
    prob, u0 = random_gate_problem(rng, d, n_t=8, n_members=3, dt=0.3 / np.sqrt(d))
    p = to_gpu(pg, prob, mode, precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    check(F, G, Fo, Go)
    p.close()


def test_mixed_lindblad_superoperator(pg):
    prob, u0 = fx.lindblad_3q(n_t=3, n_draws=2)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    check(F, G, Fo, Go)
    p.close()


def test_mixed_needs_squarings(pg):
    rng = np.random.default_rng(11)
    prob, u0 = random_gate_problem(rng, 8, n_t=5, dt=0.9, scale=3.0)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    check(F, G, Fo, Go)
    p.close()


def test_mixed_full_size_bench_workload(pg):
    """231 members x 1000 slices, d = 16: |dF| <= 1e-8 against the FP64 C
    oracle; the FP64 GPU path is the second reference for the gradient."""
    from oracle import cpu_port
    prob, u0 = fx.spin4_ensemble()
    pm = to_gpu(pg, prob, "exact", precision="mixed")
    F, G = pm.eval(u0)
    Fo, Go = cpu_port.CpuProblem(prob, "exact").eval(u0)
    dF, dG = check(F, G, Fo, Go)
    print(f"mixed vs FP64 oracle: |dF| = {dF:.3e}, grad rel = {dG:.3e}")
    pm.close()


@pytest.mark.parametrize("d", [4, 16, 32])
def test_autotune_keeps_results_bit_identical(pg, d):
    rng = np.random.default_rng(500 + d)
    prob, u0 = random_gate_problem(rng, d, n_t=12, n_members=5, dt=0.3 / np.sqrt(d))
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F1, G1 = p.eval(u0)
    report = p.autotune(u0, reps=2)
    assert "expm_mx" in report and "grad_mx" in report and "-> T=" in report
    F2, G2 = p.eval(u0)
    assert F1 == F2 and np.array_equal(G1, G2)
    p.close()


def test_mixed_states_target_is_refused(pg):
    prob, u0 = fx.single_qubit_transfer()
    with pytest.raises(pg._abi.PgxError) as ei:
        to_gpu(pg, prob, "exact", precision="mixed")
    assert ei.value.status == 6
