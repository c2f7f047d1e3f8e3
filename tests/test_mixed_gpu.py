"""Mixed-precision path (PGX_PREC_MIXED) against the FP64 oracle.

Bars: |dF| <= 1e-8 (the objective runs through double-float propagators and
chain) and max|dG|/max|G| <= 1e-4 (the gradient is FP32 by design).
"""
import numpy as np
import pytest

from oracle import members as mb
import fx
from test_parity_gpu import rand_herm, random_gate_problem, to_gpu

pytestmark = pytest.mark.gpu

F_TOL_MIXED = 1e-8
G_RTOL_MIXED = 1e-4


def check(F, G, Fo, Go):
    assert abs(F - Fo) <= F_TOL_MIXED, (F, Fo, abs(F - Fo))
    err = np.max(np.abs(G - Go)) / max(np.max(np.abs(Go)), 1e-300)
    assert err <= G_RTOL_MIXED, err
    return abs(F - Fo), err


@pytest.mark.parametrize("mode", ["ref_grape", "ref_mr", "exact"])
@pytest.mark.parametrize("d", [2, 4, 7, 16, 32, 40])
def test_mixed_random_gate(pg, mode, d):
    rng = np.random.default_rng(300 + d)
    prob, u0 = random_gate_problem(rng, d, n_t=8, n_members=3, dt=0.3 / np.sqrt(d))
    p = to_gpu(pg, prob, mode, precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    check(F, G, Fo, Go)
    p.close()


@pytest.mark.parametrize("d", [2, 8, 16])
@pytest.mark.parametrize("target_norm", [0.004, 0.03, 0.1, 0.16, 0.4, 1.5, 6.0])
def test_mixed_expm_schedules_across_norms(pg, target_norm, d):
    """The df expm picks its Paterson-Stockmeyer block size (2, 3, 4), degree
    and squarings per slice from ||A||_1: these norms walk through each kind
    of schedule (q = 2 at the smallest, q = 3 degree 9, q = 4 degree 12 / 16,
    squarings at the largest).  F stays at df accuracy against the oracle,
    for the register-resident kernel (d = 2, 8: one slice per 2 and per 16
    lanes) and the shared-memory teams (d = 16)."""
    rng = np.random.default_rng(int(1e4 * target_norm) + d)
    prob, u0 = random_gate_problem(rng, d, n_t=12, n_members=2, dt=1.0)
    A = [prob.drifts[0] + sum(u0[j, k] * prob.controls[j] for j in range(prob.n_c)) for k in range(prob.n_t)]
    nrm = max(np.abs(a).sum(axis=0).max() for a in A)
    prob.dt = np.full(prob.n_t, target_norm / nrm)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    dF, _ = check(F, G, Fo, Go)
    assert dF <= 1e-12, dF
    p.close()


def test_mixed_one_qubit_lindblad_register_path(pg):
    """A 1-qubit Lindblad gate (D = 4 superoperators, non-Hermitian): the
    register-resident expm against the FP64 oracle."""
    prob, u0 = fx.lindblad_gate(n_qubits=1, n_t=20, n_draws=3)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F, G = p.eval(u0)
    p.close()
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    dF, dG = check(F, G, Fo, Go)
    print(f"1-qubit Lindblad mixed: |dF| = {dF:.2e}, grad rel = {dG:.2e}")


def test_mixed_lindblad_superoperator(pg):
    prob, u0 = fx.lindblad_3q(n_t=3, n_draws=2)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    check(F, G, Fo, Go)
    p.close()


def test_mixed_lindblad_symmetric_products_parallel_in_time(pg):
    """D = 64 Lindblad superoperators preserve Hermiticity, so the mixed expm
    and forward chain keep half of each product and mirror the rest; 60
    slices put the forward chain in its parallel-in-time form."""
    prob, u0 = fx.lindblad_3q(n_t=60, n_draws=2)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    check(F, G, Fo, Go)
    p.close()


def test_mixed_lindblad_symmetric_path_matches_full_path(pg):
    """A ramp operator that breaks the symmetry but enters with tau = 0 leaves
    the generator unchanged and sends the evaluation through the full
    products: both paths agree to df rounding."""
    prob, u0 = fx.lindblad_3q(n_t=40, n_draws=2)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F1, G1 = p.eval(u0)
    rng = np.random.default_rng(5)
    D = prob.D
    R = rng.standard_normal((1, D, D)) + 1j * rng.standard_normal((1, D, D))
    p.set_drift_ramp(R, np.zeros(prob.n_members, int), np.zeros(prob.n_t))
    F2, G2 = p.eval(u0)
    assert abs(F1 - F2) <= 1e-12, (F1, F2)
    assert np.max(np.abs(G1 - G2)) <= 1e-6 * np.max(np.abs(G1))
    p.set_drift_ramp(np.zeros((0, D, D)), [], [])
    F3, G3 = p.eval(u0)
    assert F3 == F1 and np.array_equal(G3, G1)
    p.close()


def test_mixed_lindblad_set_drifts_updates_symmetry(pg):
    """Replacing the drifts re-checks the symmetry: asymmetric drifts take the
    full products (parity with the oracle), symmetric ones the halved ones."""
    prob, u0 = fx.lindblad_3q(n_t=6, n_draws=2)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F0, G0 = p.eval(u0)
    orig = prob.drifts.copy()
    rng = np.random.default_rng(12)
    pert = 1e-6 * np.abs(orig).max() * (rng.standard_normal(orig.shape) + 1j * rng.standard_normal(orig.shape))
    prob.drifts = orig + pert
    p.set_drifts(prob.drifts)
    F1, G1 = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    check(F1, G1, Fo, Go)
    p.set_drifts(orig)
    F2, G2 = p.eval(u0)
    assert F2 == F0 and np.array_equal(G2, G0)
    p.close()


def test_mixed_lindblad_asymmetric_generator(pg):
    """A Liouvillian whose drift does not preserve Hermiticity (relative
    defect 1e-6, far above the 1e-12 the symmetric path admits, small enough
    to keep the dynamics bounded) takes the full products."""
    prob, u0 = fx.lindblad_3q(n_t=6, n_draws=2)
    rng = np.random.default_rng(8)
    prob.drifts = prob.drifts + 1e-6 * np.abs(prob.drifts).max() * (
        rng.standard_normal(prob.drifts.shape) + 1j * rng.standard_normal(prob.drifts.shape))
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


@pytest.mark.parametrize("d", [4, 16, 32, 40])
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


@pytest.mark.parametrize("d,teams", [(16, (32, 64, 128, 256)), (32, (128, 256)), (64, (256, 512))])
def test_gradient_team_sizes_bit_identical(pg, d, teams):
    """Every CUDA-core gradient team gives the same bits: the Frechet product
    pairs run in one pass over k up to 8 outputs per lane (d = 16 at T = 32,
    d = 64 at T = 512) and in two passes beyond (d = 64 at T = 256), with the
    same order of terms."""
    rng = np.random.default_rng(900 + d)
    prob, u0 = random_gate_problem(rng, d, n_t=8, n_members=3, dt=0.3 / np.sqrt(d))
    p = to_gpu(pg, prob, "exact", precision="mixed")
    ref = None
    for t in teams:
        p.set_teams(grad=t)
        assert p.teams[1] == t
        F, G = p.eval(u0)
        if ref is None:
            ref = (F, G)
        else:
            assert F == ref[0] and np.array_equal(G, ref[1]), t
    p.close()


MODES = ("ref_grape", "ref_mr", "exact")


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("explicit", [False, True])
def test_mixed_single_qubit_transfer(pg, mode, explicit):
    """The reference's CPU-runnable case (1 qubit, 100 slices, state target),
    legacy and explicit initial-state semantics."""
    prob, u0 = fx.single_qubit_transfer(explicit_init=explicit)
    p = to_gpu(pg, prob, mode, precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    check(F, G, Fo, Go)
    p.close()


def _state_pairs(rng, d, fid, n_t=9):
    drifts = np.stack([rand_herm(rng, d, 0.5) for _ in range(3)])
    ctrls = np.stack([rand_herm(rng, d, 0.5) for _ in range(2)])
    si = np.stack([fx.haar_unitary(rng, d)[:, 0] for _ in range(3)])
    st = np.stack([fx.haar_unitary(rng, d)[:, 0] for _ in range(3)])
    prob = mb.Problem(drifts=drifts, controls=ctrls, dt=rng.uniform(0.05, 0.2, n_t),
                      member_drift=np.repeat(np.arange(3), 2), member_scale=np.tile([0.8, 1.3], 3),
                      n_members=6, target="states", fidelity=fid, states_init=si, states_target=st)
    return prob, rng.uniform(-1, 1, (2, n_t))


@pytest.mark.parametrize("fid", ["square", "real", "modulus"])
@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("d", [2, 3, 6, 16, 40])
def test_mixed_state_pairs(pg, fid, mode, d):
    """MR state transfer (GRAPEState.jl:136-250) with three pairs per member,
    drifts x pwr members; d = 40 pads to the D = 64 kernels."""
    prob, u0 = _state_pairs(np.random.default_rng(11 * d), d, fid)
    p = to_gpu(pg, prob, mode, precision="mixed")
    F, G = p.eval(u0)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    check(F, G, Fo, Go)
    F1, _ = p.eval(u0, want_grad=False)
    assert F1 == F
    p.close()


@pytest.mark.parametrize("mode", MODES)
def test_mixed_lindblad_states(pg, mode):
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
    p = to_gpu(pg, prob, mode, precision="mixed")
    F, G, st = p.eval(u0, stats=True)
    Fo, Go = mb.eval_problem(prob, u0, mode)
    check(F, G, Fo, Go)
    assert st["residual_kind"] == "state_trace" and st["residual"] <= 1e-12
    p.close()


def test_mixed_legacy_gradient_states(pg):
    """grape_optimize's gradient runs from the target state while F uses
    the initial state (Gradients.jl:153-157): both passes in mixed precision
    against the FP64 path."""
    prob, u0 = _state_pairs(np.random.default_rng(3), 4, "square")
    gs = np.roll(prob.states_init, 1, axis=0)
    kw = dict(grad_states_init=gs)
    p64, pmx = to_gpu(pg, prob, "exact", **kw), to_gpu(pg, prob, "exact", precision="mixed", **kw)
    (F, G), (Fm, Gm) = p64.eval(u0), pmx.eval(u0)
    assert abs(Fm - F) <= F_TOL_MIXED
    assert np.max(np.abs(Gm - G)) <= G_RTOL_MIXED * np.max(np.abs(G))
    assert abs(Fm - pmx.eval(u0, want_grad=False)[0]) == 0.0
    p64.close()
    pmx.close()


def test_mixed_states_residual_and_autotune(pg):
    prob, u0 = _state_pairs(np.random.default_rng(5), 16, "real", n_t=20)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F1, G1, st = p.eval(u0, stats=True)
    assert st["residual_kind"] == "norm" and st["residual"] <= 1e-12, st
    report = p.autotune(u0, reps=1)
    assert "expm_mx" in report and "grad_mx" in report
    F2, G2 = p.eval(u0)
    assert F1 == F2 and np.array_equal(G1, G2)
    p.close()


def test_mixed_states_full_size_mr_ensemble(pg):
    """The benchmark system as an MR state-transfer ensemble (231 members x
    1000 slices, d = 16, |0000> -> |1111> and a second pair): mixed against
    the FP64 GPU path at the mixed bars."""
    spec, u0 = fx.W.spin4_ensemble()
    kw = spec.problem_kwargs("exact", "fp64")
    e = np.eye(16, dtype=complex)
    kw.update(target="states", fidelity="square", target_op=None, states_init=np.stack([e[0], e[5]]),
              states_target=np.stack([e[15], e[10]]), member_weight=None)
    p64 = pg.Problem(**kw)
    pmx = pg.Problem(**dict(kw, precision="mixed"))
    (F, G), (Fm, Gm) = p64.eval(u0), pmx.eval(u0)
    print(f"mixed states vs FP64: |dF| = {abs(Fm - F):.3e}, "
          f"grad rel = {np.max(np.abs(Gm - G)) / np.max(np.abs(G)):.3e}")
    assert abs(Fm - F) <= F_TOL_MIXED
    assert np.max(np.abs(Gm - G)) <= G_RTOL_MIXED * np.max(np.abs(G))
    p64.close()
    pmx.close()
