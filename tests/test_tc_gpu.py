"""The tensor-core (tcgen05) product engine: batched complex 64 x 64
products P Q against numpy in FP64.

3xTF32 (hi/lo operand split, FP32 accumulation) must reach FP32-class
accuracy; plain TF32 (one pass) must not, which shows that the split passes
actually run.  The batch is larger than one item per SM, so the persistent
CTAs loop over several items and reuse TMEM and the staging buffers.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cmm(pg, P, Q, passes, a_in_tmem=0):
    A = pg._abi
    n = P.shape[0]
    f = A.lib().pgx_diag_tc_cmatmul64
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
    buf = lambda M: np.ascontiguousarray(np.swapaxes(M, -1, -2)).astype(np.complex128)  # column-major
    Pb, Qb = buf(P), buf(Q)
    Cb = np.zeros_like(Pb)
    st = f(Pb.ctypes.data, Qb.ctypes.data, Cb.ctypes.data, n, passes, a_in_tmem)
    assert st == 0, st
    return np.swapaxes(Cb, -1, -2)


def _rel(Cg, Cr):
    return np.max(np.abs(Cg - Cr), axis=(1, 2)) / np.max(np.abs(Cr), axis=(1, 2))


@pytest.mark.parametrize("a_in_tmem", [0, 1])
def test_tc_cmatmul64_3xtf32_is_fp32_accurate(pg, a_in_tmem):
    """modes 0 and 1: 3xTF32 with the left factor in shared memory / in TMEM"""
    rng = np.random.default_rng(64)
    n = 300
    P = rng.standard_normal((n, 64, 64)) + 1j * rng.standard_normal((n, 64, 64))
    Q = rng.standard_normal((n, 64, 64)) + 1j * rng.standard_normal((n, 64, 64))
    # near-identity factors with small off-diagonal parts, as in Taylor products
    P[:8] = np.eye(64) + 0.01 * P[:8]
    Q[:8] = np.eye(64) + 0.03 * Q[:8]
    # the FP32 rounding of the inputs is part of the kernel's input
    P32 = P.astype(np.complex64).astype(np.complex128)
    Q32 = Q.astype(np.complex64).astype(np.complex128)
    ref = P32 @ Q32
    C3 = _cmm(pg, P, Q, 3, a_in_tmem)
    e3 = _rel(C3, ref)
    assert np.all(np.isfinite(C3))
    assert e3.max() <= 5e-6, e3.max()
    C1 = _cmm(pg, P, Q, 1, a_in_tmem)
    e1 = _rel(C1, ref)
    assert 1e-5 <= np.median(e1) <= 2e-2, np.median(e1)
    print(f"3xTF32 max rel {e3.max():.2e}, TF32 median rel {np.median(e1):.2e}")


def test_tc_cmatmul64_3xfp16_is_fp32_accurate(pg):
    """mode 2, the gradient's path: 3xFP16 with the left factor in TMEM"""
    rng = np.random.default_rng(65)
    n = 300
    P = rng.standard_normal((n, 64, 64)) + 1j * rng.standard_normal((n, 64, 64))
    Q = rng.standard_normal((n, 64, 64)) + 1j * rng.standard_normal((n, 64, 64))
    P[:8] = np.eye(64) + 0.01 * P[:8]
    Q[:8] = np.eye(64) + 0.03 * Q[:8]
    P32 = P.astype(np.complex64).astype(np.complex128)
    Q32 = Q.astype(np.complex64).astype(np.complex128)
    ref = P32 @ Q32
    C3 = _cmm(pg, P, Q, 3, 2)
    e3 = _rel(C3, ref)
    assert np.all(np.isfinite(C3))
    assert e3.max() <= 5e-6, e3.max()
    print(f"3xFP16 max rel {e3.max():.2e}")


def test_tc_cmatmul64_rejects_bad_arguments(pg):
    f = pg._abi.lib().pgx_diag_tc_cmatmul64
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
    buf = np.zeros(2 * 4096)
    assert f(buf.ctypes.data, buf.ctypes.data, buf.ctypes.data, 1, 2, 0) == 1
    assert f(buf.ctypes.data, buf.ctypes.data, buf.ctypes.data, 0, 3, 0) == 1
    assert f(buf.ctypes.data, buf.ctypes.data, buf.ctypes.data, 1, 1, 2) == 1


# ---- df-class products: CUDA-core df against tensor-core slicing ----------

def _dfcmm(pg, P, Q, engine, reps=1):
    f = pg._abi.lib().pgx_diag_dfcmatmul64
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_float)]
    buf = lambda M: np.ascontiguousarray(np.swapaxes(M, -1, -2)).astype(np.complex128)
    Pb, Qb = buf(P), buf(Q)
    Cb = np.zeros_like(Pb)
    ms = C.c_float(0.0)
    st = f(Pb.ctypes.data, Qb.ctypes.data, Cb.ctypes.data, P.shape[0], engine, reps, C.byref(ms))
    assert st == 0, st
    return np.swapaxes(Cb, -1, -2), ms.value


def _df_inputs(rng, n):
    """Random Gaussian factors, near-identity factors (Taylor terms), unitary
    factors (squarings), and factors with every entry of one sign and near
    the slicing range's edge (every level sum near its bound)."""
    P = rng.standard_normal((n, 64, 64)) + 1j * rng.standard_normal((n, 64, 64))
    Q = rng.standard_normal((n, 64, 64)) + 1j * rng.standard_normal((n, 64, 64))
    P[:8] = np.eye(64) + 0.01 * P[:8]
    Q[:8] = np.eye(64) + 0.03 * Q[:8]
    for k in range(8, 16):
        P[k] = np.linalg.qr(P[k])[0]
        Q[k] = P[k]
    P[16:24] = rng.uniform(0.45, 0.5, (8, 64, 64)) * (1 + 1j)
    Q[16:24] = rng.uniform(0.45, 0.5, (8, 64, 64)) * (1 - 1j)
    return P, Q


def _df_ref(P, Q):
    """The FP64 product of the df roundings of the inputs (the kernels'
    input); its own rounding is ~1e-16."""
    def rdf(x):
        hi = x.astype(np.float32).astype(np.float64)
        return hi + (x - hi).astype(np.float32).astype(np.float64)
    rd = lambda M: rdf(M.real) + 1j * rdf(M.imag)
    return rd(P) @ rd(Q)


# Errors relative to each product's largest entry.  The CUDA-core df product
# (compensated dot products, ~2^-42 here) is the bar the expm was built on;
# the sliced forms drop the levels beyond the last and the bits below slice 5
# (2^-47 of the operand scale): about 2^-41 with levels 0..5 for
# near-identity factors, about 2^-45 with level 6 (numpy emulation of the
# slicing, exact level sums and the FP32 combine: 5.0e-13 and 2.2e-14).
DF_REL = {0: 5e-13, 1: 1e-12, 2: 5e-14}


def test_df_product_engines_reach_df_accuracy(pg):
    """engine 0: the df expm's CUDA-core product; 1, 2: the tensor-core
    product by exact bf16 slicing (levels 0..5, 0..6), on the same inputs."""
    rng = np.random.default_rng(640)
    P, Q = _df_inputs(rng, 300)
    ref = _df_ref(P, Q)
    errs = {}
    for engine in (0, 1, 2):
        Cg, _ = _dfcmm(pg, P, Q, engine)
        assert np.all(np.isfinite(Cg))
        err = np.max(np.abs(Cg - ref), axis=(1, 2)) / np.max(np.abs(ref), axis=(1, 2))
        errs[engine] = err
        print(f"df product engine {engine}: max rel {err.max():.2e}, median {np.median(err):.2e}")
    for engine, err in errs.items():
        assert err.max() <= DF_REL[engine], (engine, err.max(), int(err.argmax()))
    assert errs[2].max() < errs[0].max()


def test_df_product_tensor_core_is_faster_and_deterministic(pg):
    """Times both engines on the same batch (8 products per SM): the
    tensor-core form must beat the CUDA-core df product and reproduce its own
    bits on a rerun."""
    rng = np.random.default_rng(77)
    n = 1216
    P = rng.standard_normal((n, 64, 64)) + 1j * rng.standard_normal((n, 64, 64))
    Q = rng.standard_normal((n, 64, 64)) + 1j * rng.standard_normal((n, 64, 64))
    C0, ms0 = _dfcmm(pg, P, Q, 0, reps=10)
    C1, ms1 = _dfcmm(pg, P, Q, 1, reps=10)
    C1b, _ = _dfcmm(pg, P, Q, 1, reps=1)
    C2, ms2 = _dfcmm(pg, P, Q, 2, reps=10)
    assert np.array_equal(C1, C1b)
    print(f"df products, {n} per launch: CUDA-core {ms0:.3f} ms, tensor-core 21 pairs {ms1:.3f} ms, "
          f"26 pairs {ms2:.3f} ms; speed-up {ms0 / ms1:.2f}x / {ms0 / ms2:.2f}x")
    assert ms1 < ms0


# ---- the D = 64 exact gradient on the tensor-core engine -------------------

from oracle import members as mb  # noqa: E402
import fx  # noqa: E402
from test_parity_gpu import random_gate_problem, to_gpu  # noqa: E402

G_RTOL_MIXED = 1e-4     # the mixed path's gradient bar against the FP64 oracle
G_RTOL_ENGINES = 2e-5   # tensor-core (3xTF32) against CUDA-core (FP32) gradients


def _rel_g(G, Go):
    return np.max(np.abs(G - Go)) / np.max(np.abs(Go))


def test_tc_gradient_lindblad_vs_cuda_core_and_oracle(pg):
    prob, u0 = fx.lindblad_3q(n_t=40, n_draws=4)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    assert p.teams[1] == 1                      # the tensor-core engine is the default here
    F_tc, G_tc = p.eval(u0)
    p.set_teams(0, 512)                         # the CUDA-core FP32 team
    F_cc, G_cc = p.eval(u0)
    p.close()
    assert F_tc == F_cc                         # F does not depend on the gradient kernel
    assert _rel_g(G_tc, G_cc) <= G_RTOL_ENGINES, _rel_g(G_tc, G_cc)
    Fo, Go = mb.eval_gate_exact_adjoint(prob, u0)
    assert abs(F_tc - Fo) <= 1e-8
    assert _rel_g(G_tc, Go) <= G_RTOL_MIXED, _rel_g(G_tc, Go)
    print(f"lindblad D=64: tc vs cuda-core {_rel_g(G_tc, G_cc):.2e}, tc vs oracle {_rel_g(G_tc, Go):.2e}, "
          f"cuda-core vs oracle {_rel_g(G_cc, Go):.2e}")


@pytest.mark.parametrize("d", [40, 64])
def test_tc_gradient_hermitian_padded_vs_oracle(pg, d):
    rng = np.random.default_rng(900 + d)
    prob, u0 = random_gate_problem(rng, d, n_t=10, n_members=3, dt=0.3 / np.sqrt(d))
    p = to_gpu(pg, prob, "exact", precision="mixed")
    assert p.teams[1] == 1
    F, G = p.eval(u0)
    p.close()
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    assert abs(F - Fo) <= 1e-8
    assert _rel_g(G, Go) <= G_RTOL_MIXED, _rel_g(G, Go)


def test_tc_gradient_runs_twice_bit_identically(pg):
    """Persistent CTAs reuse TMEM, the staging buffers and the barrier phase
    across units and launches: a second evaluation reproduces the first."""
    prob, u0 = fx.lindblad_3q(n_t=200, n_draws=2)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F1, G1 = p.eval(u0)
    F2, G2 = p.eval(u0)
    p.close()
    assert F1 == F2 and np.array_equal(G1, G2)


def test_state_targets_at_64_keep_the_cuda_core_gradient(pg):
    rng = np.random.default_rng(77)
    prob, u0 = random_gate_problem(rng, 40, n_t=6, n_members=2, dt=0.05)
    kw = dict(generator=prob.generator, target="states", fidelity="square",
              states_init=np.eye(40)[:2], states_target=np.eye(40)[2:4], grad_mode="exact", precision="mixed")
    p = pg.Problem(prob.drifts, prob.controls, prob.dt, **kw)
    assert p.teams[1] == 512
    with pytest.raises(pg._abi.PgxError):
        p.set_teams(0, 1)                        # not admitted for state targets
    p.close()


def test_kernel_shared_memory_limits_grow_with_later_problems():
    """A fresh process evaluates a D = 64 problem with 2 controls, then one with
    6: kernels whose shared memory depends on the problem (the trace pass
    holds the controls) must accept the larger launch after the smaller one."""
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    code = (
        "import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
        "import numpy as np, __graft_entry__ as ge\n"
        "pg = ge.load_package()\n"
        "import fx\n"
        "from test_parity_gpu import random_gate_problem, to_gpu\n"
        "prob, u0 = random_gate_problem(np.random.default_rng(1), 40, n_t=4, n_members=2, dt=0.05)\n"
        "p = to_gpu(pg, prob, 'exact', precision='mixed'); p.eval(u0); p.close()\n"
        "prob, u0 = fx.lindblad_3q(n_t=4, n_draws=2)\n"
        "p = to_gpu(pg, prob, 'exact', precision='mixed'); F, G = p.eval(u0); p.close()\n"
        "assert np.all(np.isfinite(G)); print('ok')\n" % (str(root), str(root / "tests")))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]


def test_tc_gradient_refuses_values_beyond_fp16_range(pg):
    """A (non-physical) D = 64 Liouvillian that grows by e^24 per slice drives
    the squarings past the FP16 operand limit (the last squaring's factor
    exp(A/2) reaches e^12 ~ 1.6e5 > 32768; F ~ e^48 and G stay finite in FP32
    and FP64): the tensor-core gradient
    reports PGX_ERR_NONFINITE instead of returning a wrong gradient, and the
    CUDA-core team evaluates the same problem."""
    D = 64
    rng = np.random.default_rng(3)
    drift = 24.0 * np.eye(D, dtype=complex)
    ctrl = 0.01 * (rng.standard_normal((1, D, D)) + 1j * rng.standard_normal((1, D, D)))
    kw = dict(generator="liouvillian", target="gate", target_op=np.eye(D), grad_mode="exact", precision="mixed")
    p = pg.Problem(drift[None], ctrl, np.array([1.0]), **kw)
    assert p.teams[1] == 1
    with pytest.raises(pg._abi.PgxError) as ei:
        p.eval(np.zeros((1, 1)))
    assert ei.value.status == 10          # PGX_ERR_NONFINITE
    p.set_teams(0, 512)                   # the CUDA-core FP32 gradient
    F, G = p.eval(np.zeros((1, 1)))
    assert np.isfinite(F) and np.all(np.isfinite(G))
    p.close()


# ---- the D = 64 df expm on the tensor cores -------------------------------

@pytest.mark.parametrize("dt", [0.002, 0.02, 0.1, 0.5])
def test_tc_expm_matches_cuda_core_expm_and_oracle(pg, dt):
    """Hermitian D = 64 gate problems whose slice norms (~0.1 .. ~25) select
    different degrees, block sizes and squaring counts: the tensor-core expm
    (the default at D = 64) against the CUDA-core df expm (team 256) and the
    FP64 oracle."""
    rng = np.random.default_rng(int(dt * 1000) + 11)
    prob, u0 = random_gate_problem(rng, 64, n_t=6, n_members=2, dt=dt)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    assert p.teams[0] == 1
    F_tc, G_tc = p.eval(u0)
    p.set_teams(256, 0)
    F_cc, G_cc = p.eval(u0)
    p.close()
    Fo, Go = mb.eval_problem(prob, u0, "exact")
    assert abs(F_tc - F_cc) <= 1e-11, (F_tc, F_cc)
    assert abs(F_tc - Fo) <= 1e-8
    assert _rel_g(G_tc, Go) <= G_RTOL_MIXED, _rel_g(G_tc, Go)
    print(f"dt {dt}: |F_tc - F_cc| {abs(F_tc - F_cc):.1e}, |F_tc - F_oracle| {abs(F_tc - Fo):.1e}")


def test_tc_expm_lindblad_and_state_targets(pg):
    """The 3-qubit Lindblad gate (non-Hermitian superoperators) and a D = 64
    state-transfer problem: the tensor-core expm against the CUDA-core expm
    and the oracle."""
    prob, u0 = fx.lindblad_3q(n_t=30, n_draws=2)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F_tc, G_tc = p.eval(u0)
    p.set_teams(256, 0)
    F_cc, _ = p.eval(u0)
    p.close()
    Fo, Go = mb.eval_gate_exact_adjoint(prob, u0)
    assert abs(F_tc - F_cc) <= 1e-11 and abs(F_tc - Fo) <= 1e-8
    assert _rel_g(G_tc, Go) <= G_RTOL_MIXED
    rng = np.random.default_rng(78)
    gp, u1 = random_gate_problem(rng, 64, n_t=5, n_members=2, dt=0.04)
    kw = dict(generator=gp.generator, target="states", fidelity="square", states_init=np.eye(64)[:2],
              states_target=np.eye(64)[2:4], grad_mode="exact", precision="mixed")
    ps = pg.Problem(gp.drifts, gp.controls, gp.dt, **kw)
    assert ps.teams[0] == 1
    F1, _ = ps.eval(u1)
    ps.set_teams(256, 0)
    F2, _ = ps.eval(u1)
    ps.close()
    assert abs(F1 - F2) <= 1e-11, (F1, F2)


def test_tc_expm_and_chains_f_only_evaluation_matches(pg):
    """An F-only evaluation (no prefix stores, as the optimisers' line
    searches run) through the tensor-core expm and chain kernels gives the F
    of the full evaluation, bit for bit."""
    prob, u0 = fx.lindblad_3q(n_t=60, n_draws=3)
    p = to_gpu(pg, prob, "exact", precision="mixed")
    F_full, _ = p.eval(u0)
    F_only, G = p.eval(u0, want_grad=False)
    p.close()
    assert G is None and F_only == F_full


def test_context_released_by_its_last_problem():
    """Closing a context while problems still point to it only marks it
    closing; the last problem's destruction releases it (a fresh process, so
    the check does not depend on other tests' contexts)."""
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    code = (
        "import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
        "import numpy as np, __graft_entry__ as ge\n"
        "pg = ge.load_package()\n"
        "from test_parity_gpu import random_gate_problem, to_gpu\n"
        "ctx = pg.Context(0)\n"
        "prob, u0 = random_gate_problem(np.random.default_rng(2), 4, n_t=4, n_members=2)\n"
        "ps = [to_gpu(pg, prob, 'exact', ctx=ctx) for _ in range(2)]\n"
        "F0, _ = ps[0].eval(np.zeros((2, 4)))\n"
        "ctx.close()\n"
        "F1, _ = ps[1].eval(np.zeros((2, 4)))\n"
        "assert F1 == F0\n"
        "ps[0].close(); ps[1].close(); print('ok')\n" % (str(root), str(root / "tests")))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, (r.stdout[-500:], r.stderr[-2000:])
