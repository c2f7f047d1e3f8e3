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


def _cmm(pg, P, Q, passes):
    A = pg._abi
    n = P.shape[0]
    f = A.lib().pgx_diag_tc_cmatmul64
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]
    buf = lambda M: np.ascontiguousarray(np.swapaxes(M, -1, -2)).astype(np.complex128)  # column-major
    Pb, Qb = buf(P), buf(Q)
    Cb = np.zeros_like(Pb)
    st = f(Pb.ctypes.data, Qb.ctypes.data, Cb.ctypes.data, n, passes)
    assert st == 0, st
    return np.swapaxes(Cb, -1, -2)


def _rel(Cg, Cr):
    return np.max(np.abs(Cg - Cr), axis=(1, 2)) / np.max(np.abs(Cr), axis=(1, 2))


def test_tc_cmatmul64_3xtf32_is_fp32_accurate(pg):
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
    C3 = _cmm(pg, P, Q, 3)
    e3 = _rel(C3, ref)
    assert np.all(np.isfinite(C3))
    assert e3.max() <= 5e-6, e3.max()
    C1 = _cmm(pg, P, Q, 1)
    e1 = _rel(C1, ref)
    assert 1e-5 <= np.median(e1) <= 2e-2, np.median(e1)
    print(f"3xTF32 max rel {e3.max():.2e}, TF32 median rel {np.median(e1):.2e}")


def test_tc_cmatmul64_rejects_bad_arguments(pg):
    f = pg._abi.lib().pgx_diag_tc_cmatmul64
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]
    buf = np.zeros(2 * 4096)
    assert f(buf.ctypes.data, buf.ctypes.data, buf.ctypes.data, 1, 2) == 1
    assert f(buf.ctypes.data, buf.ctypes.data, buf.ctypes.data, 0, 3) == 1
