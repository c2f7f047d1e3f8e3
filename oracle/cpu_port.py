"""ctypes driver of the oracle's C restatement (oracle/cpu_baseline.c).

TEST INFRASTRUCTURE ONLY: used by the tests as a second checker and by the
CPU-baseline leg of bench.py.  It has its own copy of the pgx_problem_desc
layout so that the oracle does not depend on the product package.

The restatement runs the reference's arithmetic stack: LAPACK zheevr (what
Julia's ``eigen(Hermitian(H))`` calls, Propagators.jl:663) and BLAS zgemm
(``mul!``, :673), taken from the OpenBLAS/LAPACK that SciPy bundles through
``scipy.linalg.cython_lapack`` / ``cython_blas``.  BLAS is pinned to one
thread per OpenMP member thread, as GRAPEState.jl:168-174 pins it with
``BLAS.set_num_threads(1)``.  Without SciPy it falls back to its own Jacobi
eigensolver and loops (``backend()`` says which).
"""
from __future__ import annotations

import ctypes as C
import os
import time

# one BLAS thread inside each member thread; read when the OpenBLAS library loads
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np

from . import build_oracle
from .members import Problem

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class _Desc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("dim", C.c_int32), ("n_controls", C.c_int32),
        ("n_slices", C.c_int32), ("generator", C.c_int32), ("target", C.c_int32),
        ("fidelity", C.c_int32), ("grad_mode", C.c_int32), ("precision", C.c_int32),
        ("n_drifts", C.c_int32), ("n_members", C.c_int32), ("n_pairs", C.c_int32),
        ("dt", _dp), ("drifts", _dp), ("controls", _dp), ("offset_op", _dp),
        ("member_drift", _ip), ("member_scale", _dp), ("member_offset", _dp),
        ("member_weight", _dp), ("target_op", _dp), ("states_init", _dp),
        ("states_target", _dp), ("grad_states_init", _dp),
    ]


_LIB = None
_LAPACK = None


def _capsule_ptr(capsule) -> int:
    """Function pointer held by a Cython __pyx_capi__ capsule."""
    api = C.pythonapi
    api.PyCapsule_GetName.restype = C.c_char_p
    api.PyCapsule_GetName.argtypes = [C.py_object]
    api.PyCapsule_GetPointer.restype = C.c_void_p
    api.PyCapsule_GetPointer.argtypes = [C.py_object, C.c_char_p]
    return api.PyCapsule_GetPointer(capsule, api.PyCapsule_GetName(capsule))


def lapack_pointers():
    """(zheevr, zgemm) function pointers of SciPy's bundled LAPACK/BLAS, or None."""
    global _LAPACK
    if _LAPACK is None:
        try:
            from scipy.linalg import cython_blas, cython_lapack
            _LAPACK = (_capsule_ptr(cython_lapack.__pyx_capi__["zheevr"]),
                       _capsule_ptr(cython_blas.__pyx_capi__["zgemm"]))
        except (ImportError, KeyError, AttributeError):
            _LAPACK = ()
    return _LAPACK or None


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = C.CDLL(str(path))
        L.pgx_cpu_eval.restype = C.c_int
        L.pgx_cpu_eval.argtypes = [C.POINTER(_Desc), _dp, _dp, _dp, C.c_int]
        L.pgx_cpu_max_threads.restype = C.c_int
        L.pgx_cpu_set_lapack.restype = C.c_int
        L.pgx_cpu_set_lapack.argtypes = [C.c_void_p, C.c_void_p]
        L.pgx_cpu_backend.restype = C.c_int
        ptrs = lapack_pointers()
        if ptrs:
            L.pgx_cpu_set_lapack(ptrs[0], ptrs[1])
        _LIB = L
    return _LIB


BACKENDS = {"lapack": (True, True), "zheevr": (True, False), "zgemm": (False, True), "jacobi": (False, False)}
BACKEND_TEXT = {"lapack": "LAPACK zheevr + BLAS zgemm", "zheevr": "LAPACK zheevr + plain product loops",
                "zgemm": "Jacobi eigensolver + BLAS zgemm", "jacobi": "Jacobi eigensolver + plain product loops"}


def set_backend(name: str) -> None:
    """'lapack' (SciPy's zheevr + zgemm), 'zheevr' or 'zgemm' (one of the two,
    built-in code for the other), or 'jacobi' (built-in Jacobi and loops)."""
    if name not in BACKENDS:
        raise ValueError(name)
    ev, gm = BACKENDS[name]
    ptrs = lapack_pointers()
    if (ev or gm) and not ptrs:
        raise RuntimeError("SciPy's cython_lapack / cython_blas are not available")
    lib().pgx_cpu_set_lapack(ptrs[0] if ev else None, ptrs[1] if gm else None)


def backend() -> str:
    b = lib().pgx_cpu_backend()
    return {3: "lapack", 1: "zheevr", 2: "zgemm", 0: "jacobi"}[b]


def calibrate(prob: Problem, u, grad_mode: str, threads: int, members: int = 0) -> str:
    """Select the fastest backend for this host and thread count.

    OpenBLAS serialises concurrent small calls on its buffer-pool lock, so on
    some hosts LAPACK + BLAS from every member thread is slower than either
    routine alone or than the built-in code.  Each backend evaluates the same
    sub-problem (2 members per thread, up to 50 slices) once after a warm-up;
    the fastest stays selected (best of two timings each), and its name is
    returned."""
    names = [n for n in BACKENDS if n == "jacobi" or lapack_pointers()]
    nm = min(prob.n_members, members or 4 * max(threads, 1))
    nt = min(prob.n_t, 50)
    sub = prob.subproblem(nm, nt)
    best, best_t = "jacobi", float("inf")
    for n in names:
        set_backend(n)
        cp = CpuProblem(sub, grad_mode)
        cp.eval(u[:, :nt], True, threads)
        t = float("inf")
        for _ in range(2):
            t0 = time.perf_counter()
            cp.eval(u[:, :nt], True, threads)
            t = min(t, time.perf_counter() - t0)
        if t < best_t:
            best, best_t = n, t
    set_backend(best)
    return best


def _mat(a):
    a = np.swapaxes(np.asarray(a, np.complex128), -1, -2)
    return np.ascontiguousarray(a).view(np.float64).ravel()


def _vec(a):
    return np.ascontiguousarray(np.asarray(a, np.complex128)).view(np.float64).ravel()


class CpuProblem:
    """Holds the marshalled descriptor of a members.Problem."""

    GRAD = {"ref_grape": 0, "ref_mr": 1, "exact": 2}
    FID = {"square": 0, "real": 1, "modulus": 2}

    def __init__(self, prob: Problem, grad_mode: str):
        if prob.generator != "hermitian":
            raise ValueError("the C restatement covers Hermitian generators")
        self.prob = prob
        k = self._keep = {}

        def p(name, arr):
            k[name] = arr
            return arr.ctypes.data_as(_dp)

        d = _Desc()
        d.struct_size = C.sizeof(_Desc)
        d.dim, d.n_controls, d.n_slices = prob.D, prob.n_c, prob.n_t
        d.generator, d.target = 0, 0 if prob.target == "gate" else 1
        d.fidelity, d.grad_mode, d.precision = self.FID[prob.fidelity], self.GRAD[grad_mode], 0
        d.n_drifts, d.n_members = prob.drifts.shape[0], prob.n_members
        d.dt = p("dt", np.ascontiguousarray(prob.dt, np.float64))
        d.drifts = p("dr", _mat(prob.drifts))
        d.controls = p("ct", _mat(prob.controls))
        if prob.offset_op is not None:
            d.offset_op = p("of", _mat(prob.offset_op))
        di, sc, of, w = prob.members()
        md = np.ascontiguousarray(di, np.int32)
        k["md"] = md
        d.member_drift = md.ctypes.data_as(_ip)
        d.member_scale = p("ms", np.ascontiguousarray(sc, np.float64))
        d.member_offset = p("mo", np.ascontiguousarray(of, np.float64))
        d.member_weight = p("mw", np.ascontiguousarray(w, np.float64))
        if prob.target == "gate":
            d.n_pairs = 0
            d.target_op = p("tg", _mat(prob.target_op))
        else:
            d.n_pairs = prob.n_pairs
            d.states_init = p("si", _vec(prob.states_init))
            d.states_target = p("st", _vec(prob.states_target))
        self.desc = d

    def eval(self, u, want_grad=True, threads: int = 0):
        u = np.asarray(u, np.float64)
        ub = np.ascontiguousarray(u.T).ravel()
        F = C.c_double()
        G = np.zeros(ub.size) if want_grad else None
        st = lib().pgx_cpu_eval(C.byref(self.desc), ub.ctypes.data_as(_dp), C.byref(F),
                                G.ctypes.data_as(_dp) if want_grad else None, int(threads))
        if st != 0:
            raise RuntimeError(f"pgx_cpu_eval failed with status {st}")
        return F.value, (G.reshape(u.shape[1], u.shape[0]).T.copy() if want_grad else None)


def max_threads() -> int:
    return int(lib().pgx_cpu_max_threads())


def time_eval(prob: Problem, u, grad_mode: str, threads: int = 0, repeats: int = 1):
    cp = CpuProblem(prob, grad_mode)
    ts = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        cp.eval(u, True, threads)
        ts.append(time.perf_counter() - t0)
    return ts
