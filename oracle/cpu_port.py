"""ctypes driver of the oracle's C restatement (oracle/cpu_baseline.c).

TEST INFRASTRUCTURE ONLY: used by the tests as a second checker and by the
CPU-baseline leg of bench.py.  It has its own copy of the pgx_problem_desc
layout so that the oracle does not depend on the product package.
"""
from __future__ import annotations

import ctypes as C
import time

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


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = C.CDLL(str(path))
        L.pgx_cpu_eval.restype = C.c_int
        L.pgx_cpu_eval.argtypes = [C.POINTER(_Desc), _dp, _dp, _dp, C.c_int]
        L.pgx_cpu_max_threads.restype = C.c_int
        _LIB = L
    return _LIB


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
