"""ctypes mirror of include/pgx.h and the loader of libpulsar_gb300.so.

The library is the only compute path: if it is missing or cannot be loaded,
``lib()`` raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libpulsar_gb300.so"

PGX_OK = 0
STATUS = {
    1: "invalid argument", 2: "dimension mismatch", 3: "out of device memory",
    4: "HBM budget exceeded", 5: "CUDA error", 6: "unsupported", 7: "timeout",
    8: "cancelled", 9: "invalid state", 10: "non-finite value",
}
GEN = {"hermitian": 0, "liouvillian": 1}
TARGET = {"gate": 0, "states": 1}
FID = {"square": 0, "real": 1, "modulus": 2}
GRAD = {"ref_grape": 0, "ref_mr": 1, "exact": 2}
PREC = {"fp64": 0, "mixed": 1}
OPT = {"grape": 0, "ensemble_lbfgs": 1, "mr_lbfgs": 2, "mr_grape": 3}

dptr = C.POINTER(C.c_double)
iptr = C.POINTER(C.c_int32)


class ProblemDesc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("dim", C.c_int32), ("n_controls", C.c_int32),
        ("n_slices", C.c_int32), ("generator", C.c_int32), ("target", C.c_int32),
        ("fidelity", C.c_int32), ("grad_mode", C.c_int32), ("precision", C.c_int32),
        ("n_drifts", C.c_int32), ("n_members", C.c_int32), ("n_pairs", C.c_int32),
        ("dt", dptr), ("drifts", dptr), ("controls", dptr), ("offset_op", dptr),
        ("member_drift", iptr), ("member_scale", dptr), ("member_offset", dptr),
        ("member_weight", dptr), ("target_op", dptr), ("states_init", dptr),
        ("states_target", dptr), ("grad_states_init", dptr),
    ]


class EvalStats(C.Structure):
    _fields_ = [("ms_device", C.c_double), ("ms_host", C.c_double), ("units", C.c_int64),
                ("n_launches", C.c_int32), ("max_taylor_degree", C.c_int32), ("residual", C.c_double),
                ("residual_kind", C.c_int32), ("reserved", C.c_int32)]


RESIDUAL_KIND = {0: "none", 1: "unitarity", 2: "trace", 3: "norm", 4: "state_trace"}


class OptDesc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("method", C.c_int32), ("max_iter", C.c_int32),
        ("adapt_step_size", C.c_int32), ("lbfgs_memory", C.c_int32), ("reserved", C.c_int32),
        ("convergence_tol", C.c_double), ("step_size", C.c_double), ("min_step_size", C.c_double),
        ("max_step_size", C.c_double), ("gradient_norm_tol", C.c_double),
        ("amplitude_limit", C.c_double), ("l_bound", C.c_double), ("u_bound", C.c_double),
    ]


class OptResult(C.Structure):
    _fields_ = [
        ("fidelity", C.c_double), ("total_time_s", C.c_double), ("step_size_final", C.c_double),
        ("n_iterations", C.c_int32), ("converged", C.c_int32), ("n_fidelity_evals", C.c_int32),
        ("n_gradient_evals", C.c_int32), ("history_len", C.c_int32),
        ("gnorm_history_len", C.c_int32), ("reason", C.c_char * 100),
    ]


JOB_STATE = {0: "queued", 1: "running", 2: "done", 3: "failed", 4: "cancelled"}
PENALTY = {"NS": 0, "SNS": 1, "SNSA": 2, "DNS": 3, "energy": 4}
AGGREGATOR = {"mean": 0, "worst_case": 1, "cvar": 2}


class Penalty(C.Structure):
    _fields_ = [("type", C.c_int32), ("reserved", C.c_int32), ("weight", C.c_double),
                ("l_bound", C.c_double), ("u_bound", C.c_double)]


class ServerDesc(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("max_inflight", C.c_int32),
                ("hbm_budget_bytes", C.c_uint64), ("target_fidelity", C.c_double)]


class JobStatus(C.Structure):
    _fields_ = [
        ("state", C.c_int32), ("status", C.c_int32), ("iterations", C.c_int32),
        ("reserved", C.c_int32), ("fidelity", C.c_double), ("best_fidelity", C.c_double),
        ("queue_s", C.c_double), ("latency_s", C.c_double), ("reason", C.c_char * 96),
    ]


class ServeStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
        ("cancelled", C.c_int64), ("running", C.c_int64), ("queued", C.c_int64),
        ("kernel_launches", C.c_int64), ("units", C.c_int64), ("hbm_in_use", C.c_uint64),
        ("hbm_peak", C.c_uint64), ("elapsed_s", C.c_double), ("jobs_per_s", C.c_double),
        ("p50_latency_s", C.c_double), ("p99_latency_s", C.c_double),
        ("mean_iterations", C.c_double),
    ]


class JobExtras(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("n_penalties", C.c_int32), ("penalties", C.c_void_p),
        ("n_tracking", C.c_int32), ("n_ramp_ops", C.c_int32), ("tracking_steps", iptr),
        ("tracking_weights", dptr), ("tracking_targets", dptr), ("ramp_ops", dptr), ("ramp_member_op", iptr),
        ("ramp_tau", dptr),
    ]


class CheckpointInfo(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("version", C.c_int32), ("flags", C.c_int32),
        ("system_dim", C.c_int32), ("n_controls", C.c_int32), ("n_timesteps", C.c_int32),
        ("n_members", C.c_int32), ("iteration", C.c_int32), ("history_len", C.c_int32),
        ("gnorm_history_len", C.c_int32), ("lbfgs_pairs", C.c_int32), ("metadata_len", C.c_int32),
        ("F_opt", C.c_double), ("F", C.c_double), ("timestamp", C.c_double),
        ("fingerprint", C.c_uint64), ("opt", OptDesc),
    ]


CKPT_EXACT, CKPT_CONVERGED = 1, 2
CHECKPOINT_HEADER_BYTES = 208
RESUME = {"restart": 0, "continue": 1}

# name -> (restype, argtypes); every symbol declared in include/pgx.h
SIGNATURES = {
    "pgx_abi_version": (C.c_int, []),
    "pgx_status_string": (C.c_char_p, [C.c_int]),
    "pgx_ctx_create": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]),
    "pgx_ctx_destroy": (C.c_int, [C.c_void_p]),
    "pgx_last_error": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "pgx_ctx_hbm_used": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "pgx_ctx_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "pgx_ctx_timer_start": (C.c_int, [C.c_void_p]),
    "pgx_ctx_timer_stop": (C.c_int, [C.c_void_p, dptr]),
    "pgx_ctx_synchronize": (C.c_int, [C.c_void_p]),
    "pgx_ctx_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "pgx_ctx_set_stage_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "pgx_ctx_stage_times": (C.c_int, [C.c_void_p, dptr, C.POINTER(C.c_int32)]),
    "pgx_ctx_measure_peak": (C.c_int, [C.c_void_p, C.c_int32, dptr]),
    "pgx_problem_footprint": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(C.c_uint64)]),
    "pgx_problem_create": (C.c_int, [C.c_void_p, C.POINTER(ProblemDesc), C.POINTER(C.c_void_p)]),
    "pgx_problem_destroy": (C.c_int, [C.c_void_p]),
    "pgx_eval": (C.c_int, [C.c_void_p, dptr, dptr, dptr, C.POINTER(EvalStats)]),
    "pgx_eval_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "pgx_member_fidelities": (C.c_int, [C.c_void_p, dptr]),
    "pgx_total_propagator": (C.c_int, [C.c_void_p, dptr, C.c_int32, dptr]),
    "pgx_propagator": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, dptr, C.c_double, dptr]),
    "pgx_total_hamiltonian": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, dptr, dptr, dptr, dptr]),
    "pgx_propagator_stack": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, dptr, dptr, C.c_int32,
                                       dptr]),
    "pgx_propagator_chains": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, dptr, dptr, dptr, dptr, dptr]),
    "pgx_overlap": (C.c_int, [C.c_void_p, C.c_int64, dptr, dptr, dptr]),
    "pgx_trace_products": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, dptr, dptr, dptr, dptr]),
    "pgx_autotune": (C.c_int, [C.c_void_p, dptr, C.c_int32, C.c_char_p, C.c_size_t]),
    "pgx_problem_set_penalties": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "pgx_eval_aggregate": (C.c_int, [C.c_void_p, dptr, C.c_int32, C.c_double, dptr, dptr]),
    "pgx_problem_set_drifts": (C.c_int, [C.c_void_p, dptr]),
    "pgx_penalty_eval": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, dptr, dptr, C.c_void_p, dptr, dptr]),
    "pgx_problem_set_team": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "pgx_problem_get_team": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "pgx_plan_lookup": (C.c_int, [C.c_int, C.POINTER(ProblemDesc), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "pgx_plan_clear": (C.c_int, []),
    "pgx_problem_set_tracking": (C.c_int, [C.c_void_p, C.c_int32, iptr, dptr, dptr]),
    "pgx_eval_phase": (C.c_int, [C.c_void_p, dptr, dptr, dptr, dptr]),
    "pgx_problem_set_drift_ramp": (C.c_int, [C.c_void_p, C.c_int32, dptr, iptr, dptr]),
    "pgx_batch_create": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.c_int32,
                                   C.POINTER(C.c_void_p)]),
    "pgx_batch_destroy": (C.c_int, [C.c_void_p]),
    "pgx_batch_set_controls": (C.c_int, [C.c_void_p, C.c_int32, dptr]),
    "pgx_batch_get_controls": (C.c_int, [C.c_void_p, C.c_int32, dptr, dptr]),
    "pgx_batch_units": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "pgx_batch_eval": (C.c_int, [C.c_void_p, dptr]),
    "pgx_batch_iterate": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(OptDesc), dptr]),
    "pgx_total_propagator_noalloc": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p,
                                               C.c_size_t]),
    "pgx_optimize": (C.c_int, [C.c_void_p, C.POINTER(OptDesc), dptr, dptr, dptr, C.c_int32,
                               C.POINTER(OptResult)]),
    "pgx_server_create": (C.c_int, [C.c_void_p, C.POINTER(ServerDesc), C.POINTER(C.c_void_p)]),
    "pgx_server_destroy": (C.c_int, [C.c_void_p]),
    "pgx_submit": (C.c_int, [C.c_void_p, C.POINTER(ProblemDesc), C.POINTER(OptDesc), dptr,
                             C.POINTER(C.c_uint64)]),
    "pgx_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(JobStatus)]),
    "pgx_fetch": (C.c_int, [C.c_void_p, C.c_uint64, dptr, C.POINTER(OptResult)]),
    "pgx_cancel": (C.c_int, [C.c_void_p, C.c_uint64]),
    "pgx_server_drain": (C.c_int, [C.c_void_p, C.c_double]),
    "pgx_server_stats": (C.c_int, [C.c_void_p, C.POINTER(ServeStats)]),
    "pgx_job_history": (C.c_int, [C.c_void_p, C.c_uint64, dptr, dptr, C.c_int32, C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int32)]),
    "pgx_job_checkpoint": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double, C.POINTER(C.c_uint64)]),
    "pgx_job_checkpoint_read": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64]),
    "pgx_submit_ex": (C.c_int, [C.c_void_p, C.POINTER(ProblemDesc), C.POINTER(OptDesc), dptr,
                                C.POINTER(JobExtras), C.POINTER(C.c_uint64)]),
    "pgx_submit_resume": (C.c_int, [C.c_void_p, C.POINTER(ProblemDesc), C.POINTER(OptDesc),
                                    C.POINTER(JobExtras), C.c_void_p, C.c_uint64, C.c_int32,
                                    C.POINTER(C.c_uint64)]),
    "pgx_checkpoint_parse": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(CheckpointInfo), dptr, dptr, dptr]),
    "pgx_checkpoint_metadata": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64]),
    "pgx_checkpoint_create": (C.c_int, [C.POINTER(CheckpointInfo), dptr, dptr, dptr, C.c_char_p, C.c_void_p,
                                        C.c_uint64, C.POINTER(C.c_uint64)]),
    "pgx_checkpoint_set_metadata": (C.c_int, [C.c_void_p, C.c_uint64, C.c_char_p, C.c_uint64, C.c_void_p,
                                              C.c_uint64, C.POINTER(C.c_uint64)]),
    "pgx_problem_fingerprint": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(C.c_uint64)]),
}

_LIB = None


def lib() -> C.CDLL:
    """Load libpulsar_gb300.so (raises if it is absent: no fallback path)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first; "
                               "there is no CPU fallback for the GRAPE hot path")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class PgxError(RuntimeError):
    def __init__(self, status: int, detail: str = ""):
        self.status = status
        super().__init__(f"pgx status {status} ({STATUS.get(status, 'unknown')}): {detail}")


def check(status: int, ctx=None):
    if status != PGX_OK:
        detail = ""
        if ctx:
            buf = C.create_string_buffer(512)
            lib().pgx_last_error(ctx, buf, 512)
            detail = buf.value.decode(errors="replace")
        raise PgxError(status, detail)


def as_dptr(a: np.ndarray):
    return a.ctypes.data_as(dptr)


def cmat_buf(mats) -> np.ndarray:
    """[row, col] complex matrix or stack [..., D, D] -> interleaved
    column-major float64 buffer (Julia Matrix{ComplexF64} memory)."""
    a = np.swapaxes(np.asarray(mats, dtype=np.complex128), -1, -2)
    return np.ascontiguousarray(a).view(np.float64).ravel()


def cvec_buf(vecs) -> np.ndarray:
    """Complex vectors [n, D] -> interleaved float64 buffer."""
    return np.ascontiguousarray(np.asarray(vecs, dtype=np.complex128)).view(np.float64).ravel()


def cmat_from_buf(buf: np.ndarray, D: int) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(buf, np.float64)).view(np.complex128).reshape(D, D).T.copy()
