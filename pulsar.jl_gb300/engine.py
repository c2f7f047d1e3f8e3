"""Thin Python handles over the C ABI: ``Context`` and ``Problem``.

Everything computes inside libpulsar_gb300.so; this module only marshals
numpy arrays into the column-major interleaved buffers of include/pgx.h.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _abi as A


class Context:
    """One device, one stream, an HBM budget (0 = unlimited)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._h = C.c_void_p()
        st = A.lib().pgx_ctx_create(int(device), int(hbm_budget), C.byref(self._h))
        A.check(st)

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            A.lib().pgx_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def hbm_used(self) -> int:
        v = C.c_uint64()
        A.check(A.lib().pgx_ctx_hbm_used(self._h, C.byref(v)), self._h)
        return int(v.value)

    def launch_count(self) -> int:
        v = C.c_int64()
        A.check(A.lib().pgx_ctx_launch_count(self._h, C.byref(v)), self._h)
        return int(v.value)

    def stream(self) -> int:
        v = C.c_void_p()
        A.check(A.lib().pgx_ctx_stream(self._h, C.byref(v)), self._h)
        return int(v.value or 0)

    def timer_start(self):
        A.check(A.lib().pgx_ctx_timer_start(self._h), self._h)

    def timer_stop(self) -> float:
        ms = C.c_double()
        A.check(A.lib().pgx_ctx_timer_stop(self._h, C.byref(ms)), self._h)
        return float(ms.value)

    def synchronize(self):
        A.check(A.lib().pgx_ctx_synchronize(self._h), self._h)

    STAGES = ("expm", "chain_fwd", "chain_bwd", "grad", "reduce")

    def set_stage_timing(self, on: bool):
        A.check(A.lib().pgx_ctx_set_stage_timing(self._h, int(bool(on))), self._h)

    def stage_times(self):
        """({stage: summed ms}, evaluations recorded) since the last call."""
        ms = np.zeros(len(self.STAGES))
        n = C.c_int32()
        A.check(A.lib().pgx_ctx_stage_times(self._h, A.as_dptr(ms), C.byref(n)), self._h)
        return dict(zip(self.STAGES, ms.tolist())), int(n.value)

    def measure_peak(self, pipe: str = "fp64") -> float:
        """Measured FMA peak of the FP64 or FP32 pipe, GFLOP/s."""
        g = C.c_double()
        A.check(A.lib().pgx_ctx_measure_peak(self._h, {"fp64": 0, "fp32": 1}[pipe], C.byref(g)), self._h)
        return float(g.value)

    def propagator(self, G: np.ndarray, dt: float, generator: str = "hermitian") -> np.ndarray:
        """exp(-i G dt) (Hermitian) or exp(G dt) (Liouvillian) on the device."""
        G = np.asarray(G, np.complex128)
        D = G.shape[0]
        gb = A.cmat_buf(G)
        out = np.zeros(2 * D * D)
        A.check(A.lib().pgx_propagator(self._h, D, A.GEN[generator], A.as_dptr(gb), float(dt),
                                       A.as_dptr(out)), self._h)
        return A.cmat_from_buf(out, D)


_DEFAULT: Optional[Context] = None


def default_context() -> Context:
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Context(0)
    return _DEFAULT


def opt_desc(method: str = "grape", *, max_iter: int = 1000, convergence_tol: float = 1e-8,
             step_size: float = 0.01, adapt_step_size: bool = True, min_step_size: float = 1e-10,
             max_step_size: float = 10.0, gradient_norm_tol: float = 1e-6, lbfgs_memory: int = 10,
             amplitude_limit: float = math.inf, l_bound: float = -1.0, u_bound: float = 1.0) -> "A.OptDesc":
    """pgx_opt_desc with GRAPEConfig's defaults (GRAPE.jl:94-127)."""
    o = A.OptDesc()
    o.struct_size = C.sizeof(A.OptDesc)
    o.method = A.OPT[method]
    o.max_iter, o.adapt_step_size, o.lbfgs_memory = int(max_iter), int(bool(adapt_step_size)), int(lbfgs_memory)
    o.convergence_tol, o.step_size = float(convergence_tol), float(step_size)
    o.min_step_size, o.max_step_size = float(min_step_size), float(max_step_size)
    o.gradient_norm_tol, o.amplitude_limit = float(gradient_norm_tol), float(amplitude_limit)
    o.l_bound, o.u_bound = float(l_bound), float(u_bound)
    return o


class Batch:
    """Uneven problems evaluated / iterated together, one CUDA graph per call."""

    def __init__(self, problems, n_streams: int = 8):
        if not problems:
            raise ValueError("a batch needs at least one problem")
        self.problems = list(problems)
        self.ctx = self.problems[0].ctx
        arr = (C.c_void_p * len(self.problems))(*[p._h for p in self.problems])
        self._h = C.c_void_p()
        A.check(A.lib().pgx_batch_create(self.ctx.handle, len(self.problems), arr, int(n_streams),
                                         C.byref(self._h)), self.ctx.handle)

    def close(self):
        if getattr(self, "_h", None):
            A.lib().pgx_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def units(self) -> int:
        v = C.c_int64()
        A.check(A.lib().pgx_batch_units(self._h, C.byref(v)), self.ctx.handle)
        return int(v.value)

    def set_controls(self, i: int, u):
        p = self.problems[i]
        ub = p._load_u(u)
        A.check(A.lib().pgx_batch_set_controls(self._h, int(i), A.as_dptr(ub)), self.ctx.handle)

    def get_controls(self, i: int):
        p = self.problems[i]
        u = np.zeros(p.n_c * p.n_t)
        G = np.zeros(p.n_c * p.n_t)
        A.check(A.lib().pgx_batch_get_controls(self._h, int(i), A.as_dptr(u), A.as_dptr(G)), self.ctx.handle)
        return u.reshape(p.n_t, p.n_c).T.copy(), G.reshape(p.n_t, p.n_c).T.copy()

    def eval(self) -> np.ndarray:
        F = np.zeros(len(self.problems))
        A.check(A.lib().pgx_batch_eval(self._h, A.as_dptr(F)), self.ctx.handle)
        return F

    def iterate(self, n_iter: int, trace: bool = True, **opt):
        o = opt_desc("grape", **opt)
        tr = np.zeros((n_iter, len(self.problems))) if trace else None
        A.check(A.lib().pgx_batch_iterate(self._h, int(n_iter), C.byref(o),
                                          A.as_dptr(tr) if trace else None), self.ctx.handle)
        return tr


@dataclass
class JobResult:
    job_id: int
    state: str
    controls: Optional[np.ndarray]
    fidelity: float
    n_iterations: int
    converged: bool
    termination_reason: str
    latency_s: float
    step_size_final: float
    fidelity_history: list = field(default_factory=list)
    gradient_norm_history: list = field(default_factory=list)
    n_fidelity_evaluations: int = 0
    n_gradient_evaluations: int = 0


OPT_NAMES = {v: k for k, v in A.OPT.items()}


def opt_settings(o: "A.OptDesc") -> dict:
    """pgx_opt_desc -> (method name, opt_desc keywords)."""
    kw = {k: getattr(o, k) for k in ("max_iter", "convergence_tol", "step_size", "min_step_size",
                                     "max_step_size", "gradient_norm_tol", "lbfgs_memory",
                                     "amplitude_limit", "l_bound", "u_bound")}
    kw["adapt_step_size"] = bool(o.adapt_step_size)
    return {"method": OPT_NAMES.get(int(o.method), str(o.method)), **kw}


def checkpoint_parse(blob: bytes) -> dict:
    """Verify and decode a checkpoint blob on the host (pgx_checkpoint_parse):
    its Checkpoint fields (Checkpoint.jl:64-80) with w_opt as [n_c, n_t]."""
    b = bytes(blob)
    info = A.CheckpointInfo()
    buf = C.create_string_buffer(b, len(b))
    A.check(A.lib().pgx_checkpoint_parse(buf, len(b), C.byref(info), None, None, None))
    n_c, n_t = info.n_controls, info.n_timesteps
    w = np.zeros(n_c * n_t)
    fh = np.zeros(max(info.history_len, 1))
    gh = np.zeros(max(info.gnorm_history_len, 1))
    A.check(A.lib().pgx_checkpoint_parse(buf, len(b), C.byref(info), A.as_dptr(w), A.as_dptr(fh),
                                         A.as_dptr(gh)))
    return {"w_opt": w.reshape(n_t, n_c).T.copy(), "F_opt": info.F_opt, "F": info.F,
            "n_controls": n_c, "n_timesteps": n_t, "iteration": info.iteration,
            "fidelity_history": fh[:info.history_len].tolist(),
            "gradient_norm_history": gh[:info.gnorm_history_len].tolist(),
            "system_dim": info.system_dim, "n_members": info.n_members, "timestamp": info.timestamp,
            "fingerprint": int(info.fingerprint), "exact": bool(info.flags & A.CKPT_EXACT),
            "converged": bool(info.flags & A.CKPT_CONVERGED), "lbfgs_pairs": info.lbfgs_pairs,
            "optimizer": opt_settings(info.opt), "metadata": _checkpoint_metadata(buf, len(b), info.metadata_len)}


def _checkpoint_metadata(buf, n: int, m: int) -> bytes:
    out = C.create_string_buffer(max(m, 1))
    A.check(A.lib().pgx_checkpoint_metadata(buf, n, out, m))
    return out.raw[:m]


def checkpoint_set_metadata(blob: bytes, metadata: bytes) -> bytes:
    """The same checkpoint with its metadata section replaced (pgx_checkpoint_set_metadata)."""
    b, m = bytes(blob), bytes(metadata)
    need = C.c_uint64()
    A.check(A.lib().pgx_checkpoint_set_metadata(b, len(b), m, len(m), None, 0, C.byref(need)))
    out = C.create_string_buffer(need.value)
    A.check(A.lib().pgx_checkpoint_set_metadata(b, len(b), m, len(m), out, need.value, C.byref(need)))
    return out.raw[:need.value]


def checkpoint_create(w_opt, F_opt: float, *, iteration: int = 0, fidelity_history=(),
                      gradient_norm_history=(), system_dim: int = 0, n_members: int = 0,
                      converged: bool = False, timestamp: float = 0.0, fingerprint: int = 0,
                      method: str = "grape", opt: Optional[dict] = None, metadata: bytes = b"") -> bytes:
    """create_checkpoint (Checkpoint.jl:143-164) as a warm-start blob
    (pgx_checkpoint_create); w_opt is [n_c, n_t]."""
    w = np.asarray(w_opt, np.float64)
    if w.ndim != 2:
        raise ValueError("w_opt must be a [n_controls, n_timesteps] matrix")
    n_c, n_t = w.shape
    wb = np.ascontiguousarray(w.T.ravel())
    fh = np.ascontiguousarray(np.asarray(list(fidelity_history), np.float64))
    gh = np.ascontiguousarray(np.asarray(list(gradient_norm_history), np.float64))
    info = A.CheckpointInfo()
    info.struct_size = C.sizeof(A.CheckpointInfo)
    info.version = 1
    info.flags = A.CKPT_CONVERGED if converged else 0
    info.system_dim, info.n_controls, info.n_timesteps = int(system_dim), n_c, n_t
    info.n_members, info.iteration = int(n_members), int(iteration)
    info.history_len, info.gnorm_history_len = fh.size, gh.size
    info.F_opt, info.F, info.timestamp = float(F_opt), float(F_opt), float(timestamp)
    info.fingerprint = int(fingerprint)
    info.opt = opt_desc(method, **(opt or {}))
    meta = bytes(metadata)
    info.metadata_len = len(meta)
    need = C.c_uint64()
    fp = A.as_dptr(fh) if fh.size else None
    gp = A.as_dptr(gh) if gh.size else None
    A.check(A.lib().pgx_checkpoint_create(C.byref(info), A.as_dptr(wb), fp, gp, meta, None, 0, C.byref(need)))
    out = C.create_string_buffer(need.value)
    A.check(A.lib().pgx_checkpoint_create(C.byref(info), A.as_dptr(wb), fp, gp, meta, out, need.value,
                                          C.byref(need)))
    return out.raw[:need.value]


def plan_lookup(drifts, controls, dt, *, device: int = 0, **problem):
    """(expm, gradient) team sizes pgx_autotune recorded for problems of this
    key, or None (pgx_plan_lookup)."""
    d, keep, _ = problem_desc(drifts, controls, dt, **problem)
    te, tg = C.c_int32(), C.c_int32()
    rc = A.lib().pgx_plan_lookup(int(device), C.byref(d), C.byref(te), C.byref(tg))
    if rc == 9:
        return None
    A.check(rc)
    return int(te.value), int(tg.value)


def plan_clear():
    A.check(A.lib().pgx_plan_clear())


def problem_fingerprint(drifts, controls, dt, **problem) -> int:
    """FNV-1a-64 of the problem descriptor (what an exact resumption checks)."""
    d, keep, _ = problem_desc(drifts, controls, dt, **problem)
    fp = C.c_uint64()
    A.check(A.lib().pgx_problem_fingerprint(C.byref(d), C.byref(fp)))
    return int(fp.value)


def penalty_array(penalties):
    """[(type, weight[, l_bound, u_bound]), ...] -> pgx_penalty array."""
    arr = (A.Penalty * max(len(penalties), 1))()
    for i, pen in enumerate(penalties):
        t, wgt = pen[0], pen[1]
        lo, hi = (pen[2], pen[3]) if len(pen) > 2 else (-1.0, 1.0)
        if t not in A.PENALTY:
            raise ValueError(f"Unknown penalty ':{t}'. Valid: {', '.join(A.PENALTY)}")
        arr[i].type, arr[i].weight, arr[i].l_bound, arr[i].u_bound = A.PENALTY[t], float(wgt), float(lo), float(hi)
    return arr


def job_extras(D: int, penalties=None, tracking=None, drift_ramp=None):
    """pgx_job_extras of a server job (None when nothing is set) and the
    buffers it points into."""
    if not penalties and tracking is None and drift_ramp is None:
        return None, None
    x = A.JobExtras()
    x.struct_size = C.sizeof(A.JobExtras)
    keep = []
    if penalties:
        arr = penalty_array(penalties)
        keep.append(arr)
        x.n_penalties, x.penalties = len(penalties), C.cast(arr, C.c_void_p)
    if tracking is not None:
        steps, weights, targets = tracking
        st = np.ascontiguousarray(np.asarray(steps, np.int64).astype(np.int32).ravel())
        wt = np.ascontiguousarray(np.asarray(weights, np.float64).ravel())
        tg = A.cmat_buf(np.asarray(targets, np.complex128).reshape(-1, D, D))
        keep += [st, wt, tg]
        x.n_tracking = st.size
        x.tracking_steps, x.tracking_weights, x.tracking_targets = st.ctypes.data_as(A.iptr), A.as_dptr(wt), \
            A.as_dptr(tg)
    if drift_ramp is not None:
        ops, member_op, tau = drift_ramp
        ob = A.cmat_buf(np.asarray(ops, np.complex128).reshape(-1, D, D))
        mo = np.ascontiguousarray(np.asarray(member_op, np.int64).astype(np.int32).ravel())
        tv = np.ascontiguousarray(np.asarray(tau, np.float64).ravel())
        keep += [ob, mo, tv]
        x.n_ramp_ops = np.asarray(ops).reshape(-1, D, D).shape[0]
        x.ramp_ops, x.ramp_member_op, x.ramp_tau = A.as_dptr(ob), mo.ctypes.data_as(A.iptr), A.as_dptr(tv)
    return x, keep


class Server:
    """Continuous-batching GRAPE server (pgx_server): jobs are admitted by HBM
    footprint and iterate on the device, each at its own pace."""

    def __init__(self, ctx: Optional[Context] = None, *, max_inflight: int = 64,
                 hbm_budget_bytes: int = 0, target_fidelity: float = 0.999):
        self.ctx = ctx or default_context()
        d = A.ServerDesc()
        d.struct_size = C.sizeof(A.ServerDesc)
        d.max_inflight, d.hbm_budget_bytes = int(max_inflight), int(hbm_budget_bytes)
        d.target_fidelity = float(target_fidelity)
        self._h = C.c_void_p()
        A.check(A.lib().pgx_server_create(self.ctx.handle, C.byref(d), C.byref(self._h)), self.ctx.handle)
        self._shape = {}

    def close(self):
        if getattr(self, "_h", None):
            A.lib().pgx_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, drifts, controls, dt, u0, *, opt: Optional[dict] = None, method: str = "grape",
               penalties=None, tracking=None, drift_ramp=None, **problem) -> int:
        """Queue one job: grape_optimize ("grape"), the ensemble L-BFGS of
        grape_optimize_ensemble ("ensemble_lbfgs") or optimcon's MR loops
        ("mr_lbfgs", "mr_grape").  ``problem`` takes Problem's keywords, ``opt``
        opt_desc's (GRAPEConfig defaults).  Optional job extras:
        ``penalties`` as Problem.set_penalties, ``tracking`` = (steps, weights,
        targets), ``drift_ramp`` = (ops, member_op, tau).  Returns the job id."""
        d, keep, (D, n_c, n_t, _, _) = problem_desc(drifts, controls, dt, **problem)
        u = np.asarray(u0, np.float64)
        if u.shape != (n_c, n_t):
            raise ValueError(f"controls have shape {u.shape}, expected {(n_c, n_t)}")
        ub = np.ascontiguousarray(u.T.ravel())
        o = opt_desc(method, **(opt or {}))
        x, xkeep = job_extras(D, penalties, tracking, drift_ramp)
        jid = C.c_uint64()
        A.check(A.lib().pgx_submit_ex(self._h, C.byref(d), C.byref(o), A.as_dptr(ub),
                                      C.byref(x) if x is not None else None, C.byref(jid)), self.ctx.handle)
        self._shape[int(jid.value)] = (n_c, n_t)
        return int(jid.value)

    def submit_resume(self, drifts, controls, dt, checkpoint: bytes, *, mode: str = "restart",
                      opt: Optional[dict] = None, method: Optional[str] = None, penalties=None, tracking=None,
                      drift_ramp=None, **problem) -> int:
        """Queue a job resumed from a checkpoint blob.  ``mode`` "restart" is
        resume_optimization (Checkpoint.jl:220-298): a fresh run from w_opt
        whose histories and iteration count follow the checkpoint's (opt's
        max_iter = the additional iterations); "continue" resumes an exact
        snapshot bit-identically.  With neither opt nor method the
        checkpoint's own settings are used."""
        d, keep, (D, n_c, n_t, _, _) = problem_desc(drifts, controls, dt, **problem)
        b = bytes(checkpoint)
        buf = C.create_string_buffer(b, len(b))
        o = None
        if opt is not None or method is not None:
            base = checkpoint_parse(b)["optimizer"]
            kw = {k: v for k, v in base.items() if k != "method"}
            kw.update(opt or {})
            o = opt_desc(method or base["method"], **kw)
        x, xkeep = job_extras(D, penalties, tracking, drift_ramp)
        jid = C.c_uint64()
        A.check(A.lib().pgx_submit_resume(self._h, C.byref(d), C.byref(o) if o is not None else None,
                                          C.byref(x) if x is not None else None, buf, len(b), A.RESUME[mode],
                                          C.byref(jid)), self.ctx.handle)
        self._shape[int(jid.value)] = (n_c, n_t)
        return int(jid.value)

    def checkpoint(self, job_id: int, timeout_s: float = 0.0) -> bytes:
        """Checkpoint blob of a job: a running job is snapshotted at its next
        iteration boundary; a finished one gives its final state."""
        n = C.c_uint64()
        rc = A.lib().pgx_job_checkpoint(self._h, int(job_id), float(timeout_s), C.byref(n))
        if rc == 7:
            raise TimeoutError("no iteration boundary within the timeout")
        A.check(rc)
        out = C.create_string_buffer(n.value)
        A.check(A.lib().pgx_job_checkpoint_read(self._h, int(job_id), out, n.value))
        return out.raw[:n.value]

    def history(self, job_id: int):
        """(fidelity history, gradient-norm history) of a job so far."""
        nf, ng = C.c_int32(), C.c_int32()
        A.check(A.lib().pgx_job_history(self._h, int(job_id), None, None, 0, C.byref(nf), C.byref(ng)))
        cap = max(nf.value, ng.value, 1)
        fh, gh = np.zeros(cap), np.zeros(cap)
        A.check(A.lib().pgx_job_history(self._h, int(job_id), A.as_dptr(fh), A.as_dptr(gh), cap, C.byref(nf),
                                        C.byref(ng)))
        return fh[:nf.value].tolist(), gh[:ng.value].tolist()

    def poll(self, job_id: int) -> dict:
        st = A.JobStatus()
        A.check(A.lib().pgx_poll(self._h, int(job_id), C.byref(st)))
        return {"state": A.JOB_STATE[st.state], "status": int(st.status), "iterations": int(st.iterations),
                "fidelity": st.fidelity, "best_fidelity": st.best_fidelity, "queue_s": st.queue_s,
                "latency_s": st.latency_s, "reason": st.reason.decode(errors="replace")}

    def fetch(self, job_id: int) -> JobResult:
        """Result of a finished job (raises PgxError(9) while it runs)."""
        n_c, n_t = self._shape[int(job_id)]
        st = self.poll(job_id)["state"]
        if st in ("queued", "running"):
            A.check(9)
        fh, gh = self.history(job_id)
        u = np.zeros(n_c * n_t)
        r = A.OptResult()
        rc = A.lib().pgx_fetch(self._h, int(job_id), A.as_dptr(u), C.byref(r))
        if rc == 9:
            A.check(rc)
        self._shape.pop(int(job_id), None)
        state = "done" if rc == 0 else ("cancelled" if rc == 8 else "failed")
        return JobResult(int(job_id), state, u.reshape(n_t, n_c).T.copy(), r.fidelity, int(r.n_iterations),
                         bool(r.converged), r.reason.decode(errors="replace"), r.total_time_s,
                         r.step_size_final, fh, gh, int(r.n_fidelity_evals), int(r.n_gradient_evals))

    def cancel(self, job_id: int):
        A.check(A.lib().pgx_cancel(self._h, int(job_id)))

    def drain(self, timeout_s: float = 0.0) -> bool:
        rc = A.lib().pgx_server_drain(self._h, float(timeout_s))
        if rc == 7:
            return False
        A.check(rc)
        return True

    def stats(self) -> dict:
        s = A.ServeStats()
        A.check(A.lib().pgx_server_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in A.ServeStats._fields_}


@dataclass
class OptOutcome:
    controls: np.ndarray
    fidelity: float
    fidelity_history: list
    gradient_norm_history: list
    n_iterations: int
    converged: bool
    termination_reason: str
    total_time: float
    n_fidelity_evaluations: int
    n_gradient_evaluations: int
    step_size_final: float


def problem_desc(drifts, controls, dt, *, generator: str = "hermitian", offset_op=None,
                 member_drift=None, member_scale=None, member_offset=None, member_weight=None,
                 target: str = "gate", fidelity: str = "square", grad_mode: str = "exact",
                 precision: str = "fp64", target_op=None, states_init=None, states_target=None,
                 grad_states_init=None, n_members: Optional[int] = None):
    """pgx_problem_desc of an ensemble problem; returns (desc, keep, (D, n_c, n_t,
    n_members, n_pairs)) where ``keep`` holds the buffers desc points into."""
    drifts = np.asarray(drifts, np.complex128)
    if drifts.ndim == 2:
        drifts = drifts[None]
    controls = np.asarray(controls, np.complex128)
    dt = np.ascontiguousarray(np.asarray(dt, np.float64).ravel())
    D = drifts.shape[-1]
    n_c, n_t = controls.shape[0], dt.size
    nm = n_members
    for arr in (member_drift, member_scale, member_offset, member_weight):
        if arr is not None:
            nm = len(arr) if nm is None else nm
    n_members = nm if nm is not None else 1
    keep = {}

    def buf(name, val):
        keep[name] = val
        return A.as_dptr(val) if val is not None else None

    d = A.ProblemDesc()
    d.struct_size = C.sizeof(A.ProblemDesc)
    d.dim, d.n_controls, d.n_slices = D, n_c, n_t
    d.generator, d.target = A.GEN[generator], A.TARGET[target]
    d.fidelity, d.grad_mode, d.precision = A.FID[fidelity], A.GRAD[grad_mode], A.PREC[precision]
    d.n_drifts, d.n_members = drifts.shape[0], n_members
    d.dt = buf("dt", dt)
    d.drifts = buf("drifts", A.cmat_buf(drifts))
    d.controls = buf("controls", A.cmat_buf(controls))
    d.offset_op = buf("off", None if offset_op is None else A.cmat_buf(offset_op))
    if member_drift is not None:
        md = np.ascontiguousarray(np.asarray(member_drift, np.int32))
        keep["md"] = md
        d.member_drift = md.ctypes.data_as(A.iptr)
    for field, name, arr in (("member_scale", "ms", member_scale),
                             ("member_offset", "mo", member_offset),
                             ("member_weight", "mw", member_weight)):
        if arr is not None:
            setattr(d, field, buf(name, np.ascontiguousarray(np.asarray(arr, np.float64))))
    if target == "gate":
        d.n_pairs = 0
        d.target_op = buf("tgt", A.cmat_buf(target_op))
    else:
        si = np.atleast_2d(np.asarray(states_init, np.complex128))
        stt = np.atleast_2d(np.asarray(states_target, np.complex128))
        d.n_pairs = si.shape[0]
        d.states_init = buf("si", A.cvec_buf(si))
        d.states_target = buf("st", A.cvec_buf(stt))
        if grad_states_init is not None:
            d.grad_states_init = buf("sg", A.cvec_buf(np.atleast_2d(
                np.asarray(grad_states_init, np.complex128))))
    return d, keep, (D, n_c, n_t, n_members, d.n_pairs)


class Problem:
    """An ensemble GRAPE problem resident in device memory (pgx_problem)."""

    def __init__(self, drifts, controls, dt, *, ctx: Optional[Context] = None,
                 generator: str = "hermitian", offset_op=None, member_drift=None,
                 member_scale=None, member_offset=None, member_weight=None,
                 target: str = "gate", fidelity: str = "square", grad_mode: str = "exact",
                 precision: str = "fp64", target_op=None, states_init=None, states_target=None,
                 grad_states_init=None, n_members: Optional[int] = None):
        self.ctx = ctx or default_context()
        d, keep, dims = problem_desc(
            drifts, controls, dt, generator=generator, offset_op=offset_op,
            member_drift=member_drift, member_scale=member_scale, member_offset=member_offset,
            member_weight=member_weight, target=target, fidelity=fidelity, grad_mode=grad_mode,
            precision=precision, target_op=target_op, states_init=states_init,
            states_target=states_target, grad_states_init=grad_states_init, n_members=n_members)
        self.D, self.n_c, self.n_t, self.n_members, _ = dims
        self._keep = keep
        self.n_pairs = d.n_pairs
        self._h = C.c_void_p()
        A.check(A.lib().pgx_problem_create(self.ctx.handle, C.byref(d), C.byref(self._h)),
                self.ctx.handle)
        self._desc = d
        self._u = np.zeros(self.n_c * self.n_t)
        self._G = np.zeros(self.n_c * self.n_t)

    def close(self):
        if getattr(self, "_h", None):
            A.lib().pgx_problem_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _load_u(self, u) -> np.ndarray:
        u = np.asarray(u, np.float64)
        if u.shape != (self.n_c, self.n_t):
            raise ValueError(f"controls have shape {u.shape}, expected {(self.n_c, self.n_t)}")
        self._u[:] = u.T.ravel()   # column-major [n_c x n_t]
        return self._u

    def eval(self, u, want_grad: bool = True, stats: bool = False):
        """(F, G[n_c, n_t]) at controls u[n_c, n_t]; G is None when not wanted."""
        ub = self._load_u(u)
        F = C.c_double()
        st = A.EvalStats()
        A.check(A.lib().pgx_eval(self._h, A.as_dptr(ub), C.byref(F),
                                 A.as_dptr(self._G) if want_grad else None, C.byref(st) if stats else None),
                self.ctx.handle)
        G = self._G.reshape(self.n_t, self.n_c).T.copy() if want_grad else None
        if stats:
            return float(F.value), G, {"ms_device": st.ms_device, "ms_host": st.ms_host,
                                       "units": int(st.units), "n_launches": int(st.n_launches),
                                       "residual": st.residual,
                                       "residual_kind": A.RESIDUAL_KIND.get(int(st.residual_kind), "?")}
        return float(F.value), G

    def eval_device(self, d_u: int, d_F: int, d_G: Optional[int]):
        A.check(A.lib().pgx_eval_device(self._h, C.c_void_p(d_u), C.c_void_p(d_F),
                                        C.c_void_p(d_G) if d_G else None), self.ctx.handle)

    def autotune(self, u, reps: int = 3) -> str:
        """Pick the fastest team size of each tunable kernel for this problem
        (results are identical for every choice); returns the timing report."""
        ub = self._load_u(u)
        buf = C.create_string_buffer(1024)
        A.check(A.lib().pgx_autotune(self._h, A.as_dptr(ub), int(reps), buf, 1024), self.ctx.handle)
        return buf.value.decode()

    def set_drifts(self, drifts):
        """Replace the drift matrices [n_drifts, D, D] (same count as at creation)."""
        d = np.asarray(drifts, np.complex128)
        if d.ndim == 2:
            d = d[None]
        A.check(A.lib().pgx_problem_set_drifts(self._h, A.as_dptr(A.cmat_buf(d))), self.ctx.handle)

    def eval_aggregate(self, u, aggregator: str = "mean", alpha: float = 0.2, want_grad: bool = True):
        """(F, G) of the member-aggregated objective: "mean", "worst_case" or
        "cvar" with tail fraction alpha (EnsembleObjective.jl:169-217)."""
        ub = self._load_u(u)
        F = C.c_double()
        A.check(A.lib().pgx_eval_aggregate(self._h, A.as_dptr(ub), A.AGGREGATOR[aggregator], float(alpha),
                                           C.byref(F), A.as_dptr(self._G) if want_grad else None),
                self.ctx.handle)
        G = self._G.reshape(self.n_t, self.n_c).T.copy() if want_grad else None
        return float(F.value), G

    def set_penalties(self, penalties):
        """Subtract waveform penalties from every later evaluation:
        penalties = [(type, weight[, l_bound, u_bound]), ...] with type one of
        NS, SNS, SNSA, DNS, energy (Penalties.jl:197-330)."""
        arr = penalty_array(penalties)
        A.check(A.lib().pgx_problem_set_penalties(self._h, len(penalties), C.cast(arr, C.c_void_p)), self.ctx.handle)

    def set_tracking(self, steps, weights, targets):
        """Trajectory-tracking objective (pgx_problem_set_tracking,
        GRAPETracking.jl): checkpoints at 1-based steps with weights and
        target density matrices [n, D, D]; empty lists restore the terminal
        objective."""
        st = np.ascontiguousarray(np.asarray(steps, np.int64).astype(np.int32).ravel())
        wt = np.ascontiguousarray(np.asarray(weights, np.float64).ravel())
        n = int(st.size)
        if wt.size != n:
            raise ValueError("steps and weights must have the same length")
        if n == 0:
            A.check(A.lib().pgx_problem_set_tracking(self._h, 0, None, None, None), self.ctx.handle)
            return
        tg = np.asarray(targets, np.complex128)
        if tg.shape != (n, self.D, self.D):
            raise ValueError(f"targets have shape {tg.shape}, expected {(n, self.D, self.D)}")
        tb = A.cmat_buf(tg)
        A.check(A.lib().pgx_problem_set_tracking(self._h, n, st.ctypes.data_as(A.iptr), A.as_dptr(wt),
                                                 A.as_dptr(tb)), self.ctx.handle)

    def set_drift_ramp(self, ops, member_op, tau):
        """Per-slice drift ramp (pgx_problem_set_drift_ramp): member m adds
        tau[k] ops[member_op[m]] at slice k; empty ops remove it."""
        ops = np.asarray(ops, np.complex128)
        if ops.size == 0:
            A.check(A.lib().pgx_problem_set_drift_ramp(self._h, 0, None, None, None), self.ctx.handle)
            return
        if ops.ndim != 3 or ops.shape[1:] != (self.D, self.D):
            raise ValueError(f"ops have shape {ops.shape}, expected (n, {self.D}, {self.D})")
        mo = np.ascontiguousarray(np.asarray(member_op, np.int64).astype(np.int32).ravel())
        tv = np.ascontiguousarray(np.asarray(tau, np.float64).ravel())
        if mo.size != self.n_members or tv.size != self.n_t:
            raise ValueError("member_op needs one entry per member and tau one per slice")
        ob = A.cmat_buf(ops)
        A.check(A.lib().pgx_problem_set_drift_ramp(self._h, ops.shape[0], A.as_dptr(ob), mo.ctypes.data_as(A.iptr),
                                                   A.as_dptr(tv)), self.ctx.handle)

    def eval_phase(self, phi, amplitudes=None, want_grad: bool = True):
        """Phase-only evaluation (pgx_eval_phase, GRAPEPhase.jl): phases and
        amplitudes [n_c / 2, n_t]; returns (F, dF/dphi or None)."""
        ph = np.asarray(phi, np.float64)
        if ph.shape != (self.n_c // 2, self.n_t):
            raise ValueError(f"phases have shape {ph.shape}, expected {(self.n_c // 2, self.n_t)}")
        pb = np.ascontiguousarray(ph.T.ravel())
        ab = None if amplitudes is None else np.ascontiguousarray(np.asarray(amplitudes, np.float64).T.ravel())
        F = C.c_double()
        G = np.zeros(pb.size) if want_grad else None
        A.check(A.lib().pgx_eval_phase(self._h, A.as_dptr(pb), None if ab is None else A.as_dptr(ab), C.byref(F),
                                       None if G is None else A.as_dptr(G)), self.ctx.handle)
        return float(F.value), (None if G is None else G.reshape(self.n_t, self.n_c // 2).T.copy())

    @property
    def teams(self) -> tuple:
        """(expm, gradient) team sizes of the mixed kernels in use."""
        out = []
        for k in (0, 1):
            t = C.c_int32()
            A.check(A.lib().pgx_problem_get_team(self._h, k, C.byref(t)), self.ctx.handle)
            out.append(int(t.value))
        return tuple(out)

    def set_teams(self, expm: int = 0, grad: int = 0):
        """Fix the team sizes (0 = default), e.g. a plan from an earlier autotune."""
        for k, t in ((0, expm), (1, grad)):
            A.check(A.lib().pgx_problem_set_team(self._h, k, int(t)), self.ctx.handle)

    def member_fidelities(self) -> np.ndarray:
        out = np.zeros(self.n_members)
        A.check(A.lib().pgx_member_fidelities(self._h, A.as_dptr(out)), self.ctx.handle)
        return out

    def total_propagator(self, u, member: int = 0) -> np.ndarray:
        ub = self._load_u(u)
        out = np.zeros(2 * self.D * self.D)
        A.check(A.lib().pgx_total_propagator(self._h, A.as_dptr(ub), int(member), A.as_dptr(out)),
                self.ctx.handle)
        return A.cmat_from_buf(out, self.D)

    def optimize(self, u0, method: str, *, max_iter: int = 1000, convergence_tol: float = 1e-8,
                 step_size: float = 0.01, adapt_step_size: bool = True, min_step_size: float = 1e-10,
                 max_step_size: float = 10.0, gradient_norm_tol: float = 1e-6,
                 lbfgs_memory: int = 10, amplitude_limit: float = math.inf,
                 l_bound: float = -1.0, u_bound: float = 1.0, history_cap: int = 0) -> OptOutcome:
        o = opt_desc(method, max_iter=max_iter, convergence_tol=convergence_tol, step_size=step_size,
                     adapt_step_size=adapt_step_size, min_step_size=min_step_size,
                     max_step_size=max_step_size, gradient_norm_tol=gradient_norm_tol,
                     lbfgs_memory=lbfgs_memory, amplitude_limit=amplitude_limit, l_bound=l_bound,
                     u_bound=u_bound)
        ub = self._load_u(u0).copy()
        cap = history_cap or (4 * max_iter + 8)
        fh, gh = np.zeros(cap), np.zeros(cap)
        r = A.OptResult()
        A.check(A.lib().pgx_optimize(self._h, C.byref(o), A.as_dptr(ub), A.as_dptr(fh),
                                     A.as_dptr(gh), cap, C.byref(r)), self.ctx.handle)
        n = min(r.history_len, cap)
        n_g = min(r.gnorm_history_len, cap)
        return OptOutcome(ub.reshape(self.n_t, self.n_c).T.copy(), float(r.fidelity),
                          fh[:n].tolist(), gh[:n_g].tolist(),
                          int(r.n_iterations), bool(r.converged), r.reason.decode(),
                          float(r.total_time_s), int(r.n_fidelity_evals), int(r.n_gradient_evals),
                          float(r.step_size_final))
