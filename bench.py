"""Benchmark: ensemble-slice gradients per second of the GRAPE hot path.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload spin4|uneven512|lindblad3q|serve] [--precision mixed|fp64]

Workloads (seeded synthetic inputs with the configurations' shapes):
  spin4 (default)  broadband robust gate: 4 coupled spin-1/2 (d = 16), 231
                   members (21 offsets x 11 B1 scales), 1000 slices of 1 us, two
                   controls, exact Frechet gradient.  Step = one evaluation
                   (F, dF/du) = 231,000 member-slice units.
  uneven512        512 independent problems, d in {2,4,8,16,32}, 50-2000 slices,
                   1-128 members, 2-6 controls; step = one batched GRAPE
                   iteration (one CUDA graph).
  spin4_states     the spin4 system as an MR state-transfer ensemble (two
                   basis-state pairs per member; grape_state_kernel's form).
  lindblad3q       3-qubit Lindblad gate (superoperator D = 64), 32 detuning
                   draws, 500 slices, exact gradient.
  serve            Poisson job stream through the continuous-batching server
                   (pgx_server): uneven-distribution jobs plus 20 % Lindblad
                   gate jobs on 2-3 qubits, submitted in real time; reports
                   served units/s, jobs/s, p50/p99 time-to-converged-pulse and
                   |dF| of the served results against the FP64 GPU path.

value : units/s with controls and results resident in HBM, CUDA events on the
        library's stream; each step's working set (propagator and chain stacks)
        is far larger than the 129 MB L2, so no flush is needed.
e2e   : the same metric through the reference-facing calls with host buffers:
        H2D of the controls from pinned memory and D2H of (F, G) inside the
        timed region, wall clock.
--impl reference : the reference's CPU algorithm as the oracle's multi-threaded
        C restatement on the host cores, on the reference's arithmetic stack
        (LAPACK zheevr eigendecompositions, BLAS zgemm products, one BLAS thread
        per member thread), computing the same gradient as this arm (Julia, the
        reference's language, is not installed, so the reference itself cannot
        run).

The default spin4 line also carries extra keys measured in the same run:
first_order (the reference's first-order gradient on the GPU and CPU),
lbfgs200 (200 L-BFGS iterations of the ensemble end to end through the
optimiser API), uneven512 (one batched iteration over 512 uneven problems,
mixed and FP64) and serve (a Poisson job stream through the server with the
served-job stop rule F >= 0.999 or 500 iterations, plus the server's capacity
on a fixed job set, mixed and FP64).  --no-extras skips them.
"""
from __future__ import annotations

import os

# the CPU baseline pins BLAS to one thread per member thread; OpenBLAS reads
# this when it loads
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import argparse
import json
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ensemble-slice grads/s"
UNIT = "units/s"
K_EXP = 8  # conventional matrix-product count of one expm in the FLOP model

# DRAM bytes per launch of the dominant kernel from ncu captures of a smaller
# case (spin-4: 200 of 1000 slices; lindblad3q: 100 of 500), scaled by the
# units a full launch processes (every unit reads or writes the same bytes).
TRAFFIC = {("spin4", "fp64", "grad"): 5 * (190.615296e6 + 4.743936e6),
           # k_expm_mx<16,128,Herm>, 200-slice capture: 0.1 MB read, the df U stack written
           ("spin4", "mixed", "expm"): 5 * (0.095232e6 + 127.364352e6),
           ("spin4", "mixed", "grad"): 5 * (94.700544e6 + 2.850816e6),
           ("spin4", "mixed", "chain_fwd"): 5 * (189.268736e6 + 67.549952e6),
           # k_expm_oz64 (tensor cores), 100-slice capture: the prologue's planar
           # generator read once, the df U stack written once
           ("lindblad3q", "mixed", "expm"): 5 * (210.639104e6 + 194.420224e6)}
# Tensor-pipe activity of k_expm_oz64 from an ncu capture (lindblad3q, 100 of
# 500 slices): sm__pipe_tensor_cycles_active, % of peak while active.
TENSOR_ACTIVE_PCT = {("lindblad3q", "mixed", "expm"): 17.3}
# FP32 operations one df32 complex MAC executes (error-free two_prod / two_sum
# accumulation) per 8 FLOPs of the FP64 model: the model-FLOP rate a fully
# busy FP32 pipe could reach on df32 work is the FP32 peak / (DF_OPS / 8).
DF_OPS_PER_CMAC = 46


def flops_per_unit(stage: str, D: int, n_c: int, grad_mode: str, n_pairs: int = 0) -> float:
    """Algorithmic FLOPs per member-slice unit (complex MAC = 8 FLOPs), the
    conventional model W = 8 D^3 (K_exp (1 + 2 n_c) + 3) + 8 n_c D^2 split by
    stage: expm K_exp products, forward chain 1, backward chain + costate 2,
    gradient the Frechet terms 2 n_c K_exp products + n_c traces.  State
    targets (n_pairs > 0) follow the state-vector model W_v = 8 D^3 K_exp
    (1 + 2 n_c) + 8 D^2 (2 + n_c): matrix-vector chains, n_c contractions."""
    d3 = 8.0 * D ** 3
    if stage == "expm":
        return d3 * K_EXP
    if stage == "chain_fwd":
        return d3 if not n_pairs else 8.0 * D ** 2
    if stage == "chain_bwd":
        return 2 * d3 if not n_pairs else 8.0 * D ** 2
    if stage == "grad":
        return (d3 * K_EXP * 2 * n_c if grad_mode == "exact" else 0.0) + 8.0 * n_c * D ** 2
    if stage == "all":
        return sum(flops_per_unit(s, D, n_c, grad_mode, n_pairs) for s in ("expm", "chain_fwd", "chain_bwd", "grad"))
    return 0.0


def executed_flops_per_unit(D: int, n_c: int, grad_mode: str, n_pairs: int = 0) -> float:
    """FLOPs per unit counting the work the kernels execute: the same stage
    model as flops_per_unit, except that the exact gradient runs ONE Frechet
    derivative per slice (the pair (f, L_f) = 2 K_exp products) whatever n_c,
    where the conventional model counts 2 n_c K_exp products."""
    if grad_mode != "exact":
        return flops_per_unit("all", D, n_c, grad_mode, n_pairs)
    d3 = 8.0 * D ** 3
    rest = sum(flops_per_unit(s, D, n_c, grad_mode, n_pairs) for s in ("expm", "chain_fwd", "chain_bwd"))
    return rest + d3 * 2 * K_EXP + 8.0 * n_c * D ** 2


def measured_peaks() -> dict:
    """Roofline denominators: the machine's measured HBM copy bandwidth and cuBLAS
    bf16 GEMM rate (MEASURED_PEAKS.json beside this file), else the earlier
    GB300 measurement used as a fallback."""
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "bf16_tflops_sustained": float(d.get("bf16_tflops_sustained", d["bf16_tflops"])),
                "source": "of measured (MEASURED_PEAKS.json: bf16 GEMM burst)"}
    except (OSError, ValueError, KeyError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "source": "of fallback (6.8 TB/s, 1.9 PFLOP/s bf16)"}


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """x of the slowest rank, on every rank: the job takes as long as its
    slowest replica."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, units_per_rank: float, seconds: float) -> float:
    """Whole-job throughput of `world` replicas that each processed
    units_per_rank within `seconds` (the slowest rank's time)."""
    return world * units_per_rank / seconds


def guarded(fn, *a, **k):
    """Run an extra measurement; a failure is recorded in the line, not raised."""
    try:
        return fn(*a, **k)
    except Exception as e:  # noqa: BLE001 - the headline line must still print
        return {"error": f"{type(e).__name__}: {e}"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.proc, self.lines = gpu, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_problem(pg, ctx, spec, grad_mode: str, precision: str):
    return pg.Problem(ctx=ctx, **spec.problem_kwargs(grad_mode, precision))


def single_config(name: str, spec, grad_mode: str, n_gpus: int) -> dict:
    """The workload's config, identical in both arms (nothing arm-specific)."""
    cfg = {"workload": name, "members": spec.n_members, "slices": spec.n_t, "d": spec.D,
           "n_controls": spec.n_c, "generator": spec.generator, "grad_mode": grad_mode,
           "parallelism": f"replicas x{n_gpus}", "l2": "per-step working set >> 129 MB L2 (no flush needed)"}
    if spec.target != "gate":
        cfg.update(target=spec.target, n_pairs=spec.n_pairs)
    return cfg


def single_workload(name: str, n_t):
    from pulsar_gb300 import workloads as W
    if name == "spin4":
        prob, u0 = W.spin4_ensemble(n_t=n_t or 1000)
        return f"spin4_d16_231members_{prob.n_t}slices", prob, u0
    if name == "spin4_states":
        prob, u0 = W.spin4_state_transfer(n_t=n_t or 1000)
        return f"spin4_states_d16_231members_2pairs_{prob.n_t}slices", prob, u0
    if name == "lindblad3q":
        prob, u0 = W.lindblad_3q(n_t=n_t or 500)
        return f"lindblad3q_D64_32members_{prob.n_t}slices", prob, u0
    raise ValueError(name)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

class Single:
    """One ensemble problem; step = one (F, G) evaluation."""

    def __init__(self, name, prob, u0, pg, ctx, grad_mode, precision, torch, dev, teams=None, tune=True):
        self.name, self.prob, self.u0, self.grad_mode, self.precision = name, prob, u0, grad_mode, precision
        self.ctx = ctx
        self.p = gpu_problem(pg, ctx, prob, grad_mode, precision)
        self.units_per_step = prob.n_members * prob.n_t
        if precision != "mixed":
            self.tune = "FP64 path: no tunable kernels"
        elif teams:
            self.p.set_teams(*teams)
            self.tune = f"fixed teams (expm, grad) = {self.p.teams}"
        elif tune:
            self.tune = self.p.autotune(u0, reps=2) + f" -> (expm, grad) = {self.p.teams}"
        else:
            self.tune = f"default teams (expm, grad) = {self.p.teams}"
        self.d_u = torch.tensor(np.ascontiguousarray(u0.T).ravel(), dtype=torch.float64, device=dev)
        self.d_F = torch.zeros(2, dtype=torch.float64, device=dev)
        self.d_G = torch.zeros(u0.size, dtype=torch.float64, device=dev)
        self.h2d, self.d2h = int(u0.size * 8), int(u0.size * 8 + 8)

    def step_device(self):
        self.p.eval_device(self.d_u.data_ptr(), self.d_F.data_ptr(), self.d_G.data_ptr())

    def step_e2e(self):
        self.F, self.G = self.p.eval(self.u0)

    def run_device(self, K):
        for _ in range(K):
            self.step_device()
        return K * self.units_per_step

    def timed(self, warm: int, K: int) -> float:
        """Device-resident units/s over K evaluations after `warm` untimed ones."""
        for _ in range(warm):
            self.step_device()
        self.ctx.synchronize()
        self.ctx.timer_start()
        u = self.run_device(K)
        return u / (self.ctx.timer_stop() * 1e-3)

    def stage_flops(self, stage):
        return flops_per_unit(stage, self.prob.D, self.prob.n_c, self.grad_mode, self.prob.n_pairs) * self.units_per_step

    def cpu_sample(self, budget_s):
        return cpu_baseline_single(self.prob, self.u0, budget_s, self.grad_mode)

    def objective(self):
        return float(self.p.eval(self.u0, want_grad=False)[0])

    def close(self):
        self.p.close()


class Uneven:
    """512 uneven problems; step = one batched GRAPE iteration (CUDA graph)."""

    def __init__(self, name, cases, pg, ctx, grad_mode, precision):
        self.name, self.cases, self.grad_mode, self.precision = name, cases, grad_mode, precision
        self.ctx = ctx
        self.probs = [gpu_problem(pg, ctx, pr, grad_mode, precision) for pr, _ in cases]
        # autotuned tiles: one problem per (d, n_controls) key is tuned at its
        # own controls and the others take its plan (variants are bit-identical)
        self.tune = "defaults (FP64 path: no tunable kernels)"
        if precision == "mixed":
            plans = {}
            for p, (pr, u0) in zip(self.probs, cases):
                key = (pr.D, pr.n_c)
                if key not in plans:
                    p.autotune(u0, reps=2)
                    plans[key] = p.teams
                else:
                    p.set_teams(*plans[key])
            self.tune = (f"autotuned per (d, n_controls) key at load time ({len(plans)} keys tuned, "
                         f"{len(self.probs) - len(plans)} problems took the plan of their key)")
        self.batch = pg.Batch(self.probs, n_streams=16)
        for i, (_, u0) in enumerate(cases):
            self.batch.set_controls(i, u0)
        self.units_per_step = self.batch.units
        self.h2d = int(sum(u0.size * 8 for _, u0 in cases))
        self.d2h = int(sum(u0.size * 8 + 8 for _, u0 in cases))

    def run_device(self, K):
        # iterate(K) performs one extra evaluation at the start (the initial history entry)
        self.batch.iterate(K, trace=False, step_size=0.01)
        return (K + 1) * self.units_per_step

    def timed(self, warm: int, K: int) -> tuple:
        """(units/s, ms per evaluation of all problems) over one K-iteration call."""
        if warm:
            self.run_device(warm)
        self.ctx.synchronize()
        self.ctx.timer_start()
        u = self.run_device(K)
        ms = self.ctx.timer_stop()
        return u / (ms * 1e-3), ms / (K + 1)

    def step_e2e(self):
        for i, (_, u0) in enumerate(self.cases):
            self.batch.set_controls(i, u0)
        self.trace = self.batch.iterate(1, trace=True, step_size=0.01)
        for i in range(len(self.cases)):
            self.batch.get_controls(i)

    def e2e_units(self):
        return 2 * self.units_per_step

    def total_flops(self):
        return sum(flops_per_unit("all", pr.D, pr.n_c, self.grad_mode) * pr.n_members * pr.n_t
                   for pr, _ in self.cases)

    def config(self, n_gpus: int):
        ds = [pr.D for pr, _ in self.cases]
        return {"workload": self.name, "problems": len(self.cases), "d_values": sorted(set(ds)),
                "units_per_iteration": self.units_per_step, "execution": "one CUDA graph per iteration",
                "grad_mode": self.grad_mode, "parallelism": f"replicas x{n_gpus}",
                "l2": "per-step working set >> 129 MB L2 (no flush needed)"}

    def cpu_sample(self, budget_s):
        sample = [c for c in self.cases if c[0].D <= 16][:16]
        return cpu_baseline_multi(sample, budget_s, self.grad_mode)

    def objective(self):
        return float(np.mean(self.batch.eval()))

    def close(self):
        self.batch.close()
        for p in self.probs:
            p.close()


# ---------------------------------------------------------------------------
# serving
# ---------------------------------------------------------------------------

SERVE_TARGET_F = 0.999  # the served-job stop rule: F >= 0.999 (or the iteration cap)


def _pct(a, q):
    return float(np.percentile(a, q)) if len(a) else None


def serve_latency(pg, ctx, precision: str, *, rate: float, seconds: float, seed: int, max_slices: int,
                  max_members: int, lindblad_slices: int, lindblad_draws: int, max_iter: int, method: str,
                  slots: int, budget_gb: float, step: float, check: int) -> dict:
    """A Poisson job stream submitted in real time through the public server
    API (host buffers in, best controls out), then a drain.  Every job stops
    at F >= 0.999 or `max_iter` iterations (or its method's own rules).
    Latency = submit -> finished job; it splits into the queueing delay
    (submit -> admission) and the run time (admission -> finished)."""
    from pulsar_gb300 import workloads as W
    warm = W.serve_stream(seed=1, rate=50.0, duration_s=0.08, lindblad_frac=0.5, max_slices=60,
                          max_members=4, lindblad_slices=20, lindblad_draws=2)
    jobs = W.serve_stream(seed=seed, rate=rate, duration_s=seconds, max_slices=max_slices,
                          max_members=max_members, lindblad_slices=lindblad_slices,
                          lindblad_draws=lindblad_draws)
    opt = dict(max_iter=max_iter, step_size=step)
    if method == "ensemble_lbfgs":
        opt["lbfgs_memory"] = 10
    kw = [j.spec.problem_kwargs("exact", precision) for j in jobs]
    srv = pg.Server(ctx, max_inflight=slots, hbm_budget_bytes=int(budget_gb * 1e9), target_fidelity=SERVE_TARGET_F)
    for j in warm:  # first-use costs (module load, shared-memory limits) stay out of the timed region
        srv.submit(u0=j.u0, opt=dict(max_iter=3, step_size=step), **j.spec.problem_kwargs("exact", precision))
    srv.drain()
    s0 = srv.stats()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t0 = time.perf_counter()
        ids = []
        for j, k in zip(jobs, kw):
            dt = t0 + j.arrival_s - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            ids.append(srv.submit(u0=j.u0, opt=opt, method=method, **k))
        srv.drain()
        el = time.perf_counter() - t0
    st = srv.stats()
    polls = [srv.poll(i) for i in ids]
    res = [srv.fetch(i) for i in ids]
    srv.close()
    done = [(r, q) for r, q in zip(res, polls) if r.state == "done"]
    lat = np.array([q["latency_s"] for _, q in done])
    queue = np.array([q["queue_s"] for _, q in done])
    conv = np.array([q["latency_s"] for r, q in done if r.fidelity >= SERVE_TARGET_F])
    run = lat - queue
    # |dF| of the served result against the plain FP64 GPU path at the returned controls
    rng = np.random.default_rng(0)
    pick = rng.choice(len(jobs), size=min(check, len(jobs)), replace=False)
    dF = []
    for i in pick:
        if res[i].state != "done":
            continue
        p = pg.Problem(ctx=ctx, **jobs[i].spec.problem_kwargs("exact", "fp64"))
        dF.append(abs(p.eval(res[i].controls, want_grad=False)[0] - res[i].fidelity))
        p.close()
    kinds = {}
    for j in jobs:
        kinds[j.kind] = kinds.get(j.kind, 0) + 1
    flops = sum(flops_per_unit("all", j.spec.D, j.spec.n_c, "exact") * j.spec.n_members * j.spec.n_t *
                (r.n_iterations + 1) for j, r in zip(jobs, res))
    h2d = sum(8 * (k["drifts"].size * 2 + k["controls"].size * 2 + j.u0.size) for j, k in zip(jobs, kw))
    return {
        "stream": {"offered_rate_jobs_s": rate, "arrival_window_s": seconds, "jobs": len(jobs), "job_kinds": kinds,
                   "max_slices": max_slices, "max_members": max_members,
                   "lindblad": f"2-3 qubits, {lindblad_slices} slices, {lindblad_draws} draws", "method": method,
                   "stop": f"F >= {SERVE_TARGET_F} or {max_iter} iterations (or the method's own rules)",
                   "slots": slots, "hbm_budget_gb": budget_gb, "precision": precision, "grad_mode": "exact",
                   "shape_vs_full_stream": "scaled down from 200 jobs/s for 60 s with up to 2000 slices x 128 "
                                           "members (80 %) and 500-slice x 32-draw Lindblad jobs (20 %)"},
        "elapsed_s": el, "units": int(st["units"] - s0["units"]),
        "units_per_s": (st["units"] - s0["units"]) / el,
        "model_tflops": flops / el / 1e12,
        "completed": len(done), "failed": int(sum(r.state == "failed" for r in res)),
        "jobs_per_s": len(done) / el,
        "converged_frac": float(len(conv) / max(len(done), 1)),
        "p50_latency_s": _pct(lat, 50), "p99_latency_s": _pct(lat, 99),
        "p50_latency_converged_s": _pct(conv, 50), "p99_latency_converged_s": _pct(conv, 99),
        "p50_queue_s": _pct(queue, 50), "p99_queue_s": _pct(queue, 99),
        "p50_run_s": _pct(run, 50), "p99_run_s": _pct(run, 99),
        "mean_iterations": float(np.mean([r.n_iterations for r in res])),
        "hbm_peak_gb": st["hbm_peak"] / 1e9,
        "max_abs_dF_vs_fp64_gpu": max(dF) if dF else None,
        "median_abs_dF_vs_fp64_gpu": float(np.median(dF)) if dF else None, "dF_sample": len(dF),
        "launches": int(st["kernel_launches"] - s0["kernel_launches"]),
        "h2d_bytes": int(h2d), "d2h_bytes": int(sum(8 * j.u0.size for j in jobs)),
        "clocks": clk.summary(),
    }


def serve_capacity(pg, ctx, *, n_jobs: int = 64, max_iter: int = 50, slots: int = 128) -> dict:
    """The server's throughput on one fixed job set submitted at once (the
    device saturated), mixed and plain FP64, every job running exactly
    `max_iter` GRAPE iterations (the fidelity target and the stall and
    gradient-norm rules are off, so both precisions do the same work)."""
    from pulsar_gb300 import workloads as W
    jobs = W.serve_stream(seed=9, rate=1000.0, duration_s=1.0, max_slices=200, max_members=16,
                          lindblad_slices=50, lindblad_draws=4)[:n_jobs]
    opt = dict(max_iter=max_iter, step_size=0.01, convergence_tol=1e-300, gradient_norm_tol=1e-300)
    out = {"jobs": len(jobs), "iterations_per_job": max_iter, "method": "grape",
           "job_set": "first jobs of the served stream's distribution (up to 200 slices x 16 members, "
                      "20 % Lindblad 2-3 qubits x 50 slices x 4 draws), all submitted at t = 0"}
    for prec in ("mixed", "fp64"):
        srv = pg.Server(ctx, max_inflight=slots, hbm_budget_bytes=int(80e9), target_fidelity=2.0)
        for j in jobs[:4]:  # warm the kernels of this precision
            srv.submit(u0=j.u0, opt=dict(opt, max_iter=2), **j.spec.problem_kwargs("exact", prec))
        srv.drain()
        s0 = srv.stats()
        t0 = time.perf_counter()
        for j in jobs:
            srv.submit(u0=j.u0, opt=opt, method="grape", **j.spec.problem_kwargs("exact", prec))
        srv.drain()
        el = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        out[prec] = {"units_per_s": (st["units"] - s0["units"]) / el, "elapsed_s": el,
                     "jobs_per_s": len(jobs) / el, "units": int(st["units"] - s0["units"])}
    out["mixed_over_fp64"] = out["mixed"]["units_per_s"] / out["fp64"]["units_per_s"]
    return out


def run_serve(args, pg, ctx, rank: int, world: int, dist=None, dev=None):
    """--workload serve: the Poisson stream as the line's value; with several
    ranks every rank serves its own copy of the stream (replicas), and the
    value is all ranks' units over the slowest rank's wall time."""
    r = serve_latency(pg, ctx, args.precision, rate=args.serve_rate, seconds=args.serve_seconds,
                      seed=args.serve_seed, max_slices=args.serve_max_slices,
                      max_members=args.serve_max_members, lindblad_slices=args.serve_lindblad_slices,
                      lindblad_draws=args.serve_lindblad_draws, max_iter=args.serve_max_iter,
                      method=args.serve_method, slots=args.serve_slots, budget_gb=args.serve_budget_gb,
                      step=args.serve_step, check=args.serve_check)
    elapsed = max_over_ranks(r["elapsed_s"], dist, dev)
    value = job_rate(world, r["units"], elapsed)
    pk = measured_peaks()
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        from pulsar_gb300 import workloads as W
        jobs = W.serve_stream(seed=args.serve_seed, rate=args.serve_rate, duration_s=args.serve_seconds,
                              max_slices=args.serve_max_slices, max_members=args.serve_max_members)
        herm = [(j.spec, j.u0) for j in jobs if j.spec.generator == "hermitian" and j.spec.D <= 16][:16]
        cpu = cpu_baseline_multi(herm, args.cpu_budget_s, "exact")
    cfg = dict(r["stream"], workload="serve", parallelism=f"replicas x{world}",
               l2="many concurrent jobs; working set of the stream >> 129 MB L2",
               timed_region="first submission -> drain (wall clock)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": 1,
            "warmup": 3, "ms_per_step": elapsed * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+df32(f64 overlap)",
            "data": "synthetic (seeded Poisson job stream)", "config": cfg,
            "serve": {k: v for k, v in r.items() if k not in ("stream", "clocks", "h2d_bytes", "d2h_bytes")},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": r["h2d_bytes"],
                    "d2h_bytes_per_step": r["d2h_bytes"]},
            "gpu_launches": r["launches"],
            "roofline": {"kernel": "whole served stream", "bound": "tensor", "achieved": r["model_tflops"],
                         "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": r["model_tflops"] / pk["bf16_tflops"], "traffic": None,
                         "peak_source": pk["source"]},
            "clocks": r["clocks"], "cpu_baseline": cpu}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# CPU baselines (the oracle's C restatement on the reference's LAPACK/BLAS)
# ---------------------------------------------------------------------------

def _cpu_kind():
    from oracle import cpu_port
    return (f"C restatement on {cpu_port.BACKEND_TEXT[cpu_port.backend()]} (SciPy's bundled OpenBLAS/LAPACK, "
            "one BLAS thread per member thread); the fastest of the four LAPACK/BLAS/built-in combinations "
            "on this host and thread count")


def cpu_baseline_single(prob, u0, budget_s: float, grad_mode: str = "exact"):
    """The oracle's C restatement of the reference algorithm on all host cores
    (Hermitian generators), or the numpy oracle on a bounded sample otherwise."""
    threads = os.cpu_count() or 1
    from oracle import members as mb
    prob = mb.Problem.from_spec(prob)
    cmode = grad_mode if grad_mode in ("exact", "ref_grape", "ref_mr") else "ref_grape"
    if prob.generator == "hermitian":
        from oracle import cpu_port
        cpu_port.calibrate(prob, u0, cmode, threads)
        cp = cpu_port.CpuProblem(prob, cmode)
        cp.eval(u0, True, threads)
        n, t0 = 0, time.perf_counter()
        while True:
            cp.eval(u0, True, threads)
            n += 1
            el = time.perf_counter() - t0
            if el >= budget_s or n >= 50:
                break
        return {"value": n * prob.n_members * prob.n_t / el, "unit": UNIT, "cores": threads, "kind": "port",
                "backend": _cpu_kind(), "grad_mode": cmode,
                "sample": f"{n} full evaluations ({prob.n_members} members x {prob.n_t} slices), reference "
                          f"algorithm (eigendecomposition propagators; {cmode} gradient), OpenMP over "
                          f"members, {el:.1f} s"}
    sub = mb.Problem(drifts=prob.drifts[:1], controls=prob.controls, dt=prob.dt[:25], generator=prob.generator,
                     target=prob.target, fidelity=prob.fidelity, target_op=prob.target_op, n_members=1)
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < budget_s:
        mb.eval_problem(sub, u0[:, :25], cmode)
        n += 1
    el = time.perf_counter() - t0
    return {"value": n * 25 / el, "unit": UNIT, "cores": 1, "kind": "port", "grad_mode": cmode,
            "sample": f"{n} evaluations of 1 member x 25 slices with the numpy oracle (scipy Pade expm, "
                      f"{cmode} gradient), {el:.1f} s"}


def cpu_baseline_multi(cases, budget_s: float, grad_mode: str = "exact"):
    from oracle import cpu_port
    from oracle import members as mb
    threads = os.cpu_count() or 1
    big = max(cases, key=lambda c: c[0].n_members * c[0].n_t)
    cpu_port.calibrate(mb.Problem.from_spec(big[0]), big[1], grad_mode, threads)
    cps = [(cpu_port.CpuProblem(mb.Problem.from_spec(pr), grad_mode), u0, pr.n_members * pr.n_t)
           for pr, u0 in cases]
    units, t0 = 0, time.perf_counter()
    while True:
        for cp, u0, un in cps:
            cp.eval(u0, True, threads)
            units += un
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    return {"value": units / el, "unit": UNIT, "cores": threads, "kind": "port", "backend": _cpu_kind(),
            "grad_mode": grad_mode,
            "sample": f"{len(cps)} problems with d <= 16 evaluated repeatedly, reference algorithm, "
                      f"{grad_mode} gradient, OpenMP over members, {el:.1f} s"}


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------

def run_reference(args, rank: int):
    if rank != 0:
        return 0
    import __graft_entry__ as ge
    ge.load_package()
    from pulsar_gb300 import workloads as W
    from oracle import cpu_port
    from oracle import members as mb
    if args.workload in ("spin4", "spin4_states"):
        name, prob, u0 = single_workload(args.workload, args.slices)
        cases = [(prob, u0)]
        cfg = single_config(name, prob, args.grad_mode, args.gpus)
    elif args.workload == "uneven512":
        cases = [c for c in W.uneven_batch(512) if c[0].D <= 16][:16]
        cfg = {"workload": "uneven512 (sample: first 16 problems with d <= 16)", "grad_mode": args.grad_mode}
    else:
        print(json.dumps({"impl": "reference", "unavailable": "the oracle's C restatement covers Hermitian "
                          "generators; the Liouvillian workload has no multi-core CPU port"}), flush=True)
        return 0
    threads = os.cpu_count() or 1
    big = max(cases, key=lambda c: c[0].n_members * c[0].n_t)
    cpu_port.calibrate(mb.Problem.from_spec(big[0]), big[1], args.grad_mode, threads)
    cps = [(cpu_port.CpuProblem(mb.Problem.from_spec(pr), args.grad_mode), u0, pr.n_members * pr.n_t)
           for pr, u0 in cases]
    for _ in range(args.warmup):
        for cp, u0, _ in cps:
            cp.eval(u0, True, threads)
    units, t0 = 0, time.perf_counter()
    for _ in range(args.steps):
        for cp, u0, un in cps:
            cp.eval(u0, True, threads)
            units += un
    el = time.perf_counter() - t0
    v = units / el
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "backend": _cpu_kind(),
                             "sample": f"{args.steps} evaluations of the workload: Hermitian eigendecomposition "
                                       "propagators (Propagators.jl:659-674), chains, "
                                       f"{args.grad_mode} gradient ('exact': the spectral Frechet derivative "
                                       "in the eigenbasis; 'ref_grape': Gradients.jl:254-291), OpenMP over "
                                       "members"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.grad_mode != "ref_grape" and args.workload == "spin4":
        # the reference's own first-order gradient on the same stack, bounded sample
        fo = cpu_baseline_single(prob, u0, min(args.cpu_budget_s, 10.0), "ref_grape")
        line["first_order"] = {"value": fo["value"], "unit": UNIT, "sample": fo["sample"]}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# extras of the default line
# ---------------------------------------------------------------------------

def extra_first_order(wl, pg, ctx, torch, dev, cpu_budget_s, with_cpu: bool):
    """The reference's first-order gradient (Gradients.jl:254-291) on the GPU,
    mixed and FP64, beside the CPU port on the same gradient."""
    mx = Single(wl.name, wl.prob, wl.u0, pg, ctx, "ref_grape", "mixed", torch, dev, teams=wl.p.teams)
    v_mx = mx.timed(3, 10)
    mx.close()
    fp = Single(wl.name, wl.prob, wl.u0, pg, ctx, "ref_grape", "fp64", torch, dev)
    v_fp = fp.timed(1, 3)
    fp.close()
    out = {"grad_mode": "ref_grape", "gpu_mixed_value": v_mx, "gpu_fp64_value": v_fp, "unit": UNIT,
           "mixed_over_fp64_gpu": v_mx / v_fp}
    if with_cpu:
        cpu = cpu_baseline_single(wl.prob, wl.u0, cpu_budget_s, "ref_grape")
        out.update(cpu_value=cpu["value"], cpu_cores=cpu["cores"], gpu_mixed_over_cpu=v_mx / cpu["value"],
                   cpu_sample=cpu["sample"])
    return out


def extra_lbfgs200(wl):
    """grape_optimize_ensemble's L-BFGS (m = 10, GRAPE.jl:1012-1230) for 200
    iterations on the device, end to end through the optimiser call (host
    controls in, optimised controls out).  The controls are in rad/s and the
    gradient entries ~1e-6, so the stall and gradient-norm rules are off and
    the run takes all 200 iterations."""
    t0 = time.perf_counter()
    o = wl.p.optimize(wl.u0, "ensemble_lbfgs", max_iter=200, lbfgs_memory=10, step_size=0.01,
                      convergence_tol=1e-300, gradient_norm_tol=1e-300)
    el = time.perf_counter() - t0
    return {"wall_s": el, "iterations": o.n_iterations, "gradient_evaluations": o.n_gradient_evaluations,
            "fidelity_only_evaluations": o.n_fidelity_evaluations, "F_initial": o.fidelity_history[0],
            "F_final": o.fidelity, "stop": o.termination_reason,
            "grad_units_per_s": o.n_gradient_evaluations * wl.units_per_step / el,
            "per_iteration_ms": 1e3 * el / max(o.n_iterations, 1)}


def extra_uneven(pg, ctx):
    """One batched GRAPE iteration over the 512 uneven problems, mixed and
    plain FP64 (the same problems, the same CUDA-graph execution)."""
    from pulsar_gb300 import workloads as W
    cases = W.uneven_batch(512)
    out = {"problems": len(cases), "unit": UNIT}
    for prec, (warm, K) in (("mixed", (1, 2)), ("fp64", (0, 1))):
        u = Uneven("uneven512", cases, pg, ctx, "exact", prec)
        v, ms = u.timed(warm, K)
        out[prec] = {"value": v, "ms_per_evaluation": ms, "units_per_evaluation": u.units_per_step}
        if prec == "mixed":
            out["autotune"] = u.tune
        u.close()
    out["value"] = out["mixed"]["value"]
    out["mixed_over_fp64_gpu"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def extra_serve(pg, ctx):
    lat = serve_latency(pg, ctx, "mixed", rate=10.0, seconds=4.0, seed=5, max_slices=100, max_members=8,
                        lindblad_slices=40, lindblad_draws=2, max_iter=500, method="ensemble_lbfgs",
                        slots=128, budget_gb=80.0, step=0.01, check=8)
    lat.pop("h2d_bytes")
    lat.pop("d2h_bytes")
    cap = serve_capacity(pg, ctx)
    return {"latency_stream": lat, "capacity": cap}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="spin4",
                    choices=["spin4", "spin4_states", "uneven512", "lindblad3q", "serve"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--grad-mode", default="exact", choices=["exact", "ref_grape", "ref_mr"])
    ap.add_argument("--cpu-budget-s", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true",
                    help="skip timing the plain FP64 GPU form beside the mixed one")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the extra keys of the default line (first_order, lbfgs200, uneven512, serve)")
    ap.add_argument("--teams", type=lambda v: tuple(int(x) for x in v.split(",")), default=None,
                    help="fixed mixed-kernel team sizes EXPM,GRAD instead of autotuning (e.g. for profiling)")
    ap.add_argument("--slices", type=int, default=None,
                    help="slices per member (spin4: 1000, lindblad3q: 500 = the benchmark workloads; "
                         "smaller for profiling)")
    sv = ap.add_argument_group("serve workload (Poisson job stream through pgx_server)")
    sv.add_argument("--serve-rate", type=float, default=200.0, help="offered jobs/s")
    sv.add_argument("--serve-seconds", type=float, default=10.0, help="arrival window")
    sv.add_argument("--serve-seed", type=int, default=5)
    sv.add_argument("--serve-max-slices", type=int, default=200)
    sv.add_argument("--serve-max-members", type=int, default=16)
    sv.add_argument("--serve-lindblad-slices", type=int, default=50)
    sv.add_argument("--serve-lindblad-draws", type=int, default=4)
    sv.add_argument("--serve-max-iter", type=int, default=500, help="iteration cap of a served job")
    sv.add_argument("--serve-step", type=float, default=0.01)
    sv.add_argument("--serve-method", default="ensemble_lbfgs", choices=["ensemble_lbfgs", "grape"],
                    help="L-BFGS (history device-resident) or the GRAPE ascent")
    sv.add_argument("--serve-slots", type=int, default=128)
    sv.add_argument("--serve-budget-gb", type=float, default=80.0)
    sv.add_argument("--serve-check", type=int, default=48, help="jobs re-evaluated in FP64 for |dF|")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    import __graft_entry__ as ge
    ge._load_builder().build()
    pg = ge.load_package()
    ctx = pg.Context(local)
    dev = torch.device(f"cuda:{local}")
    if args.workload == "serve":
        rc = run_serve(args, pg, ctx, rank, world, dist, dev)
        ctx.close()
        if dist:
            dist.destroy_process_group()
        return rc
    if args.workload == "uneven512":
        from pulsar_gb300 import workloads as W
        wl = Uneven("uneven512", W.uneven_batch(512), pg, ctx, args.grad_mode, args.precision)
        cfg = wl.config(args.gpus)
    else:
        name, prob, u0 = single_workload(args.workload, args.slices)
        wl = Single(name, prob, u0, pg, ctx, args.grad_mode, args.precision, torch, dev, teams=args.teams)
        cfg = single_config(name, prob, args.grad_mode, args.gpus)
    torch.cuda.synchronize(dev)

    # ---- device-resident throughput (value) ----
    single = isinstance(wl, Single)
    if single:
        for _ in range(args.warmup):
            wl.step_device()
    else:
        wl.run_device(args.warmup)
    ctx.synchronize()
    if dist:
        dist.barrier()
    ctx.set_stage_timing(single)
    ctx.stage_times()  # clear
    l0 = ctx.launch_count()
    with ClockSampler(local) as clk:
        ctx.synchronize()
        ctx.timer_start()
        units = wl.run_device(args.steps)
        ms = ctx.timer_stop()
    launches = ctx.launch_count() - l0
    stages, n_rec = ctx.stage_times()
    ctx.set_stage_timing(False)
    ms = max_over_ranks(ms, dist, dev)
    value = job_rate(world, units, ms * 1e-3)

    # ---- end to end through the C ABI with host buffers (e2e) ----
    wl.step_e2e()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        wl.step_e2e()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, dist, dev)
    e2e_units = wl.e2e_units() if hasattr(wl, "e2e_units") else wl.units_per_step
    e2e = job_rate(world, e2e_units * args.steps, e2e_s)

    if rank == 0:
        pipe = "fp64" if args.precision == "fp64" else "fp32"
        pipe_peak = ctx.measure_peak(pipe) * 1e9
        pk = measured_peaks()
        peak = pk["bf16_tflops"] * 1e12
        if single:
            dom = max(stages, key=stages.get)
            dom_ms = stages[dom] / max(n_rec, 1)
            achieved = wl.stage_flops(dom) / (dom_ms * 1e-3)
            share = {k: round(v / max(sum(stages.values()), 1e-30), 4) for k, v in stages.items()}
            # at padded dimension 64 the mixed expm runs on the tensor cores by
            # default (team 1): the prologue plus the sliced-bf16 kernel
            tc_expm = pipe == "fp32" and dom == "expm" and wl.p.teams[0] == 1
            kname = ("k_" + dom) if pipe == "fp64" else {"expm": "k_expm_mx", "chain_fwd": "k_chain_gate_fwd_mx",
                                                         "chain_bwd": "k_chain_gate_bwd_mx",
                                                         "grad": "k_grad_gate_mx", "reduce": "k_reduce"}[dom]
            if tc_expm:
                kname = "k_expm_prep_oz64 + k_expm_oz64"
            roof = {"kernel": kname, "ms_per_launch": dom_ms, "stage_share": share,
                    "traffic": TRAFFIC.get((args.workload, args.precision, dom))}
            pr = wl.prob
            ex_unit = executed_flops_per_unit(pr.D, pr.n_c, args.grad_mode, pr.n_pairs)
            model_unit = flops_per_unit("all", pr.D, pr.n_c, args.grad_mode, pr.n_pairs)
            flops_acct = {"model_flops_per_unit": model_unit, "executed_flops_per_unit": ex_unit,
                          "model_tflops": model_unit * value / 1e12,
                          "executed_tflops": ex_unit * value / 1e12,
                          "note": "model = 8 D^3 (K_exp (1 + 2 n_c) + 3) + 8 n_c D^2 (K_exp = 8); executed "
                                  "counts the one Frechet derivative per slice the gradient runs"}
        else:
            tc_expm = False
            achieved = wl.total_flops() * (units / wl.units_per_step) / (ms * 1e-3)
            roof = {"kernel": "whole batched iteration (CUDA graph)", "ms_per_launch": ms / (args.steps + 1),
                    "traffic": None}
            flops_acct = None
        roof.update({"bound": "tensor", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak, "peak_source": pk["source"],
                     "pipe": f"{pipe.upper()} CUDA cores",
                     "fp_pipe_peak": pipe_peak / 1e12,
                     "frac_of_fp_pipe": achieved / pipe_peak if pipe_peak else None,
                     "fp_pipe_peak_source": f"measured in this run: independent-FMA loop kernel on the "
                                            f"{pipe.upper()} pipe",
                     "flop_model": "conventional per-unit W = 8 D^3 (K_exp (1 + 2 n_c) + 3) + 8 n_c D^2 "
                                   "(K_exp = 8) split by stage"})
        if single and tc_expm:
            roof.update({"pipe": "tensor cores (tcgen05, df products by exact bf16 slicing)",
                         "tensor_pipe_active_pct_ncu": TENSOR_ACTIVE_PCT.get((args.workload, args.precision, dom)),
                         "tensor_note": "each df product runs 26 bf16 slice-pair products (12 MMAs of N = 128 and "
                                        "2 of N = 64 per K step group); achieved counts model FLOPs, so frac "
                                        "is the df-product rate against the bf16 peak"})
        elif args.precision == "mixed" and single and dom in ("expm", "chain_fwd"):
            # df32 stages: each model FLOP costs DF_OPS_PER_CMAC / 8 FP32 operations
            eff = pipe_peak / (DF_OPS_PER_CMAC / 8.0)
            roof.update({"df32_effective_peak": eff / 1e12, "frac_of_df32_effective": achieved / eff,
                         "df32_note": f"df32 arithmetic: one complex MAC = {DF_OPS_PER_CMAC} FP32 operations "
                                      "vs 8 model FLOPs; frac_of_df32_effective is the model-FLOP rate over "
                                      "what a fully busy FP32 pipe reaches on df32 work"})
        extra = {}
        if args.precision == "mixed" and single and not args.no_fp64_compare:
            # the plain FP64 GPU form of the same workload, timed in the same run
            ref = Single(wl.name, wl.prob, wl.u0, pg, ctx, args.grad_mode, "fp64", torch, dev)
            v_ref = ref.timed(2, max(2, args.steps // 3))
            F64, Fmx = ref.objective(), wl.objective()
            extra = {"fp64_gpu_value": v_ref, "vs_fp64_gpu": value / v_ref, "abs_dF_vs_fp64": abs(Fmx - F64)}
            ref.close()
        if flops_acct:
            extra["flops"] = flops_acct
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            cpu = wl.cpu_sample(args.cpu_budget_s)
        if args.workload == "spin4" and args.precision == "mixed" and not args.no_extras and world == 1:
            extra["first_order"] = guarded(extra_first_order, wl, pg, ctx, torch, dev, min(args.cpu_budget_s, 10.0),
                                           not args.no_cpu_baseline)
            extra["lbfgs200"] = guarded(extra_lbfgs200, wl)
            extra["uneven512"] = guarded(extra_uneven, pg, ctx)
            extra["serve"] = guarded(extra_serve, pg, ctx)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else "f32+df32(f64 overlap)",
                "data": "synthetic (seeded)", "config": cfg, "precision": args.precision, "autotune": wl.tune,
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": wl.h2d, "d2h_bytes_per_step": wl.d2h},
                "gpu_launches": int(launches), "roofline": roof, "clocks": clk.summary(),
                "cpu_baseline": cpu}
        line.update(extra)
        print(json.dumps(line), flush=True)
    wl.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
