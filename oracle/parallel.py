"""Member-parallel evaluation of the numpy oracle in spawned worker processes.

TEST INFRASTRUCTURE ONLY: lets the tests check full-size workloads (for
instance 32 Liouvillian members x 500 slices at D = 64) against the oracle in
seconds.  Members are independent (EnsembleObjective.jl:272-307 sums them), so
each worker evaluates single-member problems (members.Problem.member_problem)
and the parent sums the contributions in member order.  The pool is created
with the "spawn" start method, which is safe after the parent has used a GPU.
BLAS runs one thread per worker.
"""
from __future__ import annotations

import multiprocessing as mp
import os

import numpy as np

from . import members as mb


def _member(args):
    prob, m, u, grad_mode, want_grad = args
    sub = prob.member_problem(m)
    if grad_mode == "exact" and prob.target == "gate" and want_grad:
        return mb.eval_gate_exact_adjoint(sub, u)
    return mb.eval_problem(sub, u, grad_mode, want_grad=want_grad)


def eval_problem_parallel(prob: mb.Problem, u, grad_mode: str = "exact", want_grad: bool = True,
                          processes: int = 0):
    """(F, G) as members.eval_problem, members spread over worker processes."""
    n = processes or min(os.cpu_count() or 1, prob.n_members)
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")   # inherited by the spawned workers
    u = np.asarray(u, float)
    tasks = [(prob, m, u, grad_mode, want_grad) for m in range(prob.n_members)]
    with mp.get_context("spawn").Pool(n) as pool:
        parts = pool.map(_member, tasks, chunksize=1)
    F = 0.0
    G = np.zeros((prob.n_c, prob.n_t))
    for f, g in parts:
        F += f
        if want_grad:
            G += g
    return F, (G if want_grad else None)
