"""Checkpoint and resume (IO/Checkpoint.jl) over portable checkpoint blobs.

The reference stores its ``Checkpoint`` struct (Checkpoint.jl:64-131) with
Julia ``Serialization``; here a checkpoint file is the byte blob of
include/pgx.h (little-endian header, f64 arrays, a JSON metadata section and
a checksum), written atomically as temp file + rename like save_checkpoint
(:166-177).  Blobs taken from a served job (``Server.checkpoint``) also carry
its device state, so ``Server.submit_resume(..., mode="continue")`` resumes it
bit-identically; ``resume_optimization`` keeps the reference's semantics (a
fresh run from ``w_opt`` with concatenated histories, :220-298).
"""
from __future__ import annotations

import json
import os
import warnings
from dataclasses import dataclass, field
from datetime import datetime
from typing import Optional

import numpy as np

from . import engine as E

# File names list_checkpoints picks up: this library's, and the reference's
# own (:347-351), so existing naming keeps working.
CHECKPOINT_EXTS = (".ckpt", ".jls")

_TAGS = ("domain", "drive_max_hz", "T_pulse", "system_kind")


def _jsonable(x):
    if isinstance(x, dict):
        return {str(k): _jsonable(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_jsonable(v) for v in x]
    if isinstance(x, np.ndarray):
        return _jsonable(x.tolist())
    if isinstance(x, np.generic):
        return x.item()
    if isinstance(x, complex):
        return [x.real, x.imag]
    return x


@dataclass
class Checkpoint:
    """Checkpoint.jl:64-80.  ``blob`` is the encoded form a served job gave
    (it keeps the job's device state); it is re-used by ``to_bytes`` as long
    as the decoded fields still match it."""
    w_opt: np.ndarray
    F_opt: float
    n_controls: int
    n_timesteps: int
    iteration: int = 0
    fidelity_history: list = field(default_factory=list)
    gradient_norm_history: list = field(default_factory=list)
    optimizer_state: dict = field(default_factory=dict)
    system_dim: int = 0
    domain: str = "generic"
    drive_max_hz: float = 0.0
    T_pulse: float = 0.0
    system_kind: str = "generic"
    timestamp: str = field(default_factory=lambda: datetime.now().isoformat())
    metadata: dict = field(default_factory=dict)
    blob: Optional[bytes] = field(default=None, repr=False)

    def __post_init__(self):
        self.w_opt = np.array(self.w_opt, np.float64)
        if self.w_opt.shape != (int(self.n_controls), int(self.n_timesteps)):
            raise ValueError(f"w_opt has shape {self.w_opt.shape}, expected "
                             f"{(int(self.n_controls), int(self.n_timesteps))}")
        self.F_opt, self.n_controls, self.n_timesteps = float(self.F_opt), int(self.n_controls), int(self.n_timesteps)
        self.iteration, self.system_dim = int(self.iteration), int(self.system_dim)
        self.fidelity_history = [float(v) for v in self.fidelity_history]
        self.gradient_norm_history = [float(v) for v in self.gradient_norm_history]
        self.optimizer_state = {str(k): v for k, v in dict(self.optimizer_state).items()}
        self.metadata = {str(k): v for k, v in dict(self.metadata).items()}

    @property
    def exact(self) -> bool:
        """True when the blob holds a served job's device state."""
        return self.blob is not None and self._decoded()["exact"]

    def _decoded(self) -> dict:
        return E.checkpoint_parse(self.blob)

    def _meta_bytes(self) -> bytes:
        doc = {k: getattr(self, k) for k in _TAGS}
        doc.update(timestamp=self.timestamp, optimizer_state=_jsonable(self.optimizer_state),
                   metadata=_jsonable(self.metadata))
        return json.dumps(doc, sort_keys=True).encode()

    def _matches_blob(self) -> bool:
        d = self._decoded()
        return (np.array_equal(d["w_opt"], self.w_opt) and d["F_opt"] == self.F_opt
                and d["iteration"] == self.iteration and d["system_dim"] == self.system_dim
                and d["fidelity_history"] == self.fidelity_history
                and d["gradient_norm_history"] == self.gradient_norm_history)

    def to_bytes(self) -> bytes:
        meta = self._meta_bytes()
        if self.blob is not None and self._matches_blob():
            return E.checkpoint_set_metadata(self.blob, meta)
        return E.checkpoint_create(self.w_opt, self.F_opt, iteration=self.iteration,
                                   fidelity_history=self.fidelity_history,
                                   gradient_norm_history=self.gradient_norm_history,
                                   system_dim=self.system_dim, metadata=meta)

    @classmethod
    def from_bytes(cls, blob: bytes) -> "Checkpoint":
        d = E.checkpoint_parse(blob)
        try:
            doc = json.loads(d["metadata"].decode()) if d["metadata"] else {}
        except (UnicodeDecodeError, json.JSONDecodeError):
            doc = {}
        ts = doc.get("timestamp") or datetime.fromtimestamp(d["timestamp"]).isoformat()
        return cls(d["w_opt"], d["F_opt"], d["n_controls"], d["n_timesteps"], iteration=d["iteration"],
                   fidelity_history=d["fidelity_history"], gradient_norm_history=d["gradient_norm_history"],
                   optimizer_state=doc.get("optimizer_state", {}), system_dim=d["system_dim"],
                   domain=doc.get("domain", "generic"), drive_max_hz=doc.get("drive_max_hz", 0.0),
                   T_pulse=doc.get("T_pulse", 0.0), system_kind=doc.get("system_kind", "generic"),
                   timestamp=ts, metadata=doc.get("metadata", {}), blob=bytes(blob))


def create_checkpoint(iter: int, controls, fidelity: float, fidelity_history, gradient_norms,
                      optimizer_state: dict, system, metadata: Optional[dict] = None) -> Checkpoint:
    """Checkpoint.jl:143-164."""
    c = np.asarray(controls, np.float64)
    return Checkpoint(c.copy(), fidelity, system.n_controls, c.shape[1], iteration=iter,
                      fidelity_history=list(fidelity_history), gradient_norm_history=list(gradient_norms),
                      optimizer_state=optimizer_state, system_dim=system.dim, metadata=metadata or {})


def save_checkpoint(filepath: str, ckpt) -> None:
    """Atomic write (temp file + rename, Checkpoint.jl:166-177) of a
    Checkpoint or a raw blob."""
    data = ckpt.to_bytes() if isinstance(ckpt, Checkpoint) else bytes(ckpt)
    E.checkpoint_parse(data)  # never write an invalid blob
    tmp = str(filepath) + ".tmp"
    with open(tmp, "wb") as f:
        f.write(data)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, filepath)


def load_checkpoint(filepath: str) -> Checkpoint:
    """Checkpoint.jl:186-208 (ValueError where the reference throws ArgumentError)."""
    if not os.path.isfile(filepath):
        raise ValueError(f"Checkpoint file not found: {filepath}")
    with open(filepath, "rb") as f:
        data = f.read()
    try:
        return Checkpoint.from_bytes(data)
    except E.A.PgxError as e:
        raise ValueError(f"File {filepath} does not contain a checkpoint ({e})") from None


def checkpoint_compatible(ckpt: Checkpoint, n_controls: int, n_timesteps: int) -> bool:
    """Checkpoint.jl:320-336."""
    ok = ckpt.n_controls == n_controls and ckpt.n_timesteps == n_timesteps
    if not ok:
        print(f"  [checkpoint] Dimension mismatch: checkpoint [{ckpt.n_controls} x {ckpt.n_timesteps}] "
              f"!= current [{n_controls} x {n_timesteps}].")
        print("               Falling back to default warm start.")
    return ok


def list_checkpoints(directory: str) -> list:
    """Checkpoint files in a directory, sorted by name (Checkpoint.jl:347-351)."""
    if not os.path.isdir(directory):
        return []
    return sorted(os.path.join(directory, f) for f in os.listdir(directory) if f.endswith(CHECKPOINT_EXTS))


def checkpoint_summary(filepath: str) -> str:
    """One line per file (Checkpoint.jl:358-369)."""
    if not os.path.isfile(filepath):
        return f"File not found: {filepath}"
    try:
        c = load_checkpoint(filepath)
        return f"{os.path.basename(filepath)} | iter={c.iteration} | F={c.F_opt:.6f} | saved {c.timestamp}"
    except Exception as e:  # the reference reports any failure as text
        return f"Could not read checkpoint: {e}"


def auto_checkpoint_callback(filepath: str, interval: int):
    """Checkpoint.jl:306-318: a callback (iter, controls, fidelity, grad_norm,
    system) that saves every ``interval`` iterations."""
    def callback(iter: int, controls, fidelity: float, grad_norm: float, system):
        if iter % interval == 0:
            chk = create_checkpoint(iter, controls, fidelity, [fidelity], [grad_norm], {}, system,
                                    {"callback_interval": interval})
            save_checkpoint(filepath, chk)
    return callback


def resume_optimization(checkpoint: Checkpoint, system, target, *, additional_iterations: int = 500,
                        optimizer: str = "grape", verbose: bool = True):
    """Checkpoint.jl:220-298: validates dim / n_controls, runs a fresh
    optimisation from w_opt for additional_iterations and returns a result
    whose histories and iteration count follow the checkpoint's.
    optimizer "lbfgs" runs the ensemble L-BFGS of grape_optimize_ensemble on
    the one system (the generic lbfgs_optimize of QuasiNewton.jl is not on
    this path)."""
    from .api import (ControlSequence, GRAPEConfig, OptimizationResult, grape_optimize,
                      grape_optimize_ensemble)
    if checkpoint.system_dim > 0 and system.dim != checkpoint.system_dim:
        raise ValueError(f"System dimension mismatch: checkpoint has dim={checkpoint.system_dim}, "
                         f"provided system has dim={system.dim}")
    if system.n_controls != checkpoint.n_controls:
        raise ValueError(f"n_controls mismatch: checkpoint={checkpoint.n_controls}, system={system.n_controls}")
    if verbose:
        print(f"Resuming from checkpoint (iter={checkpoint.iteration}, F={checkpoint.F_opt:.6f}, "
              f"saved {checkpoint.timestamp})")
    dt = checkpoint.metadata.get("dt")
    if dt is None:
        dt = 10e-9
        if verbose:
            warnings.warn("dt not stored in checkpoint; assuming dt=10 ns")
    cs = ControlSequence.from_controls(checkpoint.w_opt.copy(), float(dt), float(dt) * checkpoint.n_timesteps,
                                       checkpoint.n_timesteps)
    cfg = GRAPEConfig(max_iter=additional_iterations, verbose=verbose)
    r = (grape_optimize_ensemble([system], target, cs, cfg) if optimizer == "lbfgs"
         else grape_optimize(system, target, cs, cfg))
    md = dict(r.metadata)
    md["resumed_from_iter"] = checkpoint.iteration
    return OptimizationResult(r.controls, r.fidelity, checkpoint.fidelity_history + list(r.fidelity_history),
                              checkpoint.gradient_norm_history + list(r.gradient_norm_history),
                              checkpoint.iteration + r.n_iterations, r.converged, r.termination_reason,
                              r.total_time, r.n_fidelity_evaluations, r.n_gradient_evaluations, md)
