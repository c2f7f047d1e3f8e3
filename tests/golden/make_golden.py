"""Writes the golden fixtures of tests/golden/*.npz from the FP64 oracle.

    python tests/golden/make_golden.py

Each fixture holds one problem in the pgx_problem_desc member model (complex
matrices indexed [row, col]), the controls u[n_c, n_t], and the oracle's
(F, G) for every gradient mode listed in `modes`.  The oracle restates the
reference functions (oracle/ref_semantics.py cites them by file:line); the
reference itself (Julia) cannot run here.  Its test-suite holds no numeric
vectors, only invariants and thresholds, which tests/test_oracle_kats.py pins.
These fixtures freeze the oracle's outputs on small seeded cases:
- tests/test_golden_cpu.py re-derives them with the oracle;
- tests/test_golden_gpu.py checks the CUDA path against them.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import fx  # noqa: E402
from oracle import members as mb  # noqa: E402

FIELDS = ("drifts", "controls", "dt", "offset_op", "member_drift", "member_scale", "member_offset",
          "member_weight", "target_op", "states_init", "states_target")


def _herm(rng, d, s=1.0):
    A = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    return s * (A + A.conj().T) / 2


def cases():
    rng = np.random.default_rng(2024)
    out = {}
    p, u = fx.single_qubit_transfer(explicit_init=True)
    out["quickstart_transfer"] = (p, u, ("ref_grape", "ref_mr", "exact"))
    p, u = fx.spin4_ensemble(n_t=8, n_off=2, n_b1=2)
    out["spin4_8slices_4members"] = (p, u, ("exact", "ref_grape", "ref_mr"))
    # odd dimension (padded to 4), modulus and real metrics, gate target
    for fid in ("modulus", "real"):
        d, n_t, n_c, nm = 3, 7, 2, 3
        p = mb.Problem(drifts=np.stack([_herm(rng, d) for _ in range(2)]),
                       controls=np.stack([_herm(rng, d) for _ in range(n_c)]),
                       dt=rng.uniform(0.02, 0.08, n_t), member_drift=np.array([0, 1, 1]),
                       member_scale=rng.uniform(0.9, 1.1, nm), member_weight=rng.uniform(0.2, 0.5, nm),
                       target="gate", fidelity=fid, target_op=fx.haar_unitary(rng, d), n_members=nm)
        out[f"gate_d3_{fid}"] = (p, rng.uniform(-1, 1, (n_c, n_t)), ("exact", "ref_grape", "ref_mr"))
    # several state pairs, d = 5 (padded to 8), real metric, offset operator
    d, n_t, n_c, nm = 5, 9, 3, 2
    psi_i = rng.standard_normal((2, d)) + 1j * rng.standard_normal((2, d))
    psi_t = rng.standard_normal((2, d)) + 1j * rng.standard_normal((2, d))
    psi_i /= np.linalg.norm(psi_i, axis=1, keepdims=True)
    psi_t /= np.linalg.norm(psi_t, axis=1, keepdims=True)
    p = mb.Problem(drifts=_herm(rng, d)[None], controls=np.stack([_herm(rng, d) for _ in range(n_c)]),
                   dt=np.full(n_t, 0.05), offset_op=np.diag(rng.uniform(-1, 1, d)).astype(complex),
                   member_offset=np.array([-0.3, 0.4]), member_scale=np.array([1.0, 0.95]),
                   target="states", fidelity="real", states_init=psi_i, states_target=psi_t, n_members=nm)
    out["states_d5_2pairs_real"] = (p, rng.uniform(-1, 1, (n_c, n_t)), ("exact", "ref_grape", "ref_mr"))
    # uneven-distribution problem at d = 32
    p, u = fx.uneven_problem(rng, d=32, n_t=4, n_members=2)
    out["uneven_d32_4slices"] = (p, u, ("exact",))
    # Lindblad gate superoperators: 2 qubits (D = 16) and 3 qubits (D = 64)
    p, u = fx.lindblad_gate(seed=7, n_qubits=2, n_t=6, n_draws=2)
    out["lindblad2q_D16"] = (p, u, ("exact", "ref_mr"))
    p, u = fx.lindblad_gate(seed=8, n_qubits=3, n_t=3, n_draws=1)
    out["lindblad3q_D64"] = (p, u, ("exact",))
    return out


def save(name, prob, u, modes):
    arrs = {"u": np.asarray(u, float), "modes": np.array(modes), "generator": np.array(prob.generator),
            "target": np.array(prob.target), "fidelity": np.array(prob.fidelity),
            "n_members": np.array(prob.n_members)}
    for f in FIELDS:
        v = getattr(prob, f)
        if v is not None:
            arrs[f] = np.asarray(v)
    for mode in modes:
        F, G = mb.eval_problem(prob, u, mode)
        arrs[f"F_{mode}"] = np.array(F)
        arrs[f"G_{mode}"] = G
    np.savez_compressed(HERE / f"{name}.npz", **arrs)


def load(path) -> tuple:
    """(oracle Problem, u, modes, {mode: (F, G)}) of a fixture."""
    z = np.load(path)
    kw = {f: z[f] for f in FIELDS if f in z.files}
    prob = mb.Problem(generator=str(z["generator"]), target=str(z["target"]), fidelity=str(z["fidelity"]),
                      n_members=int(z["n_members"]), **kw)
    modes = [str(m) for m in z["modes"]]
    return prob, z["u"], modes, {m: (float(z[f"F_{m}"]), z[f"G_{m}"]) for m in modes}


if __name__ == "__main__":
    for name, (prob, u, modes) in cases().items():
        save(name, prob, u, modes)
        print(name, prob.D, prob.n_members, prob.n_t, modes)
