"""The package's seeded workloads as oracle problems (test inputs).

The generators live in ``pulsar_gb300.workloads`` (the benchmark uses them);
tests hand the same arrays to the oracle through ``members.Problem.from_spec``.
"""
import __graft_entry__ as ge

from oracle import members as mb

ge.load_package()
from pulsar_gb300 import workloads as W  # noqa: E402

SX, SY, SZ, I2 = W.SX, W.SY, W.SZ, W.I2
embed = W.embed
haar_unitary = W.haar_unitary


def _as_oracle(pair):
    spec, u0 = pair
    return mb.Problem.from_spec(spec), u0


def single_qubit_transfer(*a, **k):
    return _as_oracle(W.single_qubit_transfer(*a, **k))


def spin4_ensemble(*a, **k):
    return _as_oracle(W.spin4_ensemble(*a, **k))


def uneven_problem(*a, **k):
    return _as_oracle(W.uneven_problem(*a, **k))


def uneven_batch(*a, **k):
    return [_as_oracle(p) for p in W.uneven_batch(*a, **k)]


def lindblad_3q(*a, **k):
    return _as_oracle(W.lindblad_3q(*a, **k))


def lindblad_gate(*a, **k):
    return _as_oracle(W.lindblad_gate(*a, **k))
