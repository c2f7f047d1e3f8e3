"""pulsar_gb300 -- GB300-native GRAPE fidelity-and-gradient hot path of Pulsar.jl.

The compute lives in ``libpulsar_gb300.so`` (sm_103a CUDA kernels behind the C
ABI of ``include/pgx.h``).  This package is the host-side mirror of the
reference's Julia API (``api``) plus thin handles over the C ABI (``engine``).
The directory is named ``pulsar.jl_gb300``; import it as ``pulsar_gb300``
through ``__graft_entry__.load_package()``.
"""
from . import _abi
from .engine import (Batch, Context, Problem, Server, checkpoint_create, checkpoint_parse,
                     checkpoint_set_metadata, default_context, opt_desc, plan_clear, plan_lookup,
                     problem_desc, problem_fingerprint)
from .checkpoint import (Checkpoint, auto_checkpoint_callback, checkpoint_compatible, checkpoint_summary,
                         create_checkpoint, list_checkpoints, load_checkpoint, resume_optimization,
                         save_checkpoint)
from .api import (
    ControlSequence, EnsembleObjective, GRAPEConfig, LindbladMRControl, MRControl,
    OptimizationResult, QuantumSystem, QuantumTarget, build_control_liouvillian,
    build_drift_liouvillian, build_ensemble_from_systems, compute_fidelity,
    compute_grape_gradient, compute_propagator, fidelity_forward, grape_lindblad_kernel,
    grape_optimize, grape_optimize_ensemble, grape_state_kernel, mat_rho, optimcon, propagate,
    pure_state_to_vec_rho, quantum_system, random_controls, state_target, unitary_target, vec_rho,
    CUDABackend, batch_propagators_cuda, build_ensemble_from_mrcontrol, build_total_hamiltonian,
    compute_backward_propagators, compute_forward_propagators, compute_propagators,
    compute_total_propagator, cuda_backend, ensemble_value, ensemble_value_and_grad,
    fidelity_cuda, fidelity_grad_prefactor, finite_difference_gradient, gate_fidelity, gradient_cuda,
    grape_gradient_check, lindblad_grad_prefactor, matrix_exponential_cuda, state_fidelity,
    penalty_gradient, penalty_value, penalty_value_and_gradient,
    PerturbationEnsemble, build_ensemble_from_perturbations, sample_parametric_perturbations,
    drift_ramp_schedule, sample_drift_trajectories,
    TrackingPoint, grape_phase_kernel, grape_tracking_kernel,
)

LIB_PATH = _abi.LIB_PATH
