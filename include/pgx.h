/* pgx.h -- C ABI of libpulsar_gb300.so: the GRAPE fidelity-and-gradient hot
 * path of Pulsar.jl, GB300-native (sm_103a).
 *
 * Conventions
 *   - Every function returns an int status (PGX_OK = 0); no exception crosses
 *     the boundary.  pgx_last_error() gives the detail of the last failure on
 *     a context.
 *   - Complex matrices are column-major with interleaved (re, im) doubles:
 *     exactly the memory of a Julia Matrix{ComplexF64}.  Element (r, c) of a
 *     D x D matrix sits at doubles [2*(r + D*c)], [2*(r + D*c) + 1].
 *   - Control amplitudes u and gradients G are [n_controls x n_slices]
 *     column-major (u[j + n_controls*k]): the memory of the reference's
 *     OptimizationResult.controls / ControlSequence.controls.
 *   - A context is externally synchronised: calls on one context (and on the
 *     problems it owns) must not overlap.  Distinct contexts are independent.
 *
 * Replaced reference interfaces (paths inside the Pulsar.jl project) are cited
 * beside each entry point.  The reference has no FFI of its own; its plugin
 * points are Julia dispatch hooks (GRAPEConfig.backend, the physics-hook
 * grape_optimize overload, EnsembleObjective.batched_eval, MRControl.backend).
 */
#ifndef PGX_H
#define PGX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGX_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
  PGX_OK = 0,
  PGX_ERR_INVALID = 1,     /* bad argument / descriptor (reference: ArgumentError) */
  PGX_ERR_DIMS = 2,        /* inconsistent sizes (reference: DimensionMismatch)    */
  PGX_ERR_NOMEM = 3,       /* device allocation failed                              */
  PGX_ERR_BUDGET = 4,      /* admission refused: HBM budget of the context exceeded */
  PGX_ERR_CUDA = 5,        /* CUDA runtime error                                    */
  PGX_ERR_UNSUPPORTED = 6, /* valid request this build does not implement           */
  PGX_ERR_TIMEOUT = 7,     /* a bounded device wait gave up                         */
  PGX_ERR_CANCELLED = 8,   /* job cancelled                                          */
  PGX_ERR_STATE = 9,       /* call not valid in the object's current state          */
  PGX_ERR_NONFINITE = 10   /* non-finite input or result                            */
};

/* ---- problem description ----------------------------------------------- */
enum { PGX_GEN_HERMITIAN = 0,   /* U_k = exp(-i H_k dt_k)   (Propagators.jl:659-674)   */
       PGX_GEN_LIOUVILLIAN = 1  /* U_k = exp(L_k dt_k)      (GRAPELindblad.jl:146-153) */ };
enum { PGX_TARGET_GATE = 0,     /* z = Tr(T' U_total)/D    (Objectives.jl:239-246)    */
       PGX_TARGET_STATES = 1    /* z_s = <t_s|U_total i_s>  (Objectives.jl:221)        */ };
enum { PGX_FID_SQUARE = 0,      /* f = |z|^2 (gate: the :normalized fidelity)          */
       PGX_FID_REAL = 1,        /* f = Re z                                            */
       PGX_FID_MODULUS = 2      /* f = |z|                                             */ };
enum { PGX_GRAD_REF_GRAPE = 0,  /* first-order formula of Gradients.jl:254-291,357-399 */
       PGX_GRAD_REF_MR = 1,     /* first-order formula of GRAPEState.jl:220-230 /
                                   GRAPELindblad.jl:183-195                            */
       PGX_GRAD_EXACT = 2       /* exact Frechet-derivative gradient                    */ };
enum { PGX_PREC_FP64 = 0,       /* plain FP64 everywhere                                */
       PGX_PREC_MIXED = 1       /* df32 propagators and forward chain, FP64 overlap and
                                   objective, FP32 backward chain and gradient         */ };

/* A problem is an ensemble of members.  Member m evolves under
 *   G_m(u_k) = drifts[member_drift[m]] + member_offset[m] * offset_op
 *              + member_scale[m] * sum_j u[j,k] controls[j]
 * and F = sum_m member_weight[m] * sum_s f(z_ms).  One member with scale 1 is
 * a reference QuantumSystem; members = drifts x pwr_levels is an MRControl
 * ensemble (GRAPEState.jl:145-146); offsets x B1 scales is a broadband
 * ensemble without replicating the drift (SystemBuilder.jl:49-87).        */
typedef struct pgx_problem_desc {
  uint32_t struct_size;        /* sizeof(pgx_problem_desc)                       */
  int32_t dim;                 /* D <= 64 (Hilbert d, or N*N for Liouvillians)    */
  int32_t n_controls;          /* >= 1                                            */
  int32_t n_slices;            /* >= 1                                            */
  int32_t generator;           /* PGX_GEN_*                                       */
  int32_t target;              /* PGX_TARGET_*                                    */
  int32_t fidelity;            /* PGX_FID_*                                       */
  int32_t grad_mode;           /* PGX_GRAD_*                                      */
  int32_t precision;           /* PGX_PREC_*                                      */
  int32_t n_drifts;            /* >= 1                                            */
  int32_t n_members;           /* >= 1                                            */
  int32_t n_pairs;             /* state pairs (PGX_TARGET_STATES), else 0         */
  const double* dt;            /* [n_slices] slice durations                      */
  const double* drifts;        /* [n_drifts][D*D] complex                         */
  const double* controls;      /* [n_controls][D*D] complex                       */
  const double* offset_op;     /* [D*D] complex, or NULL                          */
  const int32_t* member_drift; /* [n_members] or NULL (all 0)                     */
  const double* member_scale;  /* [n_members] or NULL (all 1)                     */
  const double* member_offset; /* [n_members] or NULL (all 0)                     */
  const double* member_weight; /* [n_members] or NULL (1/(n_members*max(n_pairs,1))) */
  const double* target_op;     /* gate: [D*D] complex                             */
  const double* states_init;   /* states: [n_pairs][D] complex (used for F)       */
  const double* states_target; /* states: [n_pairs][D] complex                    */
  const double* grad_states_init; /* states: initial states for the gradient, or
                                     NULL (= states_init).  grape_optimize passes
                                     the target here (Gradients.jl:153-157).      */
} pgx_problem_desc;

/* Oracle-free error estimate of an evaluation, the largest over members:
 *   UNITARITY  gate, Hermitian:      max_ij |(U'U - I)_ij| of U_total
 *   TRACE      gate, Liouvillian:    max_c |sum_i Phi[i + N i, c] - [c = j + N j]|,
 *              the trace-preservation defect of Phi = U_total
 *   NORM       states, Hermitian:    max_s | ||psi_s(T)||^2 - ||psi_s(0)||^2 |
 *   STATE_TRACE states, Liouvillian: max_s |Tr rho_s(T) - Tr rho_s(0)|
 * (state targets: evaluations that compute G; NONE otherwise).  For mixed
 * Hermitian gate problems it is measured before the FP64 Newton-Schulz
 * refinement of U_total, so it reports the defect the refinement removed. */
enum { PGX_RESID_NONE = 0, PGX_RESID_UNITARITY = 1, PGX_RESID_TRACE = 2, PGX_RESID_NORM = 3,
       PGX_RESID_STATE_TRACE = 4 };

typedef struct pgx_eval_stats {
  double ms_device;            /* device time of the call (CUDA events)           */
  double ms_host;              /* wall time of the call                           */
  int64_t units;               /* member-slice units processed                    */
  int32_t n_launches;          /* kernels launched by the call (residual excluded) */
  int32_t max_taylor_degree;   /* largest degree chosen (0 = not recorded)        */
  double residual;             /* PGX_RESID_* estimate (after the timed region)   */
  int32_t residual_kind;       /* PGX_RESID_*                                      */
  int32_t reserved;
} pgx_eval_stats;

typedef struct pgx_ctx pgx_ctx;
typedef struct pgx_problem pgx_problem;

/* ---- library / context ------------------------------------------------- */
int pgx_abi_version(void);
const char* pgx_status_string(int status);

/* Context on one device with an HBM budget (0 = no limit).  Owns one stream.
 * pgx_ctx_destroy on a context that still has live problems only marks it
 * closing: the last pgx_problem_destroy releases it (no problem outlives the
 * context it points to).  Destroying a closing context again is
 * PGX_ERR_INVALID. */
int pgx_ctx_create(int device, uint64_t hbm_budget_bytes, pgx_ctx** out);
int pgx_ctx_destroy(pgx_ctx* ctx);
int pgx_last_error(const pgx_ctx* ctx, char* buf, size_t len);
int pgx_ctx_hbm_used(const pgx_ctx* ctx, uint64_t* bytes);
/* The context's cudaStream_t (as void*), for callers that order their own work. */
int pgx_ctx_stream(pgx_ctx* ctx, void** stream);
/* Device-time stopwatch on the context stream (CUDA events). */
int pgx_ctx_timer_start(pgx_ctx* ctx);
int pgx_ctx_timer_stop(pgx_ctx* ctx, double* ms);
int pgx_ctx_synchronize(pgx_ctx* ctx);
/* Kernels launched on this context since creation (monotone counter). */
int pgx_ctx_launch_count(const pgx_ctx* ctx, int64_t* count);
/* Per-stage device timing.  While enabled, every evaluation records CUDA
 * events around its stages (PGX_STAGE_*).  pgx_ctx_stage_times waits for the
 * recorded work, writes the summed milliseconds of each stage into
 * ms[PGX_N_STAGES], the number of recorded evaluations into *count, and
 * clears the record.                                                        */
enum { PGX_STAGE_EXPM = 0, PGX_STAGE_CHAIN_FWD = 1, PGX_STAGE_CHAIN_BWD = 2, PGX_STAGE_GRAD = 3,
       PGX_STAGE_REDUCE = 4, PGX_N_STAGES = 5 };
int pgx_ctx_set_stage_timing(pgx_ctx* ctx, int enabled);
int pgx_ctx_stage_times(pgx_ctx* ctx, double* ms, int32_t* count);
/* Measured FMA peak (GFLOP/s) of one pipe of this device, from a timed loop
 * of independent FMAs: PGX_PIPE_FP64 (the FP64 path's roofline denominator)
 * or PGX_PIPE_FP32 (the mixed path's).                                      */
enum { PGX_PIPE_FP64 = 0, PGX_PIPE_FP32 = 1 };
int pgx_ctx_measure_peak(pgx_ctx* ctx, int32_t pipe, double* gflops);

/* ---- problems ---------------------------------------------------------- */
/* HBM bytes pgx_problem_create would hold for desc (admission control).    */
int pgx_problem_footprint(const pgx_problem_desc* desc, uint64_t* bytes);
/* Validates desc (Hermiticity of H for PGX_GEN_HERMITIAN, 1e-10 as
 * QuantumSystem.jl:318-341; unitarity of a gate target, 1e-8 as
 * Targets.jl:131-144), copies every input to device memory and owns it.    */
int pgx_problem_create(pgx_ctx* ctx, const pgx_problem_desc* desc, pgx_problem** out);
int pgx_problem_destroy(pgx_problem* prob);

/* ---- evaluation -------------------------------------------------------- */
/* (F, G) at controls u, host buffers, synchronous.  G may be NULL (forward
 * only, the line-search evaluation).  Replaces, per member and averaged:
 *   compute_fidelity + compute_grape_gradient   (Objectives.jl:632-639,
 *       Gradients.jl:80-163), ensemble_value_and_grad (EnsembleObjective.jl:
 *       272-307), grape_state_kernel (GRAPEState.jl:73-250),
 *       grape_lindblad_kernel (GRAPELindblad.jl:83-215), gradient_cuda /
 *       batch_propagators_cuda / fidelity_cuda (CUDABackend.jl:126-373).  */
int pgx_eval(pgx_problem* prob, const double* u, double* F, double* G, pgx_eval_stats* stats);
/* Same on device buffers, asynchronous on the context stream.  d_G may be
 * NULL.  d_F receives one double.                                           */
int pgx_eval_device(pgx_problem* prob, const double* d_u, double* d_F, double* d_G);
/* Per-member objective sum_s f(z_ms) of the last evaluation ([n_members]). */
int pgx_member_fidelities(pgx_problem* prob, double* F_members);
/* Total propagator U_total of one member at controls u ([D*D] complex):
 * compute_total_propagator(compute_propagators(...)) (Propagators.jl:212-238). */
int pgx_total_propagator(pgx_problem* prob, const double* u, int32_t member, double* U_total);
/* Single-slice propagator exp(c dt G) of a D x D generator G ([D*D] complex in
 * and out); the compute_propagator / _expm_neg_i hook (Propagators.jl:64-90,
 * PropagatorRegistry.jl:138-191).                                           */
int pgx_propagator(pgx_ctx* ctx, int32_t dim, int32_t generator, const double* gen, double dt,
                   double* U);

/* ---- propagator stacks and chains (standalone building blocks) ---------- */
/* The pieces of Propagators.jl / Objectives.jl the evaluation fuses, as
 * device calls on host buffers (all FP64, column-major complex):
 *   H[k] = H_drift + sum_j u[j + n_controls k] H_controls[j]
 *        (build_total_hamiltonian, Propagators.jl:485-544; H [n][dim^2]) */
int pgx_total_hamiltonian(pgx_ctx* ctx, int32_t dim, int32_t n_controls, int32_t n, const double* H_drift,
                          const double* H_controls, const double* u, double* H);
/*   U[k] = exp(c dt_k H[k]), c = -i (Hermitian) or 1 (Liouvillian), dt_count
 *   = 1 (uniform) or n (compute_propagators, Propagators.jl:127-184). */
int pgx_propagator_stack(pgx_ctx* ctx, int32_t dim, int32_t generator, int32_t n, const double* H,
                         const double* dt, int32_t dt_count, double* U);
/*   P[0] = I, P[k+1] = U[k] P[k]          (compute_forward_propagators, :291-325)
 *   Q[n] = seed (NULL: I), Q[k] = U[k]' Q[k+1]
 *                                         (compute_backward_propagators(!), :390-440)
 *   U_total = U[n-1] ... U[0]             (compute_total_propagator, :212-238)
 * P and Q hold n + 1 matrices; any of P, Q, U_total may be NULL. */
int pgx_propagator_chains(pgx_ctx* ctx, int32_t dim, int32_t n, const double* U, const double* seed, double* P,
                          double* Q, double* U_total);
/*   z = sum_i conj(A_i) B_i over n complex entries: Tr(A'B) for matrices,
 *   <a|b> for vectors (the overlaps of Objectives.jl:221,239-246). */
int pgx_overlap(pgx_ctx* ctx, int64_t n, const double* A, const double* B, double* z);
/*   out[j + m k] = Tr(X[k] E[j] Y[k]) for k < n, j < m (complex): the per-slice
 *   traces of a first-order GRAPE gradient (CUDABackend.jl:352-356). */
int pgx_trace_products(pgx_ctx* ctx, int32_t dim, int32_t n, int32_t m, const double* X, const double* E,
                       const double* Y, double* out);

/* Replaces the drift matrices ([n_drifts][dim^2], same count and checks as at
 * creation), e.g. the redrawn perturbations of a resampling robust ensemble
 * (PerturbationBuilder.jl:52-133). */
int pgx_problem_set_drifts(pgx_problem* prob, const double* drifts);

/* ---- ensemble aggregators ---------------------------------------------- */
/* The aggregated objective of EnsembleObjective.jl:169-217 with each member a
 * sample: F_m = mean over the member's state pairs of f(z) (gates: f(z)),
 * dF_m/du its gradient.  MEAN averages the members, WORST_CASE takes the first
 * member of least F_m (argmin), CVAR the mean over the max(1, round(alpha n))
 * members of least F_m (stable order, round half to even).  G (nullable)
 * receives the aggregated gradient [n_c x n_t].  Member weights must be
 * positive (the per-member gradient is recovered from the weighted one). */
enum { PGX_AGG_MEAN = 0, PGX_AGG_WORST_CASE = 1, PGX_AGG_CVAR = 2 };
int pgx_eval_aggregate(pgx_problem* prob, const double* u, int32_t aggregator, double alpha, double* F, double* G);

/* ---- penalties ---------------------------------------------------------- */
/* Waveform penalties of Penalties.jl:197-330 (the PENALTY_TYPES of :205):
 *   NS     sum w^2                       SNS   sum max(0, w-u_b)^2 + max(0, l_b-w)^2
 *   SNSA   sum_k max(0, ||w[:,k]|| - u_b)^2                 DNS   sum (w[:,k+1] - w[:,k])^2
 *   ENERGY sum w^2 dt_k                                     (w = the control amplitudes u). */
enum { PGX_PEN_NS = 0, PGX_PEN_SNS = 1, PGX_PEN_SNSA = 2, PGX_PEN_DNS = 3, PGX_PEN_ENERGY = 4 };
#define PGX_MAX_PENALTIES 8
typedef struct pgx_penalty {
  int32_t type;                /* PGX_PEN_*                                        */
  int32_t reserved;
  double weight;
  double l_bound, u_bound;     /* SNS / SNSA bounds (reference defaults -1, 1)     */
} pgx_penalty;
/* Every later evaluation of the problem returns F - sum weight P and
 * G - sum weight dP/du, as _apply_penalties! (GRAPEState.jl:571-584); n = 0
 * removes them.  n <= PGX_MAX_PENALTIES. */
int pgx_problem_set_penalties(pgx_problem* prob, int32_t n, const pgx_penalty* penalties);
/* Standalone penalty_value_and_gradient (Penalties.jl:260-271): P = weight
 * P(u), G = weight dP/du ([n_c x n_t], nullable); dt nullable (uniform 1). */
int pgx_penalty_eval(pgx_ctx* ctx, int32_t n_controls, int32_t n_slices, const double* u, const double* dt,
                     const pgx_penalty* penalty, double* P, double* G);

/* ---- autotuning --------------------------------------------------------- */
/* Times every team-size variant (threads per matrix problem, with the
 * matching register blocking) of the problem's slice-parallel mixed-precision
 * kernels at controls u, `reps` launches each, keeps the fastest for this
 * problem and writes a one-line report (nullable).  Variants only re-map work
 * to threads; every dot product is summed in the same order, so results are
 * bit-identical whatever is chosen.  The FP64 path has no variants.  At
 * padded dimension 64 the expm, and the gradient of gate targets with the
 * exact gradient, have one candidate each: the tensor-core engine
 * (PGX_TEAM_TENSOR).                                                        */
int pgx_autotune(pgx_problem* prob, const double* u, int32_t reps, char* report, size_t report_len);
/* Sets the team sizes directly (a plan kept from an earlier pgx_autotune);
 * 0 = the built-in default.  Values the dimension does not admit are refused
 * with PGX_ERR_INVALID.  Kernel indices: 0 = mixed expm, 1 = mixed gradient.
 * Admitted by padded dimension: 32 (<= 8); 32, 64, 128, 256 (16); 128, 256
 * (32); 256 (64), plus 512 for the gradient at 64.  PGX_TEAM_TENSOR (1)
 * selects a tensor-core engine, the default where it exists:
 *   - the expm at 64 (every generator and target): df products by exact bf16
 *     slicing (six 8-bit slices per operand, levels 0..6 accumulated exactly
 *     in FP32), df-class like the CUDA-core team 256 but not bit-identical;
 *   - the gradient at 64 of gate targets with the exact gradient: 3xFP16
 *     tcgen05 products, FP32-class like the CUDA-core teams but not
 *     bit-identical to them.
 * The CUDA-core teams stay admitted there for comparisons.                   */
#define PGX_TUNE_EXPM 0
#define PGX_TUNE_GRAD 1
#define PGX_TEAM_TENSOR 1
int pgx_problem_set_team(pgx_problem* prob, int32_t kernel, int32_t team);
int pgx_problem_get_team(const pgx_problem* prob, int32_t kernel, int32_t* team);
/* Plans: pgx_autotune records its choice process-wide under (device, padded
 * dimension, n_controls, generator, target, precision, grad_mode), and
 * problems created later with the same key -- on any context, a server's
 * private one included -- start from it.  pgx_plan_lookup reports the plan
 * for a descriptor (PGX_ERR_STATE and zeros when none); pgx_plan_clear
 * forgets every plan.  Plans never change results, only time.              */
int pgx_plan_lookup(int device, const pgx_problem_desc* desc, int32_t* team_expm, int32_t* team_grad);
int pgx_plan_clear(void);

/* ---- allocation-free total propagator ----------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need a propagator (real-time loops that forbid allocation
 * once started, or hosts whose device memory all comes from their own pool
 * allocator): computes
 *   U_total = exp(c dt_{n-1} G_{n-1}) ... exp(c dt_0 G_0),
 * c = -i (PGX_GEN_HERMITIAN) or 1 (PGX_GEN_LIOUVILLIAN), with every piece of
 * working memory in one static device array of PGX_NOALLOC_SCRATCH_BYTES that
 * each GPU loading the library holds until the process exits.  It calls no
 * cudaMalloc/cudaFree.  d_gens ([n_slices][dim*dim] complex), d_dt
 * ([n_slices]) and d_U_total ([dim*dim] complex) are device pointers the
 * caller owns; the work is enqueued on `stream` (cudaStream_t, NULL = legacy
 * default stream) and is asynchronous.  Sizes whose propagator stack
 * (n_slices * Dp^2 * 16 bytes, Dp = next power of two >= dim, plus 5 MiB of
 * Taylor workspace when Dp = 64) exceeds the array are rejected with
 * PGX_ERR_BUDGET and a message in err (err may be NULL).  The first call on a
 * device sets that device up (resolves the array's address and loads every
 * kernel the entry point uses); make it before any stream capture.  All calls share the array: calls whose GPU work
 * overlaps race and must be serialised by the caller.  Input contents are not
 * validated (Hermiticity, finiteness are the caller's responsibility).     */
#define PGX_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)
int pgx_total_propagator_noalloc(int32_t dim, int32_t generator, int32_t n_slices,
                                 const double* d_gens, const double* d_dt, double* d_U_total,
                                 void* stream, char* err, size_t err_len);

/* ---- diagnostics ------------------------------------------------------------ */
/* No counterpart in the reference.  Batched complex 64 x 64 products
 * C_i = P_i Q_i (i < n; each matrix column-major interleaved re/im, FP64 on the
 * host, rounded to FP32) through the tensor-core (tcgen05) product engine that
 * the D = 64 mixed gradient uses: 3xTF32 with FP32 accumulation (passes = 3)
 * or plain TF32 (passes = 1), the left factor as an expanded operand in
 * shared memory (mode 0) or in tensor memory (mode 1); or 3xFP16 with the
 * left factor in tensor memory (mode 2, passes = 3: the gradient's path).
 * Synchronous, on the current device; allocates its own device buffers.
 * PGX_ERR_TIMEOUT when an MMA-completion wait gave up.  For tests and
 * profiling of the engine alone.                                             */
int pgx_diag_tc_cmatmul64(const double* P, const double* Q, double* C, int32_t n, int32_t passes,
                          int32_t mode);
/* The same batched products in df (double-float, ~48-bit) arithmetic, the
 * precision of the mixed expm: engine 0 = the CUDA-core df product of the
 * D = 64 expm (FP32 pipe); engine 1 = the tensor-core form, each operand cut
 * into six exact 8-bit bf16 slices whose 21 slice pairs of levels 0..5 are
 * accumulated exactly in FP32 TMEM and summed in df; engine 2 = the same
 * with level 6 (26 pairs).  Inputs are rounded to df from FP64.  The kernel
 * runs reps times after one warm-up launch; *ms (may be NULL) receives the
 * mean time per launch.  PGX_ERR_TIMEOUT when an MMA-completion wait gave
 * up.                                                                          */
int pgx_diag_dfcmatmul64(const double* P, const double* Q, double* C, int32_t n, int32_t engine, int32_t reps,
                         float* ms);

/* ---- drift ramps ----------------------------------------------------------- */
/* Robust drift trajectories (sample_drift_trajectories, RobustOpt.jl:168-182;
 * build_ensemble_from_perturbations(:drift), PerturbationBuilder.jl:52-133):
 * member m adds tau[k] ops[member_op[m]] to its generator at slice k (ops
 * [n_ops][D*D] complex, Hermitian for Hermitian problems; member_op
 * [n_members] in -1..n_ops-1, -1 = none; tau [n_slices]).  The reference's
 * linear ramp is tau[k] = k / max(1, n_slices - 1).  n_ops = 0 removes the
 * ramp.  Calling it again redraws the ensemble in place.                    */
int pgx_problem_set_drift_ramp(pgx_problem* prob, int32_t n_ops, const double* ops, const int32_t* member_op,
                               const double* tau);

/* ---- trajectory tracking and phase-only controls ------------------------ */
/* Tracking (MR/GRAPETracking.jl:166-277): on a Hermitian state-target
 * problem, n > 0 checkpoints replace the terminal objective by
 *   F = sum_m w_m sum_s sum_c weights[c] Re Tr(rho_c rho_ms(steps[c])),
 * rho(k) the state after k slices from rho(0) = psi_s psi_s' (states_init;
 * states_target and the fidelity metric are not used).  steps are 1..n_slices
 * (PGX_ERR_INVALID outside, GRAPETracking.jl:190-191), targets [n][D*D]
 * complex Hermitian density matrices.  PGX_GRAD_REF_MR gives the reference's
 * co-state formula (twice the first-order derivative: its co-state carries
 * 2 w_c), PGX_GRAD_EXACT the exact gradient.  n = 0 restores the terminal
 * objective.  pgx_optimize's MR methods on a tracking problem are
 * _optimcon_lbfgs_tracking / _optimcon_grape_tracking (OptControl.jl:1040-1236). */
int pgx_problem_set_tracking(pgx_problem* prob, int32_t n, const int32_t* steps, const double* weights,
                             const double* targets);
/* Phase-only evaluation (grape_phase_kernel, MR/GRAPEPhase.jl:52-93): the
 * n_controls / 2 channels of phases phi [n_ch x n_t] (column-major) and
 * amplitudes (same shape, >= 0, NULL = 1) become w[2ch] = a cos(phi),
 * w[2ch+1] = a sin(phi); F as pgx_eval, G_phase = -G_x sin(phi) + G_y cos(phi)
 * (nullable).                                                               */
int pgx_eval_phase(pgx_problem* prob, const double* phi, const double* amplitudes, double* F, double* G_phase);

/* ---- optimisation ------------------------------------------------------ */
enum { PGX_OPT_GRAPE = 0,          /* grape_optimize ascent loop (GRAPE.jl:469-643)       */
       PGX_OPT_ENSEMBLE_LBFGS = 1, /* grape_optimize_ensemble (GRAPE.jl:1012-1230)        */
       PGX_OPT_MR_LBFGS = 2,       /* optimcon :lbfgs (OptControl.jl:380-482,565-611)     */
       PGX_OPT_MR_GRAPE = 3        /* optimcon :grape (OptControl.jl:486-561)             */ };

typedef struct pgx_opt_desc {
  uint32_t struct_size;
  int32_t method;              /* PGX_OPT_*                                        */
  int32_t max_iter;
  int32_t adapt_step_size;     /* GRAPE only                                       */
  int32_t lbfgs_memory;
  int32_t reserved;
  double convergence_tol;      /* GRAPEConfig defaults: 1e-8                       */
  double step_size;            /* 0.01                                             */
  double min_step_size;        /* 1e-10                                            */
  double max_step_size;        /* 10.0                                             */
  double gradient_norm_tol;    /* 1e-6 (MR: grad_tol 1e-7)                         */
  double amplitude_limit;      /* ensemble L-BFGS clip, +inf = none                */
  double l_bound, u_bound;     /* MR bounds (-1, 1)                                */
} pgx_opt_desc;

typedef struct pgx_opt_result {
  double fidelity;             /* best fidelity (GRAPE: re-evaluated at the best controls) */
  double total_time_s;
  double step_size_final;
  int32_t n_iterations;
  int32_t converged;
  int32_t n_fidelity_evals;
  int32_t n_gradient_evals;
  int32_t history_len;         /* fidelity-history entries (<= history_cap written) */
  int32_t gnorm_history_len;   /* gradient-norm-history entries                    */
  char reason[100];
} pgx_opt_result;

/* Runs the optimiser on the device-resident problem.  u_inout holds the
 * initial controls and receives the best controls.  Histories (nullable,
 * capacity history_cap) receive fidelity / gradient-norm traces as the
 * reference's OptimizationResult does (GRAPE.jl:158-170).                   */
int pgx_optimize(pgx_problem* prob, const pgx_opt_desc* opt, double* u_inout,
                 double* fidelity_history, double* gnorm_history, int32_t history_cap,
                 pgx_opt_result* result);

/* ---- batches of uneven problems ----------------------------------------- */
/* A batch groups problems of any dimensions, slice counts and ensemble sizes
 * on one context.  pgx_batch_eval / pgx_batch_iterate enqueue every problem's
 * pipeline -- fanned out over n_streams streams, largest problems first --
 * as ONE CUDA graph per call / per iteration, captured on first use.  Each
 * problem runs the kernels of its solo evaluation, so batched results are
 * bit-identical to solo results.  No reference counterpart: Pulsar.jl runs
 * problems one after another (grape_multistart, GRAPE.jl:745-768).          */
typedef struct pgx_batch pgx_batch;
int pgx_batch_create(pgx_ctx* ctx, int32_t n, pgx_problem* const* problems, int32_t n_streams,
                     pgx_batch** out);
int pgx_batch_destroy(pgx_batch* batch);
/* Controls of problem i (host buffer, [n_c x n_t]); they stay on the device. */
int pgx_batch_set_controls(pgx_batch* batch, int32_t i, const double* u);
/* Device-resident controls and last gradient of problem i (either nullable). */
int pgx_batch_get_controls(pgx_batch* batch, int32_t i, double* u, double* G);
/* Member-slice units one evaluation of the whole batch processes. */
int pgx_batch_units(const pgx_batch* batch, int64_t* units);
/* (F, G) of every problem at its device-resident controls; F[n] (nullable)
 * receives the objectives, gradients stay on the device.                    */
int pgx_batch_eval(pgx_batch* batch, double* F);
/* n_iter iterations of the grape_optimize ascent (GRAPE.jl:536-610: evaluate,
 * adapt_grape_step_size, u += step G) for every problem, one graph launch per
 * iteration, controls / gradients / step state device-resident.  Uses
 * step_size, adapt_step_size, min_step_size and max_step_size of opt.
 * F_trace ([n_iter][n], nullable) receives the objective of every iteration. */
int pgx_batch_iterate(pgx_batch* batch, int32_t n_iter, const pgx_opt_desc* opt, double* F_trace);

/* ---- serving -------------------------------------------------------------
 * A continuous-batching optimisation server.  Jobs (a problem descriptor,
 * grape_optimize settings and initial controls) are queued by pgx_submit and
 * admitted, oldest first, while their HBM footprint fits the server budget
 * and a slot is free.  Every admitted job runs the grape_optimize ascent
 * (GRAPE.jl:536-610) with controls, gradient, step state and best controls
 * device-resident; each job advances one iteration (one CUDA graph: ascent
 * step, evaluation, 24-byte read-back) as soon as its previous one finished,
 * so jobs of different sizes overlap on the device and a job that arrives
 * while others run starts as soon as memory and a slot free up.  A job stops
 * under check_grape_convergence (GRAPE.jl:371-402), at max_iter, or once its
 * fidelity reaches the server's target_fidelity; its result is the best
 * controls seen, as grape_optimize returns them.  A job runs the kernels of a
 * solo run, so its result is bit-identical alone and in any mix.
 * PGX_OPT_ENSEMBLE_LBFGS jobs run grape_optimize_ensemble's L-BFGS
 * (GRAPE.jl:1012-1230) with the direction, line-search trial points and the
 * (s, y) history in HBM, one evaluation per step; PGX_OPT_MR_LBFGS and
 * PGX_OPT_MR_GRAPE jobs run optimcon's MR loops (OptControl.jl:380-561,
 * 594-611: bounds, Armijo-like line search with its fall-back, max|G|-scaled
 * ascent) the same way.  The server uses a private context on the
 * device of ctx; errors of pgx_submit are recorded on ctx.  No reference
 * counterpart: Pulsar.jl optimises one problem per call.                   */
enum { PGX_JOB_QUEUED = 0, PGX_JOB_RUNNING = 1, PGX_JOB_DONE = 2, PGX_JOB_FAILED = 3,
       PGX_JOB_CANCELLED = 4 };

typedef struct pgx_server_desc {
  uint32_t struct_size;
  int32_t max_inflight;        /* slots: jobs on the device at once (one stream each)  */
  uint64_t hbm_budget_bytes;   /* admission budget over the jobs' footprints, 0 = none */
  double target_fidelity;      /* serving stop rule F >= target; > 1 disables it       */
} pgx_server_desc;

typedef struct pgx_job_status {
  int32_t state;               /* PGX_JOB_*                                             */
  int32_t status;              /* PGX_OK or the error that failed the job               */
  int32_t iterations;          /* ascent steps applied                                  */
  int32_t reserved;
  double fidelity;             /* objective at the current controls                     */
  double best_fidelity;
  double queue_s;              /* submit -> admission (so far, while queued)            */
  double latency_s;            /* submit -> finish (so far, while unfinished)           */
  char reason[96];
} pgx_job_status;

typedef struct pgx_serve_stats {
  int64_t submitted, completed, failed, cancelled, running, queued;
  int64_t kernel_launches;     /* kernels the server launched (graph nodes counted)     */
  int64_t units;               /* member-slice gradient units evaluated                 */
  uint64_t hbm_in_use, hbm_peak;
  double elapsed_s;            /* since pgx_server_create                               */
  double jobs_per_s;           /* completed / elapsed                                   */
  double p50_latency_s, p99_latency_s;  /* submit -> converged pulse, completed jobs    */
  double mean_iterations;
} pgx_serve_stats;

typedef struct pgx_server pgx_server;
int pgx_server_create(pgx_ctx* ctx, const pgx_server_desc* desc, pgx_server** out);
/* Cancels queued and running jobs, then frees the server. */
int pgx_server_destroy(pgx_server* server);
/* Deep-copies desc, opt and u0 ([n_c x n_t]); PGX_ERR_BUDGET when the job's
 * footprint alone exceeds the server budget.                                */
int pgx_submit(pgx_server* server, const pgx_problem_desc* desc, const pgx_opt_desc* opt,
               const double* u0, uint64_t* job_id);
/* What a job's problem carries beyond its descriptor, applied at admission
 * with pgx_problem_set_penalties / _set_tracking / _set_drift_ramp (each
 * part unused when its count is 0; arrays as those calls take them).  A
 * part the problem refuses fails the job at admission with the reason.     */
typedef struct pgx_job_extras {
  uint32_t struct_size;
  int32_t n_penalties;
  const pgx_penalty* penalties;
  int32_t n_tracking;
  int32_t n_ramp_ops;
  const int32_t* tracking_steps;
  const double* tracking_weights;
  const double* tracking_targets;  /* [n_tracking][D*D] complex                    */
  const double* ramp_ops;          /* [n_ramp_ops][D*D] complex                    */
  const int32_t* ramp_member_op;   /* [n_members]                                  */
  const double* ramp_tau;          /* [n_slices]                                   */
} pgx_job_extras;
/* pgx_submit with extras (nullable).                                        */
int pgx_submit_ex(pgx_server* server, const pgx_problem_desc* desc, const pgx_opt_desc* opt, const double* u0,
                  const pgx_job_extras* extras, uint64_t* job_id);
int pgx_poll(pgx_server* server, uint64_t job_id, pgx_job_status* status);
/* Result of a finished job: best controls u ([n_c x n_t], nullable) and the
 * grape_optimize summary (nullable; history lengths filled, the traces come
 * from pgx_job_history).  Returns PGX_ERR_STATE while the job is queued or
 * running, the job's error when it failed, PGX_ERR_CANCELLED when cancelled.
 * A fetched job is forgotten.                                               */
int pgx_fetch(pgx_server* server, uint64_t job_id, double* u, pgx_opt_result* result);
/* Fidelity and gradient-norm traces of a job so far, with the conventions of
 * OptimizationResult (GRAPE.jl:158-170): grape_optimize's F(u0), then F at
 * each iteration's controls (+ the post-step F of a converged run);
 * ||G|| per iteration.  A resumed job's traces start with its checkpoint's
 * (Checkpoint.jl:279-280).  Either buffer nullable; *n_fidelity / *n_gnorm
 * receive the full lengths, at most cap entries are written.               */
int pgx_job_history(pgx_server* server, uint64_t job_id, double* fidelity_history, double* gnorm_history,
                    int32_t cap, int32_t* n_fidelity, int32_t* n_gnorm);
/* Queued jobs are dropped at once; running ones stop after their current
 * iteration (an L-BFGS job finishes its line search and history update), so
 * a cancelled job's checkpoint can continue exactly.                        */
int pgx_cancel(pgx_server* server, uint64_t job_id);
/* Waits until no job is queued or running; timeout_s <= 0 waits forever.   */
int pgx_server_drain(pgx_server* server, double timeout_s);
int pgx_server_stats(pgx_server* server, pgx_serve_stats* stats);

/* ---- checkpoints of served jobs ----------------------------------------- */
/* A checkpoint is a self-contained byte blob replacing the Julia
 * Serialization of Checkpoint (IO/Checkpoint.jl:64-131,166-208): the fields
 * of Checkpoint that describe an optimisation (w_opt, F_opt, n_controls,
 * n_timesteps, iteration, both histories, system_dim, a timestamp) plus, for
 * an exact snapshot, the job's device state: its current controls, gradient
 * and objective, the GRAPE step-size state or the L-BFGS (s, y) history.
 * Layout: little-endian, a fixed 208-byte header (magic "PGXCKPT\0",
 * version 1), f64 payload arrays, a metadata section (opaque UTF-8 text,
 * JSON by convention: the reference's domain tags and metadata dict, e.g.
 * "dt"), and an FNV-1a-64 checksum of everything before it as the last 8
 * bytes; identical on every host.                                          */
#define PGX_CHECKPOINT_VERSION 1
#define PGX_CHECKPOINT_HEADER_BYTES 208
enum { PGX_CKPT_EXACT = 1,       /* carries the device state (PGX_RESUME_CONTINUE) */
       PGX_CKPT_CONVERGED = 2 };
enum { PGX_RESUME_RESTART = 0,   /* resume_optimization (Checkpoint.jl:220-298): a fresh
                                    run from w_opt; histories and iteration counts add up */
       PGX_RESUME_CONTINUE = 1   /* the interrupted trajectory itself: the resumed job's
                                    iterates, histories and result are bit-identical to a
                                    run that was never interrupted                       */ };

typedef struct pgx_checkpoint_info {
  uint32_t struct_size;
  int32_t version;
  int32_t flags;               /* PGX_CKPT_*                                              */
  int32_t system_dim;          /* 0 = unknown (resume then skips the dim check)           */
  int32_t n_controls;
  int32_t n_timesteps;
  int32_t n_members;
  int32_t iteration;           /* iterations done (the n_iterations pgx_fetch reports)    */
  int32_t history_len;
  int32_t gnorm_history_len;
  int32_t lbfgs_pairs;         /* stored (s, y) pairs of an exact L-BFGS snapshot         */
  int32_t metadata_len;        /* bytes of the metadata section                           */
  double F_opt;                /* best fidelity                                           */
  double F;                    /* objective at the current controls (exact snapshots)     */
  double timestamp;            /* seconds since the Unix epoch when written               */
  uint64_t fingerprint;        /* FNV-1a-64 of the problem (0 = none)                     */
  pgx_opt_desc opt;            /* settings of the job that was snapshotted                */
} pgx_checkpoint_info;

/* Takes a checkpoint of a job: a running job is snapshotted (exactly) at its
 * next iteration boundary -- the call waits up to timeout_s (<= 0: forever;
 * PGX_ERR_TIMEOUT) -- while a finished or cancelled job gives its final
 * state (exact for cancelled jobs).  The blob stays with the job; *blob_len
 * receives its size, pgx_job_checkpoint_read copies it out.  PGX_ERR_STATE
 * for a job that never started.                                            */
int pgx_job_checkpoint(pgx_server* server, uint64_t job_id, double timeout_s, uint64_t* blob_len);
int pgx_job_checkpoint_read(pgx_server* server, uint64_t job_id, void* blob, uint64_t cap);
/* Queues a job that resumes from a checkpoint.  Validation as
 * resume_optimization (Checkpoint.jl:236-247): system_dim (when > 0) and
 * n_controls must match desc, and n_timesteps its n_slices.  opt (nullable:
 * the checkpoint's own settings) gives the new run's settings; under
 * RESTART its max_iter is the number of additional iterations.  CONTINUE
 * also requires an exact checkpoint of the same problem (fingerprint of the
 * descriptor and the extras), the same method and, for L-BFGS,
 * lbfgs_memory >= the stored pairs.                                         */
int pgx_submit_resume(pgx_server* server, const pgx_problem_desc* desc, const pgx_opt_desc* opt,
                      const pgx_job_extras* extras, const void* blob, uint64_t blob_len, int32_t mode,
                      uint64_t* job_id);
/* Host-only (no device work): parses and verifies a blob (magic, version,
 * sizes, checksum; PGX_ERR_INVALID otherwise) into info and, when non-null,
 * w_opt ([n_c x n_t]) and the histories (history_len / gnorm_history_len
 * entries).                                                                */
int pgx_checkpoint_parse(const void* blob, uint64_t blob_len, pgx_checkpoint_info* info, double* w_opt,
                         double* fidelity_history, double* gnorm_history);
/* Host-only: the metadata bytes (info.metadata_len of them; PGX_ERR_DIMS
 * when cap is smaller).                                                    */
int pgx_checkpoint_metadata(const void* blob, uint64_t blob_len, char* metadata, uint64_t cap);
/* Host-only: create_checkpoint (Checkpoint.jl:143-164) from host arrays, a
 * warm-start (non-exact) blob.  info supplies dims, iteration, F_opt,
 * history lengths, the timestamp (0 = now), fingerprint, settings and
 * metadata_len bytes of metadata; blob NULL (or cap too small:
 * PGX_ERR_DIMS) reports the size in *blob_len.                             */
int pgx_checkpoint_create(const pgx_checkpoint_info* info, const double* w_opt, const double* fidelity_history,
                          const double* gnorm_history, const char* metadata, void* blob, uint64_t cap,
                          uint64_t* blob_len);
/* Host-only: the same checkpoint with its metadata replaced (an exact
 * snapshot stays exact); out NULL reports the size in *out_len.             */
int pgx_checkpoint_set_metadata(const void* blob, uint64_t blob_len, const char* metadata, uint64_t metadata_len,
                                void* out, uint64_t cap, uint64_t* out_len);
/* FNV-1a-64 of a problem descriptor: sizes, kinds and every array's bits. */
int pgx_problem_fingerprint(const pgx_problem_desc* desc, uint64_t* fingerprint);

#ifdef __cplusplus
}
#endif
#endif /* PGX_H */
