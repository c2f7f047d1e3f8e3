// Internal types shared by the kernels and the host runtime.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pgx {

constexpr int kMaxDim = 64;

// Device view of a problem.  Matrices are padded to Dp (the kernel's
// compile-time size, a power of two >= the true dimension D); padding rows
// and columns of every generator, target and state are zero, so exp() acts as
// the identity there and no padded entry reaches F or G.
struct ProbDev {
  int D;          // true dimension (normalises the gate overlap)
  int Dp;         // padded dimension
  int n_c, n_t, n_members, n_pairs;
  int gen;        // PGX_GEN_*
  int lsym;       // Liouvillian pieces preserve Hermiticity: X[a][b] = conj(X[sigma a][sigma b])
  int target;     // PGX_TARGET_*
  int fid;        // PGX_FID_*
  int grad_mode;  // PGX_GRAD_*
  const double* dt;          // [n_t]
  const double2* drifts;     // [n_drifts][Dp*Dp]
  const double2* ctrls;      // [n_c][Dp*Dp]
  const double2* offset_op;  // [Dp*Dp] (zeros when absent)
  const int* m_drift;        // [n_members]
  const double* m_scale;     // [n_members]
  const double* m_offset;    // [n_members]
  const double* m_weight;    // [n_members]
  const double2* target_op;  // gate: [Dp*Dp]
  const double2* psi_init;   // states: [n_pairs][Dp]
  const double2* psi_targ;   // states: [n_pairs][Dp]
  // per-slice drift ramp (robust drift trajectories): member m adds
  // tau[k] ramp_ops[m_ramp[m]] to its generator at slice k
  int n_ramp;                  // 0 = none
  const int* m_ramp;           // [n_members], -1 = no ramp
  const double2* ramp_ops;     // [n_ramp][Dp*Dp]
  const double* tau;           // [n_t]
  const float4* ramp_ops_df;   // mixed: df copies
  const float2* tau_df;        // mixed: [n_t] df pairs
  // trajectory tracking (states targets): checkpoints in ascending step order
  int n_ck;                  // 0 = the terminal objective
  const int* ck_step;        // [n_ck] 1..n_t: the state after that many slices
  const double* ck_weight;   // [n_ck]
  const double2* ck_target;  // [n_ck][Dp*Dp] Hermitian target density matrices
  // mixed precision only: the same constants as df pairs
  // {re.hi, im.hi, re.lo, im.lo} (the first two floats are the FP32 rounding)
  const float4* drifts_df;   // [n_drifts][Dp*Dp]
  const float4* ctrls_df;    // [n_c][Dp*Dp]
  const float4* offset_df;   // [Dp*Dp]
  const float2* dt_df;       // [n_t] df pairs {hi, lo}
  const float2* m_scale_df;  // [n_members]
  const float2* m_offset_df; // [n_members]
  // mixed precision only: the FP32 roundings (the leading halves of the df
  // copies), read by the FP32 stages
  const float2* drifts_f32;  // [n_drifts][Dp*Dp]
  const float2* ctrls_f32;   // [n_c][Dp*Dp]
  const float2* offset_f32;  // [Dp*Dp]
};

// Device work buffers of one evaluation.
struct WorkDev {
  double2* U;       // [n_members][n_t][Dp*Dp] slice propagators
  double2* P;       // gate: [n_members][n_t][Dp*Dp] forward chain, then M_k (then, for the
                    // tensor-core gradient, L(A_k, M_k))
  double2* Utot;    // [n_members][Dp*Dp]
  double2* psi;     // states: [n_members][n_t+1][n_pairs][Dp]
  double2* lam;     // states: [n_members][n_t+1][n_pairs][Dp]
  double2* z;       // [n_members][max(n_pairs,1)] overlaps
  double2* kap;     // [n_members][max(n_pairs,1)] weighted chain-rule coefficients
  double* Fm;       // [n_members] sum_s f(z_ms)
  double* Gm;       // [n_members][n_t][n_c] per-member weighted gradient
  double2* slab;    // global Taylor workspace for Dp = 64: [slab_teams][10][Dp*Dp]
  int slab_teams;
  int* expm_plan;   // mixed, Dp = 64: [n_members][n_t] degree choice of each slice's expm
  const double* u;  // [n_t][n_c]  (column-major [n_c x n_t])
  double* G;        // [n_t][n_c]
  double* F;        // [1]
  float2* u_df;     // mixed: [n_t][n_c] df pairs of u, written once per evaluation
  // mixed gate chains, parallel in time over pit_blocks blocks of pit_len slices
  int pit_blocks, pit_len;
  float4* pit_tot;  // [n_members][pit_blocks][Dp*Dp] df block products
  float2* pit_pre;  // [n_members][pit_blocks][Dp*Dp] prefix at each block start
  float2* pit_r;    // [n_members][n_t][Dp*Dp] backward: in-block suffixes U_{k1-1}...U_k
  float2* pit_lam;  // [n_members][pit_blocks][Dp*Dp] costate at each block end
};

// Tunable kernels: their team size (threads per matrix problem) is chosen per
// problem by pgx_autotune; 0 = the built-in default for the dimension.
enum { kTuneExpmMx = 0, kTuneGradMx = 1, kNumTunable = 2 };

struct LaunchInfo {
  int num_sms;
  cudaStream_t stream;
  int64_t* launches;   // counter incremented per kernel launch
  int team[kNumTunable] = {0, 0};
};

// Device state of the grape_optimize ascent (GRAPE.jl:536-610) run on the
// device by batches and the server.
struct AscentState {
  double step;     // current step size
  double F_prev;   // objective of the previous iteration
  int iter;        // steps applied
  int pad;
};

constexpr int kStepThreads = 128;  // threads of the ascent-step CTA

struct StepArgs {
  double** u;            // [n] controls
  double* const* G;      // [n] gradients
  double* const* F;      // [n] objectives (F[i][0])
  const int* len;        // [n] n_c * n_t
  AscentState* st;       // [n]
  double* trace;         // [cap][n] objective per step, or null
  double* F_all;         // [n] gathered objectives
  double* gnorm;         // [n] ||G|| of the gradient the step uses, or null
  int n, trace_cap;
  int adapt;
  double lo, hi;         // step clamp
};

// adapt_grape_step_size (GRAPE.jl:309-334) then grape_step! (:261-268) for
// the n problems of `a`, one CTA each.
cudaError_t launch_ascent_step(const StepArgs& a, cudaStream_t stream);

// Device state of one L-BFGS job run by the server: grape_optimize_ensemble
// (GRAPE.jl:1012-1230) or the MR L-BFGS of optimcon (OptControl.jl:380-482).
// dmax, gnorm, zero and gnew come first: the host reads them back as one
// 32-byte block.
constexpr int kLbMaxMemory = 64;
struct LbState {
  double dmax;    // max |d| of the last direction (before normalisation)
  double gnorm;   // ||g|| at the current controls
  double zero;    // 1.0 when dmax < 1e-14
  double gnew;    // ||gn|| at the trial point of the last F-and-G evaluation (MR)
  double a;       // current trial step
  int head;       // next history slot
  int count;      // stored pairs (<= m)
  int m, n;       // memory, control count
};
struct LbArgs {
  LbState* st;
  double* S;          // [m][n]
  double* Y;          // [m][n]
  double* rho;        // [m]
  double* u;          // current controls (accept: <- ut)
  double* g;          // gradient at u (accept: <- gn)
  double* d;          // direction
  double* ut;         // trial controls
  const double* gn;   // gradient at the accepted trial point
  double a0;          // first trial step
  double lo, hi;      // trial points are clamped to [lo, hi] when clip != 0
  int clip;
  int mr;             // MR rules: s = ut - u, no 1e-14 floors in the recursion
  int n;              // control count (n_c x n_t)
};
enum { kTrialFirst = 0, kTrialHalve = 1, kTrialZero = 2 };
cudaError_t launch_lb_direction(const LbArgs& a, cudaStream_t stream);
cudaError_t launch_lb_trial(const LbArgs& a, int mode, cudaStream_t stream);
cudaError_t launch_lb_accept(const LbArgs& a, cudaStream_t stream);
// st->gnew = ||gn|| (fixed-order reduction)
cudaError_t launch_lb_gnorm(const LbArgs& a, cudaStream_t stream);
// MR gradient ascent step (OptControl.jl:513-518): u += 0.05 (hi - lo) / max|G|
// G, clamped to [lo, hi] (no step when max|G| <= 1e-14)
cudaError_t launch_mr_step(double* u, const double* G, int n, double lo, double hi, cudaStream_t stream);
// *out = ||v|| (one CTA, fixed-order reduction)
cudaError_t launch_norm(const double* v, int n, double* out, cudaStream_t stream);

// Raises a kernel's dynamic shared-memory limit (once per kernel and device).
void set_smem_once(const void* fn, size_t bytes);

// Team sizes the mixed slice-parallel kernel `kernel` (kTune*) admits at
// padded dimension Dp (writes up to 4 values, returns the count), and the
// default choice.
// Team values of the tunable mixed kernels: candidates the autotuner times,
// values pgx_problem_set_team admits, and the default.  kTeamTensor (1)
// selects the tensor-core engine: of the D = 64 gate-target exact gradient,
// and of the D = 64 df expm.
constexpr int kTeamTensor = 1;
bool grad_tc_eligible(const ProbDev& p);
// Whether an evaluation may run tensor-core kernels (the D = 64 expm, the
// gate chains' fix-up products, the gradient).
bool tc_kernels_used(const ProbDev& p);
int mixed_variants(const ProbDev& p, int kernel, int* out);
int mixed_admitted(const ProbDev& p, int kernel, int* out);
int mixed_default_team(const ProbDev& p, int kernel);
// (member, block) prefix chains of the mixed gate chain that the GPU holds at
// once (the CUDA-core prefix kernel at its occupancy on the current device,
// times num_sms); 0 when Dp has no such kernel here (Dp > 32).
long chain_prefix_capacity(int Dp, int num_sms);
// The df expm over the items of n mixed problems of padded dimension Dp = 2
// (the only one batches share; device tables ps, ws; problem i's members x
// slices items start at first[i], a multiple of expm_small_align(Dp);
// items = first[n]): one launch for a batch's class, each unit computed as in
// the problem's solo launch (the register-resident kernel).
int expm_small_align(int Dp);
cudaError_t launch_expm_small_set(int Dp, const ProbDev* ps, const WorkDev* ws, const long* first, int n,
                                  long items, const LaunchInfo& li);
// Error bits of the tensor-core kernels since the last call (the flags are
// cleared): 1 = an MMA-completion wait gave up, 2 = a value beyond the FP16
// operand limit of the gradient; 0 = none, -1 = a flag cannot be read.
int grad_tc_check();

// Stage launchers (pgx_kernels.cu).  Each returns cudaGetLastError() after
// launching on li.stream.
cudaError_t launch_expm(const ProbDev& p, const WorkDev& w, const LaunchInfo& li);
cudaError_t launch_chain_fwd(const ProbDev& p, const WorkDev& w, const LaunchInfo& li,
                             bool store_history);
cudaError_t launch_chain_bwd(const ProbDev& p, const WorkDev& w, const LaunchInfo& li);
cudaError_t launch_grad(const ProbDev& p, const WorkDev& w, const LaunchInfo& li);
cudaError_t launch_reduce(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool want_grad);
// Largest PGX_RESID_* residual over members into *out (bits of a
// non-negative double; *out must hold 0 before the launch).  kResidPairs:
// the per-pair residuals the mixed state chain left in Utot[m np + s].
constexpr int kResidPairs = 100;
cudaError_t launch_residual(const ProbDev& p, const WorkDev& w, int kind, int N, unsigned long long* out,
                            const LaunchInfo& li);
// G[q] = sum_i coef[i] Gm[idx[i]][q] (len = n_c n_t), in the order of idx.
cudaError_t launch_select_sum(const double* Gm, const int* idx, const double* coef, int n_sel, int len, double* G,
                              const LaunchInfo& li);
// Mixed-precision stages (pgx_mixed.cu), gate targets: df expm and forward
// chain, FP32 backward chain and gradient.  U stack holds df (float4), the P
// stack float2.
cudaError_t launch_expm_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li);
cudaError_t launch_chain_fwd_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool store);
// skip_local: the in-block suffixes were already enqueued (launch_chain_bwd_local_mx,
// gate targets with pit_blocks > 1; a no-op otherwise).
cudaError_t launch_chain_bwd_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool skip_local = false);
cudaError_t launch_chain_bwd_local_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li);
cudaError_t launch_grad_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li);
// FP64 re-unitarisation of U_total after the mixed forward chain (Hermitian
// gate problems; a no-op otherwise): z, f and kappa from the refined U.
bool refine_applies(const ProbDev& p);
cudaError_t launch_refine_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li);
// u -> w.u_df (df pairs), the first stage of a mixed evaluation.
cudaError_t launch_prep_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li);
// Global slab size (in double2 elements) the Dp = 64 path needs.
size_t slab_elems(int Dp, int num_sms);
int slab_team_count(int Dp, int num_sms);
// Independent-DFMA loop used to measure the device's FP64 FMA rate; *flops
// receives the floating-point operations it performs.
cudaError_t launch_fp64_peak(double* sink, const LaunchInfo& li, double* flops);
cudaError_t launch_fp32_peak(float* sink, const LaunchInfo& li, double* flops);
// One propagator exp(c dt G) of a padded Dp x Dp generator (device buffers).
cudaError_t launch_single_expm(int Dp, int gen, const double2* G, double dt, double2* U,
                               double2* slab, const LaunchInfo& li);

}  // namespace pgx
