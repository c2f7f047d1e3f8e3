// Host-side object layouts behind the opaque handles of pgx.h.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pgx.h"
#include "pgx_internal.h"

struct pgx_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;    // per-evaluation timing
  cudaEvent_t tev0 = nullptr, tev1 = nullptr;  // caller stopwatch
  uint64_t budget = 0;                         // bytes, 0 = unlimited
  uint64_t used = 0;                           // bytes held by live problems
  int64_t launches = 0;
  std::string err;
  // Stream-ordered allocation: when set, problem buffers come from this pool
  // on `stream` and are released with cudaFreeAsync (no device-wide sync).
  cudaMemPool_t pool = nullptr;
  // per-stage timing (pgx_ctx_set_stage_timing)
  bool stage_timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::vector<cudaEvent_t>> stage_marks;  // one vector of 6 events per evaluation
  // Problems alive on this context; pgx_ctx_destroy with live problems only
  // marks it closing, and the last pgx_problem_destroy releases it.
  int live = 0;
  bool closing = false;
};

struct pgx_problem {
  static constexpr int kMaxPairs = 8;
  pgx_ctx* ctx = nullptr;
  pgx_problem_desc desc{};
  int Dp = 0;
  pgx::ProbDev pd{};       // F pass (states_init)
  pgx::ProbDev pd_grad{};  // gradient pass (grad_states_init)
  bool split_grad_states = false;
  pgx::WorkDev w{};
  double* d_u = nullptr;
  double* d_G = nullptr;
  double* d_F = nullptr;   // [2]: objective, scratch
  double* h_stage = nullptr;  // pinned: u | G | F (allocated on first host evaluation)
  std::vector<double> h_weight;
  std::vector<void*> owned;
  uint64_t bytes = 0;
  int team[pgx::kNumTunable] = {0, 0};  // tuned team sizes (0 = default)
  pgx_penalty* d_pen = nullptr;         // [PGX_MAX_PENALTIES] on the device
  int n_pen = 0;
  void* d_track = nullptr;              // tracking checkpoints (steps | weights | targets)
  uint64_t track_bytes = 0;
  void* d_ramp = nullptr;               // drift ramp (member index | tau | operators | df copies)
  uint64_t ramp_bytes = 0;
  // mixed gate problems in parallel in time: stream and fork/join events of
  // the backward chain's in-block suffixes
  cudaStream_t side = nullptr;
  // ProbDev::lsym = lsym_fixed && lsym_drift && lsym_ramp: the controls and
  // offset (and dimension) at creation, the current drifts, the current ramp
  // operators each preserve Hermiticity
  bool lsym_fixed = false, lsym_drift = false, lsym_ramp = true;
  // bumped by every setter that changes what run_pipeline enqueues (kernel
  // parameters, team sizes): graphs captured earlier (batches) are stale
  uint64_t generation = 0;
  void refresh_lsym() {
    pd.lsym = pd_grad.lsym = (lsym_fixed && lsym_drift && lsym_ramp) ? 1 : 0;
  }
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  pgx::LaunchInfo launch_info() const {
    pgx::LaunchInfo li{ctx->num_sms, ctx->stream, &ctx->launches};
    for (int i = 0; i < pgx::kNumTunable; ++i) li.team[i] = team[i];
    return li;
  }
};

int ctx_fail(pgx_ctx* c, int status, const std::string& msg);
// Host helpers: padded size (power of two >= max(d, 2)), finiteness, the
// Hermiticity defect max |A - A'|, and n column-major D x D complex matrices
// copied into zero-padded Dp x Dp ones.
int pad_dim(int d);
bool finite_all(const double* x, size_t n);
double herm_dev(const double* m, int D);
std::vector<double> pad_mats(const double* src, int n, int D, int Dp);
// Descriptor validation (errors recorded on c) and device footprint in bytes.
int validate_desc(pgx_ctx* c, const pgx_problem_desc* d);
uint64_t problem_footprint(const pgx_problem_desc* d, int num_sms);
int ctx_cuda(pgx_ctx* c, cudaError_t e, const char* where);
namespace pgx {
// Subtracts the problem's penalties from F and G (G nullable) on li.stream.
cudaError_t launch_penalties(const pgx_penalty* d_pens, int n_pen, const double* u, const double* dt, int n_c,
                             int n_t, double* F, double* G, const LaunchInfo& li);
}  // namespace pgx
// Enqueues one evaluation; stream = nullptr means the context stream.
// skip_expm: the slice propagators of d_u are already in p->w.U (a batch's
// shared launch wrote them).
int run_pipeline(pgx_problem* p, const double* d_u, double* d_F, double* d_G, cudaStream_t stream = nullptr,
                 bool skip_expm = false);
int eval_host(pgx_problem* p, const double* u, double* F, double* G, pgx_eval_stats* stats);
