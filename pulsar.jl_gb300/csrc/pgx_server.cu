// Continuous-batching optimisation server.
//
// A worker thread owns the GPU side and a private context.  Its loop:
//   1. admission: queued jobs, oldest first, take a free slot (stream, event,
//      pinned read-back block) while their HBM footprint fits the budget; the
//      problem is created, the controls uploaded and the first evaluation
//      enqueued -- everything stays device-resident from here on;
//   2. progress: every job whose in-flight iteration has finished (its slot
//      event) is checked against the stop rules of grape_optimize and either
//      retired (best controls copied out, HBM and slot freed) or given its
//      next iteration -- one CUDA graph: the ascent step, the evaluation at the
//      new controls and a 24-byte read-back of (F, ||G||, step).
// Jobs never wait for each other: a small job iterates at its own pace while a
// large one runs, and a job that arrives while others are on the device is
// admitted as soon as memory and a slot free up.  Each job runs exactly the
// kernels of a solo run on its own stream, so its trajectory is bit-identical
// alone and in any mix.
// L-BFGS jobs (grape_optimize_ensemble, GRAPE.jl:1012-1230) advance one
// evaluation at a time instead: the direction, the trial points of the
// backtracking line search and the history update are device kernels on the
// job's stream (pgx_lbfgs.cu); each step reads back (F, max|d|, ||g||).
// Checkpoints: at an iteration boundary (nothing of the job in flight) the
// worker can copy a job's device state out -- on request, or when the job is
// cancelled -- and a job submitted with that snapshot uploads it back and
// continues with the iteration that would have come next (pgx_ckpt.h holds
// the state, pgx_checkpoint.cpp its byte encoding).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pgx.h"
#include "pgx_ckpt.h"
#include "pgx_runtime.h"

namespace {

using clk = std::chrono::steady_clock;

double secs(clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); }

// Device block of one job: the one-problem tables of its StepArgs.
struct JobDev {
  double* u;
  double* G;
  double* F;
  int len;
  int pad;
  double gnorm;              // ||G|| the last step used
  pgx::AscentState st;       // st.step follows gnorm: both read back together
  double F_out;
};

// Host read-back block of a slot (pinned): F at the new controls, ||G|| and
// step of the step that produced them.
struct Readback {
  double F;
  double gnorm;
  double step;
  double lb[4];  // L-BFGS jobs: dmax, gnorm, zero of the last direction, ||gn|| (MR)
};

// Phases of an L-BFGS job: the evaluation in flight is F and G at the initial
// controls, F at a trial point, F at the MR line search's last fall-back
// point, or F and G at the accepted point.
enum { LB_INIT = 0, LB_TRIAL = 1, LB_ACCEPT = 2, LB_FALLBACK = 3 };
enum { G_START = 0, G_HALVE = 1, G_FG = 2, G_HALVE_FG = 3, G_ACC_START = 4, G_ZERO_FG = 5, G_COUNT = 6 };

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  Readback* hb = nullptr;
};

struct Job {
  uint64_t id = 0;
  int state = PGX_JOB_QUEUED;   // guarded by the server mutex
  int status = PGX_OK;
  std::string reason;
  std::atomic<bool> cancel{false};
  // owned copies of the descriptor's arrays
  std::vector<double> dt, drifts, controls, offset, mscale, moffset, mweight, target, sinit, starg, sgrad;
  std::vector<int32_t> mdrift;
  pgx_problem_desc desc{};
  pgx_opt_desc opt{};
  std::vector<double> u;        // initial controls, then the result
  // owned copies of the job extras (penalties, tracking, drift ramp)
  std::vector<pgx_penalty> pens;
  std::vector<int32_t> tr_steps, ramp_mo;
  std::vector<double> tr_w, tr_t, ramp_ops, ramp_tau;
  uint64_t footprint = 0;
  int64_t units = 0;            // member-slice units per evaluation
  // device side (worker thread only)
  int slot = -1;
  pgx_problem* prob = nullptr;
  JobDev* dev = nullptr;
  double* d_best = nullptr;
  cudaGraphExec_t iter_exec = nullptr;
  int64_t iter_kernels = 0;
  bool inflight = false;
  // ascent bookkeeping (written by the worker under the server mutex)
  int round = -1;               // completed evaluations - 1 = steps applied
  std::vector<double> fh;       // grape_optimize fidelity history
  double F = 0.0, bestF = -INFINITY, step = 0.0;
  bool converged = false;
  clk::time_point t_submit, t_start, t_end;
  // L-BFGS jobs (PGX_OPT_ENSEMBLE_LBFGS, PGX_OPT_MR_LBFGS); MR rules (MR_LBFGS, MR_GRAPE)
  bool lbfgs = false, mr = false, mrgrape = false;
  int lb_phase = LB_INIT, lb_bt = 0, lb_it = 0;
  bool lb_grad_eval = true;      // the evaluation in flight computes G
  double lb_gnorm = 0.0;         // ||g|| at the start of the current iteration
  pgx::LbState* lb = nullptr;
  double *S = nullptr, *Yh = nullptr, *rho = nullptr, *own_u = nullptr, *own_g = nullptr, *dvec = nullptr;
  double *ucur = nullptr, *utry = nullptr, *gcur = nullptr, *gtry = nullptr;
  cudaGraphExec_t lb_exec[G_COUNT] = {};
  int64_t lb_kernels[G_COUNT] = {};
  bool lb_boundary = false;      // an iteration ended and its successor is not enqueued yet
  // histories and resumption
  std::vector<double> gh;        // gradient-norm history
  uint64_t fingerprint = 0;      // of the problem descriptor
  int prior_iter = 0;            // a resumed job: iterations and history entries of the
  std::vector<double> prior_fh, prior_gh;  // runs before it (reported ahead of its own)
  std::unique_ptr<pgx::Ckpt> restore;      // exact state to upload at admission
  // checkpoints (guarded by the server mutex)
  bool snap_req = false;         // a caller waits for a snapshot at the next boundary
  uint64_t snap_seq = 0;         // snapshots taken
  std::unique_ptr<pgx::Ckpt> snap;
  bool snap_final = false;       // snap holds the state the job ended in
  std::vector<uint8_t> blob;     // the last checkpoint taken by pgx_job_checkpoint
};

template <class T>
std::vector<T> copy_of(const T* p, size_t n) {
  return p ? std::vector<T>(p, p + n) : std::vector<T>();
}

}  // namespace

struct pgx_server {
  pgx_ctx* user = nullptr;   // submit errors are recorded here
  pgx_ctx* ctx = nullptr;    // private: used by the worker thread only
  cudaStream_t ctx_stream = nullptr;  // the private context's own stream
  cudaMemPool_t pool = nullptr;       // stream-ordered job memory (kept for reuse)
  pgx_server_desc cfg{};
  std::vector<Slot> slots;
  std::vector<int> free_slots;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv, done_cv;
  bool stop = false;
  uint64_t next_id = 1;
  std::deque<std::shared_ptr<Job>> queue;
  std::vector<std::shared_ptr<Job>> running;  // mutated by the worker under mu
  std::map<uint64_t, std::shared_ptr<Job>> jobs;
  uint64_t hbm_in_use = 0, hbm_peak = 0;
  int64_t submitted = 0, completed = 0, failed = 0, cancelled = 0;
  std::atomic<int64_t> units{0}, launches{0};  // written by the worker, read by stats
  std::vector<double> latencies;
  std::vector<int> iters_done;
  clk::time_point t0;
};

namespace {

// Points the private context at a slot stream for the duration of a scope, so
// a job's allocations, uploads and frees are ordered on its own stream (and
// never synchronise the device).
struct OnStream {
  pgx_server* s;
  OnStream(pgx_server* srv, cudaStream_t st) : s(srv) { s->ctx->stream = st; }
  ~OnStream() { s->ctx->stream = s->ctx_stream; }
};

// Copies the best controls out, frees the job's device side.  Worker thread,
// mutex NOT held.
void release_device(pgx_server* s, Job& j) {
  if (j.slot < 0) return;
  const cudaStream_t stm = s->slots[j.slot].stream;
  OnStream on(s, stm);
  cudaStreamSynchronize(stm);
  if (j.prob) {
    const size_t n = (size_t)j.desc.n_controls * j.desc.n_slices;
    if (j.round >= 0 && j.d_best) {
      j.u.resize(n);
      cudaMemcpy(j.u.data(), j.d_best, n * sizeof(double), cudaMemcpyDeviceToHost);
    }
    pgx_problem_destroy(j.prob);
    j.prob = nullptr;
  }
  if (j.iter_exec) cudaGraphExecDestroy(j.iter_exec);
  j.iter_exec = nullptr;
  for (auto& g : j.lb_exec) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  if (j.dev) cudaFreeAsync(j.dev, stm);
  j.dev = nullptr;
  if (j.d_best) cudaFreeAsync(j.d_best, stm);
  j.d_best = nullptr;
  for (void* q : {(void*)j.lb, (void*)j.S, (void*)j.Yh, (void*)j.rho, (void*)j.own_u, (void*)j.own_g,
                  (void*)j.dvec})
    if (q) cudaFreeAsync(q, stm);
  j.lb = nullptr;
  j.S = j.Yh = j.rho = j.own_u = j.own_g = j.dvec = nullptr;
  cudaGetLastError();
}

// Iterations a job reports: grape_optimize counts steps, grape_optimize_ensemble
// the entries of its fidelity history (GRAPE.jl:1218), optimcon one less
// (OptControl.jl:476, 555).
int own_iterations(const Job& j) {
  if (j.mr) return std::max((int)j.fh.size() - 1, 0);
  return j.lbfgs ? (int)j.fh.size() : std::max(j.round, 0);
}

template <class T>
std::vector<T> joined(const std::vector<T>& a, const std::vector<T>& b) {
  std::vector<T> out(a);
  out.insert(out.end(), b.begin(), b.end());
  return out;
}

// Mutex held: the fields of Checkpoint (Checkpoint.jl:64-80) a job's host
// side knows.  A resumed job's histories are its checkpoint's followed by
// its own, its iteration count their sum (resume_optimization, :279-287).
void fill_checkpoint(const Job& j, pgx::Ckpt* c) {
  pgx_checkpoint_info& I = c->info;
  I.struct_size = sizeof(pgx_checkpoint_info);
  I.version = PGX_CHECKPOINT_VERSION;
  I.system_dim = j.desc.dim;
  I.n_controls = j.desc.n_controls;
  I.n_timesteps = j.desc.n_slices;
  I.n_members = j.desc.n_members;
  I.iteration = j.prior_iter + own_iterations(j);
  I.F_opt = j.bestF;
  I.F = j.F;
  I.timestamp = pgx::unix_now();
  I.fingerprint = j.fingerprint;
  I.opt = j.opt;
  if (j.converged) I.flags |= PGX_CKPT_CONVERGED;
  c->prior_iteration = j.prior_iter;
  c->prior_history_len = (int32_t)j.prior_fh.size();
  c->prior_gnorm_len = (int32_t)j.prior_gh.size();
  c->fh = joined(j.prior_fh, j.fh);
  c->gh = joined(j.prior_gh, j.gh);
  c->round = j.lbfgs ? j.lb_it : j.round;
}

// Worker thread, mutex NOT held, job at an iteration boundary (nothing of it
// in flight): copies its device state into an exact snapshot -- best and
// current controls, the gradient there, the step-size state (GRAPE) or the
// (s, y) pairs oldest first (L-BFGS) -- and wakes callers waiting for it.
int take_snapshot(pgx_server* s, Job& j, bool final_state) {
  const cudaStream_t stm = s->slots[j.slot].stream;
  const size_t n = (size_t)j.desc.n_controls * j.desc.n_slices;
  auto c = std::make_unique<pgx::Ckpt>();
  c->w.resize(n);
  c->u.resize(n);
  c->g.resize(n);
  auto d2h = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stm) == cudaSuccess;
  };
  bool ok = d2h(c->w.data(), j.d_best, n * sizeof(double));
  int32_t pairs = 0;
  JobDev h{};
  pgx::LbState ls{};
  std::vector<double> S, Y, rho;
  if (j.lbfgs) {
    const size_t m = (size_t)j.opt.lbfgs_memory;
    S.resize(m * n);
    Y.resize(m * n);
    rho.resize(m);
    ok = ok && d2h(c->u.data(), j.ucur, n * sizeof(double)) && d2h(c->g.data(), j.gcur, n * sizeof(double)) &&
         d2h(&ls, j.lb, sizeof ls) && d2h(S.data(), j.S, m * n * sizeof(double)) &&
         d2h(Y.data(), j.Yh, m * n * sizeof(double)) && d2h(rho.data(), j.rho, m * sizeof(double));
  } else {
    ok = ok && d2h(c->u.data(), j.prob->d_u, n * sizeof(double)) &&
         d2h(c->g.data(), j.prob->d_G, n * sizeof(double)) && d2h(&h, j.dev, sizeof h);
  }
  if (!ok || cudaStreamSynchronize(stm) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  if (j.lbfgs) {
    const int m = j.opt.lbfgs_memory;
    if (ls.count < 0 || ls.count > m || ls.head < 0 || ls.head >= m) return PGX_ERR_STATE;
    pairs = ls.count;
    c->rho.resize(pairs);
    c->S.resize((size_t)pairs * n);
    c->Y.resize((size_t)pairs * n);
    for (int t = 0; t < pairs; ++t) {  // slot of the t-th oldest pair
      const int idx = (ls.head - pairs + t + 2 * m) % m;
      c->rho[t] = rho[idx];
      std::copy(S.begin() + (size_t)idx * n, S.begin() + (size_t)(idx + 1) * n, c->S.begin() + (size_t)t * n);
      std::copy(Y.begin() + (size_t)idx * n, Y.begin() + (size_t)(idx + 1) * n, c->Y.begin() + (size_t)t * n);
    }
  } else {
    c->step = h.st.step;
    c->F_prev = h.st.F_prev;
    c->step_iter = h.st.iter;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  fill_checkpoint(j, c.get());
  c->info.flags |= PGX_CKPT_EXACT;
  c->info.lbfgs_pairs = pairs;
  j.snap = std::move(c);
  j.snap_final = final_state;
  j.snap_req = false;
  ++j.snap_seq;
  s->done_cv.notify_all();
  return PGX_OK;
}

// Worker thread, mutex held: final bookkeeping of a job that left `running`;
// frees its slot and budget share.
void record_end(pgx_server* s, Job& j, int state, const std::string& why) {
  j.state = state;
  j.reason = why;
  j.t_end = clk::now();
  if (j.slot >= 0) {
    s->free_slots.push_back(j.slot);
    j.slot = -1;
    s->hbm_in_use -= j.footprint;
  }
  if (state == PGX_JOB_DONE) {
    ++s->completed;
    s->latencies.push_back(secs(j.t_submit, j.t_end));
    s->iters_done.push_back(std::max(j.round, 0));
  } else if (state == PGX_JOB_FAILED) {
    ++s->failed;
  } else {
    ++s->cancelled;
  }
}

int admit_restored(pgx_server* s, Job& j);

// Creates the job's problem and device block on its slot and enqueues the
// evaluation at the initial controls (a job resumed with its exact state
// enqueues its next iteration instead).
int admit(pgx_server* s, Job& j) {
  pgx_ctx* c = s->ctx;
  const Slot& sl = s->slots[j.slot];
  OnStream on(s, sl.stream);
  int st = pgx_problem_create(c, &j.desc, &j.prob);
  if (st) return st;
  if ((!j.pens.empty() && (st = pgx_problem_set_penalties(j.prob, (int32_t)j.pens.size(), j.pens.data()))) ||
      (!j.tr_steps.empty() && (st = pgx_problem_set_tracking(j.prob, (int32_t)j.tr_steps.size(), j.tr_steps.data(),
                                                             j.tr_w.data(), j.tr_t.data()))) ||
      (!j.ramp_mo.empty() &&
       (st = pgx_problem_set_drift_ramp(j.prob, (int32_t)(j.ramp_ops.size() / (2 * (size_t)j.desc.dim * j.desc.dim)),
                                        j.ramp_ops.data(), j.ramp_mo.data(), j.ramp_tau.data()))))
    return st;
  const size_t n = (size_t)j.desc.n_controls * j.desc.n_slices;
  if (cudaMallocFromPoolAsync((void**)&j.dev, sizeof(JobDev), s->pool, sl.stream) != cudaSuccess ||
      cudaMallocFromPoolAsync((void**)&j.d_best, n * sizeof(double), s->pool, sl.stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_NOMEM;
  }
  if (j.lbfgs) {
    const int mm = j.opt.lbfgs_memory;
    auto alloc = [&](double** q, size_t count) {
      return cudaMallocFromPoolAsync((void**)q, sizeof(double) * count, s->pool, sl.stream) == cudaSuccess;
    };
    if (cudaMallocFromPoolAsync((void**)&j.lb, sizeof(pgx::LbState), s->pool, sl.stream) != cudaSuccess ||
        !alloc(&j.S, (size_t)mm * n) || !alloc(&j.Yh, (size_t)mm * n) || !alloc(&j.rho, (size_t)mm) ||
        !alloc(&j.own_u, n) || !alloc(&j.own_g, n) || !alloc(&j.dvec, n)) {
      cudaGetLastError();
      return PGX_ERR_NOMEM;
    }
    pgx::LbState ls{};
    ls.m = mm;
    ls.n = (int)n;
    if (j.restore) {  // the pairs go to slots 0 .. count-1, oldest first
      ls.count = (int)j.restore->rho.size();
      ls.head = ls.count % mm;
    }
    if (cudaMemcpyAsync(j.lb, &ls, sizeof ls, cudaMemcpyHostToDevice, sl.stream) != cudaSuccess) {
      cudaGetLastError();
      return PGX_ERR_CUDA;
    }
    j.ucur = j.prob->d_u;
    j.gcur = j.prob->d_G;
    j.utry = j.own_u;
    j.gtry = j.own_g;
  }
  JobDev h{};
  h.u = j.prob->d_u;
  h.G = j.prob->d_G;
  h.F = j.prob->d_F;
  h.len = (int)n;
  h.st = pgx::AscentState{j.opt.step_size, 0.0, 0, 0};
  if (j.restore && !j.lbfgs) h.st = pgx::AscentState{j.restore->step, j.restore->F_prev, j.restore->step_iter, 0};
  j.step = h.st.step;
  if (cudaMemcpyAsync(j.dev, &h, sizeof(JobDev), cudaMemcpyHostToDevice, sl.stream) != cudaSuccess ||
      cudaMemcpyAsync(j.prob->d_u, j.u.data(), n * sizeof(double), cudaMemcpyHostToDevice, sl.stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(sl.stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  if (j.restore) return admit_restored(s, j);
  const int64_t l0 = c->launches;
  if ((st = run_pipeline(j.prob, j.prob->d_u, j.prob->d_F, j.prob->d_G, sl.stream))) return st;
  s->launches += c->launches - l0;
  if (j.mrgrape) {  // ||G(u0)|| opens the gradient-norm history (OptControl.jl:501)
    if (pgx::launch_norm(j.prob->d_G, (int)n, &j.dev->gnorm, sl.stream) != cudaSuccess ||
        cudaMemcpyAsync(&sl.hb->gnorm, &j.dev->gnorm, sizeof(double), cudaMemcpyDeviceToHost, sl.stream) !=
            cudaSuccess) {
      cudaGetLastError();
      return PGX_ERR_CUDA;
    }
    s->launches += 1;
  }
  if (cudaMemcpyAsync(&sl.hb->F, j.prob->d_F, sizeof(double), cudaMemcpyDeviceToHost, sl.stream) !=
          cudaSuccess ||
      cudaEventRecord(sl.done, sl.stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  j.inflight = true;
  return PGX_OK;
}

// One iteration of a job as a graph: step, evaluation, read-back.  grape_optimize
// reads back (F, ||G|| and step of the step); MR GRAPE (OptControl.jl:512-531)
// steps by 0.05 (u - l) / max|G|, clamps, and reads back (F, ||G||) at the new point.
int capture_iteration(pgx_server* s, Job& j) {
  pgx_ctx* c = s->ctx;
  const Slot& sl = s->slots[j.slot];
  JobDev* d = j.dev;
  const int n = j.desc.n_controls * j.desc.n_slices;
  const pgx::StepArgs a{&d->u, &d->G, &d->F, &d->len, &d->st, nullptr, &d->F_out, &d->gnorm,
                        1, 0, j.opt.adapt_step_size, j.opt.min_step_size, j.opt.max_step_size};
  const int64_t l0 = c->launches;
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  int st = (j.mrgrape ? pgx::launch_mr_step(j.prob->d_u, j.prob->d_G, n, j.opt.l_bound, j.opt.u_bound, sl.stream)
                      : pgx::launch_ascent_step(a, sl.stream)) == cudaSuccess ? PGX_OK : PGX_ERR_CUDA;
  if (!st) st = run_pipeline(j.prob, j.prob->d_u, j.prob->d_F, j.prob->d_G, sl.stream);
  if (!st && j.mrgrape && pgx::launch_norm(j.prob->d_G, n, &d->gnorm, sl.stream) != cudaSuccess) st = PGX_ERR_CUDA;
  if (!st && (cudaMemcpyAsync(&sl.hb->F, j.prob->d_F, sizeof(double), cudaMemcpyDeviceToHost, sl.stream) !=
                  cudaSuccess ||
              cudaMemcpyAsync(&sl.hb->gnorm, &d->gnorm, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                              sl.stream) != cudaSuccess))
    st = PGX_ERR_CUDA;
  const cudaError_t e = cudaStreamEndCapture(sl.stream, &g);
  j.iter_kernels = (j.mrgrape ? 2 : 1) + (c->launches - l0);
  c->launches = l0;  // recorded, not launched: each replay counts them
  if (!st && e != cudaSuccess) st = PGX_ERR_CUDA;
  if (!st && cudaGraphInstantiate(&j.iter_exec, g, 0) != cudaSuccess) st = PGX_ERR_CUDA;
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
  return st;
}

// check_grape_convergence (GRAPE.jl:371-402) on the history as grape_optimize
// holds it at iteration `round`: F(u0) twice, then F(u_1) .. F(u_{round-1}).
bool ref_converged(const Job& j, double gnorm, const char** why) {
  const size_t n = j.fh.size();
  if (j.fh.back() >= 1.0 - 1e-12) { *why = "perfect fidelity (F >= 1 - 1e-12)"; return true; }
  if (gnorm < j.opt.gradient_norm_tol) { *why = "gradient norm below tolerance"; return true; }
  if (n >= 3 && std::fabs(j.fh[n - 1] - j.fh[n - 2]) < j.opt.convergence_tol) {
    *why = "fidelity change below tolerance";
    return true;
  }
  return false;
}

// A finished evaluation of job j: the ascent bookkeeping of grape_optimize
// (GRAPE.jl:536-610) shifted by one -- the evaluation just read is F(u_round),
// which the reference computes at the start of iteration round+1 (or as F_post
// when iteration `round` converged).  Returns false when the job stops; *why
// then names the rule.
bool advance(pgx_server* s, Job& j, const Readback& rb, const char** why, int* err) {
  const Slot& sl = s->slots[j.slot];
  j.round += 1;
  j.F = rb.F;
  if (!std::isfinite(rb.F)) {
    *err = PGX_ERR_NONFINITE;
    *why = "non-finite objective";
    return false;
  }
  bool consider = true;   // does grape_optimize ever compare F(u_round) with the best?
  bool stop = false;
  if (j.round == 0) {
    j.fh.assign(2, rb.F);  // the initial F and iteration 1's F_curr
    // the step rule's previous objective starts at F(u0), as in the history
    if (cudaMemcpyAsync(&j.dev->st.F_prev, j.prob->d_F, sizeof(double), cudaMemcpyDeviceToDevice, sl.stream) !=
        cudaSuccess) {
      cudaGetLastError();
      *err = PGX_ERR_CUDA;
      *why = "step state initialisation failed";
      return false;
    }
  } else {
    j.step = rb.step;
    j.gh.push_back(rb.gnorm);  // ||G(u_{round-1})||: the step's gradient
    if (ref_converged(j, rb.gnorm, why)) {
      j.converged = true;  // F(u_round) is the reference's F_post, recorded too
      j.fh.push_back(rb.F);
      stop = true;
    } else if (rb.F >= s->cfg.target_fidelity) {
      *why = "target fidelity reached";
      j.converged = true;
      j.fh.push_back(rb.F);
      stop = true;
    } else if (j.round >= j.opt.max_iter) {
      *why = "maximum iterations reached";
      consider = false;  // the reference never evaluates the last step's controls
      stop = true;
    } else {
      j.fh.push_back(rb.F);
    }
  }
  if (consider && rb.F > j.bestF) {
    j.bestF = rb.F;
    const size_t n = (size_t)j.desc.n_controls * j.desc.n_slices;
    if (cudaMemcpyAsync(j.d_best, j.prob->d_u, n * sizeof(double), cudaMemcpyDeviceToDevice, sl.stream) !=
        cudaSuccess) {
      cudaGetLastError();
      *err = PGX_ERR_CUDA;
      *why = "best-controls copy failed";
      return false;
    }
  }
  return !stop;
}

// A finished evaluation of an MR GRAPE job (_optimcon_grape, OptControl.jl:
// 486-561): every evaluation enters both histories and the best-controls
// bookkeeping; the stop rules apply from the first step on.
bool advance_mrgrape(pgx_server* s, Job& j, const Readback& rb, const char** why, int* err) {
  const Slot& sl = s->slots[j.slot];
  j.round += 1;
  j.F = rb.F;
  if (!std::isfinite(rb.F)) {
    *err = PGX_ERR_NONFINITE;
    *why = "non-finite objective";
    return false;
  }
  j.fh.push_back(rb.F);
  j.gh.push_back(rb.gnorm);
  if (rb.F > j.bestF) {
    j.bestF = rb.F;
    const size_t n = (size_t)j.desc.n_controls * j.desc.n_slices;
    if (cudaMemcpyAsync(j.d_best, j.prob->d_u, n * sizeof(double), cudaMemcpyDeviceToDevice, sl.stream) !=
        cudaSuccess) {
      cudaGetLastError();
      *err = PGX_ERR_CUDA;
      *why = "best-controls copy failed";
      return false;
    }
  }
  if (j.round == 0) return true;
  if (rb.F >= 1.0 - 1e-8) {
    j.converged = true;
    *why = "near-perfect fidelity";
  } else if (rb.gnorm < j.opt.gradient_norm_tol) {
    j.converged = true;
    *why = "gradient norm below tolerance";
  } else if (rb.F >= s->cfg.target_fidelity) {
    j.converged = true;
    *why = "target fidelity reached";
  } else if (j.round >= j.opt.max_iter) {
    *why = "max iterations reached";
  } else {
    return true;
  }
  return false;
}

// ---- L-BFGS jobs (GRAPE.jl:1012-1230; MR: OptControl.jl:380-482, 594-611) --
// A job's buffers never move (the accept kernel copies ut -> u and gn -> g),
// so each kind of step is captured once per job as a CUDA graph:
//   start       direction, first trial point, F there, read-back
//   halve       halved trial point, F there, read-back
//   fg          F and G at the trial point, read-back
//   halve_fg    halved trial point, F and G there, read-back (after 20 halvings)
//   acc_start   accept (history, u, g), then as start
//   zero_fg     trial point = u, F and G there (MR fall-back: no move)
// MR jobs add ||gn|| at the trial point to every F-and-G read-back.

// First trial step: grape_optimize_ensemble's step_size (x amplitude_limit
// when clipping); MR's 0.05 (u - l) (OptControl.jl:418).
double lb_a0(const Job& j) {
  if (j.mr) return 0.05 * (j.opt.u_bound - j.opt.l_bound);
  const double lim = j.opt.amplitude_limit;
  return std::isfinite(lim) ? j.opt.step_size * lim : j.opt.step_size;
}

pgx::LbArgs lb_args(const Job& j) {
  const double lim = j.opt.amplitude_limit;
  const bool clip = j.mr || std::isfinite(lim);
  const double lo = j.mr ? j.opt.l_bound : -lim, hi = j.mr ? j.opt.u_bound : lim;
  return pgx::LbArgs{j.lb, j.S, j.Yh, j.rho, j.ucur, j.gcur, j.dvec, j.utry, j.gtry, lb_a0(j),
                     clip ? lo : 0.0, clip ? hi : 0.0, clip ? 1 : 0, j.mr ? 1 : 0,
                     j.desc.n_controls * j.desc.n_slices};
}

// Evaluation at the trial point (with G when `grad`) and the read-back of
// (F, dmax, gnorm, zero, gnew); *extra counts the kernels enqueued outside
// the pipeline.
int lb_enqueue_eval(pgx_server* s, Job& j, bool grad, int* extra) {
  const Slot& sl = s->slots[j.slot];
  const int st = run_pipeline(j.prob, j.utry, j.prob->d_F, grad ? j.gtry : nullptr, sl.stream);
  if (st) return st;
  if (grad && j.mr) {
    if (pgx::launch_lb_gnorm(lb_args(j), sl.stream) != cudaSuccess) {
      cudaGetLastError();
      return PGX_ERR_CUDA;
    }
    ++*extra;
  }
  if (cudaMemcpyAsync(&sl.hb->F, j.prob->d_F, sizeof(double), cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess ||
      cudaMemcpyAsync(sl.hb->lb, j.lb, 4 * sizeof(double), cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  return PGX_OK;
}

bool lb_kind_grad(int kind) { return kind == G_FG || kind == G_HALVE_FG || kind == G_ZERO_FG; }

int lb_enqueue_step(pgx_server* s, Job& j, int kind, int* extra) {
  const cudaStream_t stm = s->slots[j.slot].stream;
  const pgx::LbArgs a = lb_args(j);
  auto ok = [&](cudaError_t e) {
    ++*extra;
    return e == cudaSuccess;
  };
  bool good = true;
  if (kind == G_ACC_START) good = ok(pgx::launch_lb_accept(a, stm));
  if (good && (kind == G_START || kind == G_ACC_START))
    good = ok(pgx::launch_lb_direction(a, stm)) && ok(pgx::launch_lb_trial(a, pgx::kTrialFirst, stm));
  if (good && (kind == G_HALVE || kind == G_HALVE_FG)) good = ok(pgx::launch_lb_trial(a, pgx::kTrialHalve, stm));
  if (good && kind == G_ZERO_FG) good = ok(pgx::launch_lb_trial(a, pgx::kTrialZero, stm));
  if (!good) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  return lb_enqueue_eval(s, j, lb_kind_grad(kind), extra);
}

// Launches step `kind` of job j (capturing its graph on first use).
int lb_launch(pgx_server* s, Job& j, int kind) {
  if (!j.lb || !j.S || !j.Yh || !j.rho || !j.ucur || !j.gcur || !j.utry || !j.gtry || !j.dvec)
    return PGX_ERR_STATE;  // never launch on a job whose L-BFGS state is not allocated
  pgx_ctx* c = s->ctx;
  const Slot& sl = s->slots[j.slot];
  if (!j.lb_exec[kind]) {
    const int64_t l0 = c->launches;
    int extra = 0;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return PGX_ERR_CUDA;
    }
    int st = lb_enqueue_step(s, j, kind, &extra);
    const cudaError_t e = cudaStreamEndCapture(sl.stream, &g);
    j.lb_kernels[kind] = extra + (c->launches - l0);
    c->launches = l0;  // recorded, not launched: each replay counts them
    if (!st && e != cudaSuccess) st = PGX_ERR_CUDA;
    if (!st && cudaGraphInstantiate(&j.lb_exec[kind], g, 0) != cudaSuccess) st = PGX_ERR_CUDA;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (st) return st;
  }
  if (cudaGraphLaunch(j.lb_exec[kind], sl.stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  s->launches += j.lb_kernels[kind];
  j.lb_grad_eval = lb_kind_grad(kind);
  return PGX_OK;
}

int lb_copy_best(pgx_server* s, Job& j) {
  const size_t n = (size_t)j.desc.n_controls * j.desc.n_slices;
  if (cudaMemcpyAsync(j.d_best, j.ucur, n * sizeof(double), cudaMemcpyDeviceToDevice,
                      s->slots[j.slot].stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  return PGX_OK;
}

int lb_arm(pgx_server* s, Job& j) {
  if (cudaEventRecord(s->slots[j.slot].done, s->slots[j.slot].stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  j.inflight = true;
  return PGX_OK;
}

// A finished evaluation of an L-BFGS job.  The evaluation at the start of
// each reference iteration, F and G at u, repeats the one at the end of the
// previous iteration (same controls, deterministic evaluation) and is not run
// again.  Returns false when the job stops; *why names the rule.  The next
// step is enqueued here.
bool advance_lbfgs(pgx_server* s, Job& j, const Readback& rb, const char** why, int* err) {
  auto fail = [&](int e, const char* w) {
    *err = e;
    *why = w;
    return false;
  };
  if (!std::isfinite(rb.F)) return fail(PGX_ERR_NONFINITE, "non-finite objective");
  int st = PGX_OK;
  switch (j.lb_phase) {
    case LB_INIT:  // F and G at the initial controls
      j.F = rb.F;
      j.fh.assign(1, rb.F);
      j.bestF = rb.F;
      j.round = 0;
      j.lb_it = 1;
      j.lb_phase = LB_TRIAL;
      j.lb_bt = 0;
      if ((st = lb_copy_best(s, j))) return fail(st, "launch failed");
      if (j.cancel.load() || j.snap_req) {  // a boundary: the worker snapshots or stops
        j.lb_boundary = true;
        return true;
      }
      if ((st = lb_launch(s, j, G_START)) || (st = lb_arm(s, j))) return fail(st, "launch failed");
      return true;
    case LB_TRIAL: {
      if (j.lb_bt == 0) {
        // ||g|| of the iteration (GRAPE.jl:1062); MR records ||G|| at the
        // initial point here and each accepted point's at the accept
        if (!j.mr || j.gh.empty()) j.gh.push_back(rb.lb[1]);
        j.lb_gnorm = rb.lb[1];
        if (rb.lb[2] != 0.0) {
          j.converged = true;
          *why = "zero gradient direction";
          return false;
        }
      }
      // MR accepts F >= F0 - 1e-4 |a| (OptControl.jl:603), the ensemble F >= F0
      const double a = lb_a0(j) * std::ldexp(1.0, -j.lb_bt);  // exact: the device halves the same way
      if (j.mr ? rb.F >= j.F - 1e-4 * std::fabs(a) : rb.F >= j.F) {  // accepted: F and G there
        j.lb_phase = LB_ACCEPT;
        st = lb_launch(s, j, G_FG);
      } else if (j.mr) {  // backtrack: 20 trials, then one more at a / 2 (OptControl.jl:600-610)
        j.lb_bt += 1;
        if (j.lb_bt >= 20) j.lb_phase = LB_FALLBACK;
        st = lb_launch(s, j, G_HALVE);
      } else {  // backtrack: halve (20 halvings, then take the last one)
        j.lb_bt += 1;
        if (j.lb_bt >= 20) j.lb_phase = LB_ACCEPT;
        st = lb_launch(s, j, j.lb_bt >= 20 ? G_HALVE_FG : G_HALVE);
      }
      if (st || (st = lb_arm(s, j))) return fail(st, "launch failed");
      return true;
    }
    case LB_FALLBACK:  // MR: keep the last trial point only if it improves F
      j.lb_phase = LB_ACCEPT;
      if ((st = lb_launch(s, j, rb.F > j.F ? G_FG : G_ZERO_FG)) || (st = lb_arm(s, j)))
        return fail(st, "launch failed");
      return true;
    default: {  // LB_ACCEPT: F and G at the accepted point
      const double Fprev = j.F;
      j.F = rb.F;
      j.fh.push_back(rb.F);
      j.round = (int)j.fh.size() - 1;
      const bool improved = j.F > j.bestF;
      if (improved) j.bestF = j.F;
      bool stop = true;
      if (j.mr) {  // OptControl.jl:465-471
        j.gh.push_back(rb.lb[3]);
        if (j.F >= 1.0 - 1e-8) {
          j.converged = true;
          *why = "near-perfect fidelity";
        } else if (rb.lb[3] < j.opt.gradient_norm_tol) {
          j.converged = true;
          *why = "gradient norm below tolerance";
        } else if (std::fabs(j.F - Fprev) < 1e-9) {
          j.converged = true;
          *why = "fidelity stalled";
        } else if (j.F >= s->cfg.target_fidelity) {
          j.converged = true;
          *why = "target fidelity reached";
        } else if (++j.lb_it > j.opt.max_iter) {
          *why = "max iterations reached";
        } else {
          stop = false;
        }
      } else if (j.lb_gnorm < j.opt.gradient_norm_tol) {
        j.converged = true;
        *why = "gradient norm below tolerance";
      } else if (j.F >= 1.0 - 1e-8) {
        j.converged = true;
        *why = "near-perfect fidelity";
      } else if (std::fabs(j.F - Fprev) < j.opt.convergence_tol) {
        j.converged = true;
        *why = "fidelity change below tolerance";
      } else if (j.F >= s->cfg.target_fidelity) {
        j.converged = true;
        *why = "target fidelity reached";
      } else if (++j.lb_it > j.opt.max_iter) {
        *why = "maximum iterations reached";
      } else {
        stop = false;
      }
      if (stop) {  // accept only: u <- ut for the best copy
        if (pgx::launch_lb_accept(lb_args(j), s->slots[j.slot].stream) != cudaSuccess) {
          cudaGetLastError();
          return fail(PGX_ERR_CUDA, "launch failed");
        }
        s->launches += 1;
        if (improved && (st = lb_copy_best(s, j))) return fail(st, "launch failed");
        return false;
      }
      j.lb_phase = LB_TRIAL;
      j.lb_bt = 0;
      if (j.cancel.load() || j.snap_req) {  // a boundary: accept only, the worker goes on
        if (pgx::launch_lb_accept(lb_args(j), s->slots[j.slot].stream) != cudaSuccess) {
          cudaGetLastError();
          return fail(PGX_ERR_CUDA, "launch failed");
        }
        s->launches += 1;
        if (improved && (st = lb_copy_best(s, j))) return fail(st, "launch failed");
        j.lb_boundary = true;
        return true;
      }
      // the graph's accept updates u before its trial point reads it; the
      // best copy follows the graph (nothing in it writes u after the accept)
      if ((st = lb_launch(s, j, G_ACC_START)) || (improved && (st = lb_copy_best(s, j))) || (st = lb_arm(s, j)))
        return fail(st, "launch failed");
      return true;
    }
  }
}

int launch_iteration(pgx_server* s, Job& j) {
  if (!j.iter_exec) {
    const int st = capture_iteration(s, j);
    if (st) return st;
  }
  const Slot& sl = s->slots[j.slot];
  if (cudaGraphLaunch(j.iter_exec, sl.stream) != cudaSuccess || cudaEventRecord(sl.done, sl.stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  s->launches += j.iter_kernels;
  j.inflight = true;
  return PGX_OK;
}

// The first step of the next L-BFGS iteration after a boundary.
int lb_start(pgx_server* s, Job& j) {
  j.lb_boundary = false;
  int st = lb_launch(s, j, G_START);
  if (!st) st = lb_arm(s, j);
  return st;
}

// Admission of a job resumed with its exact state: the gradient, objective,
// best controls and L-BFGS pairs join the controls admit() uploaded, the
// host bookkeeping takes the snapshot's, and the job's next iteration is
// enqueued as if it had never stopped.
int admit_restored(pgx_server* s, Job& j) {
  const pgx::Ckpt& r = *j.restore;
  const Slot& sl = s->slots[j.slot];
  const size_t n = (size_t)j.desc.n_controls * j.desc.n_slices;
  const size_t pairs = r.rho.size();
  auto h2d = [&](void* dst, const void* src, size_t bytes) {
    return bytes == 0 || cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, sl.stream) == cudaSuccess;
  };
  bool ok = h2d(j.prob->d_G, r.g.data(), n * sizeof(double)) && h2d(j.prob->d_F, &r.info.F, sizeof(double)) &&
            h2d(j.d_best, r.w.data(), n * sizeof(double));
  if (j.lbfgs)
    ok = ok && h2d(j.S, r.S.data(), pairs * n * sizeof(double)) &&
         h2d(j.Yh, r.Y.data(), pairs * n * sizeof(double)) && h2d(j.rho, r.rho.data(), pairs * sizeof(double));
  if (!ok || cudaStreamSynchronize(sl.stream) != cudaSuccess) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    j.F = r.info.F;
    j.bestF = r.info.F_opt;
    if (j.lbfgs) {
      j.round = (int)j.fh.size() - 1;
      j.lb_it = r.round;
      j.lb_phase = LB_TRIAL;
      j.lb_bt = 0;
    } else {
      j.round = r.round;
    }
  }
  j.restore.reset();
  return j.lbfgs ? lb_start(s, j) : launch_iteration(s, j);
}

void worker_loop(pgx_server* s) {
  cudaSetDevice(s->ctx->device);
  while (true) {
    // ---- admission ----
    std::vector<std::shared_ptr<Job>> admitted;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->running.empty() && s->queue.empty()) {
        s->done_cv.notify_all();
        if (s->stop) break;
        s->cv.wait(lk, [&] { return s->stop || !s->queue.empty(); });
        if (s->stop && s->queue.empty()) break;
      }
      if (s->stop)
        for (auto& j : s->running) j->cancel.store(true);
      while (!s->stop && !s->queue.empty() && !s->free_slots.empty()) {
        auto j = s->queue.front();
        if (s->cfg.hbm_budget_bytes && s->hbm_in_use + j->footprint > s->cfg.hbm_budget_bytes) break;
        s->queue.pop_front();
        j->slot = s->free_slots.back();
        s->free_slots.pop_back();
        s->hbm_in_use += j->footprint;
        s->hbm_peak = std::max(s->hbm_peak, s->hbm_in_use);
        j->state = PGX_JOB_RUNNING;
        j->t_start = clk::now();
        s->running.push_back(j);
        admitted.push_back(j);
      }
    }
    for (auto& j : admitted) {
      const int st = admit(s, *j);
      if (st) {
        release_device(s, *j);
        std::lock_guard<std::mutex> lk(s->mu);
        j->status = st;
        s->running.erase(std::find(s->running.begin(), s->running.end(), j));
        record_end(s, *j, PGX_JOB_FAILED, std::string("admission failed: ") + pgx_status_string(st));
        s->done_cv.notify_all();
      }
    }
    // ---- progress ----
    bool progress = !admitted.empty();
    std::vector<std::shared_ptr<Job>> ended;
    std::vector<std::pair<int, std::string>> end_how;
    const size_t n_run = s->running.size();  // only this thread changes `running`
    for (size_t i = 0; i < n_run; ++i) {
      auto j = s->running[i];
      if (!j->inflight) continue;
      const Slot& sl = s->slots[j->slot];
      const cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) continue;
      progress = true;
      j->inflight = false;
      int err = (q == cudaSuccess) ? PGX_OK : PGX_ERR_CUDA;
      cudaGetLastError();
      const char* why = "evaluation failed";
      bool go = false, want_snap = false;
      if (!err) {
        const Readback rb = *sl.hb;
        if (!j->lbfgs || j->lb_grad_eval) s->units += j->units;
        std::lock_guard<std::mutex> lk(s->mu);  // polls read what advance() updates
        go = j->lbfgs     ? advance_lbfgs(s, *j, rb, &why, &err)
             : j->mrgrape ? advance_mrgrape(s, *j, rb, &why, &err)
                          : advance(s, *j, rb, &why, &err);
        want_snap = j->snap_req;
      }
      // An iteration boundary: the job continues and nothing of it is in
      // flight.  Cancellation and snapshots happen only here, so a cancelled
      // job's state is one an exact resumption can continue from.
      const bool boundary = go && (!j->lbfgs || j->lb_boundary);
      bool cancelled = false;
      if (boundary && j->cancel.load()) {
        go = false;
        cancelled = true;
      }
      if (boundary && (cancelled || want_snap)) {
        const int st = take_snapshot(s, *j, cancelled);
        if (st && !cancelled) err = st;  // a cancelled job keeps its host-side checkpoint
      }
      if (go && !err) err = !j->lbfgs ? launch_iteration(s, *j) : j->lb_boundary ? lb_start(s, *j) : PGX_OK;
      if (go && !err) continue;
      ended.push_back(j);
      if (err) {
        j->status = err;
        end_how.emplace_back(PGX_JOB_FAILED, err == PGX_ERR_NONFINITE ? why : pgx_status_string(err));
      } else if (cancelled) {
        end_how.emplace_back(PGX_JOB_CANCELLED, "cancelled");
      } else {
        end_how.emplace_back(PGX_JOB_DONE, why);
      }
    }
    for (auto& j : ended) release_device(s, *j);
    if (!ended.empty()) {
      std::lock_guard<std::mutex> lk(s->mu);
      for (size_t e = 0; e < ended.size(); ++e) {
        s->running.erase(std::find(s->running.begin(), s->running.end(), ended[e]));
        record_end(s, *ended[e], end_how[e].first, end_how[e].second);
      }
      s->done_cv.notify_all();
    }
    if (!progress) {
      // Device progress is polled.  While any job is on the device the loop
      // only yields between sweeps: a timed sleep here (with the kernel's
      // timer slack) would add its wake-up latency to every step of every
      // small job.  With nothing in flight it sleeps until a submission.
      bool any_inflight = false;
      for (const auto& j : s->running) any_inflight |= j->inflight;
      if (any_inflight) {
        std::this_thread::yield();
      } else {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv.wait_for(lk, std::chrono::microseconds(200),
                       [&] { return s->stop || (!s->queue.empty() && !s->free_slots.empty()); });
      }
    }
  }
}

double pct(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

void fill_status(const Job& j, pgx_job_status* out) {
  std::memset(out, 0, sizeof(*out));
  out->state = j.state;
  out->status = j.status;
  out->iterations = j.prior_iter + own_iterations(j);
  out->fidelity = j.F;
  out->best_fidelity = j.bestF;
  const auto now = clk::now();
  const bool ended = j.state == PGX_JOB_DONE || j.state == PGX_JOB_FAILED || j.state == PGX_JOB_CANCELLED;
  const bool started = j.t_start.time_since_epoch().count() != 0;
  out->latency_s = secs(j.t_submit, ended ? j.t_end : now);
  out->queue_s = started ? secs(j.t_submit, j.t_start) : out->latency_s;
  std::snprintf(out->reason, sizeof(out->reason), "%s", j.reason.c_str());
}

}  // namespace

extern "C" int pgx_server_create(pgx_ctx* c, const pgx_server_desc* d, pgx_server** out) {
  if (!c || !d || !out) return PGX_ERR_INVALID;
  *out = nullptr;
  if (d->struct_size < sizeof(pgx_server_desc) || d->max_inflight < 1 || d->max_inflight > 4096 ||
      !(d->target_fidelity > 0.0))
    return ctx_fail(c, PGX_ERR_INVALID, "invalid server settings");
  auto* s = new pgx_server();
  s->user = c;
  s->cfg = *d;
  s->t0 = clk::now();
  int st = pgx_ctx_create(c->device, 0, &s->ctx);
  cudaSetDevice(c->device);
  if (!st) {
    s->ctx_stream = s->ctx->stream;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = c->device;
    uint64_t keep = UINT64_MAX;  // freed job memory stays in the pool for the next job
    if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
      cudaGetLastError();
      st = PGX_ERR_CUDA;
    } else {
      s->ctx->pool = s->pool;
    }
  }
  s->slots.resize(d->max_inflight);
  for (int i = 0; i < d->max_inflight && !st; ++i) {
    Slot& sl = s->slots[i];
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost((void**)&sl.hb, sizeof(Readback)) != cudaSuccess) {
      cudaGetLastError();
      st = PGX_ERR_CUDA;
    }
  }
  for (int i = d->max_inflight - 1; i >= 0; --i) s->free_slots.push_back(i);
  if (st) {
    pgx_server_destroy(s);
    return ctx_fail(c, st, "server resources could not be created");
  }
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return PGX_OK;
}

extern "C" int pgx_server_destroy(pgx_server* s) {
  if (!s) return PGX_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (auto& j : s->queue) {
      j->state = PGX_JOB_CANCELLED;
      j->reason = "server destroyed";
      ++s->cancelled;
    }
    s->queue.clear();
    for (auto& j : s->running) j->cancel.store(true);
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->ctx) cudaSetDevice(s->ctx->device);
  for (auto& j : s->running) release_device(s, *j);  // only when the worker never started
  for (auto& sl : s->slots) {
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.hb) cudaFreeHost(sl.hb);
  }
  if (s->ctx) pgx_ctx_destroy(s->ctx);
  if (s->pool) {
    cudaDeviceSynchronize();  // every cudaFreeAsync into the pool has run
    cudaMemPoolDestroy(s->pool);
  }
  delete s;
  return PGX_OK;
}

namespace {

// Validates a submission and builds its job (owned copies of every array).
int make_job(pgx_server* s, const pgx_problem_desc* d, const pgx_opt_desc* o, const double* u0,
             const pgx_job_extras* x, std::shared_ptr<Job>* out) {
  pgx_ctx* c = s->user;
  int st = validate_desc(c, d);
  if (st) return st;
  if (o->struct_size < sizeof(pgx_opt_desc) || o->max_iter < 1 || o->step_size <= 0.0 ||
      o->min_step_size <= 0.0 || o->max_step_size < o->step_size)
    return ctx_fail(c, PGX_ERR_INVALID, "invalid optimiser settings (GRAPE.jl:108-119)");
  if (o->method != PGX_OPT_GRAPE && o->method != PGX_OPT_ENSEMBLE_LBFGS && o->method != PGX_OPT_MR_LBFGS &&
      o->method != PGX_OPT_MR_GRAPE)
    return ctx_fail(c, PGX_ERR_UNSUPPORTED, "unknown optimisation method");
  const bool mr = o->method == PGX_OPT_MR_LBFGS || o->method == PGX_OPT_MR_GRAPE;
  if (o->method == PGX_OPT_ENSEMBLE_LBFGS &&
      (o->lbfgs_memory < 1 || o->lbfgs_memory > pgx::kLbMaxMemory || !(o->amplitude_limit > 0.0)))
    return ctx_fail(c, PGX_ERR_INVALID, "lbfgs_memory must be in [1, 64] and amplitude_limit positive");
  if (mr && !(std::isfinite(o->l_bound) && std::isfinite(o->u_bound) && o->l_bound < o->u_bound))
    return ctx_fail(c, PGX_ERR_INVALID, "MR methods need finite bounds l_bound < u_bound");
  if (o->method == PGX_OPT_MR_LBFGS && (o->lbfgs_memory < 1 || o->lbfgs_memory > pgx::kLbMaxMemory))
    return ctx_fail(c, PGX_ERR_INVALID, "lbfgs_memory must be in [1, 64]");
  const size_t D = d->dim, DD = D * D, nc = d->n_controls, nt = d->n_slices, nm = d->n_members;
  const size_t np = d->target == PGX_TARGET_STATES ? d->n_pairs : 0;
  for (size_t i = 0; i < nc * nt; ++i)
    if (!std::isfinite(u0[i])) return ctx_fail(c, PGX_ERR_NONFINITE, "controls must be finite");
  if (x && (x->struct_size < sizeof(pgx_job_extras) || x->n_penalties < 0 || x->n_penalties > PGX_MAX_PENALTIES ||
            x->n_tracking < 0 || x->n_ramp_ops < 0 || (x->n_penalties > 0 && !x->penalties) ||
            (x->n_tracking > 0 && (!x->tracking_steps || !x->tracking_weights || !x->tracking_targets)) ||
            (x->n_ramp_ops > 0 && (!x->ramp_ops || !x->ramp_member_op || !x->ramp_tau))))
    return ctx_fail(c, PGX_ERR_INVALID, "invalid job extras");
  auto j = std::make_shared<Job>();
  j->lbfgs = o->method == PGX_OPT_ENSEMBLE_LBFGS || o->method == PGX_OPT_MR_LBFGS;
  j->mr = mr;
  j->mrgrape = o->method == PGX_OPT_MR_GRAPE;
  j->footprint = problem_footprint(d, s->ctx->num_sms) + sizeof(JobDev) + nc * nt * sizeof(double);
  if (j->lbfgs)  // (s, y) history, rho, trial controls and gradient, direction
    j->footprint += sizeof(pgx::LbState) + sizeof(double) * ((2 * (size_t)o->lbfgs_memory + 3) * nc * nt +
                                                             (size_t)o->lbfgs_memory);
  if (s->cfg.hbm_budget_bytes && j->footprint > s->cfg.hbm_budget_bytes)
    return ctx_fail(c, PGX_ERR_BUDGET, "job footprint exceeds the server's HBM budget");
  j->units = (int64_t)nm * (int64_t)nt;
  j->fingerprint = pgx::problem_fingerprint(d, x);
  if (x) {
    j->pens = copy_of(x->penalties, (size_t)x->n_penalties);
    j->tr_steps = copy_of(x->tracking_steps, (size_t)x->n_tracking);
    j->tr_w = copy_of(x->tracking_weights, (size_t)x->n_tracking);
    j->tr_t = copy_of(x->tracking_targets, 2 * DD * (size_t)x->n_tracking);
    if (x->n_ramp_ops > 0) {
      j->ramp_ops = copy_of(x->ramp_ops, 2 * DD * (size_t)x->n_ramp_ops);
      j->ramp_mo = copy_of(x->ramp_member_op, nm);
      j->ramp_tau = copy_of(x->ramp_tau, nt);
    }
  }
  j->dt = copy_of(d->dt, nt);
  j->drifts = copy_of(d->drifts, 2 * DD * d->n_drifts);
  j->controls = copy_of(d->controls, 2 * DD * nc);
  j->offset = copy_of(d->offset_op, 2 * DD);
  j->mdrift = copy_of(d->member_drift, nm);
  j->mscale = copy_of(d->member_scale, nm);
  j->moffset = copy_of(d->member_offset, nm);
  j->mweight = copy_of(d->member_weight, nm);
  j->target = copy_of(d->target_op, 2 * DD);
  j->sinit = copy_of(d->states_init, 2 * np * D);
  j->starg = copy_of(d->states_target, 2 * np * D);
  j->sgrad = copy_of(d->grad_states_init, 2 * np * D);
  j->desc = *d;
  auto P = [](std::vector<double>& v) -> const double* { return v.empty() ? nullptr : v.data(); };
  j->desc.dt = P(j->dt);
  j->desc.drifts = P(j->drifts);
  j->desc.controls = P(j->controls);
  j->desc.offset_op = P(j->offset);
  j->desc.member_drift = j->mdrift.empty() ? nullptr : j->mdrift.data();
  j->desc.member_scale = P(j->mscale);
  j->desc.member_offset = P(j->moffset);
  j->desc.member_weight = P(j->mweight);
  j->desc.target_op = P(j->target);
  j->desc.states_init = P(j->sinit);
  j->desc.states_target = P(j->starg);
  j->desc.grad_states_init = P(j->sgrad);
  j->opt = *o;
  j->u.assign(u0, u0 + nc * nt);
  if (mr)  // optimcon clamps the guess to the bounds first (OptControl.jl:384, 491)
    for (double& x : j->u) x = std::min(std::max(x, o->l_bound), o->u_bound);
  *out = std::move(j);
  return PGX_OK;
}

int enqueue(pgx_server* s, std::shared_ptr<Job> j, uint64_t* job_id) {
  j->t_submit = clk::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return PGX_ERR_STATE;
    j->id = s->next_id++;
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    ++s->submitted;
    *job_id = j->id;
  }
  s->cv.notify_all();
  return PGX_OK;
}

std::shared_ptr<Job> find_job(pgx_server* s, uint64_t id) {
  auto it = s->jobs.find(id);
  return it == s->jobs.end() ? nullptr : it->second;
}

}  // namespace

extern "C" int pgx_submit_ex(pgx_server* s, const pgx_problem_desc* d, const pgx_opt_desc* o, const double* u0,
                             const pgx_job_extras* x, uint64_t* job_id) {
  if (!s || !d || !o || !u0 || !job_id) return PGX_ERR_INVALID;
  std::shared_ptr<Job> j;
  const int st = make_job(s, d, o, u0, x, &j);
  return st ? st : enqueue(s, std::move(j), job_id);
}

extern "C" int pgx_submit(pgx_server* s, const pgx_problem_desc* d, const pgx_opt_desc* o, const double* u0,
                          uint64_t* job_id) {
  return pgx_submit_ex(s, d, o, u0, nullptr, job_id);
}

extern "C" int pgx_submit_resume(pgx_server* s, const pgx_problem_desc* d, const pgx_opt_desc* o,
                                 const pgx_job_extras* x, const void* blob, uint64_t blob_len, int32_t mode,
                                 uint64_t* job_id) {
  if (!s || !d || !blob || !job_id) return PGX_ERR_INVALID;
  pgx_ctx* c = s->user;
  if (mode != PGX_RESUME_RESTART && mode != PGX_RESUME_CONTINUE)
    return ctx_fail(c, PGX_ERR_INVALID, "mode must be PGX_RESUME_RESTART or PGX_RESUME_CONTINUE");
  auto ck = std::make_unique<pgx::Ckpt>();
  std::string why;
  if (pgx::ckpt_decode(blob, blob_len, ck.get(), &why)) return ctx_fail(c, PGX_ERR_INVALID, why.c_str());
  const pgx_checkpoint_info& I = ck->info;
  char msg[160];
  if (I.system_dim > 0 && I.system_dim != d->dim) {  // Checkpoint.jl:236-240
    std::snprintf(msg, sizeof msg, "System dimension mismatch: checkpoint has dim=%d, provided system has dim=%d",
                  I.system_dim, d->dim);
    return ctx_fail(c, PGX_ERR_INVALID, msg);
  }
  if (I.n_controls != d->n_controls) {  // Checkpoint.jl:242-246
    std::snprintf(msg, sizeof msg, "n_controls mismatch: checkpoint=%d, system=%d", I.n_controls, d->n_controls);
    return ctx_fail(c, PGX_ERR_INVALID, msg);
  }
  if (I.n_timesteps != d->n_slices) {
    std::snprintf(msg, sizeof msg, "n_timesteps mismatch: checkpoint=%d, problem=%d", I.n_timesteps, d->n_slices);
    return ctx_fail(c, PGX_ERR_DIMS, msg);
  }
  const pgx_opt_desc opt = o ? *o : I.opt;
  const bool cont = mode == PGX_RESUME_CONTINUE;
  if (cont) {
    if (!(I.flags & PGX_CKPT_EXACT))
      return ctx_fail(c, PGX_ERR_INVALID, "exact continuation needs a snapshot of a running or cancelled job");
    if (validate_desc(c, d)) return PGX_ERR_INVALID;
    if (pgx::problem_fingerprint(d, x) != I.fingerprint)
      return ctx_fail(c, PGX_ERR_INVALID, "the checkpoint was taken on a different problem");
    if (opt.method != I.opt.method)
      return ctx_fail(c, PGX_ERR_INVALID, "exact continuation keeps the checkpoint's method");
    if ((opt.method == PGX_OPT_ENSEMBLE_LBFGS || opt.method == PGX_OPT_MR_LBFGS) && opt.lbfgs_memory < I.lbfgs_pairs)
      return ctx_fail(c, PGX_ERR_INVALID, "lbfgs_memory is below the checkpoint's stored pairs");
  }
  std::shared_ptr<Job> j;
  const int st = make_job(s, d, &opt, cont ? ck->u.data() : ck->w.data(), x, &j);
  if (st) return st;
  if (cont) {  // the run goes on: its own histories continue, earlier runs' stay ahead
    j->prior_iter = ck->prior_iteration;
    j->prior_fh.assign(ck->fh.begin(), ck->fh.begin() + ck->prior_history_len);
    j->prior_gh.assign(ck->gh.begin(), ck->gh.begin() + ck->prior_gnorm_len);
    j->fh.assign(ck->fh.begin() + ck->prior_history_len, ck->fh.end());
    j->gh.assign(ck->gh.begin() + ck->prior_gnorm_len, ck->gh.end());
    j->restore = std::move(ck);
  } else {  // resume_optimization: a fresh run after the checkpoint's
    j->prior_iter = I.iteration;
    j->prior_fh = std::move(ck->fh);
    j->prior_gh = std::move(ck->gh);
  }
  return enqueue(s, std::move(j), job_id);
}

extern "C" int pgx_job_checkpoint(pgx_server* s, uint64_t id, double timeout_s, uint64_t* blob_len) {
  if (!s || !blob_len) return PGX_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const std::shared_ptr<Job> jp = find_job(s, id);
  if (!jp) return PGX_ERR_INVALID;
  Job& j = *jp;
  if (j.state == PGX_JOB_QUEUED) return PGX_ERR_STATE;
  if (j.state == PGX_JOB_RUNNING) {
    const uint64_t seq0 = j.snap_seq;
    j.snap_req = true;
    const auto ready = [&] { return j.snap_seq != seq0 || j.state != PGX_JOB_RUNNING; };
    if (timeout_s <= 0) {
      s->done_cv.wait(lk, ready);
    } else if (!s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
      return PGX_ERR_TIMEOUT;
    }
  }
  if (j.state == PGX_JOB_RUNNING || (j.snap && j.snap_final)) {
    j.blob = pgx::ckpt_encode(*j.snap);
  } else {  // finished: the final best controls and histories
    if (j.round < 0 || j.u.size() != (size_t)j.desc.n_controls * j.desc.n_slices) return PGX_ERR_STATE;
    pgx::Ckpt c;
    fill_checkpoint(j, &c);
    c.w = j.u;
    j.blob = pgx::ckpt_encode(c);
  }
  *blob_len = j.blob.size();
  return PGX_OK;
}

extern "C" int pgx_job_checkpoint_read(pgx_server* s, uint64_t id, void* blob, uint64_t cap) {
  if (!s || !blob) return PGX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  const std::shared_ptr<Job> j = find_job(s, id);
  if (!j) return PGX_ERR_INVALID;
  if (j->blob.empty()) return PGX_ERR_STATE;
  if (cap < j->blob.size()) return PGX_ERR_DIMS;
  std::memcpy(blob, j->blob.data(), j->blob.size());
  return PGX_OK;
}

extern "C" int pgx_job_history(pgx_server* s, uint64_t id, double* fh, double* gh, int32_t cap, int32_t* n_f,
                               int32_t* n_g) {
  if (!s || cap < 0) return PGX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  const std::shared_ptr<Job> j = find_job(s, id);
  if (!j) return PGX_ERR_INVALID;
  const std::vector<double> f = joined(j->prior_fh, j->fh), g = joined(j->prior_gh, j->gh);
  if (n_f) *n_f = (int32_t)f.size();
  if (n_g) *n_g = (int32_t)g.size();
  if (fh) std::copy(f.begin(), f.begin() + std::min<size_t>(f.size(), (size_t)cap), fh);
  if (gh) std::copy(g.begin(), g.begin() + std::min<size_t>(g.size(), (size_t)cap), gh);
  return PGX_OK;
}

extern "C" int pgx_poll(pgx_server* s, uint64_t id, pgx_job_status* out) {
  if (!s || !out) return PGX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return PGX_ERR_INVALID;
  fill_status(*it->second, out);
  return PGX_OK;
}

extern "C" int pgx_fetch(pgx_server* s, uint64_t id, double* u, pgx_opt_result* res) {
  if (!s) return PGX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return PGX_ERR_INVALID;
  const Job& j = *it->second;
  if (j.state == PGX_JOB_QUEUED || j.state == PGX_JOB_RUNNING) return PGX_ERR_STATE;
  if (res) {
    std::memset(res, 0, sizeof(*res));
    res->fidelity = j.bestF;
    res->total_time_s = secs(j.t_submit, j.t_end);
    res->step_size_final = j.mrgrape ? 0.05 : j.mr ? 0.0 : j.lbfgs ? j.opt.step_size : j.step;
    res->n_iterations = j.prior_iter + own_iterations(j);
    res->history_len = (int32_t)(j.prior_fh.size() + j.fh.size());
    res->gnorm_history_len = (int32_t)(j.prior_gh.size() + j.gh.size());
    res->converged = j.converged;
    res->n_fidelity_evals = j.round + 1;
    res->n_gradient_evals = j.round + 1;
    std::snprintf(res->reason, sizeof(res->reason), "%s", j.reason.c_str());
  }
  if (u && j.u.size() == (size_t)j.desc.n_controls * j.desc.n_slices) std::copy(j.u.begin(), j.u.end(), u);
  const int rc = j.state == PGX_JOB_DONE ? PGX_OK : j.state == PGX_JOB_CANCELLED ? PGX_ERR_CANCELLED : j.status;
  s->jobs.erase(it);
  return rc;
}

extern "C" int pgx_cancel(pgx_server* s, uint64_t id) {
  if (!s) return PGX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return PGX_ERR_INVALID;
  auto& j = it->second;
  if (j->state == PGX_JOB_QUEUED) {
    s->queue.erase(std::remove(s->queue.begin(), s->queue.end(), j), s->queue.end());
    j->state = PGX_JOB_CANCELLED;
    j->reason = "cancelled";
    j->t_end = clk::now();
    ++s->cancelled;
    s->done_cv.notify_all();
    return PGX_OK;
  }
  if (j->state == PGX_JOB_RUNNING) {
    j->cancel.store(true);  // stops after its in-flight iteration
    return PGX_OK;
  }
  return PGX_ERR_STATE;
}

extern "C" int pgx_server_drain(pgx_server* s, double timeout_s) {
  if (!s) return PGX_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto idle = [&] { return s->queue.empty() && s->running.empty(); };
  if (timeout_s <= 0) {
    s->done_cv.wait(lk, idle);
    return PGX_OK;
  }
  return s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), idle) ? PGX_OK : PGX_ERR_TIMEOUT;
}

extern "C" int pgx_server_stats(pgx_server* s, pgx_serve_stats* out) {
  if (!s || !out) return PGX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->cancelled = s->cancelled;
  out->running = (int64_t)s->running.size();
  out->queued = (int64_t)s->queue.size();
  out->kernel_launches = s->launches.load();
  out->units = s->units.load();
  out->hbm_in_use = s->hbm_in_use;
  out->hbm_peak = s->hbm_peak;
  out->elapsed_s = secs(s->t0, clk::now());
  out->jobs_per_s = out->elapsed_s > 0 ? (double)s->completed / out->elapsed_s : 0.0;
  out->p50_latency_s = pct(s->latencies, 0.50);
  out->p99_latency_s = pct(s->latencies, 0.99);
  double it = 0;
  for (int k : s->iters_done) it += k;
  out->mean_iterations = s->iters_done.empty() ? 0.0 : it / (double)s->iters_done.size();
  return PGX_OK;
}
