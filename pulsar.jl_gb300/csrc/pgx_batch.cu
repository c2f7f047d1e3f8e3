// Batched uneven problems: one CUDA graph per GRAPE iteration.
//
// A batch owns N problems of any dimensions, slice counts and ensemble sizes
// (each already resident in HBM).  One iteration evaluates every problem at its
// device-resident controls and applies the grape_optimize ascent step
// (GRAPE.jl:536-610: adapt_grape_step_size :309-334, grape_step! :261-268) to
// every problem on the device.  The per-problem pipelines are fanned out over
// several streams -- largest problems first -- so small problems fill the GPU
// while large ones run, and the whole iteration (fork, pipelines, join, the
// step kernel) is captured once into a CUDA graph and relaunched; the host
// reads nothing between iterations.  Each problem runs the kernels of a solo
// evaluation, except that mixed problems of padded dimension 2 get their slice
// propagators from one shared launch (the register-resident expm over every
// (problem, member, slice) item of the class, whose per-slice arithmetic is
// the solo launch's), so batched results are bit-identical to solo ones.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "pgx.h"
#include "pgx_runtime.h"

using pgx::AscentState;
using pgx::StepArgs;
using pgx::kStepThreads;

namespace {

// One CTA per problem: the step rule of adapt_grape_step_size, then u += step G.
__global__ void k_ascent_step(StepArgs a) {
  const int i = blockIdx.x;
  if (i >= a.n) return;
  __shared__ double step;
  if (threadIdx.x == 0) {
    const double F = a.F[i][0];
    AscentState s = a.st[i];
    if (a.adapt) {
      const double d = F - s.F_prev;  // the history always holds the previous objective
      double ns = s.step;
      if (d > 0.0) ns = s.step * 1.05;
      else if (d < -1e-14) ns = s.step * 0.5;
      s.step = fmin(fmax(ns, a.lo), a.hi);
    }
    if (a.trace && s.iter < a.trace_cap) a.trace[(size_t)s.iter * a.n + i] = F;
    s.F_prev = F;
    s.iter += 1;
    a.st[i] = s;
    a.F_all[i] = F;
    step = s.step;
  }
  __syncthreads();
  double* u = a.u[i];
  const double* G = a.G[i];
  double acc = 0.0;
  for (int k = threadIdx.x; k < a.len[i]; k += blockDim.x) {
    const double g = G[k];
    acc = fma(g, g, acc);
    u[k] = fma(step, g, u[k]);
  }
  if (a.gnorm) {  // fixed-order tree: the same bits on every run
    __shared__ double red[kStepThreads];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kStepThreads / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) a.gnorm[i] = sqrt(red[0]);
  }
}

__global__ void k_gather_F(double* const* F, double* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = F[i][0];
}

}  // namespace

cudaError_t pgx::launch_ascent_step(const StepArgs& a, cudaStream_t stream) {
  k_ascent_step<<<a.n, kStepThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

struct pgx_batch {
  pgx_ctx* ctx = nullptr;
  std::vector<pgx_problem*> probs;
  std::vector<int> order;            // problems by decreasing work
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;   // fork + one join per stream
  cudaGraphExec_t eval_exec = nullptr, iter_exec = nullptr;
  std::vector<uint64_t> gens;        // the problems' generations the graphs were captured at
  // device tables
  double** d_u = nullptr;
  double** d_G = nullptr;
  double** d_F = nullptr;
  int* d_len = nullptr;
  AscentState* d_state = nullptr;
  double* d_F_all = nullptr;
  double* d_trace = nullptr;
  int trace_cap = 0;
  StepArgs step_args{};
  double opt_key[4] = {0, 0, 0, 0};  // settings baked into iter_exec
  int64_t units = 0;
  int64_t kernels_eval = 0, kernels_iter = 0;  // kernel nodes in each graph
  // Mixed problems of padded dimension 2 take their slice propagators from
  // one shared launch of the register-resident expm, walking every (problem,
  // member, slice) item of the class.
  struct Small {
    int Dp = 0;
    std::vector<int> idx;  // problems of the class
    pgx::ProbDev* d_p = nullptr;
    pgx::WorkDev* d_w = nullptr;
    long* d_first = nullptr;
  };
  std::vector<Small> small;
  std::vector<char> shared_expm;  // per problem
  cudaStream_t s_small = nullptr;
  cudaEvent_t ev_small = nullptr;
};

static int batch_cuda(pgx_batch* b, cudaError_t e, const char* where) { return ctx_cuda(b->ctx, e, where); }

// Drops both graphs when a problem was changed (pgx_problem_set_*, autotune)
// since they were captured; the next eval / iterate captures them again.
static void drop_stale_graphs(pgx_batch* b) {
  bool stale = b->gens.size() != b->probs.size();
  for (size_t i = 0; !stale && i < b->probs.size(); ++i) stale = b->gens[i] != b->probs[i]->generation;
  if (!stale) return;
  if (b->eval_exec) cudaGraphExecDestroy(b->eval_exec);
  if (b->iter_exec) cudaGraphExecDestroy(b->iter_exec);
  b->eval_exec = b->iter_exec = nullptr;
  b->gens.clear();
  for (const pgx_problem* p : b->probs) b->gens.push_back(p->generation);
}

// Fork the context stream into the batch streams, enqueue every pipeline,
// join; returns the captured graph instantiated.
static int capture(pgx_batch* b, bool with_step, cudaGraphExec_t* out) {
  pgx_ctx* c = b->ctx;
  const int64_t l0 = c->launches;  // the launchers count the kernels they record
  struct Count {
    pgx_batch* b; pgx_ctx* c; int64_t l0; bool step;
    ~Count() {
      const int64_t k = c->launches - l0;
      (step ? b->kernels_iter : b->kernels_eval) = k;
      c->launches = l0;  // recorded, not launched: replays count them
    }
  } count{b, c, l0, with_step};
  cudaStream_t s0 = c->stream;
  cudaGraph_t g = nullptr;
  int st = PGX_OK;
  for (const auto& cl : b->small) {  // the problems' current device descriptors
    const int n = (int)cl.idx.size();
    std::vector<pgx::ProbDev> hp(n);
    std::vector<pgx::WorkDev> hw(n);
    std::vector<long> first(n + 1, 0);
    for (int a = 0; a < n; ++a) {
      const pgx_problem* p = b->probs[cl.idx[a]];
      hp[a] = p->pd;
      hw[a] = p->w;
      hw[a].u = p->d_u;
      // each problem's items start where the shared launch needs them
      const long spw = pgx::expm_small_align(cl.Dp);
      const long n_items = (long)p->desc.n_members * p->desc.n_slices;
      first[a + 1] = first[a] + (n_items + spw - 1) / spw * spw;
    }
    if (!st) st = batch_cuda(b, cudaMemcpy(cl.d_p, hp.data(), sizeof(pgx::ProbDev) * n, cudaMemcpyHostToDevice), "upload");
    if (!st) st = batch_cuda(b, cudaMemcpy(cl.d_w, hw.data(), sizeof(pgx::WorkDev) * n, cudaMemcpyHostToDevice), "upload");
    if (!st) st = batch_cuda(b, cudaMemcpy(cl.d_first, first.data(), sizeof(long) * (n + 1), cudaMemcpyHostToDevice), "upload");
  }
  if (st) return st;
  st = batch_cuda(b, cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal), "begin capture");
  if (st) return st;
  const int K = (int)b->streams.size();
  cudaEventRecord(b->events[0], s0);
  for (int k = 0; k < K; ++k) cudaStreamWaitEvent(b->streams[k], b->events[0], 0);
  if (!b->small.empty()) {  // the shared small-dimension expm launches
    cudaStreamWaitEvent(b->s_small, b->events[0], 0);
    pgx::LaunchInfo li{c->num_sms, b->s_small, &c->launches};
    for (const auto& cl : b->small) {
      const long spw = pgx::expm_small_align(cl.Dp);
      long items = 0;
      for (int i : cl.idx)
        items += ((long)b->probs[i]->desc.n_members * b->probs[i]->desc.n_slices + spw - 1) / spw * spw;
      if (!st)
        st = batch_cuda(b, pgx::launch_expm_small_set(cl.Dp, cl.d_p, cl.d_w, cl.d_first, (int)cl.idx.size(), items, li),
                        "shared expm");
    }
    cudaEventRecord(b->ev_small, b->s_small);
  }
  for (size_t j = 0; j < b->order.size() && !st; ++j) {
    const int i = b->order[j];
    pgx_problem* p = b->probs[i];
    const bool shared = b->shared_expm[i] != 0;
    if (shared) cudaStreamWaitEvent(b->streams[j % K], b->ev_small, 0);
    st = run_pipeline(p, p->d_u, p->d_F, p->d_G, b->streams[j % K], shared);
  }
  for (int k = 0; k < K; ++k) {
    cudaEventRecord(b->events[1 + k], b->streams[k]);
    cudaStreamWaitEvent(s0, b->events[1 + k], 0);
  }
  if (!b->small.empty()) cudaStreamWaitEvent(s0, b->ev_small, 0);
  const int n = (int)b->probs.size();
  if (!st) {
    if (with_step) k_ascent_step<<<n, kStepThreads, 0, s0>>>(b->step_args);
    else k_gather_F<<<(n + 127) / 128, 128, 0, s0>>>(b->d_F, b->d_F_all, n);
    ++c->launches;
  }
  cudaError_t e = cudaStreamEndCapture(s0, &g);
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if ((st = batch_cuda(b, e, "end capture"))) return st;
  st = batch_cuda(b, cudaGraphInstantiate(out, g, 0), "graph instantiate");
  cudaGraphDestroy(g);
  return st;
}

extern "C" int pgx_batch_create(pgx_ctx* c, int32_t n, pgx_problem* const* problems, int32_t n_streams,
                                pgx_batch** out) {
  if (!c || !problems || !out || n < 1) return PGX_ERR_INVALID;
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!problems[i] || problems[i]->ctx != c)
      return ctx_fail(c, PGX_ERR_INVALID, "every problem must belong to the batch's context");
    for (int j = 0; j < i; ++j)
      if (problems[j] == problems[i]) return ctx_fail(c, PGX_ERR_INVALID, "a problem appears twice in a batch");
  }
  cudaSetDevice(c->device);
  auto* b = new pgx_batch();
  b->ctx = c;
  b->probs.assign(problems, problems + n);
  std::vector<double> work(n);
  for (int i = 0; i < n; ++i) {
    const pgx_problem* p = problems[i];
    const double D = p->Dp;
    work[i] = (double)p->desc.n_members * p->desc.n_slices * D * D * D;
    b->units += (int64_t)p->desc.n_members * p->desc.n_slices;
  }
  b->order.resize(n);
  std::iota(b->order.begin(), b->order.end(), 0);
  std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int z) { return work[a] > work[z]; });
  const int K = std::max(1, std::min<int>(n_streams > 0 ? n_streams : 8, n));
  b->streams.resize(K);
  b->events.resize(K + 1);
  int st = PGX_OK;
  for (auto& s : b->streams)
    if (!st) st = batch_cuda(b, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
  for (auto& e : b->events)
    if (!st) st = batch_cuda(b, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
  b->shared_expm.assign(n, 0);
  for (int Dp : {2}) {  // the dimensions whose batches share the expm launch
    pgx_batch::Small cl;
    cl.Dp = Dp;
    for (int i = 0; i < n; ++i)
      if (problems[i]->desc.precision == PGX_PREC_MIXED && problems[i]->Dp == Dp) cl.idx.push_back(i);
    if (cl.idx.empty()) continue;
    const size_t k = cl.idx.size();
    if (!st) st = batch_cuda(b, cudaMalloc((void**)&cl.d_p, sizeof(pgx::ProbDev) * k), "alloc");
    if (!st) st = batch_cuda(b, cudaMalloc((void**)&cl.d_w, sizeof(pgx::WorkDev) * k), "alloc");
    if (!st) st = batch_cuda(b, cudaMalloc((void**)&cl.d_first, sizeof(long) * (k + 1)), "alloc");
    for (int i : cl.idx) b->shared_expm[i] = 1;
    b->small.push_back(cl);
  }
  if (!b->small.empty()) {
    if (!st) st = batch_cuda(b, cudaStreamCreateWithFlags(&b->s_small, cudaStreamNonBlocking), "stream");
    if (!st) st = batch_cuda(b, cudaEventCreateWithFlags(&b->ev_small, cudaEventDisableTiming), "event");
  }
  std::vector<double*> hu(n), hG(n), hF(n);
  std::vector<int> hl(n);
  for (int i = 0; i < n; ++i) {
    hu[i] = problems[i]->d_u;
    hG[i] = problems[i]->d_G;
    hF[i] = problems[i]->d_F;
    hl[i] = problems[i]->desc.n_controls * problems[i]->desc.n_slices;
  }
  const size_t pb = sizeof(double*) * n;
  if (!st) st = batch_cuda(b, cudaMalloc((void**)&b->d_u, pb), "alloc");
  if (!st) st = batch_cuda(b, cudaMalloc((void**)&b->d_G, pb), "alloc");
  if (!st) st = batch_cuda(b, cudaMalloc((void**)&b->d_F, pb), "alloc");
  if (!st) st = batch_cuda(b, cudaMalloc((void**)&b->d_len, sizeof(int) * n), "alloc");
  if (!st) st = batch_cuda(b, cudaMalloc((void**)&b->d_state, sizeof(AscentState) * n), "alloc");
  if (!st) st = batch_cuda(b, cudaMalloc((void**)&b->d_F_all, sizeof(double) * n), "alloc");
  if (!st) st = batch_cuda(b, cudaMemcpy(b->d_u, hu.data(), pb, cudaMemcpyHostToDevice), "upload");
  if (!st) st = batch_cuda(b, cudaMemcpy(b->d_G, hG.data(), pb, cudaMemcpyHostToDevice), "upload");
  if (!st) st = batch_cuda(b, cudaMemcpy(b->d_F, hF.data(), pb, cudaMemcpyHostToDevice), "upload");
  if (!st) st = batch_cuda(b, cudaMemcpy(b->d_len, hl.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "upload");
  if (st) {
    pgx_batch_destroy(b);
    return st;
  }
  *out = b;
  return PGX_OK;
}

extern "C" int pgx_batch_destroy(pgx_batch* b) {
  if (!b) return PGX_ERR_INVALID;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  if (b->eval_exec) cudaGraphExecDestroy(b->eval_exec);
  if (b->iter_exec) cudaGraphExecDestroy(b->iter_exec);
  for (auto s : b->streams)
    if (s) cudaStreamDestroy(s);
  for (auto e : b->events)
    if (e) cudaEventDestroy(e);
  for (auto& cl : b->small) {
    cudaFree(cl.d_p);
    cudaFree(cl.d_w);
    cudaFree(cl.d_first);
  }
  if (b->s_small) cudaStreamDestroy(b->s_small);
  if (b->ev_small) cudaEventDestroy(b->ev_small);
  cudaFree(b->d_u);
  cudaFree(b->d_G);
  cudaFree(b->d_F);
  cudaFree(b->d_len);
  cudaFree(b->d_state);
  cudaFree(b->d_F_all);
  cudaFree(b->d_trace);
  delete b;
  return PGX_OK;
}

extern "C" int pgx_batch_set_controls(pgx_batch* b, int32_t i, const double* u) {
  if (!b || !u || i < 0 || i >= (int)b->probs.size()) return PGX_ERR_INVALID;
  pgx_problem* p = b->probs[i];
  const size_t n = (size_t)p->desc.n_controls * p->desc.n_slices;
  for (size_t k = 0; k < n; ++k)
    if (!std::isfinite(u[k])) return ctx_fail(b->ctx, PGX_ERR_NONFINITE, "controls must be finite");
  cudaSetDevice(b->ctx->device);
  int st = batch_cuda(b, cudaMemcpyAsync(p->d_u, u, n * sizeof(double), cudaMemcpyHostToDevice, b->ctx->stream),
                      "H2D u");
  return st ? st : batch_cuda(b, cudaStreamSynchronize(b->ctx->stream), "sync");
}

extern "C" int pgx_batch_get_controls(pgx_batch* b, int32_t i, double* u, double* G) {
  if (!b || i < 0 || i >= (int)b->probs.size()) return PGX_ERR_INVALID;
  pgx_problem* p = b->probs[i];
  const size_t n = (size_t)p->desc.n_controls * p->desc.n_slices;
  cudaSetDevice(b->ctx->device);
  int st = PGX_OK;
  if (u) st = batch_cuda(b, cudaMemcpyAsync(u, p->d_u, n * sizeof(double), cudaMemcpyDeviceToHost, b->ctx->stream), "D2H");
  if (!st && G)
    st = batch_cuda(b, cudaMemcpyAsync(G, p->d_G, n * sizeof(double), cudaMemcpyDeviceToHost, b->ctx->stream), "D2H");
  return st ? st : batch_cuda(b, cudaStreamSynchronize(b->ctx->stream), "sync");
}

extern "C" int pgx_batch_units(const pgx_batch* b, int64_t* units) {
  if (!b || !units) return PGX_ERR_INVALID;
  *units = b->units;
  return PGX_OK;
}

extern "C" int pgx_batch_eval(pgx_batch* b, double* F) {
  if (!b) return PGX_ERR_INVALID;
  pgx_ctx* c = b->ctx;
  cudaSetDevice(c->device);
  int st = PGX_OK;
  drop_stale_graphs(b);
  if (!b->eval_exec) {
    // one plain pass first: sets kernel attributes outside the capture
    for (pgx_problem* p : b->probs)
      if (!st) st = run_pipeline(p, p->d_u, p->d_F, p->d_G);
    if (!st) st = batch_cuda(b, cudaStreamSynchronize(c->stream), "warm-up");
    if (!st) st = capture(b, false, &b->eval_exec);
    if (st) return st;
  }
  if ((st = batch_cuda(b, cudaGraphLaunch(b->eval_exec, c->stream), "graph launch"))) return st;
  c->launches += b->kernels_eval;
  if (F) {
    if ((st = batch_cuda(b, cudaMemcpyAsync(F, b->d_F_all, sizeof(double) * b->probs.size(), cudaMemcpyDeviceToHost,
                                            c->stream), "D2H F")))
      return st;
    return batch_cuda(b, cudaStreamSynchronize(c->stream), "sync");
  }
  return PGX_OK;
}

extern "C" int pgx_batch_iterate(pgx_batch* b, int32_t n_iter, const pgx_opt_desc* o, double* F_trace) {
  if (!b || !o || n_iter < 0) return PGX_ERR_INVALID;
  if (o->struct_size < sizeof(pgx_opt_desc) || o->step_size <= 0.0 || o->min_step_size <= 0.0 ||
      o->max_step_size < o->step_size)
    return ctx_fail(b->ctx, PGX_ERR_INVALID, "invalid optimiser settings (GRAPE.jl:108-119)");
  pgx_ctx* c = b->ctx;
  cudaSetDevice(c->device);
  const int n = (int)b->probs.size();
  int st = PGX_OK;
  // starting point: F of the initial controls is the first history entry
  if ((st = pgx_batch_eval(b, nullptr))) return st;
  std::vector<AscentState> init(n);
  for (auto& s : init) s = AscentState{o->step_size, 0.0, 0, 0};
  if ((st = batch_cuda(b, cudaMemcpyAsync(b->d_state, init.data(), sizeof(AscentState) * n, cudaMemcpyHostToDevice,
                                          c->stream), "state")))
    return st;
  {
    // F_prev <- F(u0) (the reference's initial history entry)
    std::vector<double> F0(n);
    if ((st = batch_cuda(b, cudaMemcpyAsync(F0.data(), b->d_F_all, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                            c->stream), "D2H")) ||
        (st = batch_cuda(b, cudaStreamSynchronize(c->stream), "sync")))
      return st;
    for (int i = 0; i < n; ++i) init[i].F_prev = F0[i];
    if ((st = batch_cuda(b, cudaMemcpyAsync(b->d_state, init.data(), sizeof(AscentState) * n, cudaMemcpyHostToDevice,
                                            c->stream), "state")))
      return st;
  }
  if (F_trace && b->trace_cap < n_iter) {
    cudaFree(b->d_trace);
    b->d_trace = nullptr;
    if ((st = batch_cuda(b, cudaMalloc((void**)&b->d_trace, sizeof(double) * (size_t)n_iter * n), "trace")))
      return st;
    b->trace_cap = n_iter;
    if (b->iter_exec) { cudaGraphExecDestroy(b->iter_exec); b->iter_exec = nullptr; }
  }
  const double key[4] = {(double)o->adapt_step_size, o->min_step_size, o->max_step_size, (double)(b->d_trace != nullptr)};
  if (b->iter_exec && std::memcmp(key, b->opt_key, sizeof key) != 0) {
    cudaGraphExecDestroy(b->iter_exec);
    b->iter_exec = nullptr;
  }
  if (!b->iter_exec) {
    b->step_args = StepArgs{b->d_u, b->d_G, b->d_F, b->d_len, b->d_state, b->d_trace, b->d_F_all, nullptr, n,
                            b->trace_cap, o->adapt_step_size, o->min_step_size, o->max_step_size};
    if ((st = capture(b, true, &b->iter_exec))) return st;
    std::memcpy(b->opt_key, key, sizeof key);
  }
  for (int it = 0; it < n_iter; ++it) {
    if ((st = batch_cuda(b, cudaGraphLaunch(b->iter_exec, c->stream), "graph launch"))) return st;
    c->launches += b->kernels_iter;
  }
  if (F_trace && n_iter > 0) {
    if ((st = batch_cuda(b, cudaMemcpyAsync(F_trace, b->d_trace, sizeof(double) * (size_t)n_iter * n,
                                            cudaMemcpyDeviceToHost, c->stream), "D2H trace")))
      return st;
  }
  return batch_cuda(b, cudaStreamSynchronize(c->stream), "sync");
}
