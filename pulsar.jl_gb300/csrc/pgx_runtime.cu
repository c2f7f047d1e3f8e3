// Host runtime behind include/pgx.h: contexts, problems, evaluation.
//
// The reference keeps everything in Julia arrays and, on its CUDA path,
// uploads CPU-built propagators every call (GRAPEState.jl:329-330,
// GRAPELindblad.jl:369-410).  Here every input is copied to HBM once at
// pgx_problem_create; an evaluation moves only u (n_c*n_t doubles) in and
// (F, G) out.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "pgx.h"
#include "pgx_internal.h"
#include "pgx_runtime.h"

using pgx::ProbDev;
using pgx::WorkDev;
using cplx = std::complex<double>;

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
int ctx_fail(pgx_ctx* c, int status, const std::string& msg) {
  if (c) c->err = msg;
  return status;
}

int ctx_cuda(pgx_ctx* c, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return PGX_OK;
  const int st = (e == cudaErrorMemoryAllocation) ? PGX_ERR_NOMEM : PGX_ERR_CUDA;
  return ctx_fail(c, st, std::string(where) + ": " + cudaGetErrorString(e));
}

int ctx_alloc(pgx_ctx* c, void** p, size_t bytes, std::vector<void*>& owned, uint64_t& acct) {
  *p = nullptr;
  if (bytes == 0) return PGX_OK;
  if (c->budget && c->used + bytes > c->budget)
    return ctx_fail(c, PGX_ERR_BUDGET, "HBM budget exceeded: " + std::to_string(c->used + bytes) +
                                           " > " + std::to_string(c->budget) + " bytes");
  cudaError_t e = c->pool ? cudaMallocFromPoolAsync(p, bytes, c->pool, c->stream) : cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return ctx_cuda(c, e, "device allocation");
  }
  owned.push_back(*p);
  c->used += bytes;
  acct += bytes;
  return PGX_OK;
}

extern "C" int pgx_abi_version(void) { return PGX_ABI_VERSION; }

extern "C" const char* pgx_status_string(int s) {
  switch (s) {
    case PGX_OK: return "ok";
    case PGX_ERR_INVALID: return "invalid argument";
    case PGX_ERR_DIMS: return "dimension mismatch";
    case PGX_ERR_NOMEM: return "out of device memory";
    case PGX_ERR_BUDGET: return "HBM budget exceeded";
    case PGX_ERR_CUDA: return "CUDA error";
    case PGX_ERR_UNSUPPORTED: return "unsupported";
    case PGX_ERR_TIMEOUT: return "timeout";
    case PGX_ERR_CANCELLED: return "cancelled";
    case PGX_ERR_STATE: return "invalid state";
    case PGX_ERR_NONFINITE: return "non-finite value";
    default: return "unknown status";
  }
}

extern "C" int pgx_ctx_create(int device, uint64_t hbm_budget_bytes, pgx_ctx** out) {
  if (!out) return PGX_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return PGX_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return PGX_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return PGX_ERR_CUDA;
  pgx_ctx* c = new (std::nothrow) pgx_ctx();
  if (!c) return PGX_ERR_NOMEM;
  c->device = device;
  c->budget = hbm_budget_bytes;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaEventCreate(&c->tev0) != cudaSuccess || cudaEventCreate(&c->tev1) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return PGX_ERR_CUDA;
  }
  *out = c;
  return PGX_OK;
}

static void ctx_release(pgx_ctx* c) {
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  cudaEventDestroy(c->ev0);
  cudaEventDestroy(c->ev1);
  cudaEventDestroy(c->tev0);
  cudaEventDestroy(c->tev1);
  for (auto& ev : c->stage_marks)
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int pgx_ctx_destroy(pgx_ctx* c) {
  if (!c || c->closing) return PGX_ERR_INVALID;
  if (c->live > 0) {  // released by the last pgx_problem_destroy
    c->closing = true;
    return PGX_OK;
  }
  ctx_release(c);
  return PGX_OK;
}

extern "C" int pgx_last_error(const pgx_ctx* c, char* buf, size_t len) {
  if (!c || !buf || len == 0) return PGX_ERR_INVALID;
  std::snprintf(buf, len, "%s", c->err.c_str());
  return PGX_OK;
}

extern "C" int pgx_ctx_hbm_used(const pgx_ctx* c, uint64_t* bytes) {
  if (!c || !bytes) return PGX_ERR_INVALID;
  *bytes = c->used;
  return PGX_OK;
}

extern "C" int pgx_ctx_stream(pgx_ctx* c, void** stream) {
  if (!c || !stream) return PGX_ERR_INVALID;
  *stream = (void*)c->stream;
  return PGX_OK;
}

extern "C" int pgx_ctx_timer_start(pgx_ctx* c) {
  if (!c) return PGX_ERR_INVALID;
  return ctx_cuda(c, cudaEventRecord(c->tev0, c->stream), "timer_start");
}

extern "C" int pgx_ctx_timer_stop(pgx_ctx* c, double* ms) {
  if (!c || !ms) return PGX_ERR_INVALID;
  int st = ctx_cuda(c, cudaEventRecord(c->tev1, c->stream), "timer_stop");
  if (st) return st;
  st = ctx_cuda(c, cudaEventSynchronize(c->tev1), "timer_stop sync");
  if (st) return st;
  float f = 0.f;
  st = ctx_cuda(c, cudaEventElapsedTime(&f, c->tev0, c->tev1), "timer elapsed");
  *ms = f;
  return st;
}

extern "C" int pgx_ctx_synchronize(pgx_ctx* c) {
  if (!c) return PGX_ERR_INVALID;
  return ctx_cuda(c, cudaStreamSynchronize(c->stream), "synchronize");
}

extern "C" int pgx_ctx_launch_count(const pgx_ctx* c, int64_t* count) {
  if (!c || !count) return PGX_ERR_INVALID;
  *count = c->launches;
  return PGX_OK;
}

// ---------------------------------------------------------------------------
// problem validation / sizing
// ---------------------------------------------------------------------------
int pad_dim(int d) {
  int p = 2;
  while (p < d) p *= 2;
  return p;
}

bool finite_all(const double* x, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(x[i])) return false;
  return true;
}

double herm_dev(const double* m, int D) {
  double dev = 0.0;
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) {
      const cplx a(m[2 * (r + D * c)], m[2 * (r + D * c) + 1]);
      const cplx b(m[2 * (c + D * r)], -m[2 * (c + D * r) + 1]);
      dev = std::max(dev, std::abs(a - b));
    }
  return dev;
}

// Largest |X[a][b] - conj(X[sigma a][sigma b])| of a D x D superoperator,
// D = d^2, sigma(i + d j) = j + d i: zero for Hermiticity-preserving maps
// (every Lindblad generator).  Returns -1 when D is not a square.
static double lsym_dev(const double* m, int D) {
  int d = 1;
  while (d * d < D) ++d;
  if (d * d != D) return -1.0;
  double dev = 0.0;
  for (int a = 0; a < D; ++a)
    for (int b = 0; b < D; ++b) {
      const int sa = a / d + d * (a % d), sb = b / d + d * (b % d);
      const cplx x(m[2 * (a + D * b)], m[2 * (a + D * b) + 1]);
      const cplx y(m[2 * (sa + D * sb)], -m[2 * (sa + D * sb) + 1]);
      dev = std::max(dev, std::abs(x - y));
    }
  return dev;
}
static bool lsym_all(const double* m, int n, int D) {
  for (int i = 0; i < n; ++i) {
    const double* x = m + 2 * (size_t)i * D * D;
    double mx = 0.0;
    for (size_t k = 0; k < 2 * (size_t)D * D; ++k) mx = std::max(mx, std::abs(x[k]));
    const double dev = lsym_dev(x, D);
    if (dev < 0.0 || dev > 1e-12 * std::max(mx, 1e-300)) return false;
  }
  return true;
}

static double unitarity_dev(const double* m, int D) {
  // ||U'U - I||_F / D  (Targets.jl:135-137)
  double s = 0.0;
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) {
      cplx acc = 0.0;
      for (int k = 0; k < D; ++k)
        acc += std::conj(cplx(m[2 * (k + D * i)], m[2 * (k + D * i) + 1])) *
               cplx(m[2 * (k + D * j)], m[2 * (k + D * j) + 1]);
      if (i == j) acc -= 1.0;
      s += std::norm(acc);
    }
  return std::sqrt(s) / D;
}

static int validate(pgx_ctx* c, const pgx_problem_desc* d) {
  if (!d) return ctx_fail(c, PGX_ERR_INVALID, "descriptor is NULL");
  if (d->struct_size < sizeof(pgx_problem_desc))
    return ctx_fail(c, PGX_ERR_INVALID, "descriptor struct_size too small");
  if (d->dim < 1 || d->dim > pgx::kMaxDim)
    return ctx_fail(c, PGX_ERR_DIMS, "dim must be in [1, 64]");
  if (d->n_controls < 1 || d->n_slices < 1 || d->n_drifts < 1 || d->n_members < 1)
    return ctx_fail(c, PGX_ERR_DIMS, "n_controls, n_slices, n_drifts, n_members must be >= 1");
  if (d->generator != PGX_GEN_HERMITIAN && d->generator != PGX_GEN_LIOUVILLIAN)
    return ctx_fail(c, PGX_ERR_INVALID, "unknown generator kind");
  if (d->target != PGX_TARGET_GATE && d->target != PGX_TARGET_STATES)
    return ctx_fail(c, PGX_ERR_INVALID, "unknown target kind");
  if (d->fidelity < PGX_FID_SQUARE || d->fidelity > PGX_FID_MODULUS)
    return ctx_fail(c, PGX_ERR_INVALID, "unknown fidelity type");
  if (d->generator == PGX_GEN_LIOUVILLIAN && d->fidelity == PGX_FID_MODULUS)
    return ctx_fail(c, PGX_ERR_INVALID,
                    "modulus fidelity is not supported in Liouville space (OptControl.jl:813-816)");
  if (d->grad_mode < PGX_GRAD_REF_GRAPE || d->grad_mode > PGX_GRAD_EXACT)
    return ctx_fail(c, PGX_ERR_INVALID, "unknown gradient mode");
  if (d->precision != PGX_PREC_FP64 && d->precision != PGX_PREC_MIXED)
    return ctx_fail(c, PGX_ERR_INVALID, "unknown precision mode");
  if (!d->dt || !d->drifts || !d->controls)
    return ctx_fail(c, PGX_ERR_INVALID, "dt, drifts and controls are required");
  const size_t DD = (size_t)d->dim * d->dim;
  if (!finite_all(d->dt, d->n_slices)) return ctx_fail(c, PGX_ERR_NONFINITE, "dt not finite");
  for (int k = 0; k < d->n_slices; ++k)
    if (d->dt[k] < 0.0) return ctx_fail(c, PGX_ERR_INVALID, "dt must be non-negative");
  if (!finite_all(d->drifts, 2 * DD * d->n_drifts) || !finite_all(d->controls, 2 * DD * d->n_controls))
    return ctx_fail(c, PGX_ERR_NONFINITE, "generator entries must be finite");
  if (d->offset_op && !finite_all(d->offset_op, 2 * DD))
    return ctx_fail(c, PGX_ERR_NONFINITE, "offset_op entries must be finite");
  if (d->generator == PGX_GEN_HERMITIAN) {
    for (int i = 0; i < d->n_drifts; ++i)
      if (herm_dev(d->drifts + 2 * DD * i, d->dim) > 1e-10)
        return ctx_fail(c, PGX_ERR_INVALID, "drift " + std::to_string(i) + " is not Hermitian");
    for (int j = 0; j < d->n_controls; ++j)
      if (herm_dev(d->controls + 2 * DD * j, d->dim) > 1e-10)
        return ctx_fail(c, PGX_ERR_INVALID, "control " + std::to_string(j) + " is not Hermitian");
    if (d->offset_op && herm_dev(d->offset_op, d->dim) > 1e-10)
      return ctx_fail(c, PGX_ERR_INVALID, "offset_op is not Hermitian");
  }
  if (d->member_drift)
    for (int m = 0; m < d->n_members; ++m)
      if (d->member_drift[m] < 0 || d->member_drift[m] >= d->n_drifts)
        return ctx_fail(c, PGX_ERR_INVALID, "member_drift out of range");
  for (const double* v : {d->member_scale, d->member_offset, d->member_weight})
    if (v && !finite_all(v, d->n_members))
      return ctx_fail(c, PGX_ERR_NONFINITE, "member table entries must be finite");
  if (d->target == PGX_TARGET_GATE) {
    if (d->n_pairs != 0) return ctx_fail(c, PGX_ERR_INVALID, "gate target takes n_pairs = 0");
    if (!d->target_op) return ctx_fail(c, PGX_ERR_INVALID, "gate target needs target_op");
    if (!finite_all(d->target_op, 2 * DD)) return ctx_fail(c, PGX_ERR_NONFINITE, "target not finite");
    if (unitarity_dev(d->target_op, d->dim) > 1e-8)
      return ctx_fail(c, PGX_ERR_INVALID, "target matrix is not unitary (Targets.jl:135-140)");
  } else {
    if (d->n_pairs < 1 || d->n_pairs > pgx_problem::kMaxPairs)
      return ctx_fail(c, PGX_ERR_DIMS, "n_pairs must be in [1, 8]");
    if (!d->states_init || !d->states_target)
      return ctx_fail(c, PGX_ERR_INVALID, "state target needs states_init and states_target");
    const size_t n = 2 * (size_t)d->n_pairs * d->dim;
    if (!finite_all(d->states_init, n) || !finite_all(d->states_target, n) ||
        (d->grad_states_init && !finite_all(d->grad_states_init, n)))
      return ctx_fail(c, PGX_ERR_NONFINITE, "states not finite");
    for (int s = 0; s < d->n_pairs; ++s) {
      double ni = 0, nt = 0;
      for (int i = 0; i < 2 * d->dim; ++i) {
        ni += d->states_init[2 * (size_t)s * d->dim + i] * d->states_init[2 * (size_t)s * d->dim + i];
        nt += d->states_target[2 * (size_t)s * d->dim + i] * d->states_target[2 * (size_t)s * d->dim + i];
      }
      if (std::sqrt(ni) < 2.220446049250313e-16 || std::sqrt(nt) < 2.220446049250313e-16)
        return ctx_fail(c, PGX_ERR_INVALID, "state has zero norm (Targets.jl:85-96)");
    }
  }
  return PGX_OK;
}

struct Sizes {
  size_t U, P, Utot, psi, z, Fm, Gm, slab, u, G, plan;
};

static Sizes sizes_of(const pgx_problem_desc* d, int Dp, int num_sms) {
  Sizes s{};
  const size_t DD = (size_t)Dp * Dp;
  const size_t nm = d->n_members, nt = d->n_slices;
  const size_t np = d->target == PGX_TARGET_STATES ? d->n_pairs : 0;
  s.U = nm * nt * DD * sizeof(double2);
  s.P = d->target == PGX_TARGET_GATE ? nm * nt * DD * sizeof(double2) : 0;  // forward chain, then M_k
  // U_total per member; mixed state targets keep one residual per pair there
  s.Utot = nm * std::max<size_t>(DD, np) * sizeof(double2);
  s.psi = np ? nm * (nt + 1) * np * Dp * sizeof(double2) : 0;
  s.z = nm * std::max<size_t>(np, 1) * sizeof(double2);
  s.Fm = nm * sizeof(double);
  s.Gm = nm * nt * d->n_controls * sizeof(double);
  s.slab = pgx::slab_elems(Dp, num_sms) * sizeof(double2);
  s.plan = (Dp >= 64 && d->precision == PGX_PREC_MIXED) ? nm * nt * sizeof(int) : 0;
  s.u = nt * d->n_controls * sizeof(double);
  s.G = s.u;
  return s;
}

// Blocks of the parallel-in-time mixed gate chain: enough (member, block)
// chains to fill the GPU (about 4 teams of 256 threads per SM from D = 32, 7
// of the 12 64-thread teams an SM holds at D = 16, 16 warp-teams at
// Dp <= 8), but never more than the prefix kernel holds at once, and blocks
// of at least 8 slices; 1 = the sequential chain.
static void pit_shape(const pgx_problem_desc* d, int Dp, int num_sms, int* blocks, int* len) {
  *blocks = 1;
  *len = d->n_slices;
  if (d->precision != PGX_PREC_MIXED || d->target != PGX_TARGET_GATE) return;
  const long target = (long)(Dp <= 8 ? 16 : Dp == 16 ? 7 : 4) * num_sms;
  long b = (target + d->n_members - 1) / d->n_members;
  // never more chains than the prefix kernel holds at once: the rest would
  // run as a second wave of whole chains
  const long cap = pgx::chain_prefix_capacity(Dp, num_sms);
  if (cap > 0) b = std::min<long>(b, std::max<long>(1, cap / d->n_members));
  b = std::min<long>(b, std::max(1, d->n_slices / 8));
  if (b <= 1) return;
  const int L = (int)((d->n_slices + b - 1) / b);
  *len = L;
  *blocks = (d->n_slices + L - 1) / L;
}

static uint64_t footprint(const pgx_problem_desc* d, int num_sms) {
  const int Dp = pad_dim(d->dim);
  const Sizes s = sizes_of(d, Dp, num_sms);
  const size_t DD = (size_t)Dp * Dp * sizeof(double2);
  const size_t consts = DD * (d->n_drifts + d->n_controls + 3) +
                        2 * (size_t)std::max(d->n_pairs, 0) * Dp * sizeof(double2) * 2 +
                        (size_t)d->n_members * (sizeof(int) + 3 * sizeof(double)) +
                        (size_t)d->n_slices * sizeof(double);
  int pit_b, pit_l;
  pit_shape(d, Dp, num_sms, &pit_b, &pit_l);
  const size_t pit = pit_b > 1 ? (size_t)d->n_members * Dp * Dp *
                                     (pit_b * (sizeof(float4) + 2 * sizeof(float2)) + (size_t)d->n_slices * sizeof(float2))
                               : 0;
  // mixed: df and FP32 copies of the generator constants, df scalars and
  // controls
  const size_t mixed = pit + (d->precision == PGX_PREC_MIXED
                           ? (DD + DD / 2) * (d->n_drifts + d->n_controls + 1) +
                                 sizeof(float2) * ((size_t)d->n_slices + 2 * (size_t)d->n_members) + s.u
                           : 0);
  return s.U + s.P + s.Utot + 2 * s.psi + 2 * s.z + s.Fm + s.Gm + s.slab + s.plan + s.u + s.G +
         3 * sizeof(double) + consts + mixed;
}

int validate_desc(pgx_ctx* c, const pgx_problem_desc* d) { return validate(c, d); }
uint64_t problem_footprint(const pgx_problem_desc* d, int num_sms) { return footprint(d, num_sms); }

extern "C" int pgx_problem_footprint(const pgx_problem_desc* d, uint64_t* bytes) {
  if (!d || !bytes) return PGX_ERR_INVALID;
  if (d->struct_size < sizeof(pgx_problem_desc) || d->dim < 1 || d->dim > pgx::kMaxDim ||
      d->n_controls < 1 || d->n_slices < 1 || d->n_drifts < 1 || d->n_members < 1)
    return PGX_ERR_DIMS;
  *bytes = footprint(d, 152);
  return PGX_OK;
}

// ---------------------------------------------------------------------------
// problem create / destroy
// ---------------------------------------------------------------------------
std::vector<double> pad_mats(const double* src, int n, int D, int Dp) {
  std::vector<double> out((size_t)n * Dp * Dp * 2, 0.0);
  if (!src) return out;
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < D; ++c)
      for (int r = 0; r < D; ++r) {
        const size_t si = 2 * ((size_t)i * D * D + r + (size_t)D * c);
        const size_t di = 2 * ((size_t)i * Dp * Dp + r + (size_t)Dp * c);
        out[di] = src[si];
        out[di + 1] = src[si + 1];
      }
  return out;
}

// Interleaved complex doubles -> their FP32 roundings (the leading halves of
// the df pairs below).
static std::vector<float> to_f32(const std::vector<double>& z) {
  std::vector<float> out(z.size());
  for (size_t i = 0; i < z.size(); ++i) out[i] = (float)z[i];
  return out;
}

// Interleaved complex doubles -> df pairs {re.hi, im.hi, re.lo, im.lo}.
static std::vector<float> to_df_pairs(const std::vector<double>& z) {
  std::vector<float> out(2 * z.size());
  for (size_t i = 0; i + 1 < z.size(); i += 2) {
    const float rh = (float)z[i], ih = (float)z[i + 1];
    out[2 * i] = rh;
    out[2 * i + 1] = ih;
    out[2 * i + 2] = (float)(z[i] - (double)rh);
    out[2 * i + 3] = (float)(z[i + 1] - (double)ih);
  }
  return out;
}

// Doubles -> df pairs {hi, lo}.
static std::vector<float> to_df_scalars(const std::vector<double>& x) {
  std::vector<float> out(2 * x.size());
  for (size_t i = 0; i < x.size(); ++i) {
    out[2 * i] = (float)x[i];
    out[2 * i + 1] = (float)(x[i] - (double)out[2 * i]);
  }
  return out;
}

static std::vector<double> pad_vecs(const double* src, int n, int D, int Dp) {
  std::vector<double> out((size_t)n * Dp * 2, 0.0);
  if (!src) return out;
  for (int i = 0; i < n; ++i)
    for (int r = 0; r < D; ++r) {
      out[2 * ((size_t)i * Dp + r)] = src[2 * ((size_t)i * D + r)];
      out[2 * ((size_t)i * Dp + r) + 1] = src[2 * ((size_t)i * D + r) + 1];
    }
  return out;
}

template <class T>
static int upload(pgx_problem* p, T** dptr, const std::vector<T>& host) {
  int st = ctx_alloc(p->ctx, (void**)dptr, host.size() * sizeof(T), p->owned, p->bytes);
  if (st) return st;
  if (host.empty()) return PGX_OK;
  // pageable source: the call returns once `host` has been staged
  return ctx_cuda(p->ctx, cudaMemcpyAsync(*dptr, host.data(), host.size() * sizeof(T),
                                          cudaMemcpyHostToDevice, p->ctx->stream), "upload");
}

// Tuned plans (team sizes of the tunable kernels), process-wide: pgx_autotune
// records its choice under (device, padded dimension, n_controls, generator,
// target, precision, grad_mode) and every problem created later with the same
// key -- on any context, the server's private one included -- starts with it.
// Team sizes never change results (the variants are bit-identical), so a plan
// only moves time.
namespace {
using PlanKey = std::tuple<int, int, int, int, int, int, int>;
std::mutex g_plan_mu;
std::map<PlanKey, std::pair<int, int>> g_plans;

PlanKey plan_key(int device, const pgx_problem_desc* d) {
  return PlanKey{device, pad_dim(d->dim), d->n_controls, d->generator, d->target, d->precision, d->grad_mode};
}
}  // namespace

extern "C" int pgx_plan_lookup(int device, const pgx_problem_desc* d, int32_t* team_expm, int32_t* team_grad) {
  if (!d || !team_expm || !team_grad || d->dim < 1 || d->dim > pgx::kMaxDim) return PGX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(g_plan_mu);
  const auto it = g_plans.find(plan_key(device, d));
  if (it == g_plans.end()) {
    *team_expm = *team_grad = 0;
    return PGX_ERR_STATE;
  }
  *team_expm = it->second.first;
  *team_grad = it->second.second;
  return PGX_OK;
}

extern "C" int pgx_plan_clear(void) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  g_plans.clear();
  return PGX_OK;
}

extern "C" int pgx_problem_create(pgx_ctx* c, const pgx_problem_desc* d, pgx_problem** out) {
  if (!c || !out) return PGX_ERR_INVALID;
  *out = nullptr;
  int st = validate(c, d);
  if (st) return st;
  cudaSetDevice(c->device);
  if (c->budget && c->used + footprint(d, c->num_sms) > c->budget)
    return ctx_fail(c, PGX_ERR_BUDGET, "problem footprint exceeds the context HBM budget");
  pgx_problem* p = new (std::nothrow) pgx_problem();
  if (!p) return ctx_fail(c, PGX_ERR_NOMEM, "host allocation failed");
  p->ctx = c;
  ++c->live;  // every later failure path releases p through pgx_problem_destroy
  p->desc = *d;
  const int D = d->dim, Dp = pad_dim(D);
  p->Dp = Dp;
  const int nm = d->n_members, nt = d->n_slices, nc = d->n_controls;
  const int np = d->target == PGX_TARGET_STATES ? d->n_pairs : 0;

  // ---- constant inputs, padded ----
  std::vector<double> drifts = pad_mats(d->drifts, d->n_drifts, D, Dp);
  std::vector<double> ctrls = pad_mats(d->controls, nc, D, Dp);
  std::vector<double> offs = pad_mats(d->offset_op, 1, D, Dp);
  std::vector<double> tgt = pad_mats(d->target_op, 1, D, Dp);
  std::vector<double> dt(d->dt, d->dt + nt);
  std::vector<int> mdrift(nm, 0);
  std::vector<double> mscale(nm, 1.0), moff(nm, 0.0), mw(nm, 1.0 / ((double)nm * std::max(np, 1)));
  for (int m = 0; m < nm; ++m) {
    if (d->member_drift) mdrift[m] = d->member_drift[m];
    if (d->member_scale) mscale[m] = d->member_scale[m];
    if (d->member_offset) moff[m] = d->member_offset[m];
    if (d->member_weight) mw[m] = d->member_weight[m];
  }
  p->h_weight = mw;
  std::vector<double> psi_i = pad_vecs(d->states_init, np, D, Dp);
  std::vector<double> psi_t = pad_vecs(d->states_target, np, D, Dp);
  std::vector<double> psi_g = pad_vecs(d->grad_states_init ? d->grad_states_init : d->states_init, np, D, Dp);
  p->split_grad_states = np > 0 && d->grad_states_init &&
                         std::memcmp(d->grad_states_init, d->states_init,
                                     sizeof(double) * 2 * (size_t)np * D) != 0;

  double *g_dr, *g_ct, *g_of, *g_tg, *g_dt, *g_ms, *g_mo, *g_mw, *g_pi, *g_pt, *g_pg;
  int* g_md;
  if ((st = upload(p, &g_dr, drifts)) || (st = upload(p, &g_ct, ctrls)) || (st = upload(p, &g_of, offs)) ||
      (st = upload(p, &g_tg, tgt)) || (st = upload(p, &g_dt, dt)) || (st = upload(p, &g_md, mdrift)) ||
      (st = upload(p, &g_ms, mscale)) || (st = upload(p, &g_mo, moff)) || (st = upload(p, &g_mw, mw)) ||
      (st = upload(p, &g_pi, psi_i)) || (st = upload(p, &g_pt, psi_t)) || (st = upload(p, &g_pg, psi_g))) {
    pgx_problem_destroy(p);
    return st;
  }
  ProbDev& pd = p->pd;
  if (d->precision == PGX_PREC_MIXED) {
    // df copies of the generator constants for the mixed kernels
    float *f_dr, *f_ct, *f_of;
    if ((st = upload(p, &f_dr, to_df_pairs(drifts))) || (st = upload(p, &f_ct, to_df_pairs(ctrls))) ||
        (st = upload(p, &f_of, to_df_pairs(offs)))) {
      pgx_problem_destroy(p);
      return st;
    }
    pd.drifts_df = (const float4*)f_dr;
    pd.ctrls_df = (const float4*)f_ct;
    pd.offset_df = (const float4*)f_of;
    // FP32 copies for the FP32 stages (half the bytes of the df copies)
    float *h_dr, *h_ct, *h_of;
    if ((st = upload(p, &h_dr, to_f32(drifts))) || (st = upload(p, &h_ct, to_f32(ctrls))) ||
        (st = upload(p, &h_of, to_f32(offs)))) {
      pgx_problem_destroy(p);
      return st;
    }
    pd.drifts_f32 = (const float2*)h_dr;
    pd.ctrls_f32 = (const float2*)h_ct;
    pd.offset_f32 = (const float2*)h_of;
    float *f_dt, *f_ms, *f_mo;
    if ((st = upload(p, &f_dt, to_df_scalars(dt))) || (st = upload(p, &f_ms, to_df_scalars(mscale))) ||
        (st = upload(p, &f_mo, to_df_scalars(moff)))) {
      pgx_problem_destroy(p);
      return st;
    }
    pd.dt_df = (const float2*)f_dt;
    pd.m_scale_df = (const float2*)f_ms;
    pd.m_offset_df = (const float2*)f_mo;
  }
  pd.D = D;
  pd.Dp = Dp;
  pd.n_c = nc;
  pd.n_t = nt;
  pd.n_members = nm;
  pd.n_pairs = np;
  pd.gen = d->generator;
  // Liouvillians whose every generator piece preserves Hermiticity, at a
  // dimension without padding: the mixed expm and forward chain keep half
  // of each product (D = 64)
  p->lsym_fixed = d->generator == PGX_GEN_LIOUVILLIAN && Dp == D && lsym_all(d->controls, d->n_controls, D) &&
                  (!d->offset_op || lsym_all(d->offset_op, 1, D));
  p->lsym_drift = p->lsym_fixed && lsym_all(d->drifts, d->n_drifts, D);
  pd.lsym = (p->lsym_fixed && p->lsym_drift) ? 1 : 0;
  pd.target = d->target;
  pd.fid = d->fidelity;
  pd.grad_mode = d->grad_mode;
  pd.dt = g_dt;
  pd.drifts = (const double2*)g_dr;
  pd.ctrls = (const double2*)g_ct;
  pd.offset_op = (const double2*)g_of;
  pd.m_drift = g_md;
  pd.m_scale = g_ms;
  pd.m_offset = g_mo;
  pd.m_weight = g_mw;
  pd.target_op = (const double2*)g_tg;
  pd.psi_init = (const double2*)g_pi;
  pd.psi_targ = (const double2*)g_pt;
  p->pd_grad = pd;
  p->pd_grad.psi_init = (const double2*)g_pg;

  // ---- workspace ----
  const Sizes s = sizes_of(d, Dp, c->num_sms);
  WorkDev& w = p->w;
  void* ptr;
  auto A = [&](size_t bytes) -> void* {
    if (st) return nullptr;
    st = ctx_alloc(c, &ptr, bytes, p->owned, p->bytes);
    return st ? nullptr : ptr;
  };
  w.U = (double2*)A(s.U);
  w.P = (double2*)A(s.P);
  w.Utot = (double2*)A(s.Utot);
  w.psi = (double2*)A(s.psi);
  w.lam = (double2*)A(s.psi);
  w.z = (double2*)A(s.z);
  w.kap = (double2*)A(s.z);
  w.Fm = (double*)A(s.Fm);
  w.Gm = (double*)A(s.Gm);
  w.slab = (double2*)A(s.slab);
  w.slab_teams = pgx::slab_team_count(Dp, c->num_sms);
  w.expm_plan = (int*)A(s.plan);
  p->d_u = (double*)A(s.u);
  p->d_G = (double*)A(s.G);
  p->d_F = (double*)A(3 * sizeof(double));  // objective, gradient-pass scratch, residual bits
  if (d->precision == PGX_PREC_MIXED) w.u_df = (float2*)A(s.u);
  p->d_pen = (pgx_penalty*)A(sizeof(pgx_penalty) * PGX_MAX_PENALTIES);
  pit_shape(d, Dp, c->num_sms, &w.pit_blocks, &w.pit_len);
  if (w.pit_blocks > 1) {
    const size_t blk = (size_t)d->n_members * w.pit_blocks * Dp * Dp;
    w.pit_tot = (float4*)A(blk * sizeof(float4));
    w.pit_pre = (float2*)A(blk * sizeof(float2));
    w.pit_lam = (float2*)A(blk * sizeof(float2));
    w.pit_r = (float2*)A((size_t)d->n_members * d->n_slices * Dp * Dp * sizeof(float2));
  }
  if (st) {
    pgx_problem_destroy(p);
    return st;
  }
  if ((st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "upload sync"))) {
    pgx_problem_destroy(p);
    return st;
  }
  if (d->precision == PGX_PREC_MIXED && d->target == PGX_TARGET_GATE && p->w.pit_blocks > 1) {
    // second stream for the backward chain's in-block suffixes (run_pipeline)
    if (cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      pgx_problem_destroy(p);
      return ctx_fail(c, PGX_ERR_CUDA, "stream creation failed");
    }
  }
  if (d->precision == PGX_PREC_MIXED) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    const auto it = g_plans.find(plan_key(c->device, d));
    if (it != g_plans.end()) {
      p->team[pgx::kTuneExpmMx] = it->second.first;
      p->team[pgx::kTuneGradMx] = it->second.second;
    }
  }
  *out = p;
  return PGX_OK;
}

// Pinned staging buffer of the host-facing calls (u | G | F), made on first use.
static int stage_buffer(pgx_problem* p) {
  if (p->h_stage) return PGX_OK;
  const size_t n = (size_t)p->desc.n_controls * p->desc.n_slices;
  if (cudaMallocHost((void**)&p->h_stage, (2 * n + 2) * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    p->h_stage = nullptr;
    return ctx_fail(p->ctx, PGX_ERR_NOMEM, "pinned staging allocation failed");
  }
  return PGX_OK;
}

extern "C" int pgx_problem_destroy(pgx_problem* p) {
  if (!p) return PGX_ERR_INVALID;
  cudaSetDevice(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  for (void* q : p->owned) {
    if (p->ctx->pool) cudaFreeAsync(q, p->ctx->stream);
    else cudaFree(q);
  }
  if (p->h_stage) cudaFreeHost(p->h_stage);
  if (p->side) {
    cudaStreamSynchronize(p->side);
    cudaStreamDestroy(p->side);
  }
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->ev_join) cudaEventDestroy(p->ev_join);
  pgx_ctx* c = p->ctx;
  c->used -= p->bytes;
  delete p;
  if (--c->live == 0 && c->closing) ctx_release(c);
  return PGX_OK;
}

// ---------------------------------------------------------------------------
// evaluation
// ---------------------------------------------------------------------------
// Stage marks: event i is recorded before stage i (i = 0..4) and event 5 after
// the last stage, so stage i lasts ev[i] -> ev[i+1].
struct Marks {
  pgx_ctx* c;
  std::vector<cudaEvent_t> ev;
  explicit Marks(pgx_ctx* ctx, bool enabled = true) : c(ctx) {
    if (!c->stage_timing || !enabled) return;
    for (int i = 0; i <= PGX_N_STAGES; ++i) {
      cudaEvent_t e;
      if (!c->ev_pool.empty()) { e = c->ev_pool.back(); c->ev_pool.pop_back(); }
      else if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); ev.clear(); return; }
      ev.push_back(e);
    }
  }
  void mark(int i) {
    if (!ev.empty()) cudaEventRecord(ev[i], c->stream);
  }
  void commit() {
    if (!ev.empty()) c->stage_marks.push_back(ev);
  }
};

// F -= sum weight P(u), G -= sum weight dP/du after the member reduction.
static int apply_penalties(pgx_problem* p, const WorkDev& w, bool want_grad, const pgx::LaunchInfo& li) {
  if (p->n_pen == 0) return PGX_OK;
  return ctx_cuda(p->ctx, pgx::launch_penalties(p->d_pen, p->n_pen, w.u, p->pd.dt, p->desc.n_controls,
                                                p->desc.n_slices, w.F, want_grad ? w.G : nullptr, li),
                  "penalties");
}

int run_pipeline(pgx_problem* p, const double* d_u, double* d_F, double* d_G, cudaStream_t stream, bool skip_expm) {
  pgx_ctx* c = p->ctx;
  pgx::LaunchInfo li = p->launch_info();
  if (stream) li.stream = stream;  // batches enqueue on their own (captured) streams
  WorkDev w = p->w;
  w.u = d_u;
  w.G = d_G ? d_G : p->d_G;
  w.F = d_F;
  const bool want_grad = d_G != nullptr;
  Marks mk(c, stream == nullptr);
  int st;
  if (p->desc.precision == PGX_PREC_MIXED) {
    mk.mark(PGX_STAGE_EXPM);
    if ((st = ctx_cuda(c, pgx::launch_prep_mx(p->pd, w, li), "prep_mx"))) return st;
    if (!skip_expm && (st = ctx_cuda(c, pgx::launch_expm_mx(p->pd, w, li), "expm_mx"))) return st;
    mk.mark(PGX_STAGE_CHAIN_FWD);
    if (want_grad && p->split_grad_states) {
      // F from states_init; gradient from grad_states_init (Gradients.jl:153-157)
      if ((st = ctx_cuda(c, pgx::launch_chain_fwd_mx(p->pd, w, li, false), "chain_fwd_mx(F)")) ||
          (st = ctx_cuda(c, pgx::launch_reduce(p->pd, w, li, false), "reduce(F)")))
        return st;
      WorkDev w2 = w;
      w2.F = p->d_F + 1;  // scratch: the gradient pass's own objective
      if ((st = ctx_cuda(c, pgx::launch_chain_fwd_mx(p->pd_grad, w2, li, true), "chain_fwd_mx"))) return st;
      mk.mark(PGX_STAGE_CHAIN_BWD);
      if ((st = ctx_cuda(c, pgx::launch_chain_bwd_mx(p->pd_grad, w2, li), "chain_bwd_mx"))) return st;
      mk.mark(PGX_STAGE_GRAD);
      if ((st = ctx_cuda(c, pgx::launch_grad_mx(p->pd_grad, w2, li), "grad_mx"))) return st;
      mk.mark(PGX_STAGE_REDUCE);
      st = ctx_cuda(c, pgx::launch_reduce(p->pd_grad, w2, li, true), "reduce");
      if (!st) st = apply_penalties(p, w, true, li);
      mk.mark(PGX_N_STAGES);
      mk.commit();
      return st;
    }
    // Gate targets in parallel in time: the backward chain's in-block
    // suffixes need only U, so they run on the side stream beside the
    // forward chain (FP32 latency-bound work beside issue-bound df work).
    const bool fork = want_grad && p->side != nullptr;
    if (fork) {
      pgx::LaunchInfo ls = li;
      ls.stream = p->side;
      if ((st = ctx_cuda(c, cudaEventRecord(p->ev_fork, li.stream), "fork")) ||
          (st = ctx_cuda(c, cudaStreamWaitEvent(p->side, p->ev_fork, 0), "fork")) ||
          (st = ctx_cuda(c, pgx::launch_chain_bwd_local_mx(p->pd, w, ls), "chain_bwd_local_mx")) ||
          (st = ctx_cuda(c, cudaEventRecord(p->ev_join, p->side), "join")))
        return st;
    }
    if ((st = ctx_cuda(c, pgx::launch_chain_fwd_mx(p->pd, w, li, want_grad), "chain_fwd_mx"))) return st;
    if ((st = ctx_cuda(c, pgx::launch_refine_mx(p->pd, w, li), "refine_mx"))) return st;
    mk.mark(PGX_STAGE_CHAIN_BWD);
    if (fork && (st = ctx_cuda(c, cudaStreamWaitEvent(li.stream, p->ev_join, 0), "join"))) return st;
    if (want_grad && (st = ctx_cuda(c, pgx::launch_chain_bwd_mx(p->pd, w, li, fork), "chain_bwd_mx"))) return st;
    mk.mark(PGX_STAGE_GRAD);
    if (want_grad && (st = ctx_cuda(c, pgx::launch_grad_mx(p->pd, w, li), "grad_mx"))) return st;
    mk.mark(PGX_STAGE_REDUCE);
    st = ctx_cuda(c, pgx::launch_reduce(p->pd, w, li, want_grad), "reduce");
    if (!st) st = apply_penalties(p, w, want_grad, li);
    mk.mark(PGX_N_STAGES);
    mk.commit();
    return st;
  }
  mk.mark(PGX_STAGE_EXPM);
  if ((st = ctx_cuda(c, pgx::launch_expm(p->pd, w, li), "expm"))) return st;
  mk.mark(PGX_STAGE_CHAIN_FWD);
  if (want_grad && p->split_grad_states && p->pd.n_ck == 0) {
    // F from states_init; gradient from grad_states_init (Gradients.jl:153-157).
    if ((st = ctx_cuda(c, pgx::launch_chain_fwd(p->pd, w, li, false), "chain_fwd(F)"))) return st;
    if ((st = ctx_cuda(c, pgx::launch_reduce(p->pd, w, li, false), "reduce(F)"))) return st;
    WorkDev w2 = w;
    w2.F = p->d_F + 1;  // scratch: the gradient pass's own objective
    if ((st = ctx_cuda(c, pgx::launch_chain_fwd(p->pd_grad, w2, li, true), "chain_fwd"))) return st;
    mk.mark(PGX_STAGE_CHAIN_BWD);
    if ((st = ctx_cuda(c, pgx::launch_chain_bwd(p->pd_grad, w2, li), "chain_bwd"))) return st;
    mk.mark(PGX_STAGE_GRAD);
    if ((st = ctx_cuda(c, pgx::launch_grad(p->pd_grad, w2, li), "grad"))) return st;
    mk.mark(PGX_STAGE_REDUCE);
    st = ctx_cuda(c, pgx::launch_reduce(p->pd_grad, w2, li, true), "reduce");
    if (!st) st = apply_penalties(p, w, true, li);
    mk.mark(PGX_N_STAGES);
    mk.commit();
    return st;
  }
  if ((st = ctx_cuda(c, pgx::launch_chain_fwd(p->pd, w, li, want_grad), "chain_fwd"))) return st;
  mk.mark(PGX_STAGE_CHAIN_BWD);
  if (want_grad && (st = ctx_cuda(c, pgx::launch_chain_bwd(p->pd, w, li), "chain_bwd"))) return st;
  mk.mark(PGX_STAGE_GRAD);
  if (want_grad && (st = ctx_cuda(c, pgx::launch_grad(p->pd, w, li), "grad"))) return st;
  mk.mark(PGX_STAGE_REDUCE);
  st = ctx_cuda(c, pgx::launch_reduce(p->pd, w, li, want_grad), "reduce");
  if (!st) st = apply_penalties(p, w, want_grad, li);
  mk.mark(PGX_N_STAGES);
  mk.commit();
  return st;
}

extern "C" int pgx_autotune(pgx_problem* p, const double* u, int32_t reps, char* report, size_t len) {
  if (!p || !u) return PGX_ERR_INVALID;
  pgx_ctx* c = p->ctx;
  if (report && len) report[0] = '\0';
  if (reps < 1) reps = 1;
  const size_t n = (size_t)p->desc.n_controls * p->desc.n_slices;
  if (!finite_all(u, n)) return ctx_fail(c, PGX_ERR_NONFINITE, "controls must be finite");
  if (p->desc.precision != PGX_PREC_MIXED) {
    if (report && len) std::snprintf(report, len, "FP64 path: no tunable kernels");
    return PGX_OK;
  }
  cudaSetDevice(c->device);
  if (const int sb = stage_buffer(p)) return sb;
  std::memcpy(p->h_stage, u, n * sizeof(double));
  int st = ctx_cuda(c, cudaMemcpyAsync(p->d_u, p->h_stage, n * sizeof(double), cudaMemcpyHostToDevice,
                                       c->stream), "H2D u");
  if (st || (st = run_pipeline(p, p->d_u, p->d_F, p->d_G))) return st;
  WorkDev w = p->w;
  w.u = p->d_u;
  w.G = p->d_G;
  w.F = p->d_F;
  std::string rep;
  const char* names[pgx::kNumTunable] = {"expm_mx", "grad_mx"};
  for (int kern = 0; kern < pgx::kNumTunable; ++kern) {
    if (kern == pgx::kTuneGradMx && p->desc.grad_mode != PGX_GRAD_EXACT) continue;
    int vs[4];
    const int nv = pgx::mixed_variants(p->pd, kern, vs);
    double best_ms = 1e300;
    int best = vs[0];
    rep += std::string(rep.empty() ? "" : " | ") + names[kern] + "<" + std::to_string(p->Dp) + ">:";
    if (nv == 1) {  // nothing to choose (and the tensor-core gradient consumes its input in place)
      rep += " T=" + std::to_string(best) + " (single candidate) -> T=" + std::to_string(best);
      p->team[kern] = best;
      ++p->generation;
      continue;
    }
    for (int i = 0; i < nv; ++i) {
      pgx::LaunchInfo li = p->launch_info();
      li.team[kern] = vs[i];
      auto launch = [&]() {
        return kern == pgx::kTuneExpmMx ? pgx::launch_expm_mx(p->pd, w, li) : pgx::launch_grad_mx(p->pd, w, li);
      };
      if ((st = ctx_cuda(c, launch(), "autotune warm-up"))) return st;
      cudaEventRecord(c->tev0, c->stream);
      for (int r = 0; r < reps; ++r)
        if ((st = ctx_cuda(c, launch(), "autotune"))) return st;
      cudaEventRecord(c->tev1, c->stream);
      if ((st = ctx_cuda(c, cudaEventSynchronize(c->tev1), "autotune sync"))) return st;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->tev0, c->tev1);
      const double per = ms / reps;
      char buf[48];
      std::snprintf(buf, sizeof buf, " T=%d %.3fms", vs[i], per);
      rep += buf;
      if (per < best_ms) { best_ms = per; best = vs[i]; }
    }
    p->team[kern] = best;
    ++p->generation;
    rep += " -> T=" + std::to_string(best);
  }
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    g_plans[plan_key(c->device, &p->desc)] = {p->team[pgx::kTuneExpmMx], p->team[pgx::kTuneGradMx]};
  }
  if (report && len) std::snprintf(report, len, "%s", rep.c_str());
  return run_pipeline(p, p->d_u, p->d_F, p->d_G);
}

extern "C" int pgx_problem_set_team(pgx_problem* p, int32_t kernel, int32_t team) {
  if (!p || kernel < 0 || kernel >= pgx::kNumTunable) return PGX_ERR_INVALID;
  if (team != 0) {
    int vs[4];
    const int nv = pgx::mixed_admitted(p->pd, kernel, vs);
    if (std::find(vs, vs + nv, team) == vs + nv)
      return ctx_fail(p->ctx, PGX_ERR_INVALID, "team size not admitted at this dimension");
  }
  p->team[kernel] = team;
  ++p->generation;
  return PGX_OK;
}

extern "C" int pgx_problem_get_team(const pgx_problem* p, int32_t kernel, int32_t* team) {
  if (!p || !team || kernel < 0 || kernel >= pgx::kNumTunable) return PGX_ERR_INVALID;
  *team = p->team[kernel] ? p->team[kernel] : pgx::mixed_default_team(p->pd, kernel);
  return PGX_OK;
}

extern "C" int pgx_ctx_set_stage_timing(pgx_ctx* c, int enabled) {
  if (!c) return PGX_ERR_INVALID;
  c->stage_timing = enabled != 0;
  return PGX_OK;
}

extern "C" int pgx_ctx_stage_times(pgx_ctx* c, double* ms, int32_t* count) {
  if (!c || !ms || !count) return PGX_ERR_INVALID;
  for (int i = 0; i < PGX_N_STAGES; ++i) ms[i] = 0.0;
  int st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "stage sync");
  if (st) return st;
  for (auto& ev : c->stage_marks) {
    for (int i = 0; i < PGX_N_STAGES; ++i) {
      float f = 0.f;
      if (cudaEventElapsedTime(&f, ev[i], ev[i + 1]) == cudaSuccess) ms[i] += f;
      else cudaGetLastError();
    }
    for (cudaEvent_t e : ev) c->ev_pool.push_back(e);
  }
  *count = (int32_t)c->stage_marks.size();
  c->stage_marks.clear();
  return PGX_OK;
}

extern "C" int pgx_ctx_measure_peak(pgx_ctx* c, int32_t pipe, double* gflops) {
  if (!c || !gflops || (pipe != PGX_PIPE_FP64 && pipe != PGX_PIPE_FP32)) return PGX_ERR_INVALID;
  cudaSetDevice(c->device);
  double* sink = nullptr;
  int st = ctx_cuda(c, cudaMallocAsync((void**)&sink, sizeof(double) * 64, c->stream), "alloc");
  if (st) return st;
  pgx::LaunchInfo li{c->num_sms, c->stream, &c->launches};
  double best = 0.0;
  for (int rep = 0; rep < 4 && !st; ++rep) {
    double flops = 0.0;
    cudaEventRecord(c->tev0, c->stream);
    st = ctx_cuda(c, pipe == PGX_PIPE_FP64 ? pgx::launch_fp64_peak(sink, li, &flops)
                                           : pgx::launch_fp32_peak((float*)sink, li, &flops), "peak");
    cudaEventRecord(c->tev1, c->stream);
    if (!st) st = ctx_cuda(c, cudaEventSynchronize(c->tev1), "sync");
    float ms = 0.f;
    if (!st) cudaEventElapsedTime(&ms, c->tev0, c->tev1);
    if (rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e9);
  }
  cudaFreeAsync(sink, c->stream);
  cudaStreamSynchronize(c->stream);
  *gflops = best;
  return st;
}

// The oracle-free residual of the evaluation just run (pgx_eval_stats):
// from U_total for gate targets, from the stored states for state targets
// when the evaluation computed G (F-only state evaluations store none).
static int eval_residual(pgx_problem* p, bool had_grad, double* out, int32_t* kind_out) {
  pgx_ctx* c = p->ctx;
  const pgx_problem_desc& d = p->desc;
  const bool liou = d.generator == PGX_GEN_LIOUVILLIAN;
  int kind = PGX_RESID_NONE, N = 0;
  if (liou) {
    N = (int)std::lround(std::sqrt((double)d.dim));
    if (N * N != d.dim) N = 0;  // not a vectorised density matrix: no trace to check
  }
  if (d.target == PGX_TARGET_GATE)
    kind = liou ? (N ? PGX_RESID_TRACE : PGX_RESID_NONE) : PGX_RESID_UNITARITY;
  else if (had_grad || p->pd.n_ck > 0 || d.precision == PGX_PREC_MIXED)
    // FP64 states are stored when G is computed (tracking: always); the mixed
    // state chain records each pair's residual on every evaluation
    kind = liou ? (N ? PGX_RESID_STATE_TRACE : PGX_RESID_NONE) : PGX_RESID_NORM;
  *kind_out = kind;
  *out = 0.0;
  if (kind == PGX_RESID_NONE) return PGX_OK;
  const int dev_kind = (d.target == PGX_TARGET_STATES && d.precision == PGX_PREC_MIXED) ? pgx::kResidPairs : kind;
  unsigned long long* bits = reinterpret_cast<unsigned long long*>(p->d_F + 2);
  pgx::LaunchInfo li = p->launch_info();
  double* h = p->h_stage + 2 * (size_t)d.n_controls * d.n_slices + 1;
  int st;
  if ((st = ctx_cuda(c, cudaMemsetAsync(bits, 0, sizeof(double), c->stream), "memset")) ||
      (st = ctx_cuda(c, pgx::launch_residual(p->split_grad_states && had_grad ? p->pd_grad : p->pd, p->w, dev_kind,
                                             N, bits, li), "residual")) ||
      (st = ctx_cuda(c, cudaMemcpyAsync(h, bits, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H")) ||
      (st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync")))
    return st;
  *out = *h;
  return PGX_OK;
}

int eval_host(pgx_problem* p, const double* u, double* F, double* G, pgx_eval_stats* stats) {
  pgx_ctx* c = p->ctx;
  const auto t0 = std::chrono::steady_clock::now();
  const size_t n = (size_t)p->desc.n_controls * p->desc.n_slices;
  if (!finite_all(u, n)) return ctx_fail(c, PGX_ERR_NONFINITE, "controls must be finite");
  cudaSetDevice(c->device);
  const int64_t l0 = c->launches;
  if (const int sb = stage_buffer(p)) return sb;
  std::memcpy(p->h_stage, u, n * sizeof(double));
  int st;
  if ((st = ctx_cuda(c, cudaEventRecord(c->ev0, c->stream), "event"))) return st;
  if ((st = ctx_cuda(c, cudaMemcpyAsync(p->d_u, p->h_stage, n * sizeof(double), cudaMemcpyHostToDevice,
                                        c->stream), "H2D u")))
    return st;
  if ((st = run_pipeline(p, p->d_u, p->d_F, G ? p->d_G : nullptr))) return st;
  double* hG = p->h_stage + n;
  double* hF = p->h_stage + 2 * n;
  if (G && (st = ctx_cuda(c, cudaMemcpyAsync(hG, p->d_G, n * sizeof(double), cudaMemcpyDeviceToHost,
                                             c->stream), "D2H G")))
    return st;
  if ((st = ctx_cuda(c, cudaMemcpyAsync(hF, p->d_F, sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                     "D2H F")))
    return st;
  if ((st = ctx_cuda(c, cudaEventRecord(c->ev1, c->stream), "event"))) return st;
  if ((st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "eval sync"))) return st;
  if (p->desc.precision == PGX_PREC_MIXED && pgx::tc_kernels_used(p->pd)) {
    const int tcf = pgx::grad_tc_check();
    if (tcf & 2)
      return ctx_fail(c, PGX_ERR_NONFINITE, "tensor-core gradient: an operand exceeded the FP16 range (select the "
                                            "CUDA-core gradient team with pgx_problem_set_team)");
    if (tcf != 0) return ctx_fail(c, PGX_ERR_TIMEOUT, "tensor-core kernel: a completion wait gave up");
  }
  if (G) std::memcpy(G, hG, n * sizeof(double));
  if (F) *F = *hF;
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->ms_device = ms;
    stats->ms_host = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    stats->units = (int64_t)p->desc.n_members * p->desc.n_slices;
    stats->n_launches = (int32_t)(c->launches - l0);
    stats->max_taylor_degree = 0;
    if ((st = eval_residual(p, G != nullptr, &stats->residual, &stats->residual_kind))) return st;
  }
  if (!std::isfinite(*hF)) return ctx_fail(c, PGX_ERR_NONFINITE, "objective is not finite");
  return PGX_OK;
}

extern "C" int pgx_eval(pgx_problem* p, const double* u, double* F, double* G, pgx_eval_stats* stats) {
  if (!p || !u || !F) return PGX_ERR_INVALID;
  return eval_host(p, u, F, G, stats);
}

extern "C" int pgx_eval_device(pgx_problem* p, const double* d_u, double* d_F, double* d_G) {
  if (!p || !d_u || !d_F) return PGX_ERR_INVALID;
  cudaSetDevice(p->ctx->device);
  return run_pipeline(p, d_u, d_F, d_G);
}

extern "C" int pgx_eval_aggregate(pgx_problem* p, const double* u, int32_t agg, double alpha, double* F,
                                  double* G) {
  if (!p || !u || !F) return PGX_ERR_INVALID;
  pgx_ctx* c = p->ctx;
  if (agg < PGX_AGG_MEAN || agg > PGX_AGG_CVAR) return ctx_fail(c, PGX_ERR_INVALID, "unknown aggregator");
  if (agg == PGX_AGG_CVAR && !(alpha > 0.0 && alpha <= 1.0))
    return ctx_fail(c, PGX_ERR_INVALID, "cvar alpha must be in (0, 1]");
  const int nm = p->desc.n_members;
  for (int m = 0; m < nm; ++m)
    if (!(p->h_weight[m] > 0.0)) return ctx_fail(c, PGX_ERR_INVALID, "aggregators need positive member weights");
  double Fw = 0.0;
  int st = eval_host(p, u, &Fw, G, nullptr);  // leaves Fm (and Gm when G) of every member on the device
  if (st) return st;
  std::vector<double> Fm(nm);
  if ((st = ctx_cuda(c, cudaMemcpyAsync(Fm.data(), p->w.Fm, sizeof(double) * nm, cudaMemcpyDeviceToHost, c->stream),
                     "D2H Fm")) ||
      (st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync")))
    return st;
  const double npair = (double)std::max(p->desc.target == PGX_TARGET_STATES ? p->desc.n_pairs : 0, 1);
  std::vector<double> fs(nm);
  for (int m = 0; m < nm; ++m) fs[m] = Fm[m] / npair;   // per-sample objective
  std::vector<int> sel;
  if (agg == PGX_AGG_MEAN) {
    for (int m = 0; m < nm; ++m) sel.push_back(m);
  } else if (agg == PGX_AGG_WORST_CASE) {
    sel.push_back((int)(std::min_element(fs.begin(), fs.end()) - fs.begin()));
  } else {
    std::vector<int> order(nm);
    for (int m = 0; m < nm; ++m) order[m] = m;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return fs[a] < fs[b]; });
    const int n_tail = std::max(1, (int)std::nearbyint(alpha * nm));
    sel.assign(order.begin(), order.begin() + std::min(n_tail, nm));
  }
  double f = 0.0;
  for (int m : sel) f += fs[m];
  *F = f / (double)sel.size();
  if (!G) return PGX_OK;
  // gradient of sample m: Gm[m] / (w_m npair); averaged over the selection
  std::vector<int> idx(sel.begin(), sel.end());
  std::vector<double> coef(sel.size());
  for (size_t i = 0; i < sel.size(); ++i) coef[i] = 1.0 / (p->h_weight[sel[i]] * npair * (double)sel.size());
  const size_t len = (size_t)p->desc.n_controls * p->desc.n_slices;
  void* buf = nullptr;
  if ((st = ctx_cuda(c, cudaMallocAsync(&buf, sel.size() * (sizeof(int) + sizeof(double)) + 16, c->stream),
                     "alloc")))
    return st;
  double* d_coef = (double*)buf;
  int* d_idx = (int*)(d_coef + sel.size());
  pgx::LaunchInfo li{c->num_sms, c->stream, &c->launches};
  if (!(st = ctx_cuda(c, cudaMemcpyAsync(d_coef, coef.data(), sizeof(double) * sel.size(), cudaMemcpyHostToDevice,
                                         c->stream), "H2D")) &&
      !(st = ctx_cuda(c, cudaMemcpyAsync(d_idx, idx.data(), sizeof(int) * sel.size(), cudaMemcpyHostToDevice,
                                         c->stream), "H2D")) &&
      !(st = ctx_cuda(c, pgx::launch_select_sum(p->w.Gm, d_idx, d_coef, (int)sel.size(), (int)len, p->d_G, li),
                      "select_sum")))
    st = ctx_cuda(c, cudaMemcpyAsync(G, p->d_G, sizeof(double) * len, cudaMemcpyDeviceToHost, c->stream), "D2H G");
  cudaFreeAsync(buf, c->stream);
  const int st2 = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
  return st ? st : st2;
}

extern "C" int pgx_problem_set_drifts(pgx_problem* p, const double* drifts) {
  if (!p || !drifts) return PGX_ERR_INVALID;
  pgx_ctx* c = p->ctx;
  const int D = p->desc.dim, Dp = p->Dp, nd = p->desc.n_drifts;
  if (!finite_all(drifts, 2 * (size_t)nd * D * D)) return ctx_fail(c, PGX_ERR_NONFINITE, "drifts must be finite");
  if (p->desc.generator == PGX_GEN_HERMITIAN)
    for (int i = 0; i < nd; ++i)
      if (herm_dev(drifts + 2 * (size_t)i * D * D, D) > 1e-10)
        return ctx_fail(c, PGX_ERR_INVALID, "drift is not Hermitian (QuantumSystem.jl:318-341)");
  cudaSetDevice(c->device);
  // the flag changes only after the stream has drained the evaluations that
  // were enqueued with the old drifts
  int st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
  if (st) return st;
  p->lsym_drift = p->lsym_fixed && lsym_all(drifts, nd, D);
  p->refresh_lsym();
  ++p->generation;
  const std::vector<double> padded = pad_mats(drifts, nd, D, Dp);
  st = ctx_cuda(c, cudaMemcpyAsync((void*)p->pd.drifts, padded.data(), padded.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, c->stream), "H2D drifts");
  if (!st && p->pd.drifts_df) {
    const std::vector<float> dfp = to_df_pairs(padded), f32 = to_f32(padded);
    st = ctx_cuda(c, cudaMemcpyAsync((void*)p->pd.drifts_df, dfp.data(), dfp.size() * sizeof(float),
                                     cudaMemcpyHostToDevice, c->stream), "H2D drifts (df)");
    if (!st)
      st = ctx_cuda(c, cudaMemcpyAsync((void*)p->pd.drifts_f32, f32.data(), f32.size() * sizeof(float),
                                       cudaMemcpyHostToDevice, c->stream), "H2D drifts (FP32)");
    if (!st) st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");  // dfp lives on this stack
    return st;
  }
  return st ? st : ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
}

extern "C" int pgx_member_fidelities(pgx_problem* p, double* F_members) {
  if (!p || !F_members) return PGX_ERR_INVALID;
  pgx_ctx* c = p->ctx;
  int st = ctx_cuda(c, cudaMemcpyAsync(F_members, p->w.Fm, sizeof(double) * p->desc.n_members,
                                       cudaMemcpyDeviceToHost, c->stream), "D2H Fm");
  if (st) return st;
  return ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
}

extern "C" int pgx_total_propagator(pgx_problem* p, const double* u, int32_t member, double* U_total) {
  if (!p || !u || !U_total) return PGX_ERR_INVALID;
  pgx_ctx* c = p->ctx;
  if (member < 0 || member >= p->desc.n_members) return ctx_fail(c, PGX_ERR_INVALID, "member out of range");
  const size_t n = (size_t)p->desc.n_controls * p->desc.n_slices;
  if (!finite_all(u, n)) return ctx_fail(c, PGX_ERR_NONFINITE, "controls must be finite");
  cudaSetDevice(c->device);
  if (const int sb = stage_buffer(p)) return sb;
  std::memcpy(p->h_stage, u, n * sizeof(double));
  int st = ctx_cuda(c, cudaMemcpyAsync(p->d_u, p->h_stage, n * sizeof(double), cudaMemcpyHostToDevice,
                                       c->stream), "H2D u");
  if (st) return st;
  pgx::LaunchInfo li{c->num_sms, c->stream, &c->launches};
  ProbDev pd = p->pd;
  pd.target = PGX_TARGET_GATE;  // the gate chain forms U_total for any target kind
  pd.n_pairs = 0;
  WorkDev w = p->w;
  w.u = p->d_u;
  w.F = p->d_F + 1;
  // The gate chain writes z/kap/Fm for every member; keep those of the last
  // evaluation intact by pointing them at scratch that is large enough.
  if (!w.P) w.P = nullptr;
  double2* zsave = nullptr;
  double* fsave = nullptr;
  const size_t zbytes = (size_t)p->desc.n_members * std::max(p->pd.n_pairs, 1) * sizeof(double2);
  if ((st = ctx_cuda(c, cudaMallocAsync((void**)&zsave, 2 * zbytes, c->stream), "alloc scratch")) ||
      (st = ctx_cuda(c, cudaMallocAsync((void**)&fsave, sizeof(double) * p->desc.n_members, c->stream),
                     "alloc scratch")))
    return st;
  w.z = zsave;
  w.kap = zsave + zbytes / sizeof(double2);
  w.Fm = fsave;
  if ((st = ctx_cuda(c, pgx::launch_expm(pd, w, li), "expm")) ||
      (st = ctx_cuda(c, pgx::launch_chain_fwd(pd, w, li, false), "chain")))
    return st;
  const int D = p->desc.dim, Dp = p->Dp;
  std::vector<double> buf((size_t)Dp * Dp * 2);
  st = ctx_cuda(c, cudaMemcpyAsync(buf.data(), p->w.Utot + (size_t)member * Dp * Dp,
                                   buf.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H");
  cudaFreeAsync(zsave, c->stream);
  cudaFreeAsync(fsave, c->stream);
  if (st) return st;
  if ((st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync"))) return st;
  for (int col = 0; col < D; ++col)
    for (int r = 0; r < D; ++r) {
      U_total[2 * (r + (size_t)D * col)] = buf[2 * (r + (size_t)Dp * col)];
      U_total[2 * (r + (size_t)D * col) + 1] = buf[2 * (r + (size_t)Dp * col) + 1];
    }
  return PGX_OK;
}

extern "C" int pgx_propagator(pgx_ctx* c, int32_t dim, int32_t generator, const double* gen, double dt,
                              double* U) {
  if (!c || !gen || !U) return PGX_ERR_INVALID;
  if (dim < 1 || dim > pgx::kMaxDim) return ctx_fail(c, PGX_ERR_DIMS, "dim must be in [1, 64]");
  if (generator != PGX_GEN_HERMITIAN && generator != PGX_GEN_LIOUVILLIAN)
    return ctx_fail(c, PGX_ERR_INVALID, "unknown generator kind");
  if (!std::isfinite(dt) || !finite_all(gen, 2 * (size_t)dim * dim))
    return ctx_fail(c, PGX_ERR_NONFINITE, "generator and dt must be finite");
  if (generator == PGX_GEN_HERMITIAN && herm_dev(gen, dim) > 1e-10)
    return ctx_fail(c, PGX_ERR_INVALID, "H is not Hermitian (Propagators.jl:617-624)");
  cudaSetDevice(c->device);
  const int Dp = pad_dim(dim);
  std::vector<double> g = pad_mats(gen, 1, dim, Dp);
  const size_t mb = (size_t)Dp * Dp * sizeof(double2);
  const size_t slab = pgx::slab_elems(Dp, c->num_sms) ? (size_t)10 * Dp * Dp * sizeof(double2) : 0;
  double2* dbuf = nullptr;
  int st = ctx_cuda(c, cudaMallocAsync((void**)&dbuf, 2 * mb + slab, c->stream), "alloc");
  if (st) return st;
  pgx::LaunchInfo li{c->num_sms, c->stream, &c->launches};
  std::vector<double> out((size_t)Dp * Dp * 2);
  if (!(st = ctx_cuda(c, cudaMemcpyAsync(dbuf, g.data(), mb, cudaMemcpyHostToDevice, c->stream), "H2D")) &&
      !(st = ctx_cuda(c, pgx::launch_single_expm(Dp, generator, dbuf, dt, dbuf + Dp * Dp,
                                                 slab ? dbuf + 2 * Dp * Dp : nullptr, li), "expm")))
    st = ctx_cuda(c, cudaMemcpyAsync(out.data(), dbuf + Dp * Dp, mb, cudaMemcpyDeviceToHost, c->stream), "D2H");
  cudaFreeAsync(dbuf, c->stream);
  int st2 = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
  if (st) return st;
  if (st2) return st2;
  for (int col = 0; col < dim; ++col)
    for (int r = 0; r < dim; ++r) {
      U[2 * (r + (size_t)dim * col)] = out[2 * (r + (size_t)Dp * col)];
      U[2 * (r + (size_t)dim * col) + 1] = out[2 * (r + (size_t)Dp * col) + 1];
    }
  return PGX_OK;
}

// ---------------------------------------------------------------------------
// trajectory tracking and phase-only evaluation (MR/GRAPETracking.jl,
// MR/GRAPEPhase.jl)
// ---------------------------------------------------------------------------
// Frees an owned device buffer of a problem ahead of its destruction.
static void release_owned(pgx_problem* p, void*& ptr, uint64_t& bytes) {
  if (!ptr) return;
  pgx_ctx* c = p->ctx;
  auto it = std::find(p->owned.begin(), p->owned.end(), ptr);
  if (it != p->owned.end()) p->owned.erase(it);
  if (c->pool) cudaFreeAsync(ptr, c->stream);
  else cudaFree(ptr);
  c->used -= bytes;
  p->bytes -= bytes;
  ptr = nullptr;
  bytes = 0;
}

extern "C" int pgx_problem_set_tracking(pgx_problem* p, int32_t n, const int32_t* steps, const double* weights,
                                        const double* targets) {
  if (!p || n < 0 || (n > 0 && (!steps || !weights || !targets))) return PGX_ERR_INVALID;
  pgx_ctx* c = p->ctx;
  const pgx_problem_desc& d = p->desc;
  if (n > 0 && (d.target != PGX_TARGET_STATES || d.generator != PGX_GEN_HERMITIAN))
    return ctx_fail(c, PGX_ERR_UNSUPPORTED, "tracking needs a Hermitian problem with state targets "
                                            "(grape_tracking_kernel, GRAPETracking.jl:166-173)");
  if (n > 0 && d.precision != PGX_PREC_FP64)
    return ctx_fail(c, PGX_ERR_UNSUPPORTED, "tracking runs in FP64");
  if (n > 0 && d.grad_mode == PGX_GRAD_REF_GRAPE)
    return ctx_fail(c, PGX_ERR_UNSUPPORTED, "tracking has the MR first-order formula (PGX_GRAD_REF_MR) "
                                            "or the exact gradient");
  const int D = d.dim, Dp = p->Dp;
  for (int i = 0; i < n; ++i) {
    if (steps[i] < 1 || steps[i] > d.n_slices) {
      char msg[96];
      std::snprintf(msg, sizeof msg, "TrackingPoint.step=%d out of range [1, %d]", steps[i], d.n_slices);
      return ctx_fail(c, PGX_ERR_INVALID, msg);  // GRAPETracking.jl:190-191
    }
    if (!std::isfinite(weights[i]) || !finite_all(targets + (size_t)i * 2 * D * D, (size_t)2 * D * D))
      return ctx_fail(c, PGX_ERR_NONFINITE, "tracking weights and targets must be finite");
    if (herm_dev(targets + (size_t)i * 2 * D * D, D) > 1e-10)
      return ctx_fail(c, PGX_ERR_INVALID, "tracking target density matrices must be Hermitian");
  }
  cudaSetDevice(c->device);
  // checkpoints in ascending step order; ties keep their given order
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return steps[a] < steps[b]; });
  const size_t tb = (size_t)n * Dp * Dp * sizeof(double2);
  const size_t off_w = ((size_t)n * sizeof(int) + 15) / 16 * 16;
  const size_t off_t = off_w + ((size_t)n * sizeof(double) + 15) / 16 * 16;
  const size_t bytes = off_t + tb;
  std::vector<unsigned char> host(bytes, 0);
  int* hs = reinterpret_cast<int*>(host.data());
  double* hw = reinterpret_cast<double*>(host.data() + off_w);
  for (int i = 0; i < n; ++i) {
    hs[i] = steps[order[i]];
    hw[i] = weights[order[i]];
    const std::vector<double> t = pad_mats(targets + (size_t)order[i] * 2 * D * D, 1, D, Dp);
    std::memcpy(host.data() + off_t + (size_t)i * Dp * Dp * sizeof(double2), t.data(), Dp * Dp * sizeof(double2));
  }
  int st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
  if (st) return st;
  release_owned(p, p->d_track, p->track_bytes);  // the previous checkpoints
  if (n > 0) {
    if ((st = ctx_alloc(c, &p->d_track, bytes, p->owned, p->bytes))) return st;
    p->track_bytes = bytes;
    if ((st = ctx_cuda(c, cudaMemcpyAsync(p->d_track, host.data(), bytes, cudaMemcpyHostToDevice, c->stream),
                       "H2D tracking")) ||
        (st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync")))
      return st;
  }
  unsigned char* base = static_cast<unsigned char*>(p->d_track);
  for (pgx::ProbDev* pd : {&p->pd, &p->pd_grad}) {
    pd->n_ck = n;
    pd->ck_step = n ? reinterpret_cast<const int*>(base) : nullptr;
    pd->ck_weight = n ? reinterpret_cast<const double*>(base + off_w) : nullptr;
    pd->ck_target = n ? reinterpret_cast<const double2*>(base + off_t) : nullptr;
  }
  ++p->generation;
  return PGX_OK;
}

extern "C" int pgx_problem_set_drift_ramp(pgx_problem* p, int32_t n_ops, const double* ops, const int32_t* member_op,
                                          const double* tau) {
  if (!p || n_ops < 0 || (n_ops > 0 && (!ops || !member_op || !tau))) return PGX_ERR_INVALID;
  pgx_ctx* c = p->ctx;
  const pgx_problem_desc& d = p->desc;
  const int D = d.dim, Dp = p->Dp, nm = d.n_members, nt = d.n_slices;
  if (n_ops > 0) {
    if (!finite_all(ops, 2 * (size_t)n_ops * D * D) || !finite_all(tau, nt))
      return ctx_fail(c, PGX_ERR_NONFINITE, "ramp operators and schedule must be finite");
    if (d.generator == PGX_GEN_HERMITIAN)
      for (int i = 0; i < n_ops; ++i)
        if (herm_dev(ops + 2 * (size_t)i * D * D, D) > 1e-10)
          return ctx_fail(c, PGX_ERR_INVALID, "ramp operators of a Hermitian problem must be Hermitian");
    for (int m = 0; m < nm; ++m)
      if (member_op[m] < -1 || member_op[m] >= n_ops)
        return ctx_fail(c, PGX_ERR_INVALID, "member ramp index out of range");
  }
  cudaSetDevice(c->device);
  const bool mixed = d.precision == PGX_PREC_MIXED;
  auto up16 = [](size_t b) { return (b + 15) / 16 * 16; };
  const size_t off_tau = up16((size_t)nm * sizeof(int));
  const size_t off_ops = off_tau + up16((size_t)nt * sizeof(double));
  const size_t ops_bytes = (size_t)n_ops * Dp * Dp * sizeof(double2);
  const size_t off_tdf = off_ops + ops_bytes;
  const size_t off_odf = off_tdf + up16((size_t)nt * sizeof(float2));
  const size_t bytes = mixed ? off_odf + (size_t)n_ops * Dp * Dp * sizeof(float4) : off_tdf;
  std::vector<unsigned char> host(n_ops > 0 ? bytes : 0, 0);
  std::vector<double> opsp;
  if (n_ops > 0) {
    std::memcpy(host.data(), member_op, (size_t)nm * sizeof(int));
    std::memcpy(host.data() + off_tau, tau, (size_t)nt * sizeof(double));
    opsp = pad_mats(ops, n_ops, D, Dp);
    std::memcpy(host.data() + off_ops, opsp.data(), ops_bytes);
    if (mixed) {
      const std::vector<double> tv(tau, tau + nt);
      const std::vector<float> tdf = to_df_scalars(tv), odf = to_df_pairs(opsp);
      std::memcpy(host.data() + off_tdf, tdf.data(), tdf.size() * sizeof(float));
      std::memcpy(host.data() + off_odf, odf.data(), odf.size() * sizeof(float));
    }
  }
  int st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
  if (st) return st;
  release_owned(p, p->d_ramp, p->ramp_bytes);
  if (n_ops > 0) {
    if ((st = ctx_alloc(c, &p->d_ramp, bytes, p->owned, p->bytes))) return st;
    p->ramp_bytes = bytes;
    if ((st = ctx_cuda(c, cudaMemcpyAsync(p->d_ramp, host.data(), bytes, cudaMemcpyHostToDevice, c->stream),
                       "H2D ramp")) ||
        (st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync")))
      return st;
  }
  unsigned char* base = static_cast<unsigned char*>(p->d_ramp);
  p->lsym_ramp = n_ops == 0 || lsym_all(ops, n_ops, D);  // the symmetric products need every piece symmetric
  p->refresh_lsym();
  ++p->generation;
  for (pgx::ProbDev* pd : {&p->pd, &p->pd_grad}) {
    pd->n_ramp = n_ops;
    pd->m_ramp = n_ops ? reinterpret_cast<const int*>(base) : nullptr;
    pd->tau = n_ops ? reinterpret_cast<const double*>(base + off_tau) : nullptr;
    pd->ramp_ops = n_ops ? reinterpret_cast<const double2*>(base + off_ops) : nullptr;
    pd->tau_df = n_ops && mixed ? reinterpret_cast<const float2*>(base + off_tdf) : nullptr;
    pd->ramp_ops_df = n_ops && mixed ? reinterpret_cast<const float4*>(base + off_odf) : nullptr;
  }
  return PGX_OK;
}

extern "C" int pgx_eval_phase(pgx_problem* p, const double* phi, const double* amplitudes, double* F,
                              double* G_phase) {
  if (!p || !phi || !F) return PGX_ERR_INVALID;
  pgx_ctx* c = p->ctx;
  const int nc = p->desc.n_controls, nt = p->desc.n_slices;
  if (nc % 2 != 0)
    return ctx_fail(c, PGX_ERR_INVALID, "phase-only controls come in (x, y) pairs: n_controls must be even "
                                        "(GRAPEPhase.jl:60-66)");
  const int nch = nc / 2;
  const size_t n = (size_t)nch * nt;
  if (!finite_all(phi, n) || (amplitudes && !finite_all(amplitudes, n)))
    return ctx_fail(c, PGX_ERR_NONFINITE, "phases and amplitudes must be finite");
  for (size_t i = 0; amplitudes && i < n; ++i)
    if (amplitudes[i] < 0.0) return ctx_fail(c, PGX_ERR_INVALID, "all amplitudes must be >= 0 (GRAPEPhase.jl:72)");
  // polar -> Cartesian: w[2ch, k] = a cos(phi), w[2ch+1, k] = a sin(phi)
  std::vector<double> u((size_t)nc * nt), G(G_phase ? (size_t)nc * nt : 0);
  for (int k = 0; k < nt; ++k)
    for (int ch = 0; ch < nch; ++ch) {
      const size_t i = (size_t)ch + (size_t)nch * k;
      const double a = amplitudes ? amplitudes[i] : 1.0;
      u[(size_t)2 * ch + (size_t)nc * k] = a * std::cos(phi[i]);
      u[(size_t)2 * ch + 1 + (size_t)nc * k] = a * std::sin(phi[i]);
    }
  const int st = eval_host(p, u.data(), F, G_phase ? G.data() : nullptr, nullptr);
  if (st || !G_phase) return st;
  // dF/dphi = -G_x sin(phi) + G_y cos(phi)   (GRAPEPhase.jl:86-90)
  for (int k = 0; k < nt; ++k)
    for (int ch = 0; ch < nch; ++ch) {
      const size_t i = (size_t)ch + (size_t)nch * k;
      G_phase[i] = -G[(size_t)2 * ch + (size_t)nc * k] * std::sin(phi[i]) +
                   G[(size_t)2 * ch + 1 + (size_t)nc * k] * std::cos(phi[i]);
    }
  return PGX_OK;
}
