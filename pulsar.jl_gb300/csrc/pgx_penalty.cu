// Waveform penalties (Penalties.jl:197-330) on the device: fused after the
// member reduction of every evaluation of a problem that carries them
// (F -= weight P, G -= weight dP/du, as _apply_penalties!, GRAPEState.jl:571-584),
// and as a standalone call.  u is [n_c x n_t] column-major (u[j + n_c k] =
// w[j, k]).  One CTA, fixed-order reductions: results do not depend on launch
// timing.
#include <cuda_runtime.h>

#include <cmath>

#include "pgx.h"
#include "pgx_runtime.h"

namespace pgx {
namespace {

constexpr int kPenThreads = 512;

__device__ __forceinline__ double pen_block_sum(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = kPenThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// For each penalty: P_out (when non-null) receives weight * P; F (when
// non-null) -= weight * P; G (when non-null) gets sign * weight * dP/du added.
__global__ void __launch_bounds__(kPenThreads) k_penalties(const pgx_penalty* pens, int n_pen, const double* u,
                                                           const double* dt, int n_c, int n_t, double* F,
                                                           double* G, double sign, double* P_out) {
  __shared__ double red[kPenThreads];
  const int n = n_c * n_t;
  for (int q = 0; q < n_pen; ++q) {
    const pgx_penalty pen = pens[q];
    const double wgt = pen.weight, lo = pen.l_bound, hi = pen.u_bound;
    double acc = 0.0;
    if (pen.type == PGX_PEN_SNSA) {  // per time slice: A = ||w[:, k]||
      for (int k = threadIdx.x; k < n_t; k += kPenThreads) {
        double s2 = 0.0;
        for (int j = 0; j < n_c; ++j) s2 = fma(u[j + n_c * k], u[j + n_c * k], s2);
        const double A = sqrt(s2);
        const double sp = fmax(0.0, A - hi);
        acc = fma(sp, sp, acc);
        if (G && sp > 0.0 && A > 1e-14)
          for (int j = 0; j < n_c; ++j) G[j + n_c * k] += sign * wgt * (2.0 * sp / A) * u[j + n_c * k];
      }
    } else {
      for (int i = threadIdx.x; i < n; i += kPenThreads) {
        const int j = i % n_c, k = i / n_c;
        const double v = u[i];
        double g = 0.0;
        if (pen.type == PGX_PEN_NS) {
          acc = fma(v, v, acc);
          g = 2.0 * v;
        } else if (pen.type == PGX_PEN_SNS) {
          const double e = v > hi ? v - hi : (v < lo ? v - lo : 0.0);
          acc = fma(e, e, acc);
          g = 2.0 * e;
        } else if (pen.type == PGX_PEN_DNS) {  // sum over k < n_t - 1 of (w[j, k+1] - w[j, k])^2
          const double dn = (k + 1 < n_t) ? u[j + n_c * (k + 1)] - v : 0.0;
          const double dp = (k > 0) ? v - u[j + n_c * (k - 1)] : 0.0;
          acc = fma(dn, dn, acc);
          g = 2.0 * dp - 2.0 * dn;
        } else {  // PGX_PEN_ENERGY
          const double t = dt ? dt[k] : 1.0;
          acc = fma(v * v, t, acc);
          g = 2.0 * v * t;
        }
        if (G) G[i] += sign * wgt * g;
      }
    }
    const double P = pen_block_sum(acc, red);
    if (threadIdx.x == 0) {
      if (F) *F -= wgt * P;
      if (P_out) P_out[q] = wgt * P;
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_penalties(const pgx_penalty* d_pens, int n_pen, const double* u, const double* dt, int n_c,
                             int n_t, double* F, double* G, const LaunchInfo& li) {
  k_penalties<<<1, kPenThreads, 0, li.stream>>>(d_pens, n_pen, u, dt, n_c, n_t, F, G, -1.0, nullptr);
  ++*li.launches;
  return cudaGetLastError();
}

}  // namespace pgx

static bool valid_penalty(const pgx_penalty& p) {
  return p.type >= PGX_PEN_NS && p.type <= PGX_PEN_ENERGY && std::isfinite(p.weight) && std::isfinite(p.l_bound) &&
         std::isfinite(p.u_bound);
}

extern "C" int pgx_problem_set_penalties(pgx_problem* p, int32_t n, const pgx_penalty* pens) {
  if (!p || n < 0 || n > PGX_MAX_PENALTIES || (n > 0 && !pens)) return PGX_ERR_INVALID;
  for (int i = 0; i < n; ++i)
    if (!valid_penalty(pens[i]))
      return ctx_fail(p->ctx, PGX_ERR_INVALID, "unknown penalty type or non-finite weight / bounds "
                                               "(Penalties.jl:205)");
  cudaSetDevice(p->ctx->device);
  if (n > 0) {
    const int st = ctx_cuda(p->ctx, cudaMemcpyAsync(p->d_pen, pens, sizeof(pgx_penalty) * n, cudaMemcpyHostToDevice,
                                                    p->ctx->stream), "H2D penalties");
    if (st) return st;
    const int st2 = ctx_cuda(p->ctx, cudaStreamSynchronize(p->ctx->stream), "sync");
    if (st2) return st2;
  }
  p->n_pen = n;
  ++p->generation;
  return PGX_OK;
}

extern "C" int pgx_penalty_eval(pgx_ctx* c, int32_t n_controls, int32_t n_slices, const double* u, const double* dt,
                                const pgx_penalty* pen, double* P, double* G) {
  if (!c || !u || !pen || !P || n_controls < 1 || n_slices < 1) return PGX_ERR_INVALID;
  if (!valid_penalty(*pen)) return ctx_fail(c, PGX_ERR_INVALID, "unknown penalty type (Penalties.jl:205)");
  const size_t n = (size_t)n_controls * n_slices;
  if (!finite_all(u, n) || (dt && !finite_all(dt, n_slices)))
    return ctx_fail(c, PGX_ERR_NONFINITE, "waveform and dt must be finite");
  cudaSetDevice(c->device);
  double* buf = nullptr;
  const size_t bytes = sizeof(double) * (2 * n + n_slices + 1) + sizeof(pgx_penalty);
  int st = ctx_cuda(c, cudaMallocAsync((void**)&buf, bytes, c->stream), "alloc");
  if (st) return st;
  double* d_u = buf;
  double* d_G = d_u + n;
  double* d_dt = d_G + n;
  double* d_P = d_dt + n_slices;
  pgx_penalty* d_pen = reinterpret_cast<pgx_penalty*>(d_P + 1);
  if (!(st = ctx_cuda(c, cudaMemcpyAsync(d_u, u, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream), "H2D")) &&
      !(st = ctx_cuda(c, cudaMemsetAsync(d_G, 0, sizeof(double) * n, c->stream), "memset")) &&
      !(st = ctx_cuda(c, dt ? cudaMemcpyAsync(d_dt, dt, sizeof(double) * n_slices, cudaMemcpyHostToDevice, c->stream)
                            : cudaSuccess, "H2D")) &&
      !(st = ctx_cuda(c, cudaMemcpyAsync(d_pen, pen, sizeof(pgx_penalty), cudaMemcpyHostToDevice, c->stream),
                      "H2D"))) {
    pgx::k_penalties<<<1, pgx::kPenThreads, 0, c->stream>>>(d_pen, 1, d_u, dt ? d_dt : nullptr, n_controls, n_slices,
                                                           nullptr, G ? d_G : nullptr, 1.0, d_P);
    ++c->launches;
    st = ctx_cuda(c, cudaGetLastError(), "penalty");
    if (!st) st = ctx_cuda(c, cudaMemcpyAsync(P, d_P, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (!st && G) st = ctx_cuda(c, cudaMemcpyAsync(G, d_G, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream), "D2H");
  }
  cudaFreeAsync(buf, c->stream);
  const int st2 = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
  return st ? st : st2;
}
