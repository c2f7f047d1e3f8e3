// Device-resident L-BFGS for served jobs, in the two forms the reference has:
// grape_optimize_ensemble (GRAPE.jl:1012-1230: the two-loop recursion with its
// 1e-14 floors, clipped trial points, s = a d) and the MR L-BFGS of optimcon
// (OptControl.jl:380-482, 565-611: no floors, trial points clamped to the
// bounds, s = w_new - w).  Both: the normalised direction, the trial points of
// the backtracking line search and the (s, y) history update with its
// curvature test.  Every vector of a job (controls, gradients, direction,
// trial point, the m-entry history) stays in HBM; the host reads back only
// (F, max|d|, ||g||) to steer the line search.  One CTA per call; every
// reduction is a fixed-order tree, so a job's iterates do not depend on what
// else runs on the device.
#include <cuda_runtime.h>

#include "pgx_internal.h"

namespace pgx {
namespace {

constexpr int kLbThreads = 512;

__device__ __forceinline__ double block_sum(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = kLbThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_max(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = kLbThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// Each thread touches elements i = tid + k * kLbThreads only, so vector
// updates followed by dot products need no barrier beyond block_sum's.
__device__ __forceinline__ double dotv(const double* a, const double* b, int n, double* red) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += kLbThreads) acc = fma(a[i], b[i], acc);
  return block_sum(acc, red);
}

// d = H g by the two-loop recursion over the stored pairs, oldest first in
// the second loop; then gnorm = ||g||, dmax = max|d|, d /= dmax unless zero.
__global__ void __launch_bounds__(kLbThreads) k_lb_direction(LbArgs A) {
  __shared__ double red[kLbThreads];
  __shared__ double alpha[kLbMaxMemory];
  LbState* st = A.st;
  const int n = st->n, m = st->m, k = st->count, head = st->head;
  double* d = A.d;
  for (int i = threadIdx.x; i < n; i += kLbThreads) d[i] = A.g[i];
  for (int t = 0; t < k; ++t) {  // newest to oldest
    const int idx = (head - 1 - t + 2 * m) % m;
    const double a = A.rho[idx] * dotv(A.S + (size_t)idx * n, d, n, red);
    if (threadIdx.x == 0) alpha[t] = a;
    const double* y = A.Y + (size_t)idx * n;
    for (int i = threadIdx.x; i < n; i += kLbThreads) d[i] -= a * y[i];
  }
  if (k > 0) {
    const int nw = (head - 1 + m) % m;
    const double* s = A.S + (size_t)nw * n;
    const double* y = A.Y + (size_t)nw * n;
    const double sy = dotv(s, y, n, red);
    const double yy = dotv(y, y, n, red);
    const double gam = sy / (A.mr ? yy : fmax(yy, 1e-14));
    for (int i = threadIdx.x; i < n; i += kLbThreads) d[i] *= gam;
  }
  __syncthreads();  // alpha[] written by thread 0
  for (int t = k - 1; t >= 0; --t) {  // oldest to newest
    const int idx = (head - 1 - t + 2 * m) % m;
    const double b = A.rho[idx] * dotv(A.Y + (size_t)idx * n, d, n, red);
    const double c = alpha[t] - b;
    const double* s = A.S + (size_t)idx * n;
    for (int i = threadIdx.x; i < n; i += kLbThreads) d[i] += c * s[i];
  }
  const double gn = sqrt(dotv(A.g, A.g, n, red));
  double mx = 0.0;
  for (int i = threadIdx.x; i < n; i += kLbThreads) mx = fmax(mx, fabs(d[i]));
  const double dmax = block_max(mx, red);
  const bool zero = dmax < 1e-14;
  if (!zero)
    for (int i = threadIdx.x; i < n; i += kLbThreads) d[i] /= dmax;
  if (threadIdx.x == 0) {
    st->dmax = dmax;
    st->gnorm = gn;
    st->zero = zero ? 1.0 : 0.0;
    st->a = A.a0;
  }
}

// ut = clamp(u + a d); kTrialHalve: a <- a / 2 first; kTrialZero: a <- 0
// (the MR line search's fall-back to the current point).
__global__ void __launch_bounds__(kLbThreads) k_lb_trial(LbArgs A, int mode) {
  LbState* st = A.st;
  const double a = mode == kTrialHalve ? 0.5 * st->a : mode == kTrialZero ? 0.0 : st->a;
  __syncthreads();  // every thread has read st->a
  if (threadIdx.x == 0) st->a = a;
  const int n = st->n;
  for (int i = threadIdx.x; i < n; i += kLbThreads) {
    double v = fma(a, A.d[i], A.u[i]);
    if (A.clip) v = fmin(fmax(v, A.lo), A.hi);
    A.ut[i] = v;
  }
}

// s = a d (MR: ut - u), y = gn - g; kept when y.s > 1e-14 ||s||^2 (the oldest
// pair drops out beyond m).  Then u <- ut and g <- gn, so a job's buffers never
// move and its steps can be replayed as CUDA graphs.
__global__ void __launch_bounds__(kLbThreads) k_lb_accept(LbArgs A) {
  __shared__ double red[kLbThreads];
  LbState* st = A.st;
  const int n = st->n, m = st->m, head = st->head;
  const double a = st->a;
  double ss = 0.0, ys = 0.0;
  for (int i = threadIdx.x; i < n; i += kLbThreads) {
    const double si = A.mr ? A.ut[i] - A.u[i] : a * A.d[i], yi = A.gn[i] - A.g[i];
    ss = fma(si, si, ss);
    ys = fma(yi, si, ys);
  }
  ss = block_sum(ss, red);
  ys = block_sum(ys, red);
  const double sn = sqrt(ss);
  const bool keep = ys > 1e-14 * sn * sn;
  double* s = A.S + (size_t)head * n;
  double* y = A.Y + (size_t)head * n;
  double* u = A.u;
  double* g = A.g;
  for (int i = threadIdx.x; i < n; i += kLbThreads) {
    const double gi = A.gn[i];
    if (keep) {
      s[i] = A.mr ? A.ut[i] - u[i] : a * A.d[i];
      y[i] = gi - g[i];
    }
    g[i] = gi;
    u[i] = A.ut[i];
  }
  if (keep && threadIdx.x == 0) {
    A.rho[head] = 1.0 / (A.mr ? ys : fmax(ys, 1e-14));
    st->head = (head + 1) % m;
    st->count = st->count < m ? st->count + 1 : m;
  }
}

// *out = ||v||
__global__ void __launch_bounds__(kLbThreads) k_norm(const double* v, int n, double* out) {
  __shared__ double red[kLbThreads];
  const double s = dotv(v, v, n, red);
  if (threadIdx.x == 0) *out = sqrt(s);
}

// One MR ascent step: u <- clamp(u + (0.05 (hi - lo) / max|G|) G).
__global__ void __launch_bounds__(kLbThreads) k_mr_step(double* u, const double* G, int n, double lo, double hi) {
  __shared__ double red[kLbThreads];
  double mx = 0.0;
  for (int i = threadIdx.x; i < n; i += kLbThreads) mx = fmax(mx, fabs(G[i]));
  const double gmax = block_max(mx, red);
  if (!(gmax > 1e-14)) return;
  const double step = 0.05 * (hi - lo) / gmax;
  for (int i = threadIdx.x; i < n; i += kLbThreads) u[i] = fmin(fmax(u[i] + step * G[i], lo), hi);
}

}  // namespace

cudaError_t launch_lb_gnorm(const LbArgs& a, cudaStream_t stream) {
  k_norm<<<1, kLbThreads, 0, stream>>>(a.gn, a.n, &a.st->gnew);
  return cudaGetLastError();
}
cudaError_t launch_mr_step(double* u, const double* G, int n, double lo, double hi, cudaStream_t stream) {
  k_mr_step<<<1, kLbThreads, 0, stream>>>(u, G, n, lo, hi);
  return cudaGetLastError();
}
cudaError_t launch_norm(const double* v, int n, double* out, cudaStream_t stream) {
  k_norm<<<1, kLbThreads, 0, stream>>>(v, n, out);
  return cudaGetLastError();
}

cudaError_t launch_lb_direction(const LbArgs& a, cudaStream_t stream) {
  k_lb_direction<<<1, kLbThreads, 0, stream>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_lb_trial(const LbArgs& a, int mode, cudaStream_t stream) {
  k_lb_trial<<<1, kLbThreads, 0, stream>>>(a, mode);
  return cudaGetLastError();
}
cudaError_t launch_lb_accept(const LbArgs& a, cudaStream_t stream) {
  k_lb_accept<<<1, kLbThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace pgx
