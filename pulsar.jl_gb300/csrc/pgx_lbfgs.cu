// Device-resident L-BFGS of grape_optimize_ensemble (GRAPE.jl:1012-1230) for
// served jobs: the two-loop recursion (GRAPE.jl:1064-1084, with its 1e-14
// floors), the normalised direction, the clipped trial point of the
// backtracking line search (:1088-1104) and the (s, y) history update with its
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
    const double gam = sy / fmax(yy, 1e-14);
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

// ut = clip(u + a d); halve: a <- a / 2 first.
__global__ void __launch_bounds__(kLbThreads) k_lb_trial(LbArgs A, int halve) {
  LbState* st = A.st;
  const double a = halve ? 0.5 * st->a : st->a;
  __syncthreads();  // every thread has read st->a
  if (threadIdx.x == 0) st->a = a;
  const int n = st->n;
  for (int i = threadIdx.x; i < n; i += kLbThreads) {
    double v = fma(a, A.d[i], A.u[i]);
    if (A.clip) v = fmin(fmax(v, -A.lim), A.lim);
    A.ut[i] = v;
  }
}

// s = a d, y = gn - g; kept when y.s > 1e-14 ||s||^2 (the oldest pair drops
// out beyond m).  Then u <- ut and g <- gn, so a job's buffers never move and
// its steps can be replayed as CUDA graphs.
__global__ void __launch_bounds__(kLbThreads) k_lb_accept(LbArgs A) {
  __shared__ double red[kLbThreads];
  LbState* st = A.st;
  const int n = st->n, m = st->m, head = st->head;
  const double a = st->a;
  double ss = 0.0, ys = 0.0;
  for (int i = threadIdx.x; i < n; i += kLbThreads) {
    const double si = a * A.d[i], yi = A.gn[i] - A.g[i];
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
      s[i] = a * A.d[i];
      y[i] = gi - g[i];
    }
    g[i] = gi;
    u[i] = A.ut[i];
  }
  if (keep && threadIdx.x == 0) {
    A.rho[head] = 1.0 / fmax(ys, 1e-14);
    st->head = (head + 1) % m;
    st->count = st->count < m ? st->count + 1 : m;
  }
}

}  // namespace

cudaError_t launch_lb_direction(const LbArgs& a, cudaStream_t stream) {
  k_lb_direction<<<1, kLbThreads, 0, stream>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_lb_trial(const LbArgs& a, bool halve, cudaStream_t stream) {
  k_lb_trial<<<1, kLbThreads, 0, stream>>>(a, halve ? 1 : 0);
  return cudaGetLastError();
}
cudaError_t launch_lb_accept(const LbArgs& a, cudaStream_t stream) {
  k_lb_accept<<<1, kLbThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace pgx
