// Propagator stacks, chains, total Hamiltonians and overlaps as standalone
// device calls: the building blocks of Propagators.jl and Objectives.jl that
// the fused evaluation pipeline computes internally.
//
//   pgx_total_hamiltonian   H_k = H_d + sum_j u_jk H_j          (Propagators.jl:485-544)
//   pgx_propagator_stack    U_k = exp(c dt_k H_k)                (Propagators.jl:127-184)
//   pgx_propagator_chains   P_0 = I, P_{k+1} = U_k P_k           (Propagators.jl:291-325)
//                           Q_n = seed | I, Q_k = U_k' Q_{k+1}   (Propagators.jl:390-440)
//                           U_total = U_{n-1} ... U_0            (Propagators.jl:212-238)
//   pgx_overlap             z = sum_ij conj(A_ij) B_ij = Tr(A'B) (Objectives.jl:221,239-246)
//   pgx_trace_products      t_jk = Tr(X_k E_j Y_k)               (the traces of CUDABackend.jl:352-356)
//
// All in FP64 on padded Dp x Dp matrices (zero padding: the padded block of
// exp() is the identity and never mixes with the true block).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "pgx.h"
#include "pgx_runtime.h"
#include "pgx_stages.cuh"

namespace pgx {
namespace {

// U_k = exp(c dt_k H_k) for a stack of generators (dt_count 1: uniform dt).
template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_expm_stack(int gen, const double2* H, const double* dt,
                                                                int dt_count, int n, double2* U, double2* slab) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  double2* base;
  double2* red;
  if constexpr (G::SLAB) {
    base = slab + (size_t)blockIdx.x * G::NBUF * D * D;
    red = smem + (size_t)team * T;
  } else {
    base = smem + (size_t)team * G::NBUF * D * D;
    red = smem + (size_t)G::TPC * G::NBUF * D * D + (size_t)team * T;
  }
  const Work<double2, D> W = Work<double2, D>::at(base);
  for (long k = (long)blockIdx.x * G::TPC + team; k < n; k += (long)gridDim.x * G::TPC) {
    const double dtk = dt[dt_count == 1 ? 0 : k];
    const double2* Hk = H + (size_t)k * D * D;
    for (int e = tm.lane; e < D * D; e += T) {
      double2 v = Hk[e];
      v.x *= dtk;
      v.y *= dtk;
      W.B[e] = times_c(v, gen);
    }
    tm.sync();
    const double nrm = norm1<D, T>(tm, W.B, reinterpret_cast<double*>(red));
    int deg, s;
    choose_degree(nrm, c_theta64, deg, s);
    const double sc = ldexp(1.0, -s);
    for (int e = tm.lane; e < D * D; e += T) W.B[e] = cscale(W.B[e], sc);
    tm.sync();
    taylor_exp<D, T>(tm, W, deg, s, c_invf);
    double2* out = U + (size_t)k * D * D;
    for (int e = tm.lane; e < D * D; e += T) out[e] = W.Y[e];
    tm.sync();
  }
}

// Block 0: forward chain (P, U_total); block 1: backward chain (Q).  One team
// each, sequential over the slices.
template <int D>
__global__ void __launch_bounds__(Cfg<D>::T) k_chains(int n, const double2* U, const double2* seed, double2* P,
                                                      double2* Q, double2* Utot) {
  constexpr int T = Cfg<D>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* cur = reinterpret_cast<double2*>(smem_raw);
  double2* Ub = cur + D * D;
  const Team<T> tm{(int)threadIdx.x};
  if (blockIdx.x == 0) {
    if (!P && !Utot) return;
    for (int e = tm.lane; e < D * D; e += T) {
      cur[e] = make_double2((e % D) == (e / D) ? 1.0 : 0.0, 0.0);
      if (P) P[e] = cur[e];
    }
    tm.sync();
    for (int k = 0; k < n; ++k) {
      mm1<D, T>(tm, cur, U + (size_t)k * D * D, cur);
      if (P)
        for (int e = tm.lane; e < D * D; e += T) P[(size_t)(k + 1) * D * D + e] = cur[e];
    }
    if (Utot)
      for (int e = tm.lane; e < D * D; e += T) Utot[e] = cur[e];
  } else {
    if (!Q) return;
    for (int e = tm.lane; e < D * D; e += T) {
      cur[e] = seed ? seed[e] : make_double2((e % D) == (e / D) ? 1.0 : 0.0, 0.0);
      Q[(size_t)n * D * D + e] = cur[e];
    }
    tm.sync();
    for (int k = n - 1; k >= 0; --k) {
      const double2* Uk = U + (size_t)k * D * D;
      for (int e = tm.lane; e < D * D; e += T) {  // Ub = U_k'
        const double2 v = Uk[(e / D) + D * (e % D)];
        Ub[e] = make_double2(v.x, -v.y);
      }
      tm.sync();
      mm1<D, T>(tm, cur, Ub, cur);
      for (int e = tm.lane; e < D * D; e += T) Q[(size_t)k * D * D + e] = cur[e];
    }
  }
}

// H_k = H_d + sum_j u[j + n_c k] H_j on padded matrices, elementwise.
__global__ void k_total_hamiltonian(int DD, int n_c, int n, const double2* Hd, const double2* Hc,
                                    const double* u, double2* H) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)n * DD) return;
  const int k = (int)(i / DD), e = (int)(i % DD);
  double2 v = Hd[e];
  for (int j = 0; j < n_c; ++j) {
    const double a = u[j + (size_t)n_c * k];
    const double2 c = Hc[(size_t)j * DD + e];
    v.x = fma(a, c.x, v.x);
    v.y = fma(a, c.y, v.y);
  }
  H[i] = v;
}

// z = sum_i conj(a_i) b_i: one CTA, strided partials then a fixed tree.
constexpr int kOverlapThreads = 256;
__global__ void __launch_bounds__(kOverlapThreads) k_overlap(long n, const double2* a, const double2* b,
                                                             double2* z) {
  __shared__ double2 red[kOverlapThreads];
  double2 acc = make_double2(0.0, 0.0);
  for (long i = threadIdx.x; i < n; i += kOverlapThreads) {
    const double2 x = a[i], y = b[i];
    acc.x = fma(x.x, y.x, fma(x.y, y.y, acc.x));
    acc.y = fma(x.x, y.y, fma(-x.y, y.x, acc.y));
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kOverlapThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      red[threadIdx.x].x += red[threadIdx.x + w].x;
      red[threadIdx.x].y += red[threadIdx.x + w].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *z = red[0];
}

// out[j + m k] = Tr(X_k E_j Y_k) = Tr(E_j G_k), G_k = Y_k X_k: one team per k.
template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_trace_products(int n, int m, const double2* X,
                                                                    const double2* E, const double2* Y,
                                                                    double2* out) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  Team<T> tm{(int)(threadIdx.x % T)};
  if (G::TPC > 1 && T > 32) tm.bar = 1 + team;
  double2* Gk = smem + (size_t)team * (D * D + T);
  double2* red = Gk + D * D;
  for (long k = (long)blockIdx.x * G::TPC + team; k < n; k += (long)gridDim.x * G::TPC) {
    mm1<D, T>(tm, Gk, Y + (size_t)k * D * D, X + (size_t)k * D * D);
    for (int j = 0; j < m; ++j) {
      const double2* Ej = E + (size_t)j * D * D;
      double2 acc = make_double2(0.0, 0.0);
      for (int q = tm.lane; q < D * D; q += T) {  // E_j[b][c] G[c][b]
        const int b = q % D, c = q / D;
        acc = cmac(acc, Ej[q], Gk[c + D * b]);
      }
      acc = team_sum<T>(tm, acc, red);
      if (tm.lane == 0) out[j + (size_t)m * k] = acc;
    }
    tm.sync();
  }
}

template <int D>
cudaError_t do_trace_products(int n, int m, const double2* X, const double2* E, const double2* Y, double2* out,
                              const LaunchInfo& li) {
  using G = Cfg<D>;
  const size_t smem = (size_t)G::TPC * (D * D + G::T) * sizeof(double2);
  set_smem_once((const void*)k_trace_products<D>, smem);
  const long blocks = std::min<long>(((long)n + G::TPC - 1) / G::TPC, (long)li.num_sms * 4);
  k_trace_products<D><<<(int)std::max<long>(blocks, 1), G::THREADS, smem, li.stream>>>(n, m, X, E, Y, out);
  ++*li.launches;
  return cudaGetLastError();
}

template <int D>
cudaError_t do_expm_stack(int gen, const double2* H, const double* dt, int dt_count, int n, double2* U,
                          double2* slab, int slab_teams, const LaunchInfo& li) {
  using G = Cfg<D>;
  const size_t smem = taylor_smem_bytes<D>();
  set_smem_once((const void*)k_expm_stack<D>, smem);
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_expm_stack<D>, G::THREADS, smem);
  long blocks = std::min<long>(((long)n + G::TPC - 1) / G::TPC, (long)li.num_sms * std::max(per_sm, 1));
  if (G::SLAB) blocks = std::min<long>(blocks, slab_teams);
  k_expm_stack<D><<<(int)std::max<long>(blocks, 1), G::THREADS, smem, li.stream>>>(gen, H, dt, dt_count, n, U,
                                                                                    slab);
  ++*li.launches;
  return cudaGetLastError();
}

template <int D>
cudaError_t do_chains(int n, const double2* U, const double2* seed, double2* P, double2* Q, double2* Utot,
                      const LaunchInfo& li) {
  const size_t smem = (size_t)2 * D * D * sizeof(double2);
  set_smem_once((const void*)k_chains<D>, smem);
  k_chains<D><<<2, Cfg<D>::T, smem, li.stream>>>(n, U, seed, P, Q, Utot);
  ++*li.launches;
  return cudaGetLastError();
}

#define PGX_DISPATCH_STACK(DP, CALL)                 \
  switch (DP) {                                      \
    case 2: { constexpr int D_ = 2; CALL; } break;   \
    case 4: { constexpr int D_ = 4; CALL; } break;   \
    case 8: { constexpr int D_ = 8; CALL; } break;   \
    case 16: { constexpr int D_ = 16; CALL; } break; \
    case 32: { constexpr int D_ = 32; CALL; } break; \
    case 64: { constexpr int D_ = 64; CALL; } break; \
    default: return cudaErrorInvalidValue;           \
  }

// Device scratch of one call, released on every path.
struct Scratch {
  pgx_ctx* c;
  void* p = nullptr;
  explicit Scratch(pgx_ctx* ctx) : c(ctx) {}
  ~Scratch() {
    if (p) cudaFreeAsync(p, c->stream);
    cudaStreamSynchronize(c->stream);
  }
};

std::vector<double> unpad(const std::vector<double>& src, int n, int D, int Dp) {
  std::vector<double> out((size_t)n * D * D * 2);
  for (int i = 0; i < n; ++i)
    for (int col = 0; col < D; ++col)
      for (int r = 0; r < D; ++r) {
        const size_t si = 2 * ((size_t)i * Dp * Dp + r + (size_t)Dp * col);
        const size_t di = 2 * ((size_t)i * D * D + r + (size_t)D * col);
        out[di] = src[si];
        out[di + 1] = src[si + 1];
      }
  return out;
}

}  // namespace
}  // namespace pgx

using pgx::LaunchInfo;

extern "C" int pgx_total_hamiltonian(pgx_ctx* c, int32_t dim, int32_t n_controls, int32_t n,
                                     const double* H_drift, const double* H_controls, const double* u,
                                     double* H) {
  if (!c || !H_drift || (n_controls > 0 && (!H_controls || !u)) || !H) return PGX_ERR_INVALID;
  if (dim < 1 || n < 0 || n_controls < 0) return ctx_fail(c, PGX_ERR_DIMS, "dim >= 1, n >= 0, n_controls >= 0");
  if (n == 0) return PGX_OK;
  const size_t DD = (size_t)dim * dim;
  if (!finite_all(H_drift, 2 * DD) || !finite_all(H_controls, 2 * DD * n_controls) ||
      !finite_all(u, (size_t)n_controls * n))
    return ctx_fail(c, PGX_ERR_NONFINITE, "inputs must be finite");
  cudaSetDevice(c->device);
  pgx::Scratch sc(c);
  const size_t b_in = 2 * DD * sizeof(double) * (1 + n_controls), b_u = sizeof(double) * n_controls * n;
  const size_t b_out = 2 * DD * sizeof(double) * n;
  int st = ctx_cuda(c, cudaMallocAsync(&sc.p, b_in + b_u + b_out, c->stream), "alloc");
  if (st) return st;
  double* d_in = (double*)sc.p;
  double* d_u = d_in + 2 * DD * (1 + n_controls);
  double* d_H = d_u + (size_t)n_controls * n;
  if ((st = ctx_cuda(c, cudaMemcpyAsync(d_in, H_drift, 2 * DD * sizeof(double), cudaMemcpyHostToDevice, c->stream),
                     "H2D")) ||
      (n_controls && ((st = ctx_cuda(c, cudaMemcpyAsync(d_in + 2 * DD, H_controls, 2 * DD * sizeof(double) * n_controls,
                                                        cudaMemcpyHostToDevice, c->stream), "H2D")) ||
                      (st = ctx_cuda(c, cudaMemcpyAsync(d_u, u, b_u, cudaMemcpyHostToDevice, c->stream), "H2D")))))
    return st;
  const long total = (long)n * (long)DD;
  pgx::k_total_hamiltonian<<<(int)((total + 255) / 256), 256, 0, c->stream>>>(
      (int)DD, n_controls, n, (const double2*)d_in, (const double2*)(d_in + 2 * DD), d_u, (double2*)d_H);
  ++c->launches;
  if ((st = ctx_cuda(c, cudaGetLastError(), "total_hamiltonian")) ||
      (st = ctx_cuda(c, cudaMemcpyAsync(H, d_H, b_out, cudaMemcpyDeviceToHost, c->stream), "D2H")))
    return st;
  return ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
}

extern "C" int pgx_propagator_stack(pgx_ctx* c, int32_t dim, int32_t generator, int32_t n, const double* H,
                                    const double* dt, int32_t dt_count, double* U) {
  if (!c || !H || !dt || !U) return PGX_ERR_INVALID;
  if (dim < 1 || dim > pgx::kMaxDim) return ctx_fail(c, PGX_ERR_DIMS, "dim must be in [1, 64]");
  if (n < 0 || (dt_count != 1 && dt_count != n)) return ctx_fail(c, PGX_ERR_DIMS, "dt_count must be 1 or n");
  if (generator != PGX_GEN_HERMITIAN && generator != PGX_GEN_LIOUVILLIAN)
    return ctx_fail(c, PGX_ERR_INVALID, "unknown generator kind");
  if (n == 0) return PGX_OK;
  const size_t DD = (size_t)dim * dim;
  if (!finite_all(H, 2 * DD * n) || !finite_all(dt, dt_count))
    return ctx_fail(c, PGX_ERR_NONFINITE, "generators and dt must be finite");
  for (int i = 0; i < dt_count; ++i)
    if (!(dt[i] > 0.0)) return ctx_fail(c, PGX_ERR_INVALID, "dt must be positive (Propagators.jl:141-143)");
  if (generator == PGX_GEN_HERMITIAN)
    for (int k = 0; k < n; ++k)
      if (herm_dev(H + 2 * DD * k, dim) > 1e-10)
        return ctx_fail(c, PGX_ERR_INVALID, "H[k] is not Hermitian (Propagators.jl:617-624)");
  cudaSetDevice(c->device);
  const int Dp = pad_dim(dim);
  const std::vector<double> hp = pad_mats(H, n, dim, Dp);
  const size_t mb = (size_t)Dp * Dp * sizeof(double2);
  const int slab_teams = pgx::slab_team_count(Dp, c->num_sms);
  const size_t slab = pgx::slab_elems(Dp, c->num_sms) * sizeof(double2);
  pgx::Scratch sc(c);
  int st = ctx_cuda(c, cudaMallocAsync(&sc.p, 2 * mb * n + sizeof(double) * (dt_count + 1) + slab, c->stream),
                     "alloc");
  if (st) return st;
  double2* d_H = (double2*)sc.p;
  double2* d_U = d_H + (size_t)Dp * Dp * n;
  double* d_dt = (double*)(d_U + (size_t)Dp * Dp * n);
  double2* d_slab = slab ? (double2*)(d_dt + dt_count + (dt_count & 1)) : nullptr;
  if ((st = ctx_cuda(c, cudaMemcpyAsync(d_H, hp.data(), mb * n, cudaMemcpyHostToDevice, c->stream), "H2D")) ||
      (st = ctx_cuda(c, cudaMemcpyAsync(d_dt, dt, sizeof(double) * dt_count, cudaMemcpyHostToDevice, c->stream),
                     "H2D")))
    return st;
  LaunchInfo li{c->num_sms, c->stream, &c->launches};
  const cudaError_t e = [&]() -> cudaError_t {
    PGX_DISPATCH_STACK(Dp, return pgx::do_expm_stack<D_>(generator, d_H, d_dt, dt_count, n, d_U, d_slab,
                                                         slab_teams, li));
    return cudaErrorInvalidValue;
  }();
  if ((st = ctx_cuda(c, e, "propagator_stack"))) return st;
  std::vector<double> out(2 * (size_t)Dp * Dp * n);
  if ((st = ctx_cuda(c, cudaMemcpyAsync(out.data(), d_U, mb * n, cudaMemcpyDeviceToHost, c->stream), "D2H")) ||
      (st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync")))
    return st;
  const std::vector<double> u = pgx::unpad(out, n, dim, Dp);
  std::copy(u.begin(), u.end(), U);
  return PGX_OK;
}

extern "C" int pgx_propagator_chains(pgx_ctx* c, int32_t dim, int32_t n, const double* U, const double* seed,
                                     double* P, double* Q, double* U_total) {
  if (!c || (!U && n > 0) || (!P && !Q && !U_total)) return PGX_ERR_INVALID;
  if (dim < 1 || dim > pgx::kMaxDim || n < 0) return ctx_fail(c, PGX_ERR_DIMS, "dim in [1, 64], n >= 0");
  const size_t DD = (size_t)dim * dim;
  if ((n > 0 && !finite_all(U, 2 * DD * n)) || (seed && !finite_all(seed, 2 * DD)))
    return ctx_fail(c, PGX_ERR_NONFINITE, "inputs must be finite");
  cudaSetDevice(c->device);
  const int Dp = pad_dim(dim);
  const size_t mp = (size_t)Dp * Dp;
  const std::vector<double> up = pad_mats(U, n, dim, Dp);
  std::vector<double> sp = pad_mats(seed, 1, dim, Dp);
  pgx::Scratch sc(c);
  // U stack | seed | P (n+1) | Q (n+1) | U_total
  const size_t elems = mp * ((size_t)n + 1 + 2 * ((size_t)n + 1) + 1);
  int st = ctx_cuda(c, cudaMallocAsync(&sc.p, elems * sizeof(double2), c->stream), "alloc");
  if (st) return st;
  double2* d_U = (double2*)sc.p;
  double2* d_seed = d_U + mp * n;
  double2* d_P = d_seed + mp;
  double2* d_Q = d_P + mp * (n + 1);
  double2* d_T = d_Q + mp * (n + 1);
  if ((n > 0 && (st = ctx_cuda(c, cudaMemcpyAsync(d_U, up.data(), mp * n * sizeof(double2), cudaMemcpyHostToDevice,
                                                  c->stream), "H2D"))) ||
      (seed && (st = ctx_cuda(c, cudaMemcpyAsync(d_seed, sp.data(), mp * sizeof(double2), cudaMemcpyHostToDevice,
                                                 c->stream), "H2D"))))
    return st;
  LaunchInfo li{c->num_sms, c->stream, &c->launches};
  const cudaError_t e = [&]() -> cudaError_t {
    PGX_DISPATCH_STACK(Dp, return pgx::do_chains<D_>(n, d_U, seed ? d_seed : nullptr, P ? d_P : nullptr,
                                                     Q ? d_Q : nullptr, U_total ? d_T : nullptr, li));
    return cudaErrorInvalidValue;
  }();
  if ((st = ctx_cuda(c, e, "propagator_chains"))) return st;
  std::vector<double> hp(2 * mp * (n + 1)), hq(2 * mp * (n + 1)), ht(2 * mp);
  if ((P && (st = ctx_cuda(c, cudaMemcpyAsync(hp.data(), d_P, hp.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                              c->stream), "D2H"))) ||
      (Q && (st = ctx_cuda(c, cudaMemcpyAsync(hq.data(), d_Q, hq.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                              c->stream), "D2H"))) ||
      (U_total && (st = ctx_cuda(c, cudaMemcpyAsync(ht.data(), d_T, ht.size() * sizeof(double),
                                                    cudaMemcpyDeviceToHost, c->stream), "D2H"))) ||
      (st = ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync")))
    return st;
  if (P) {
    const std::vector<double> v = pgx::unpad(hp, n + 1, dim, Dp);
    std::copy(v.begin(), v.end(), P);
  }
  if (Q) {
    const std::vector<double> v = pgx::unpad(hq, n + 1, dim, Dp);
    std::copy(v.begin(), v.end(), Q);
  }
  if (U_total) {
    const std::vector<double> v = pgx::unpad(ht, 1, dim, Dp);
    std::copy(v.begin(), v.end(), U_total);
  }
  return PGX_OK;
}

extern "C" int pgx_overlap(pgx_ctx* c, int64_t n, const double* A, const double* B, double* z) {
  if (!c || !A || !B || !z || n < 1) return PGX_ERR_INVALID;
  if (!finite_all(A, 2 * (size_t)n) || !finite_all(B, 2 * (size_t)n))
    return ctx_fail(c, PGX_ERR_NONFINITE, "inputs must be finite");
  cudaSetDevice(c->device);
  pgx::Scratch sc(c);
  const size_t b = 2 * sizeof(double) * (size_t)n;
  int st = ctx_cuda(c, cudaMallocAsync(&sc.p, 2 * b + sizeof(double2), c->stream), "alloc");
  if (st) return st;
  double* d_a = (double*)sc.p;
  double* d_b = d_a + 2 * n;
  double2* d_z = (double2*)(d_b + 2 * n);
  if ((st = ctx_cuda(c, cudaMemcpyAsync(d_a, A, b, cudaMemcpyHostToDevice, c->stream), "H2D")) ||
      (st = ctx_cuda(c, cudaMemcpyAsync(d_b, B, b, cudaMemcpyHostToDevice, c->stream), "H2D")))
    return st;
  pgx::k_overlap<<<1, pgx::kOverlapThreads, 0, c->stream>>>(n, (const double2*)d_a, (const double2*)d_b, d_z);
  ++c->launches;
  if ((st = ctx_cuda(c, cudaGetLastError(), "overlap")) ||
      (st = ctx_cuda(c, cudaMemcpyAsync(z, d_z, sizeof(double2), cudaMemcpyDeviceToHost, c->stream), "D2H")))
    return st;
  return ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
}

extern "C" int pgx_trace_products(pgx_ctx* c, int32_t dim, int32_t n, int32_t m, const double* X, const double* E,
                                  const double* Y, double* out) {
  if (!c || !X || !E || !Y || !out) return PGX_ERR_INVALID;
  if (dim < 1 || dim > pgx::kMaxDim || n < 0 || m < 0) return ctx_fail(c, PGX_ERR_DIMS, "dim in [1, 64], n, m >= 0");
  if (n == 0 || m == 0) return PGX_OK;
  const size_t DD = (size_t)dim * dim;
  if (!finite_all(X, 2 * DD * n) || !finite_all(Y, 2 * DD * n) || !finite_all(E, 2 * DD * m))
    return ctx_fail(c, PGX_ERR_NONFINITE, "inputs must be finite");
  cudaSetDevice(c->device);
  const int Dp = pad_dim(dim);
  const size_t mp = (size_t)Dp * Dp;
  const std::vector<double> xp = pad_mats(X, n, dim, Dp), yp = pad_mats(Y, n, dim, Dp), ep = pad_mats(E, m, dim, Dp);
  pgx::Scratch sc(c);
  int st = ctx_cuda(c, cudaMallocAsync(&sc.p, (mp * (2 * (size_t)n + m) + (size_t)n * m) * sizeof(double2), c->stream),
                    "alloc");
  if (st) return st;
  double2* d_X = (double2*)sc.p;
  double2* d_Y = d_X + mp * n;
  double2* d_E = d_Y + mp * n;
  double2* d_o = d_E + mp * m;
  if ((st = ctx_cuda(c, cudaMemcpyAsync(d_X, xp.data(), mp * n * sizeof(double2), cudaMemcpyHostToDevice, c->stream),
                     "H2D")) ||
      (st = ctx_cuda(c, cudaMemcpyAsync(d_Y, yp.data(), mp * n * sizeof(double2), cudaMemcpyHostToDevice, c->stream),
                     "H2D")) ||
      (st = ctx_cuda(c, cudaMemcpyAsync(d_E, ep.data(), mp * m * sizeof(double2), cudaMemcpyHostToDevice, c->stream),
                     "H2D")))
    return st;
  LaunchInfo li{c->num_sms, c->stream, &c->launches};
  const cudaError_t e = [&]() -> cudaError_t {
    PGX_DISPATCH_STACK(Dp, return pgx::do_trace_products<D_>(n, m, d_X, d_E, d_Y, d_o, li));
    return cudaErrorInvalidValue;
  }();
  if ((st = ctx_cuda(c, e, "trace_products")) ||
      (st = ctx_cuda(c, cudaMemcpyAsync(out, d_o, (size_t)n * m * sizeof(double2), cudaMemcpyDeviceToHost, c->stream),
                     "D2H")))
    return st;
  return ctx_cuda(c, cudaStreamSynchronize(c->stream), "sync");
}
