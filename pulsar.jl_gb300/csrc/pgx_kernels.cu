// FP64 kernels of the GRAPE hot path (sm_103a).
//
// One evaluation (F, dF/du) of an ensemble problem runs five stages:
//   expm       slice-parallel   U_mk = exp(A_mk), A_mk = c dt_k G_m(u_k)
//                               (replaces Propagators.jl:166-184,659-674 and the
//                                per-slice exp of GRAPELindblad.jl:146-153)
//   chain_fwd  member-parallel  P_{k+1} = U_k P_k  or  psi_{k+1} = U_k psi_k,
//                               overlap z, f(z) and the chain-rule coefficient
//                               (Propagators.jl:309-325, Objectives.jl:609-630)
//   chain_bwd  member-parallel  Lambda_{k-1} = Lambda_k U_k, M_k = P_k Lambda_k
//                               or lambda_k = U_k' lambda_{k+1}
//                               (Propagators.jl:390-406, GRAPEState.jl:214-217)
//   grad       slice-parallel   g_jk = Re Tr(X_k E_jk), X_k = L_exp(A_k, M_k)
//                               (exact) or M_k (first-order reference formulas,
//                               Gradients.jl:254-291,357-399, GRAPEState.jl:220-230)
//   reduce     deterministic    G = sum_m G_m in member order, F = sum_m w_m F_m
//                               (EnsembleObjective.jl:169-217, GRAPEState.jl:238-244)
//
// The exact gradient uses Tr(M L(A,E)) = Tr(L(A,M) E), valid for any
// polynomial in A with scalar coefficients, so ONE Frechet derivative per
// slice serves all n_c controls.
#include <mutex>
#include <map>
#include <set>
#include <utility>

#include "pgx.h"
#include "pgx_stages.cuh"

namespace pgx {

// --------------------------------------------------------------------------
// Stage 1: slice propagators
// --------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_expm(ProbDev p, WorkDev w) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  double2* base;
  double2* red;
  if constexpr (G::SLAB) {
    base = w.slab + (size_t)blockIdx.x * G::NBUF * D * D;
    red = smem + (size_t)team * T;
  } else {
    base = smem + (size_t)team * G::NBUF * D * D;
    red = smem + (size_t)G::TPC * G::NBUF * D * D + (size_t)team * T;
  }
  const Work<double2, D> W = Work<double2, D>::at(base);
  const long items = (long)p.n_members * p.n_t;
  for (long it = (long)blockIdx.x * G::TPC + team; it < items; it += (long)gridDim.x * G::TPC) {
    const int m = (int)(it / p.n_t), k = (int)(it % p.n_t);
    build_A<D, T>(tm, p, w.u, m, k, W.B);
    tm.sync();
    const double nrm = norm1<D, T>(tm, W.B, reinterpret_cast<double*>(red));
    int deg, s;
    choose_degree(nrm, c_theta64, deg, s);
    const double sc = ldexp(1.0, -s);
    for (int e = tm.lane; e < D * D; e += T) W.B[e] = cscale(W.B[e], sc);
    tm.sync();
    taylor_exp<D, T>(tm, W, deg, s, c_invf);
    double2* out = w.U + ((size_t)m * p.n_t + k) * D * D;
    for (int e = tm.lane; e < D * D; e += T) out[e] = W.Y[e];
    tm.sync();
  }
}

template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_single_expm(int gen, const double2* Gin, double dt,
                                                                 double2* U, double2* slab) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  if (threadIdx.x >= T) return;  // one team
  const Team<T> tm{(int)threadIdx.x};
  double2* base = G::SLAB ? slab : smem;
  double2* red = G::SLAB ? smem : smem + (size_t)G::TPC * G::NBUF * D * D;
  const Work<double2, D> W = Work<double2, D>::at(base);
  for (int e = tm.lane; e < D * D; e += T) {
    double2 v = Gin[e];
    v.x *= dt;
    v.y *= dt;
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
  for (int e = tm.lane; e < D * D; e += T) U[e] = W.Y[e];
}

// --------------------------------------------------------------------------
// Stage 2: forward chains
// --------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_chain_gate_fwd(ProbDev p, WorkDev w, int store) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  constexpr int NE = (D * D + T - 1) / T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;  // whole team leaves together
  double2 *base, *red;
  team_slot<D>(smem, 2 * D * D + T, team, base, red);
  double2* Pc = base;
  double2* Ub = base + D * D;
  for (int e = tm.lane; e < D * D; e += T)
    Pc[e] = make_double2((e % D) == (e / D) ? 1.0 : 0.0, 0.0);
  const double2* Um = w.U + (size_t)m * p.n_t * D * D;
  double2 pre[NE];
#pragma unroll
  for (int i = 0; i < NE; ++i) {
    const int e = tm.lane + i * T;
    if (e < D * D) pre[i] = Um[e];
  }
  tm.sync();
  for (int k = 0; k < p.n_t; ++k) {
    if (store) {
      double2* dst = w.P + ((size_t)m * p.n_t + k) * D * D;
      for (int e = tm.lane; e < D * D; e += T) dst[e] = Pc[e];
    }
#pragma unroll
    for (int i = 0; i < NE; ++i) {
      const int e = tm.lane + i * T;
      if (e < D * D) Ub[e] = pre[i];
    }
    if (k + 1 < p.n_t) {  // prefetch U_{k+1} while U_k P_k is formed
      const double2* nx = Um + (size_t)(k + 1) * D * D;
#pragma unroll
      for (int i = 0; i < NE; ++i) {
        const int e = tm.lane + i * T;
        if (e < D * D) pre[i] = nx[e];
      }
    }
    tm.sync();
    mm1<D, T>(tm, Pc, Ub, Pc);
  }
  double2* Ut = w.Utot + (size_t)m * D * D;
  double2 acc = make_double2(0.0, 0.0);
  for (int e = tm.lane; e < D * D; e += T) {
    Ut[e] = Pc[e];
    acc = cmac_cj(acc, p.target_op[e], Pc[e]);
  }
  double2 z = team_sum<T>(tm, acc, red);
  if (tm.lane == 0) {
    z.x /= p.D;
    z.y /= p.D;
    double f;
    double2 kap;
    fid_kappa(z, p.fid, p.grad_mode, f, kap);
    const double sc = p.m_weight[m] / p.D;
    w.z[m] = z;
    w.kap[m] = make_double2(kap.x * sc, kap.y * sc);
    w.Fm[m] = f;
  }
}

template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_chain_states_fwd(ProbDev p, WorkDev w, int store) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  const int np = p.n_pairs;
  const int pan = np * D;
  const int per_team = (2 * D * D > 2 * pan ? 2 * D * D : 2 * pan) + T;
  double2 *base, *red;
  team_slot<D>(smem, per_team, team, base, red);
  double2* Ps = base;  // [np][D]
  for (int e = tm.lane; e < pan; e += T) Ps[e] = p.psi_init[e];
  tm.sync();
  const double2* Um = w.U + (size_t)m * p.n_t * D * D;
  for (int k = 0; k < p.n_t; ++k) {
    if (store) {
      double2* dst = w.psi + ((size_t)m * (p.n_t + 1) + k) * pan;
      for (int e = tm.lane; e < pan; e += T) dst[e] = Ps[e];
    }
    const double2* Uk = Um + (size_t)k * D * D;
    // Each lane forms its outputs in registers, then the team writes.
    double2 outv[(D * 8 + T - 1) / T > 0 ? (D * 8 + T - 1) / T : 1];
    int cnt = 0;
    for (int e = tm.lane; e < pan; e += T, ++cnt) {
      const int s = e / D, r = e % D;
      double2 acc = make_double2(0.0, 0.0);
      for (int q = 0; q < D; ++q) acc = cmac(acc, Uk[r + D * q], Ps[s * D + q]);
      if (cnt < (int)(sizeof(outv) / sizeof(outv[0]))) outv[cnt] = acc;
    }
    tm.sync();
    cnt = 0;
    for (int e = tm.lane; e < pan; e += T, ++cnt) Ps[e] = outv[cnt];
    tm.sync();
  }
  if (store) {
    double2* dst = w.psi + ((size_t)m * (p.n_t + 1) + p.n_t) * pan;
    for (int e = tm.lane; e < pan; e += T) dst[e] = Ps[e];
  }
  double Fm = 0.0;
  for (int s = 0; s < np; ++s) {
    double2 acc = make_double2(0.0, 0.0);
    for (int r = tm.lane; r < D; r += T) acc = cmac_cj(acc, p.psi_targ[s * D + r], Ps[s * D + r]);
    const double2 z = team_sum<T>(tm, acc, red);
    double f;
    double2 kap;
    fid_kappa(z, p.fid, p.grad_mode, f, kap);
    Fm += f;
    if (tm.lane == 0) {
      const double wgt = p.m_weight[m];
      w.z[(size_t)m * np + s] = z;
      w.kap[(size_t)m * np + s] = make_double2(kap.x * wgt, kap.y * wgt);
    }
  }
  if (tm.lane == 0) w.Fm[m] = Fm;
}

// Trajectory tracking (GRAPETracking.jl:166-277).  The reference propagates
// density matrices rho[n+1] = U_n rho[n] U_n'; with rho[0] = psi0 psi0' that
// is rho[n] = psi[n] psi[n]' exactly, so the chain carries the state vectors
// (D^2 per slice instead of 2 D^3) and the objective of member m is
//   F_m = sum_s sum_c w_c Re <psi_s[j_c]| rho_c |psi_s[j_c]>.
// Every state is stored: the backward chain and the gradient read them.
template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_track_fwd(ProbDev p, WorkDev w) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  const int np = p.n_pairs;
  const int pan = np * D;
  const int per_team = (2 * D * D > 2 * pan ? 2 * D * D : 2 * pan) + T;
  double2 *base, *red;
  team_slot<D>(smem, per_team, team, base, red);
  double2* Ps = base;  // [np][D]
  double2* Pm = w.psi + (size_t)m * (p.n_t + 1) * pan;
  for (int e = tm.lane; e < pan; e += T) {
    Ps[e] = p.psi_init[e];
    Pm[e] = Ps[e];
  }
  tm.sync();
  const double2* Um = w.U + (size_t)m * p.n_t * D * D;
  double Fm = 0.0;
  int c = 0;
  for (int k = 0; k < p.n_t; ++k) {
    const double2* Uk = Um + (size_t)k * D * D;
    double2 outv[(D * 8 + T - 1) / T > 0 ? (D * 8 + T - 1) / T : 1];
    int cnt = 0;
    for (int e = tm.lane; e < pan; e += T, ++cnt) {
      const int s = e / D, r = e % D;
      double2 acc = make_double2(0.0, 0.0);
      for (int q = 0; q < D; ++q) acc = cmac(acc, Uk[r + D * q], Ps[s * D + q]);
      if (cnt < (int)(sizeof(outv) / sizeof(outv[0]))) outv[cnt] = acc;
    }
    tm.sync();
    cnt = 0;
    double2* dst = Pm + (size_t)(k + 1) * pan;
    for (int e = tm.lane; e < pan; e += T, ++cnt) {
      Ps[e] = outv[cnt];
      dst[e] = outv[cnt];
    }
    tm.sync();
    for (; c < p.n_ck && p.ck_step[c] == k + 1; ++c) {  // checkpoints after slice k
      const double2* R = p.ck_target + (size_t)c * D * D;
      double acc = 0.0;
      for (int e = tm.lane; e < pan; e += T) {
        const int s = e / D, r = e % D;
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < D; ++q) t = cmac(t, R[r + D * q], Ps[s * D + q]);
        const double2 v = Ps[e];
        acc = fma(v.x, t.x, fma(v.y, t.y, acc));  // Re(conj(psi_r) (rho psi)_r)
      }
      Fm = fma(p.ck_weight[c], team_sum<T>(tm, make_double2(acc, 0.0), red).x, Fm);
    }
  }
  if (tm.lane == 0) w.Fm[m] = Fm;
}

// Tracking co-state as vectors: chi_s[k] = Lambda[k] psi_s[k], where the
// reference's matrix co-state (Lambda += 2 w_c (rho_c - rho) at a checkpoint,
// Lambda <- U' Lambda U) is the same for every pair, gives
//   chi_s[k] = U_k' chi_s[k+1] + sum_{c: j_c = k} 2 w_c rho_c psi_s[k].
// The -rho part of the reference's source adds -2 w_c |psi|^2 psi to chi,
// whose contribution Im <psi|Op|psi> to the gradient is identically zero; it
// is left out.  lam[k] = scale * chi[k]: scale = 2 w_m for the reference's
// formula (its gradient is -dt Re(i Tr(Lambda' [H_k, rho])) = 2 dt Im <chi|H_k|psi>),
// w_m for the exact gradient (d rho = dU rho U' + h.c. gives
// Re Tr(L(A, psi[k] chi[k+1]') E_k)).
template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_track_bwd(ProbDev p, WorkDev w) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  const int np = p.n_pairs;
  const int pan = np * D;
  const int per_team = (2 * D * D > 2 * pan ? 2 * D * D : 2 * pan) + T;
  double2 *base, *red;
  team_slot<D>(smem, per_team, team, base, red);
  double2* Ls = base;
  const double scl = (p.grad_mode == GRAD_EXACT ? 1.0 : 2.0) * p.m_weight[m];
  const double2* Pm = w.psi + (size_t)m * (p.n_t + 1) * pan;
  double2* Lm = w.lam + (size_t)m * (p.n_t + 1) * pan;
  const double2* Um = w.U + (size_t)m * p.n_t * D * D;
  for (int e = tm.lane; e < pan; e += T) Ls[e] = make_double2(0.0, 0.0);
  int c = p.n_ck - 1;
  for (int k = p.n_t; k >= 1; --k) {
    const double2* psk = Pm + (size_t)k * pan;
    for (; c >= 0 && p.ck_step[c] == k; --c) {  // each lane updates the entries it owns
      const double2* R = p.ck_target + (size_t)c * D * D;
      const double tw = 2.0 * p.ck_weight[c];
      for (int e = tm.lane; e < pan; e += T) {
        const int s = e / D, r = e % D;
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < D; ++q) t = cmac(t, R[r + D * q], psk[s * D + q]);
        Ls[e].x = fma(tw, t.x, Ls[e].x);
        Ls[e].y = fma(tw, t.y, Ls[e].y);
      }
    }
    tm.sync();
    for (int e = tm.lane; e < pan; e += T) Lm[(size_t)k * pan + e] = make_double2(scl * Ls[e].x, scl * Ls[e].y);
    const double2* Uk = Um + (size_t)(k - 1) * D * D;
    double2 outv[(D * 8 + T - 1) / T > 0 ? (D * 8 + T - 1) / T : 1];
    int cnt = 0;
    for (int e = tm.lane; e < pan; e += T, ++cnt) {
      const int s = e / D, r = e % D;
      double2 acc = make_double2(0.0, 0.0);
      for (int q = 0; q < D; ++q) acc = cmac_cj(acc, Uk[q + D * r], Ls[s * D + q]);
      if (cnt < (int)(sizeof(outv) / sizeof(outv[0]))) outv[cnt] = acc;
    }
    tm.sync();
    cnt = 0;
    for (int e = tm.lane; e < pan; e += T, ++cnt) Ls[e] = outv[cnt];
    tm.sync();
  }
  for (int e = tm.lane; e < pan; e += T) Lm[e] = make_double2(scl * Ls[e].x, scl * Ls[e].y);
  (void)red;
}

// --------------------------------------------------------------------------
// Stage 3: backward chains
// --------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_chain_gate_bwd(ProbDev p, WorkDev w) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  double2 *base, *red;
  team_slot<D>(smem, 2 * D * D + T, team, base, red);
  double2* Lam = base;
  double2* Buf = base + D * D;
  const double2 kap = w.kap[m];
  // Lambda_{n-1} = kappa T'   (kappa carries the member weight and 1/D)
  for (int e = tm.lane; e < D * D; e += T) {
    const int r = e % D, c = e / D;
    const double2 t = p.target_op[c + D * r];
    Lam[e] = cmul(kap, make_double2(t.x, -t.y));
  }
  tm.sync();
  const double2* Um = w.U + (size_t)m * p.n_t * D * D;
  double2* Pm = w.P + (size_t)m * p.n_t * D * D;
  const bool grape = (p.grad_mode == GRAD_REF_GRAPE);
  for (int k = p.n_t - 1; k >= 0; --k) {
    if (grape) {  // Gradients.jl: the costate includes the slice's own U_k
      for (int e = tm.lane; e < D * D; e += T) Buf[e] = Um[(size_t)k * D * D + e];
      tm.sync();
      mm1<D, T>(tm, Lam, Lam, Buf);
    }
    for (int e = tm.lane; e < D * D; e += T) Buf[e] = Pm[(size_t)k * D * D + e];
    tm.sync();
    mm1<D, T>(tm, Pm + (size_t)k * D * D, Buf, Lam);  // M_k = P_k Lambda
    if (!grape) {
      for (int e = tm.lane; e < D * D; e += T) Buf[e] = Um[(size_t)k * D * D + e];
      tm.sync();
      mm1<D, T>(tm, Lam, Lam, Buf);
    }
  }
  (void)red;
}

template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_chain_states_bwd(ProbDev p, WorkDev w) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  const int np = p.n_pairs;
  const int pan = np * D;
  const int per_team = (2 * D * D > 2 * pan ? 2 * D * D : 2 * pan) + T;
  double2 *base, *red;
  team_slot<D>(smem, per_team, team, base, red);
  double2* Ls = base;
  // lambda_n = conj(kappa_s) t_s, so that lambda' E psi = kappa_s <t_s|...>
  for (int e = tm.lane; e < pan; e += T) {
    const double2 kp = w.kap[(size_t)m * np + e / D];
    Ls[e] = cmul(make_double2(kp.x, -kp.y), p.psi_targ[e]);
  }
  tm.sync();
  double2* Lm = w.lam + (size_t)m * (p.n_t + 1) * pan;
  for (int e = tm.lane; e < pan; e += T) Lm[(size_t)p.n_t * pan + e] = Ls[e];
  const double2* Um = w.U + (size_t)m * p.n_t * D * D;
  for (int k = p.n_t - 1; k >= 0; --k) {
    const double2* Uk = Um + (size_t)k * D * D;
    double2 outv[(D * 8 + T - 1) / T > 0 ? (D * 8 + T - 1) / T : 1];
    int cnt = 0;
    for (int e = tm.lane; e < pan; e += T, ++cnt) {
      const int s = e / D, r = e % D;
      double2 acc = make_double2(0.0, 0.0);
      for (int q = 0; q < D; ++q) acc = cmac_cj(acc, Uk[q + D * r], Ls[s * D + q]);
      if (cnt < (int)(sizeof(outv) / sizeof(outv[0]))) outv[cnt] = acc;
    }
    tm.sync();
    cnt = 0;
    for (int e = tm.lane; e < pan; e += T, ++cnt) {
      Ls[e] = outv[cnt];
      Lm[(size_t)k * pan + e] = outv[cnt];
    }
    tm.sync();
  }
  (void)red;
}

// --------------------------------------------------------------------------
// Stage 4: per-slice gradient contributions
// --------------------------------------------------------------------------
// g_j = Re(c dt scale Tr(X C_j)), X in the team's reach (smem or global).
template <int D, int T>
__device__ __forceinline__ void trace_controls(const Team<T>& tm, const ProbDev& p, const double2* X,
                                               int m, int k, double* Gout, double2* red) {
  const double cds = p.dt[k] * p.m_scale[m];
  for (int j = 0; j < p.n_c; ++j) {
    const double2* Cj = p.ctrls + (size_t)j * D * D;
    double2 acc = make_double2(0.0, 0.0);
    for (int e = tm.lane; e < D * D; e += T) {
      const int r = e % D, c = e / D;
      acc = cmac(acc, X[e], Cj[c + D * r]);
    }
    const double2 t = team_sum<T>(tm, acc, red);
    if (tm.lane == 0) Gout[j] = cds * (p.gen == GEN_HERM ? t.y : t.x);
  }
}

template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_grad(ProbDev p, WorkDev w) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  double2* base;
  double2* red;
  if constexpr (G::SLAB) {
    base = w.slab + (size_t)blockIdx.x * G::NBUF * D * D;
    red = smem + (size_t)team * T;
  } else {
    base = smem + (size_t)team * G::NBUF * D * D;
    red = smem + (size_t)G::TPC * G::NBUF * D * D + (size_t)team * T;
  }
  const Work<double2, D> W = Work<double2, D>::at(base);
  const int np = p.n_pairs;
  const int pan = np * D;
  const bool exact = (p.grad_mode == GRAD_EXACT);
  const long items = (long)p.n_members * p.n_t;
  for (long it = (long)blockIdx.x * G::TPC + team; it < items; it += (long)gridDim.x * G::TPC) {
    const int m = (int)(it / p.n_t), k = (int)(it % p.n_t);
    double* Gout = w.Gm + ((size_t)m * p.n_t + k) * p.n_c;
    const double2* X;
    if (p.target == TGT_GATE) {
      const double2* Mk = w.P + ((size_t)m * p.n_t + k) * D * D;
      if (!exact) {
        trace_controls<D, T>(tm, p, Mk, m, k, Gout, red);
        continue;
      }
      for (int e = tm.lane; e < D * D; e += T) W.dB[e] = Mk[e];
    } else {
      // tracking's reference formula pairs the co-state with the state after
      // the slice (GRAPETracking.jl:256-262); every other form with the one before
      const int pk = (p.n_ck > 0 && !exact) ? k + 1 : k;
      const double2* psi = w.psi + ((size_t)m * (p.n_t + 1) + pk) * pan;
      const int li = (p.grad_mode == GRAD_REF_GRAPE) ? k : k + 1;
      const double2* lam = w.lam + ((size_t)m * (p.n_t + 1) + li) * pan;
      if (!exact) {
        // g_j = Re(c dt scale sum_s lambda_s' C_j psi_s)
        const double cds = p.dt[k] * p.m_scale[m];
        for (int j = 0; j < p.n_c; ++j) {
          const double2* Cj = p.ctrls + (size_t)j * D * D;
          double2 acc = make_double2(0.0, 0.0);
          for (int e = tm.lane; e < D * D; e += T) {
            const int r = e % D, c = e / D;
            double2 lp = make_double2(0.0, 0.0);
            for (int s = 0; s < np; ++s) lp = cmac_cj(lp, lam[s * D + r], psi[s * D + c]);
            acc = cmac(acc, lp, Cj[e]);
          }
          const double2 t = team_sum<T>(tm, acc, red);
          if (tm.lane == 0) Gout[j] = cds * (p.gen == GEN_HERM ? t.y : t.x);
        }
        continue;
      }
      // M = sum_s psi_s lambda_s'
      for (int e = tm.lane; e < D * D; e += T) {
        const int r = e % D, c = e / D;
        double2 acc = make_double2(0.0, 0.0);
        for (int s = 0; s < np; ++s) {
          const double2 l = lam[s * D + c];
          acc = cmac(acc, psi[s * D + r], make_double2(l.x, -l.y));
        }
        W.dB[e] = acc;
      }
    }
    // Exact: X = L_f(A_k, M_k) with the same degree/squarings as stage 1.
    build_A<D, T>(tm, p, w.u, m, k, W.B);
    tm.sync();
    const double nrm = norm1<D, T>(tm, W.B, reinterpret_cast<double*>(red));
    int deg, s;
    choose_degree(nrm, c_theta64, deg, s);
    const double sc = ldexp(1.0, -s);
    for (int e = tm.lane; e < D * D; e += T) {
      W.B[e] = cscale(W.B[e], sc);
      W.dB[e] = cscale(W.dB[e], sc);
    }
    tm.sync();
    taylor_exp_frechet<D, T>(tm, W, deg, s, c_invf);
    X = W.dY;
    trace_controls<D, T>(tm, p, X, m, k, Gout, red);
    tm.sync();
  }
}

// --------------------------------------------------------------------------
// Stage 5: deterministic ensemble reduction
// --------------------------------------------------------------------------
__global__ void k_reduce(ProbDev p, WorkDev w, int want_grad) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = p.n_t * p.n_c;
  if (want_grad && idx < n) {
    double s = 0.0;
    for (int m = 0; m < p.n_members; ++m) s += w.Gm[(size_t)m * n + idx];
    w.G[idx] = s;
  }
  if (idx == 0) {
    double f = 0.0;
    for (int m = 0; m < p.n_members; ++m) f += p.m_weight[m] * w.Fm[m];
    w.F[0] = f;
  }
}

// Oracle-free residual of one evaluation (the PGX_RESID_* kinds of pgx.h),
// one block per member.  Non-negative doubles order like their bit patterns,
// so atomicMax on the bits gives the exact maximum in any order; a NaN (sign
// cleared) sorts above +inf and survives.
constexpr int kResidThreads = 256;

__global__ void __launch_bounds__(kResidThreads) k_residual(ProbDev p, WorkDev w, int kind, int N,
                                                            unsigned long long* out) {
  __shared__ double red[kResidThreads];
  const int m = blockIdx.x;
  const int Dp = p.Dp, D = p.D;
  double r = 0.0;
  auto keep = [&r](double v) {
    v = fabs(v);
    if (!(v <= r)) r = v;
  };
  if (kind == PGX_RESID_UNITARITY) {
    const double2* U = w.Utot + (size_t)m * Dp * Dp;
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
      const int i = e % D, j = e / D;
      double2 acc = make_double2(i == j ? -1.0 : 0.0, 0.0);
      for (int k = 0; k < D; ++k) acc = cmac_cj(acc, U[k + (size_t)Dp * i], U[k + (size_t)Dp * j]);
      keep(hypot(acc.x, acc.y));
    }
  } else if (kind == PGX_RESID_TRACE) {
    const double2* U = w.Utot + (size_t)m * Dp * Dp;
    for (int c = threadIdx.x; c < D; c += blockDim.x) {
      double sx = c % (N + 1) == 0 ? -1.0 : 0.0, sy = 0.0;
      for (int i = 0; i < N; ++i) {
        const double2 v = U[(i + N * i) + (size_t)Dp * c];
        sx += v.x;
        sy += v.y;
      }
      keep(hypot(sx, sy));
    }
  } else if (kind == kResidPairs) {
    for (int s = threadIdx.x; s < p.n_pairs; s += blockDim.x) {
      const double2 v = w.Utot[(size_t)m * p.n_pairs + s];
      keep(hypot(v.x, v.y));
    }
  } else {
    const size_t pan = (size_t)p.n_pairs * Dp;
    const double2* p0 = w.psi + (size_t)m * (p.n_t + 1) * pan;
    const double2* pT = p0 + (size_t)p.n_t * pan;
    for (int s = threadIdx.x; s < p.n_pairs; s += blockDim.x) {
      double ax = 0.0, ay = 0.0;
      if (kind == PGX_RESID_NORM) {
        for (int i = 0; i < D; ++i) {
          const double2 a = pT[(size_t)s * Dp + i], b = p0[(size_t)s * Dp + i];
          ax += (a.x * a.x + a.y * a.y) - (b.x * b.x + b.y * b.y);
        }
      } else {
        for (int i = 0; i < N; ++i) {
          const double2 a = pT[(size_t)s * Dp + i + N * i], b = p0[(size_t)s * Dp + i + N * i];
          ax += a.x - b.x;
          ay += a.y - b.y;
        }
      }
      keep(hypot(ax, ay));
    }
  }
  red[threadIdx.x] = r;
  __syncthreads();
  for (int h = kResidThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h && !(red[threadIdx.x + h] <= red[threadIdx.x])) red[threadIdx.x] = red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(red[0]));
}

// G[q] = sum_i coef[i] Gm[idx[i]][q], members in the order given (the
// worst-case and CVaR ensemble gradients).
__global__ void k_select_sum(const double* Gm, const int* idx, const double* coef, int n_sel, int len, double* G) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= len) return;
  double s = 0.0;
  for (int i = 0; i < n_sel; ++i) s = fma(coef[i], Gm[(size_t)idx[i] * len + q], s);
  G[q] = s;
}

cudaError_t launch_select_sum(const double* Gm, const int* idx, const double* coef, int n_sel, int len, double* G,
                              const LaunchInfo& li) {
  k_select_sum<<<(len + 255) / 256, 256, 0, li.stream>>>(Gm, idx, coef, n_sel, len, G);
  ++*li.launches;
  return cudaGetLastError();
}

// --------------------------------------------------------------------------
// Launchers
// --------------------------------------------------------------------------
template <class K>
static void ensure_smem(K kernel, size_t bytes) {
  set_smem_once((const void*)kernel, bytes);
}

// The dynamic shared-memory limit of a kernel on a device only grows: it is
// raised when a launch needs more than any earlier one (kernels whose shared
// memory depends on the problem -- state pairs, control counts -- meet larger
// needs later), and never lowered, so launches already recorded into a CUDA
// graph stay valid.
void set_smem_once(const void* fn, size_t bytes) {
  if (bytes <= 48 * 1024) return;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> limit;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = limit[{fn, dev}];
  if (bytes > cur) {
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    cur = bytes;
  }
}

template <class K>
static int item_grid(K kernel, int threads, size_t smem, long teams_needed, int tpc, int num_sms,
                     int cap) {
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  if (per_sm < 1) per_sm = 1;
  long blocks = (teams_needed + tpc - 1) / tpc;
  long maxb = (long)num_sms * per_sm;
  if (blocks > maxb) blocks = maxb;
  if (cap > 0 && blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

int slab_team_count(int Dp, int num_sms) { return Dp >= 64 ? 2 * num_sms : 0; }
size_t slab_elems(int Dp, int num_sms) {
  return Dp >= 64 ? (size_t)slab_team_count(Dp, num_sms) * 10 * Dp * Dp : 0;
}

#define PGX_DISPATCH(DP, CALL)                      \
  switch (DP) {                                     \
    case 2: { constexpr int D_ = 2; CALL; } break;  \
    case 4: { constexpr int D_ = 4; CALL; } break;  \
    case 8: { constexpr int D_ = 8; CALL; } break;  \
    case 16: { constexpr int D_ = 16; CALL; } break; \
    case 32: { constexpr int D_ = 32; CALL; } break; \
    case 64: { constexpr int D_ = 64; CALL; } break; \
    default: return cudaErrorInvalidValue;          \
  }

template <int D>
static cudaError_t do_expm(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  using G = Cfg<D>;
  const size_t smem = taylor_smem_bytes<D>();
  ensure_smem(k_expm<D>, smem);
  const int grid = item_grid(k_expm<D>, G::THREADS, smem, (long)p.n_members * p.n_t, G::TPC,
                             li.num_sms, G::SLAB ? w.slab_teams : 0);
  k_expm<D><<<grid, G::THREADS, smem, li.stream>>>(p, w);
  ++*li.launches;
  return cudaGetLastError();
}
cudaError_t launch_expm(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  PGX_DISPATCH(p.Dp, return do_expm<D_>(p, w, li));
  return cudaSuccess;
}

template <int D>
static cudaError_t do_chain_fwd(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool store) {
  using G = Cfg<D>;
  const size_t smem = chain_smem_bytes<D>(p.n_pairs);
  const int grid = (p.n_members + G::TPC - 1) / G::TPC;
  if (p.target == TGT_GATE) {
    ensure_smem(k_chain_gate_fwd<D>, smem);
    k_chain_gate_fwd<D><<<grid, G::THREADS, smem, li.stream>>>(p, w, store ? 1 : 0);
  } else if (p.n_ck > 0) {
    ensure_smem(k_track_fwd<D>, smem);
    k_track_fwd<D><<<grid, G::THREADS, smem, li.stream>>>(p, w);
  } else {
    ensure_smem(k_chain_states_fwd<D>, smem);
    k_chain_states_fwd<D><<<grid, G::THREADS, smem, li.stream>>>(p, w, store ? 1 : 0);
  }
  ++*li.launches;
  return cudaGetLastError();
}
cudaError_t launch_chain_fwd(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool store) {
  PGX_DISPATCH(p.Dp, return do_chain_fwd<D_>(p, w, li, store));
  return cudaSuccess;
}

template <int D>
static cudaError_t do_chain_bwd(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  using G = Cfg<D>;
  const size_t smem = chain_smem_bytes<D>(p.n_pairs);
  const int grid = (p.n_members + G::TPC - 1) / G::TPC;
  if (p.target == TGT_GATE) {
    ensure_smem(k_chain_gate_bwd<D>, smem);
    k_chain_gate_bwd<D><<<grid, G::THREADS, smem, li.stream>>>(p, w);
  } else if (p.n_ck > 0) {
    ensure_smem(k_track_bwd<D>, smem);
    k_track_bwd<D><<<grid, G::THREADS, smem, li.stream>>>(p, w);
  } else {
    ensure_smem(k_chain_states_bwd<D>, smem);
    k_chain_states_bwd<D><<<grid, G::THREADS, smem, li.stream>>>(p, w);
  }
  ++*li.launches;
  return cudaGetLastError();
}
cudaError_t launch_chain_bwd(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  PGX_DISPATCH(p.Dp, return do_chain_bwd<D_>(p, w, li));
  return cudaSuccess;
}

template <int D>
static cudaError_t do_grad(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  using G = Cfg<D>;
  const size_t smem = taylor_smem_bytes<D>();
  ensure_smem(k_grad<D>, smem);
  const int grid = item_grid(k_grad<D>, G::THREADS, smem, (long)p.n_members * p.n_t, G::TPC,
                             li.num_sms, G::SLAB ? w.slab_teams : 0);
  k_grad<D><<<grid, G::THREADS, smem, li.stream>>>(p, w);
  ++*li.launches;
  return cudaGetLastError();
}
cudaError_t launch_grad(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  PGX_DISPATCH(p.Dp, return do_grad<D_>(p, w, li));
  return cudaSuccess;
}

cudaError_t launch_reduce(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool want_grad) {
  const int n = p.n_t * p.n_c;
  const int grid = want_grad ? (n + 255) / 256 : 1;
  k_reduce<<<grid, 256, 0, li.stream>>>(p, w, want_grad ? 1 : 0);
  ++*li.launches;
  return cudaGetLastError();
}

cudaError_t launch_residual(const ProbDev& p, const WorkDev& w, int kind, int N, unsigned long long* out,
                            const LaunchInfo& li) {
  k_residual<<<p.n_members, kResidThreads, 0, li.stream>>>(p, w, kind, N, out);
  ++*li.launches;
  return cudaGetLastError();
}

// 8 independent FMA chains per thread; the result is stored only when it is
// impossible (all-zero inputs keep it finite), which keeps the loop alive.
__global__ void __launch_bounds__(256) k_fp64_peak(double* sink, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-9 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 12345.678) sink[threadIdx.x & 63] = s;
}

__global__ void __launch_bounds__(256) k_fp32_peak(float* sink, int iters, float a, float b) {
  float x[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) x[i] = threadIdx.x * 1e-6f + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = fmaf(x[i], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 16; ++i) s += x[i];
  if (s == 12345.678f) sink[threadIdx.x & 63] = s;
}

cudaError_t launch_fp32_peak(float* sink, const LaunchInfo& li, double* flops) {
  const int blocks = li.num_sms * 8, threads = 256, iters = 65536;
  k_fp32_peak<<<blocks, threads, 0, li.stream>>>(sink, iters, 0.9999f, 1e-4f);
  ++*li.launches;
  *flops = 2.0 * 16.0 * iters * (double)blocks * threads;
  return cudaGetLastError();
}

cudaError_t launch_fp64_peak(double* sink, const LaunchInfo& li, double* flops) {
  const int blocks = li.num_sms * 8, threads = 256, iters = 8192;
  k_fp64_peak<<<blocks, threads, 0, li.stream>>>(sink, iters, 0.999999, 1e-7);
  ++*li.launches;
  *flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  return cudaGetLastError();
}

template <int D>
static cudaError_t do_single(int gen, const double2* Gm, double dt, double2* U, double2* slab,
                             const LaunchInfo& li) {
  using G = Cfg<D>;
  const size_t smem = taylor_smem_bytes<D>();
  ensure_smem(k_single_expm<D>, smem);
  k_single_expm<D><<<1, G::THREADS, smem, li.stream>>>(gen, Gm, dt, U, slab);
  ++*li.launches;
  return cudaGetLastError();
}
cudaError_t launch_single_expm(int Dp, int gen, const double2* Gm, double dt, double2* U,
                               double2* slab, const LaunchInfo& li) {
  PGX_DISPATCH(Dp, return do_single<D_>(gen, Gm, dt, U, slab, li));
  return cudaSuccess;
}

}  // namespace pgx
