// Stage helpers shared by the FP64 kernels (pgx_kernels.cu) and the
// mixed-precision kernels (pgx_mixed.cu): team configuration, generator
// assembly, fidelity chain-rule coefficients and the Taylor constant tables.
#pragma once
#include "pgx_device.cuh"
#include "pgx_internal.h"

namespace pgx {

static __constant__ double c_invf[PGX_N_INVFACT] = PGX_INVFACT_INIT;
static __constant__ double c_theta64[PGX_N_DEGREES] = PGX_THETA64_INIT;

enum { GEN_HERM = 0, GEN_LIOUV = 1 };
enum { TGT_GATE = 0, TGT_STATES = 1 };
enum { FID_SQUARE = 0, FID_REAL = 1, FID_MODULUS = 2 };
enum { GRAD_REF_GRAPE = 0, GRAD_REF_MR = 1, GRAD_EXACT = 2 };

template <int D> struct Cfg {
  static constexpr int T = (D <= 8) ? 32 : 256;    // threads per team
  static constexpr int TPC = (D <= 8) ? 4 : 1;     // teams per CTA
  static constexpr bool SLAB = (D >= 64);          // Taylor workspace in global memory
  static constexpr int NBUF = 10;                  // matrices of Taylor workspace
  static constexpr int THREADS = T * TPC;
};

template <int D> constexpr size_t taylor_smem_bytes() {
  using G = Cfg<D>;
  return (G::SLAB ? 0 : (size_t)G::TPC * G::NBUF * D * D * sizeof(double2)) +
         (size_t)G::TPC * G::T * sizeof(double2);
}
template <int D> constexpr size_t chain_smem_bytes(int n_pairs) {
  using G = Cfg<D>;
  // gate: two matrices; states: two n_pairs x D panels.  Plus reduction scratch.
  const size_t mats = (size_t)2 * D * D;
  const size_t vecs = (size_t)2 * (n_pairs > 0 ? n_pairs : 1) * D;
  return (size_t)G::TPC * ((mats > vecs ? mats : vecs) + G::T) * sizeof(double2);
}

__device__ __forceinline__ double2 times_c(double2 v, int gen) {
  // c = -i for a Hermitian generator, 1 for a Liouvillian.
  if (gen == GEN_HERM) return make_double2(v.y, -v.x);
  return v;
}

// A = c dt_k (drift + off O + scale sum_j u_jk C_j), assembled in FP64 and
// stored as C (double2, or float2 for the FP32 stages).
template <int D, int T, int SW = 0, class C>
__device__ __forceinline__ void build_A(const Team<T>& tm, const ProbDev& p, const double* u, int m,
                                        int k, C* A) {
  const double dt = p.dt[k];
  const double sc = p.m_scale[m], off = p.m_offset[m];
  const double2* Gd = p.drifts + (size_t)p.m_drift[m] * D * D;
  const double* uk = u + (size_t)k * p.n_c;
  const int ro = p.n_ramp ? p.m_ramp[m] : -1;
  const double2* Rm = ro >= 0 ? p.ramp_ops + (size_t)ro * D * D : nullptr;
  const double tk = ro >= 0 ? p.tau[k] : 0.0;
  for (int e = tm.lane; e < D * D; e += T) {
    double2 v = Gd[e];
    const double2 o = p.offset_op[e];
    v.x = fma(off, o.x, v.x);
    v.y = fma(off, o.y, v.y);
    if (Rm) {
      v.x = fma(tk, Rm[e].x, v.x);
      v.y = fma(tk, Rm[e].y, v.y);
    }
    for (int j = 0; j < p.n_c; ++j) {
      const double a = sc * uk[j];
      const double2 c = p.ctrls[(size_t)j * D * D + e];
      v.x = fma(a, c.x, v.x);
      v.y = fma(a, c.y, v.y);
    }
    v.x *= dt;
    v.y *= dt;
    const double2 a = times_c(v, p.gen);
    C out;
    out.x = a.x;
    out.y = a.y;
    A[Lay<D, SW>::idx(e % D, e / D)] = out;
  }
}

// f(z) and the chain-rule coefficient kappa with dF = Re(kappa dz).
__device__ __forceinline__ void fid_kappa(double2 z, int fid, int mode, double& f, double2& kap) {
  const double az = hypot(z.x, z.y);
  if (fid == FID_SQUARE) {
    f = z.x * z.x + z.y * z.y;
    kap = make_double2(2.0 * z.x, -2.0 * z.y);
  } else if (fid == FID_REAL) {
    f = z.x;
    kap = make_double2(1.0, 0.0);
  } else {
    f = az;
    if (az < 1e-14) kap = make_double2(0.0, 0.0);
    else if (mode == GRAD_EXACT) kap = make_double2(z.x / az, -z.y / az);
    else kap = make_double2(1.0 / az, 0.0);  // Objectives.jl:356-361 uses Im(inner/|z|)
  }
}

template <int D>
__device__ __forceinline__ void team_slot(double2* smem, int per_team_elems, int team, double2*& base,
                                          double2*& red) {
  base = smem + (size_t)team * per_team_elems;
  red = base + (per_team_elems - Cfg<D>::T);
}

static __constant__ float c_invf32[PGX_N_INVFACT] = PGX_INVFACT32_INIT;
// The FP32 thresholds for the mixed gradient, which chooses its degree
// without touching the FP64 pipe (the norm it compares carries a 1e-5 safety
// margin, far above the float rounding of a threshold).
static __constant__ float c_theta32f[PGX_N_DEGREES] = PGX_THETA32_INIT;

}  // namespace pgx
