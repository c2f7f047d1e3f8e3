// Mixed-precision kernels (PGX_PREC_MIXED), gate targets.
//
// GB300 issues FP32 at 64x its FP64 rate, so the FP64 pipeline is replaced
// stage by stage with the cheapest arithmetic that keeps the objective at
// near-FP64 accuracy:
//   expm       df (double-float) Paterson-Stockmeyer Taylor; degree and
//              squarings from the FP64 1-norm and the FP64 theta table, so the
//              truncation error stays at the FP64 level.  U stack = df (float4).
//   chain_fwd  df products P_{k+1} = U_k P_k; the total propagator and the
//              overlap Tr(T'U)/D are formed in FP64 from the df chain; the
//              float rounding of P_k is stored for the gradient.
//   chain_bwd  FP32: Lambda <- Lambda U_k, M_k = P_k Lambda (only the
//              gradient depends on it).
//   grad       FP32 Frechet derivative L(A_k, M_k) (degree from the FP32 theta
//              table) and traces; results accumulated as FP64.
// F therefore carries df (~1e-13 per product) rounding; G carries FP32
// (~1e-6 relative) rounding.
#include <atomic>
#include <type_traits>

#include "pgx_df.cuh"
#include "pgx_stages.cuh"

namespace pgx {

static __constant__ df c_dfcoef[PGX_N_INVFACT] = PGX_INVFACT_DF_INIT;

// Shared-memory layout of the team matrices (Lay<D, SW>).  Measured on GB300:
// the XOR swizzle removes bank conflicts but its index arithmetic costs more
// than the conflicts do, so it is not used.
// The FP32 gradient is bound by shared-memory bandwidth, not FMAs: with
// leading dimension D the columns a warp reads at one k share a bank.  It
// keeps its Taylor workspace padded to leading dimension D + 1.
constexpr int kSwzGrad = 2;
constexpr int kSwzExpm = 2;

// Teams of the slice-parallel mixed kernels.  A team of T threads owns one
// matrix problem; a CTA holds 256 / T teams (T = 32: independent warps on
// __syncwarp; 64 and 128: hardware barriers 1..; 256: the whole CTA).  Each
// lane owns an RB x CB block of every product (Blocking<D, T>).  The
// workspace is 80 bytes x D^2 per team (five df matrices for the propagator,
// ten complex-float ones for the gradient), in shared memory up to D = 32 and
// in a per-CTA global slab at D = 64.  The best T depends on the kernel and on
// D (occupancy against barrier waits); pgx_autotune picks it per problem.  All
// variants sum every dot product in the same order: results are identical.
template <int D, int T> struct CfgM {
  static constexpr bool SLAB = (D >= 64);
  static constexpr int TPC = (T >= 256) ? 1 : 256 / T;
  static constexpr int THREADS = T * TPC;
  static constexpr size_t WS = (size_t)80 * D * D;                 // workspace bytes per team
  static constexpr size_t RED = (size_t)2 * T * sizeof(float2);    // reduction scratch per team
  static constexpr size_t SMEM = (SLAB ? 0 : TPC * WS) + TPC * RED;
  // expm kernel: five df matrices in the padded layout
  static constexpr size_t WSE = (size_t)5 * Lay<D, 2>::SIZE * sizeof(float4);
  static constexpr size_t SMEM_E = (SLAB ? 0 : TPC * WSE) + TPC * RED;
  // gradient kernel: the q = 2 Paterson-Stockmeyer Frechet form, six
  // complex-float matrices in the padded layout (fits shared memory at D = 64;
  // at the norms of short slices it is also the cheaper form, below)
  static constexpr size_t WSG = (size_t)6 * Lay<D, 2>::SIZE * sizeof(float2);
  static constexpr size_t SMEM_G = TPC * WSG + TPC * RED;
};

template <int D, int T>
__device__ __forceinline__ Team<T> team_of() {
  Team<T> tm{(int)(threadIdx.x % T)};
  tm.bar = (T > 32 && CfgM<D, T>::TPC > 1) ? 1 + (int)(threadIdx.x / T) : 0;
  return tm;
}

// ---- per-slice prologue without the FP64 pipe -----------------------------------
// GB300 runs FP64 at 1/64 of its FP32 rate, so an FP64 assembly of A_k and an
// FP64 1-norm cost as much pipe time as the products they feed.  The mixed
// kernels assemble A_k from df copies of the constants (expm: df arithmetic,
// gradient: FP32) and take the 1-norm in FP32.

__global__ void k_prep_mx(const double* u, float2* u_df, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double x = u[i];
    const float hi = (float)x;
    u_df[i] = make_float2(hi, (float)(x - (double)hi));
  }
}

__device__ __forceinline__ df df_ld(const float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

// Entry q (= r + D c) of A = c dt_k (drift + off O + tau_k R + scale
// sum_j u_jk C_j) in df for member m, slice k; u(j) gives control j of slice
// k as df.
template <int D, class U>
__device__ __forceinline__ dfc gen_entry_df(const ProbDev& p, int m, int k, int q, U u) {
  const df dt = df_ld(p.dt_df[k]), sc = df_ld(p.m_scale_df[m]), off = df_ld(p.m_offset_df[m]);
  const float4* Gd = p.drifts_df + (size_t)p.m_drift[m] * D * D;
  const int ro = p.n_ramp ? p.m_ramp[m] : -1;
  dfc v = dfc_load(Gd[q]);
  if (off.hi != 0.f) v = dfc_add(v, dfc_scale(dfc_load(p.offset_df[q]), off));
  if (ro >= 0) v = dfc_add(v, dfc_scale(dfc_load(p.ramp_ops_df[(size_t)ro * D * D + q]), df_ld(p.tau_df[k])));
  for (int j = 0; j < p.n_c; ++j) {
    const df a = df_mul(sc, u(j));
    v = dfc_add(v, dfc_scale(dfc_load(p.ctrls_df[(size_t)j * D * D + q]), a));
  }
  v = dfc_scale(v, dt);
  if (p.gen == GEN_HERM) v = {v.im, df_neg(v.re)};  // times -i
  return v;
}

// The whole A into a team's matrix (layout SW).
template <int D, int T, int SW>
__device__ __forceinline__ void build_A_df(const Team<T>& tm, const ProbDev& p, const WorkDev& w, int m,
                                           int k, float4* A) {
  const float2* uk = w.u_df + (size_t)k * p.n_c;
  const auto u = [=](int j) { return df_ld(uk[j]); };
  for (int q = tm.lane; q < D * D; q += T) A[Lay<D, SW>::idx(q % D, q / D)] = dfc_store(gen_entry_df<D>(p, m, k, q, u));
}

// The same in FP32 from the FP32 copies of the constants (the leading halves
// of the df copies).
template <int D, int T, int SW>
__device__ __forceinline__ void build_A32(const Team<T>& tm, const ProbDev& p, const WorkDev& w, int m,
                                          int k, float2* A) {
  const float dt = p.dt_df[k].x, sc = p.m_scale_df[m].x, off = p.m_offset_df[m].x;
  const float2* Gd = p.drifts_f32 + (size_t)p.m_drift[m] * D * D;
  const float2* uk = w.u_df + (size_t)k * p.n_c;
  const int ro = p.n_ramp ? p.m_ramp[m] : -1;
  const float4* Rm = ro >= 0 ? p.ramp_ops_df + (size_t)ro * D * D : nullptr;
  const float tk = ro >= 0 ? p.tau_df[k].x : 0.f;
  for (int q = tm.lane; q < D * D; q += T) {
    const float2 g = Gd[q];
    const float2 o = p.offset_f32[q];
    float vx = fmaf(off, o.x, g.x), vy = fmaf(off, o.y, g.y);
    if (Rm) {
      vx = fmaf(tk, Rm[q].x, vx);
      vy = fmaf(tk, Rm[q].y, vy);
    }
    for (int j = 0; j < p.n_c; ++j) {
      const float a = sc * uk[j].x;
      const float2 c = p.ctrls_f32[(size_t)j * D * D + q];
      vx = fmaf(a, c.x, vx);
      vy = fmaf(a, c.y, vy);
    }
    vx *= dt;
    vy *= dt;
    A[Lay<D, SW>::idx(q % D, q / D)] = (p.gen == GEN_HERM) ? make_float2(vy, -vx) : make_float2(vx, vy);
  }
}

// 1-norm from the FP32 (leading) parts, enlarged by 1e-5 to cover their
// rounding: it only selects the Taylor degree and the squarings, whose
// thresholds are tail bounds.
template <int D, int T, int SW, class C>
__device__ __forceinline__ float norm1f(const Team<T>& tm, const C* A, float* scratch) {
  float best = 0.f;
  for (int c = tm.lane; c < D; c += T) {
    float s = 0.f;
    for (int r = 0; r < D; ++r) {
      const C a = A[Lay<D, SW>::idx(r, c)];
      s += sqrtf(fmaf(a.x, a.x, a.y * a.y));
    }
    best = fmaxf(best, s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
  if constexpr (T > 32) {  // max over the team's warps (exact in any order)
    if (tm.lane % 32 == 0) scratch[tm.lane / 32] = best;
    tm.sync();
#pragma unroll
    for (int w = 0; w < T / 32; ++w) best = fmaxf(best, scratch[w]);
    tm.sync();
  }
  return best * 1.00001f;
}

// First Horner step of the df Taylor polynomial (block size q) that may run
// in FP32.  Step i computes B^q Y with ||B^q|| <= a^q and ||Y|| <= e^a /
// (q(i+1))!, and its error reaches the result through i more factors B^q:
// bound D u32 a^(q(i+1)) e^a / (q(i+1))!, required below 2^-47.  Step 0 stays
// in df.
__device__ __forceinline__ int lo_horner_from(float a, int L, int D, int q) {
  float aq = a;
#pragma unroll 1
  for (int j = 1; j < q; ++j) aq *= a;
  float pw = aq, fact = 1.f;  // a^(q(i+1)), (q(i+1))! for i = 0
#pragma unroll 1
  for (int j = 2; j <= q; ++j) fact *= (float)j;
  const float lim = 7.1e-15f / (float)D / 5.96e-8f / __expf(a);
#pragma unroll 1
  for (int i = 0; i < L - 1; ++i) {
    if (i >= 1 && pw / fact <= lim) return i;
    pw *= aq;
#pragma unroll 1
    for (int j = q * (i + 1) + 1; j <= q * (i + 2); ++j) fact *= (float)j;
  }
  return 1 << 30;
}

// Degree m = q L, block size q in {2, 3, 4} and squarings s of the df expm:
// every degree whose df threshold theta_m (tail <= 2^-47) admits ||A|| / 2^s,
// costed in twentieths of a df product by what it executes:
//  - the q - 1 power products (16 each when triangular, else 20);
//  - the df Horner steps (20 each);
//  - the Horner steps lo_horner_from moves to FP32 (5 each);
//  - the s squarings (20 each).
// The 21 candidates (q = 4: L = 1..5, q = 3: L = 1..6, q = 2: L = 1..10, in
// that order) are costed one per lane of the team's first warp; the exact
// integer minimum, ties to the earlier candidate, is broadcast through
// `scratch`.  Returns m | q << 5 | s << 8 | min(lo_from, 31) << 16.
static __constant__ float c_thetadf_all[PGX_N_INVFACT - 1] = PGX_THETADF_ALL_INIT;
constexpr int kTriPowCost = 16, kPowCost = 20, kLoHornerCost = 5;
template <int T>
__device__ __forceinline__ int choose_expm_df(const Team<T>& tm, float nrm, int D, bool tri, int* scratch) {
  if (tm.lane < 32) {
    const int t = tm.lane;
    const int qq = (t < 5) ? 4 : (t < 11) ? 3 : 2;
    const int L = (t < 5) ? t + 1 : (t < 11) ? t - 4 : t - 10;
    long long key = 0x7fffffffffffffffLL;
    int packed = 0;
    if (t < 21) {
      const int mm = qq * L;
      int si = 0;
      float x = nrm;
      while (x > c_thetadf_all[mm - 1] && si < 60) { x *= 0.5f; ++si; }
      const int lo = lo_horner_from(x, L, D, qq);
      const int n_df = lo < L - 1 ? lo : L - 1;  // Horner steps i = L-2 .. 0 below lo run in df
      const int cost = (qq - 1) * (tri ? kTriPowCost : kPowCost) + 20 * n_df + kLoHornerCost * (L - 1 - n_df) + 20 * si;
      key = (long long)cost * 32 + t;
      packed = mm | (qq << 5) | (si << 8) | ((lo < 31 ? lo : 31) << 16);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ok = __shfl_xor_sync(0xffffffffu, key, o);
      const int op = __shfl_xor_sync(0xffffffffu, packed, o);
      if (ok < key) { key = ok; packed = op; }
    }
    if (t == 0) *scratch = packed;
  }
  tm.sync();
  const int r = *scratch;
  tm.sync();
  return r;
}

// Degree m and squarings s of the q = 2 Frechet form: 3 (m/2 + s) product
// units (X and dX, then per Horner step and per squaring dY and Y), fewest
// first, ties to the lower degree.  At m = 4 this is 6 units against 9 for the
// q = 4 form, which needs B^2, B^3, B^4 and their derivatives.
__device__ __forceinline__ void choose_degree_q2(float nrm, const float* theta, int& m, int& s) {
  int best = 1 << 30;
  m = 4;
  s = 0;
#pragma unroll
  for (int i = 0; i < PGX_N_DEGREES; ++i) {
    int si = 0;
    float x = nrm;
    while (x > theta[i] && si < 60) { x *= 0.5f; ++si; }
    const int cost = 2 * (i + 1) + si;  // m/2 + s
    if (cost < best) { best = cost; m = 4 * (i + 1); s = si; }
  }
}

// ---- expm in df --------------------------------------------------------------
// Register budget: as many CTAs per SM as shared memory admits (at most 5;
// two at D = 64, whose workspace lies in global memory).
template <int D, int T> constexpr int expm_min_ctas() {
  constexpr size_t kSmemSm = 227 * 1024;
  constexpr size_t n = CfgM<D, T>::SLAB ? 2 : kSmemSm / CfgM<D, T>::SMEM_E;
  return n < 1 ? 1 : n > 5 ? 5 : (int)n;
}
// KIND: kExpmFull (general generator), kExpmHerm (Hermitian: triangular
// powers), kExpmLSym (Hermiticity-preserving superoperator at D = 64: half
// of every product).
enum { kExpmFull = 0, kExpmHerm = 1, kExpmLSym = 2 };
// One unit (member m, slice k) of the df expm by one team; its five
// workspace matrices at `base`, reduction scratch `red`.  U_DOUBLE: the
// controls come from w.u (FP64) rounded to df here, with the same values as
// the prologue's df copy w.u_df.
template <int D, int T, int KIND, bool U_DOUBLE>
__device__ __forceinline__ void expm_unit(const Team<T>& tm, const ProbDev& p, const WorkDev& w, int m, int k,
                                          float4* base, float4* red) {
  constexpr bool HERM = KIND == kExpmHerm, LSYM = KIND == kExpmLSym;
  using G = CfgM<D, T>;
  using L = Lay<D, kSwzExpm>;
  float4* B = base;
  float4* B2 = base + L::SIZE;
  float4* B3 = base + 2 * L::SIZE;
  float4* B4 = base + 3 * L::SIZE;
  float4* Y = base + 4 * L::SIZE;
  if constexpr (U_DOUBLE) {
    const double* uk = w.u + (size_t)k * p.n_c;
    const auto u = [=](int c) { return df_from(uk[c]); };
    for (int q = tm.lane; q < D * D; q += T) B[L::idx(q % D, q / D)] = dfc_store(gen_entry_df<D>(p, m, k, q, u));
  } else {
    build_A_df<D, T, kSwzExpm>(tm, p, w, m, k, B);
  }
  tm.sync();
  const float nrm = norm1f<D, T, kSwzExpm>(tm, B, reinterpret_cast<float*>(red));
  const int pk = choose_expm_df<T>(tm, nrm, D, HERM && D >= 16, reinterpret_cast<int*>(red));
  const int deg = pk & 31, q = (pk >> 5) & 7, s = (pk >> 8) & 63;
  const int lo_from = (pk >> 16) >= 31 ? 1 << 30 : (pk >> 16);
  if (s > 0) {  // B <- B / 2^s, exact in df
    const float sc = ldexpf(1.f, -s);
    for (int q = tm.lane; q < D * D; q += T) {  // same lane wrote this entry above
      const int e = L::idx(q % D, q / D);
      const float4 a = B[e];
      B[e] = make_float4(a.x * sc, a.y * sc, a.z * sc, a.w * sc);
    }
    tm.sync();
  }
  taylor_exp_df<D, T, kSwzExpm, HERM, LSYM>(tm, B, B2, B3, B4, Y, deg, q, s, c_dfcoef, lo_from);
  float4* out = reinterpret_cast<float4*>(w.U) + ((size_t)m * p.n_t + k) * D * D;
  if constexpr (G::SLAB) {
    // the U stack streams out (gigabytes, read back from DRAM by the
    // chains): evict-first stores keep the per-CTA Taylor slab in L2
    for (int e = tm.lane; e < D * D; e += T) __stcs(out + e, Y[L::idx(e % D, e / D)]);
  } else {
    for (int e = tm.lane; e < D * D; e += T) out[e] = Y[L::idx(e % D, e / D)];
  }
  tm.sync();
}

template <int D, int T, int KIND>
__global__ void __launch_bounds__(CfgM<D, T>::THREADS, expm_min_ctas<D, T>()) k_expm_mx(ProbDev p, WorkDev w) {
  using G = CfgM<D, T>;
  using L = Lay<D, kSwzExpm>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int team = threadIdx.x / T;
  const Team<T> tm = team_of<D, T>();
  float4* base;
  if constexpr (G::SLAB)
    base = reinterpret_cast<float4*>(w.slab) + (size_t)blockIdx.x * 5 * L::SIZE;
  else
    base = reinterpret_cast<float4*>(smem_raw + (size_t)team * G::WSE);
  float4* red = reinterpret_cast<float4*>(smem_raw + (G::SLAB ? 0 : G::TPC * G::WSE) + (size_t)team * G::RED);
  const long items = (long)p.n_members * p.n_t;
  for (long it = (long)blockIdx.x * G::TPC + team; it < items; it += (long)gridDim.x * G::TPC)
    expm_unit<D, T, KIND, false>(tm, p, w, (int)(it / p.n_t), (int)(it % p.n_t), base, red);
}

}  // namespace pgx

// register-resident expm for D <= 8 (uses gen_entry_df, choose's tables, DfAcc)
#include "pgx_small.cuh"

namespace pgx {

// ---- forward chain in df -------------------------------------------------------
// U_total = P_n in FP64 from the df chain, the overlap z = Tr(T'U)/D in FP64,
// f(z) and the weighted chain-rule coefficient of member m.
template <int D, int T>
__device__ __forceinline__ void chain_epilogue_mx(const Team<T>& tm, const ProbDev& p, const WorkDev& w, int m,
                                                  const float4* Pc, double2* red) {
  double2* Ut = w.Utot + (size_t)m * D * D;
  double2 acc = make_double2(0.0, 0.0);
  for (int e = tm.lane; e < D * D; e += T) {
    const double2 v = dfc_to(dfc_load(Pc[e]));
    Ut[e] = v;
    acc = cmac_cj(acc, p.target_op[e], v);
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

// FP64 refinement of the chained propagator (Hermitian gate problems).  The
// df chain leaves U_total unitary to about 1e-13; one Newton-Schulz step of
// the polar decomposition, U' = U (3I - U'U) / 2, projects it back onto the
// unitary matrices (its non-unitary error goes from e to O(e^2)), all in FP64.
// The overlap z = Tr(T'U')/D, f and the chain-rule coefficient are then
// recomputed from U', so F and the gradient's costate seed both use the
// refined propagator.  U_total itself stays as the chain produced it: the
// oracle-free residual ||U'U - I|| of pgx_eval_stats reports the defect the
// refinement removed.  One CTA per member; sums in a fixed order.
constexpr int kRefThreads = 256;
template <int D>
__global__ void __launch_bounds__(kRefThreads) k_refine_unitary_mx(ProbDev p, WorkDev w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* U = reinterpret_cast<double2*>(smem_raw);
  double2* S = U + D * D;
  double2* red = S + D * D;
  const int m = blockIdx.x;
  const Team<kRefThreads> tm{(int)threadIdx.x};
  const double2* Ut = w.Utot + (size_t)m * D * D;
  for (int e = threadIdx.x; e < D * D; e += kRefThreads) U[e] = Ut[e];
  __syncthreads();
  for (int e = threadIdx.x; e < D * D; e += kRefThreads) {  // S = (3I - U'U) / 2
    const int r = e % D, c = e / D;
    double2 acc = make_double2(0.0, 0.0);
    for (int k = 0; k < D; ++k) acc = cmac_cj(acc, U[k + D * r], U[k + D * c]);
    S[e] = make_double2(0.5 * ((r == c ? 3.0 : 0.0) - acc.x), -0.5 * acc.y);
  }
  __syncthreads();
  double2 z = make_double2(0.0, 0.0);
  for (int e = threadIdx.x; e < D * D; e += kRefThreads) {  // z = sum conj(T) (U S)
    const int r = e % D, c = e / D;
    double2 v = make_double2(0.0, 0.0);
    for (int k = 0; k < D; ++k) v = cmac(v, U[r + D * k], S[k + D * c]);
    z = cmac_cj(z, p.target_op[e], v);
  }
  z = team_sum<kRefThreads>(tm, z, red);
  if (threadIdx.x == 0) {
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

// Parallel in time (members with few teams each would leave SMs idle): the
// slices of member m fall into pit_blocks blocks of pit_len.
//   local   per (m, b): local prefixes Q_i = U_{k0+i-1} ... U_{k0} in df,
//           stored as FP32 in the P slots k0 + i, the block product in df;
//   combine per m: T_0 = I, T_{b+1} = Q_b T_b in df (T_b saved as FP32),
//           P_n = T_B gives U_total and z exactly as the sequential chain;
//   fix     per (m, k), k >= pit_len: P_k <- Q_i T_b in FP32 (the gradient
//           consumes P in FP32).
// LSYM (D = 64, Hermiticity-preserving superoperators): the prefix products
// keep half of each product (mm_df_lsym).
// Teams of the in-block prefixes.  At D = 16, 64-thread teams (2 x 2
// blocks, 79 registers: 12 teams per SM) over about 7 (member, block) chains
// per SM (the runtime's block count) balance the SMs better than one
// 256-thread team per chain: spin-4 20.85 -> 21.08 M units/s.
template <int D> struct PreCfg {
  static constexpr int T = (D == 16) ? 64 : Cfg<D>::T;
  static constexpr int TPC = (D <= 8) ? Cfg<D>::TPC : (T >= 256 ? 1 : 256 / T);
  static constexpr int THREADS = T * TPC;
};

template <int D, bool LSYM>
__global__ void __launch_bounds__(PreCfg<D>::THREADS) k_chainf_local_mx(ProbDev p, WorkDev w, int store) {
  using G = PreCfg<D>;
  constexpr int T = G::T;
  constexpr int NE = (D * D + T - 1) / T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* smem = reinterpret_cast<float4*>(smem_raw);
  const int team = threadIdx.x / T;
  Team<T> tm{(int)(threadIdx.x % T)};
  tm.bar = (T > 32 && G::TPC > 1) ? 1 + team : 0;
  float4* Pc = smem + (size_t)team * (2 * D * D);
  float4* Ub = Pc + D * D;
  const long items = (long)p.n_members * w.pit_blocks;
  for (long it = (long)blockIdx.x * G::TPC + team; it < items; it += (long)gridDim.x * G::TPC) {
    const int m = (int)(it / w.pit_blocks), b = (int)(it % w.pit_blocks);
    const int k0 = b * w.pit_len, k1 = min(p.n_t, k0 + w.pit_len);
    const float4* Um = reinterpret_cast<const float4*>(w.U) + (size_t)m * p.n_t * D * D;
    float2* Pst = reinterpret_cast<float2*>(w.P) + (size_t)m * p.n_t * D * D;
    for (int e = tm.lane; e < D * D; e += T) {
      Pc[e] = make_float4((e % D) == (e / D) ? 1.f : 0.f, 0.f, 0.f, 0.f);
      if (store && k0 < k1) Pst[(size_t)k0 * D * D + e] = make_float2(Pc[e].x, Pc[e].y);
    }
    float4 pre[NE];
#pragma unroll
    for (int i = 0; i < NE; ++i) {
      const int e = tm.lane + i * T;
      if (e < D * D && k0 < k1) pre[i] = Um[(size_t)k0 * D * D + e];
    }
    tm.sync();
    for (int k = k0; k < k1; ++k) {
#pragma unroll
      for (int i = 0; i < NE; ++i) {
        const int e = tm.lane + i * T;
        if (e < D * D) Ub[e] = pre[i];
      }
      if (k + 1 < k1) {
        const float4* nx = Um + (size_t)(k + 1) * D * D;
#pragma unroll
        for (int i = 0; i < NE; ++i) {
          const int e = tm.lane + i * T;
          if (e < D * D) pre[i] = nx[e];
        }
      }
      tm.sync();
      if constexpr (LSYM)
        mm_df_lsym<D, T, false, 0>(tm, Pc, Ub, Pc, DfEpiNone{});
      else
        mm1_df<D, T>(tm, Pc, Ub, Pc);
      if (store && k + 1 < k1)
        for (int e = tm.lane; e < D * D; e += T) Pst[(size_t)(k + 1) * D * D + e] = make_float2(Pc[e].x, Pc[e].y);
    }
    float4* tot = w.pit_tot + ((size_t)m * w.pit_blocks + b) * D * D;
    for (int e = tm.lane; e < D * D; e += T) tot[e] = Pc[e];
    tm.sync();
  }
}

// Per member, the block products in order: P <- T_b P in df, each T_b staged
// in shared memory first (a latency-bound chain of few teams); LSYM as in
// k_chainf_local_mx.
template <int D, bool LSYM>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_chainf_combine_mx(ProbDev p, WorkDev w, int store) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* smem = reinterpret_cast<float4*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  float4* Pc = smem + (size_t)team * (2 * D * D + T);
  float4* Tb = Pc + D * D;
  double2* red = reinterpret_cast<double2*>(Tb + D * D);
  for (int e = tm.lane; e < D * D; e += T) Pc[e] = make_float4((e % D) == (e / D) ? 1.f : 0.f, 0.f, 0.f, 0.f);
  for (int b = 0; b < w.pit_blocks; ++b) {
    const float4* tot = w.pit_tot + ((size_t)m * w.pit_blocks + b) * D * D;
    for (int e = tm.lane; e < D * D; e += T) Tb[e] = tot[e];
    tm.sync();
    if (store) {
      float2* pre = w.pit_pre + ((size_t)m * w.pit_blocks + b) * D * D;
      for (int e = tm.lane; e < D * D; e += T) pre[e] = make_float2(Pc[e].x, Pc[e].y);
    }
    if constexpr (LSYM)
      mm_df_lsym<D, T, false, 0>(tm, Pc, Tb, Pc, DfEpiNone{});
    else
      mm1_df<D, T>(tm, Pc, Tb, Pc);
  }
  chain_epilogue_mx<D, T>(tm, p, w, m, Pc, red);
}

// Fully parallel FP32 fix-up products of the chains: operands staged from
// HBM into padded shared memory (each entry is read D times by the product).
// The products are bound by their shared-memory operand loads, so the teams
// give each lane 8 outputs (2 x 4 blocks) up to D = 32: at D = 16, T = 32
// runs the spin-4 evaluation 3 % faster than 2 x 2 blocks at T = 64; at
// D = 32, 16 outputs per lane (T = 64) were 0.5 % slower.
template <int D> struct FixCfg {
  static constexpr int T = (D <= 16) ? 32 : (D == 32) ? 128 : 256;
  static constexpr int TPC = (T >= 256) ? 1 : 256 / T;
  static constexpr int THREADS = T * TPC;
};
template <int D> __device__ __forceinline__ Team<FixCfg<D>::T> fix_team() {
  constexpr int T = FixCfg<D>::T;
  Team<T> tm{(int)(threadIdx.x % T)};
  tm.bar = (T > 32 && FixCfg<D>::TPC > 1) ? 1 + (int)(threadIdx.x / T) : 0;
  return tm;
}
// global column-major D x D <-> padded shared layout
template <int D, int T>
__device__ __forceinline__ void load_pad(const Team<T>& tm, float2* dst, const float2* src) {
  for (int e = tm.lane; e < D * D; e += T) dst[Lay<D, 2>::idx(e % D, e / D)] = src[e];
}
template <int D, int T>
__device__ __forceinline__ void store_pad(const Team<T>& tm, float2* dst, const float2* src) {
  for (int e = tm.lane; e < D * D; e += T) dst[e] = src[Lay<D, 2>::idx(e % D, e / D)];
}

// P_k <- P_k T_b for every slice after the first block (FP32).
template <int D>
__global__ void __launch_bounds__(FixCfg<D>::THREADS) k_chainf_fix_mx(ProbDev p, WorkDev w) {
  using F = FixCfg<D>;
  using L = Lay<D, 2>;
  constexpr int T = F::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int team = threadIdx.x / T;
  const Team<T> tm = fix_team<D>();
  float2* A = reinterpret_cast<float2*>(smem_raw) + (size_t)team * 2 * L::SIZE;
  float2* Tb = A + L::SIZE;
  const int Lb = w.pit_len, nk = p.n_t - Lb;
  const long items = (long)p.n_members * (nk > 0 ? nk : 0);
  for (long it = (long)blockIdx.x * F::TPC + team; it < items; it += (long)gridDim.x * F::TPC) {
    const int m = (int)(it / nk), k = Lb + (int)(it % nk), b = k / Lb;
    float2* Pk = reinterpret_cast<float2*>(w.P) + ((size_t)m * p.n_t + k) * D * D;
    load_pad<D, T>(tm, A, Pk);
    load_pad<D, T>(tm, Tb, w.pit_pre + ((size_t)m * w.pit_blocks + b) * D * D);
    tm.sync();
    mm1<D, T, 2>(tm, A, A, Tb);
    store_pad<D, T>(tm, Pk, A);
    tm.sync();
  }
}

template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_chain_gate_fwd_mx(ProbDev p, WorkDev w, int store) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  constexpr int NE = (D * D + T - 1) / T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* smem = reinterpret_cast<float4*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  float4* Pc = smem + (size_t)team * (2 * D * D + T);
  float4* Ub = Pc + D * D;
  double2* red = reinterpret_cast<double2*>(Ub + D * D);
  for (int e = tm.lane; e < D * D; e += T)
    Pc[e] = make_float4((e % D) == (e / D) ? 1.f : 0.f, 0.f, 0.f, 0.f);
  const float4* Um = reinterpret_cast<const float4*>(w.U) + (size_t)m * p.n_t * D * D;
  float2* Pst = reinterpret_cast<float2*>(w.P) + (size_t)m * p.n_t * D * D;
  float4 pre[NE];
#pragma unroll
  for (int i = 0; i < NE; ++i) {
    const int e = tm.lane + i * T;
    if (e < D * D) pre[i] = Um[e];
  }
  tm.sync();
  for (int k = 0; k < p.n_t; ++k) {
    if (store)
      for (int e = tm.lane; e < D * D; e += T) Pst[(size_t)k * D * D + e] = make_float2(Pc[e].x, Pc[e].y);
#pragma unroll
    for (int i = 0; i < NE; ++i) {
      const int e = tm.lane + i * T;
      if (e < D * D) Ub[e] = pre[i];
    }
    if (k + 1 < p.n_t) {
      const float4* nx = Um + (size_t)(k + 1) * D * D;
#pragma unroll
      for (int i = 0; i < NE; ++i) {
        const int e = tm.lane + i * T;
        if (e < D * D) pre[i] = nx[e];
      }
    }
    tm.sync();
    mm1_df<D, T>(tm, Pc, Ub, Pc);
  }
  chain_epilogue_mx<D, T>(tm, p, w, m, Pc, red);
}

// ---- backward chain in FP32 -------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_chain_gate_bwd_mx(ProbDev p, WorkDev w) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* smem = reinterpret_cast<float2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  float2* Lam = smem + (size_t)team * 2 * D * D;
  float2* Buf = Lam + D * D;
  const double2 kap = w.kap[m];
  for (int e = tm.lane; e < D * D; e += T) {
    const int r = e % D, c = e / D;
    const double2 t = p.target_op[c + D * r];
    const double2 v = cmul(kap, make_double2(t.x, -t.y));
    Lam[e] = make_float2((float)v.x, (float)v.y);
  }
  tm.sync();
  const float4* Um = reinterpret_cast<const float4*>(w.U) + (size_t)m * p.n_t * D * D;
  float2* Pm = reinterpret_cast<float2*>(w.P) + (size_t)m * p.n_t * D * D;
  const bool grape = (p.grad_mode == GRAD_REF_GRAPE);
  for (int k = p.n_t - 1; k >= 0; --k) {
    if (grape) {
      for (int e = tm.lane; e < D * D; e += T) {
        const float4 u = Um[(size_t)k * D * D + e];
        Buf[e] = make_float2(u.x, u.y);
      }
      tm.sync();
      mm1<D, T>(tm, Lam, Lam, Buf);
    }
    for (int e = tm.lane; e < D * D; e += T) Buf[e] = Pm[(size_t)k * D * D + e];
    tm.sync();
    mm1<D, T>(tm, Pm + (size_t)k * D * D, Buf, Lam);
    if (!grape) {
      for (int e = tm.lane; e < D * D; e += T) {
        const float4 u = Um[(size_t)k * D * D + e];
        Buf[e] = make_float2(u.x, u.y);
      }
      tm.sync();
      mm1<D, T>(tm, Lam, Lam, Buf);
    }
  }
}

// Backward chain in parallel in time (FP32), blocks as the forward chain's:
//   local   per (m, b): in-block suffixes R_k = U_{k1-1} ... U_k;
//   combine per m: Lambda_n = kappa T', Lambda_{k0} = Lambda_{k1} R_{k0} block
//           by block from the end (Lambda_{k1} of each block saved);
//   fix     per (m, k): Lambda_{k+1} = Lambda_{k1} R_{k+1} (or Lambda_{k1} at
//           the block end), M_k = P_k Lambda_{k+1}; the first-order GRAPE
//           formula takes Lambda_k = Lambda_{k1} R_k instead.
template <int D, int T>
__device__ __forceinline__ void load_hi(const Team<T>& tm, float2* dst, const float4* src) {
  for (int e = tm.lane; e < D * D; e += T) {
    const float4 u = src[e];
    dst[e] = make_float2(u.x, u.y);
  }
}

// Teams of the backward chain's in-block suffixes.  They run on a side
// stream beside the df forward prefixes, so the fewest SMs serve them best:
// one warp per (member, block) chain at D = 16 (spin-4 evaluation 20.68 ->
// 20.82 M units/s against T = 256; T = 64 and 128 were slower).  At D = 32
// 64-thread teams were 1 % slower than 256 on the largest uneven problems.
template <int D> struct SufCfg {
  static constexpr int T = (D == 16) ? 32 : (D == 32) ? 256 : Cfg<D>::T;
  static constexpr int TPC = (D <= 8) ? Cfg<D>::TPC : (T >= 256 ? 1 : 256 / T);
  static constexpr int THREADS = T * TPC;
};

template <int D>
__global__ void __launch_bounds__(SufCfg<D>::THREADS) k_chainb_local_mx(ProbDev p, WorkDev w) {
  using G = SufCfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* smem = reinterpret_cast<float2*>(smem_raw);
  const int team = threadIdx.x / T;
  Team<T> tm{(int)(threadIdx.x % T)};
  tm.bar = (T > 32 && G::TPC > 1) ? 1 + team : 0;
  float2* R = smem + (size_t)team * 2 * D * D;
  float2* Ub = R + D * D;
  const long items = (long)p.n_members * w.pit_blocks;
  for (long it = (long)blockIdx.x * G::TPC + team; it < items; it += (long)gridDim.x * G::TPC) {
    const int m = (int)(it / w.pit_blocks), b = (int)(it % w.pit_blocks);
    const int k0 = b * w.pit_len, k1 = min(p.n_t, k0 + w.pit_len);
    const float4* Um = reinterpret_cast<const float4*>(w.U) + (size_t)m * p.n_t * D * D;
    float2* Rm = w.pit_r + (size_t)m * p.n_t * D * D;
    for (int e = tm.lane; e < D * D; e += T) R[e] = make_float2((e % D) == (e / D) ? 1.f : 0.f, 0.f);
    for (int k = k1 - 1; k >= k0; --k) {
      load_hi<D, T>(tm, Ub, Um + (size_t)k * D * D);
      tm.sync();
      mm1<D, T>(tm, R, R, Ub);
      for (int e = tm.lane; e < D * D; e += T) Rm[(size_t)k * D * D + e] = R[e];
    }
    tm.sync();
  }
}

template <int D>
__global__ void __launch_bounds__(Cfg<D>::THREADS) k_chainb_combine_mx(ProbDev p, WorkDev w) {
  using G = Cfg<D>;
  constexpr int T = G::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* smem = reinterpret_cast<float2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * G::TPC + team;
  if (m >= p.n_members) return;
  float2* Lam = smem + (size_t)team * D * D;
  const double2 kap = w.kap[m];
  for (int e = tm.lane; e < D * D; e += T) {
    const int r = e % D, c = e / D;
    const double2 t = p.target_op[c + D * r];
    const double2 v = cmul(kap, make_double2(t.x, -t.y));
    Lam[e] = make_float2((float)v.x, (float)v.y);
  }
  tm.sync();
  const float2* Rm = w.pit_r + (size_t)m * p.n_t * D * D;
  for (int b = w.pit_blocks - 1; b >= 0; --b) {
    float2* lam_b = w.pit_lam + ((size_t)m * w.pit_blocks + b) * D * D;
    for (int e = tm.lane; e < D * D; e += T) lam_b[e] = Lam[e];
    mm1<D, T>(tm, Lam, Lam, Rm + (size_t)(b * w.pit_len) * D * D);
  }
}

template <int D>
__global__ void __launch_bounds__(FixCfg<D>::THREADS) k_chainb_fix_mx(ProbDev p, WorkDev w) {
  using F = FixCfg<D>;
  using L = Lay<D, 2>;
  constexpr int T = F::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int team = threadIdx.x / T;
  const Team<T> tm = fix_team<D>();
  float2* Lam = reinterpret_cast<float2*>(smem_raw) + (size_t)team * 3 * L::SIZE;
  float2* R = Lam + L::SIZE;
  float2* Pm = R + L::SIZE;
  const bool grape = (p.grad_mode == GRAD_REF_GRAPE);
  const long items = (long)p.n_members * p.n_t;
  for (long it = (long)blockIdx.x * F::TPC + team; it < items; it += (long)gridDim.x * F::TPC) {
    const int m = (int)(it / p.n_t), k = (int)(it % p.n_t), b = k / w.pit_len;
    const int k1 = min(p.n_t, (b + 1) * w.pit_len);
    const int kk = grape ? k : k + 1;  // costate index the formula uses
    float2* Pk = reinterpret_cast<float2*>(w.P) + ((size_t)m * p.n_t + k) * D * D;
    load_pad<D, T>(tm, Lam, w.pit_lam + ((size_t)m * w.pit_blocks + b) * D * D);
    load_pad<D, T>(tm, Pm, Pk);
    if (kk != k1) load_pad<D, T>(tm, R, w.pit_r + ((size_t)m * p.n_t + kk) * D * D);
    tm.sync();
    if (kk != k1) mm1<D, T, 2>(tm, Lam, Lam, R);  // Lambda_kk = Lambda_k1 R_kk
    mm1<D, T, 2>(tm, Pm, Pm, Lam);                 // M_k = P_k Lambda_kk
    store_pad<D, T>(tm, Pk, Pm);
    tm.sync();
  }
}

// ---- state chains -----------------------------------------------------------------
// State targets (pairs psi_s -> t_s; MR state transfer, Lindblad vec(rho)) carry
// D^2 work per slice and pair: one warp per member.  The warp streams the next
// slice's propagator (and, backward, the stored states) into a second
// shared-memory buffer with cp.async while it computes the current slice, so
// the sequential chain waits on shared memory, not on HBM.
template <int D> struct StCfg {
  static constexpr int TPC = D >= 64 ? 1 : 4;  // members (warps) per CTA
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// bytes (a multiple of 16) from global to shared, spread over the warp
__device__ __forceinline__ void warp_copy_async(int lane, void* dst, const void* src, size_t bytes) {
  const int n = (int)(bytes / 16);
  for (int i = lane; i < n; i += 32)
    cp_async16(static_cast<char*>(dst) + 16 * (size_t)i, static_cast<const char*>(src) + 16 * (size_t)i);
  cp_async_commit();
}

// The same copy into the padded layout (leading dimension D + 1): each
// 16-byte chunk is one df entry (r, c), placed at r + (D + 1) c.
template <int D>
__device__ __forceinline__ void warp_copy_async_pad(int lane, float4* dst, const float4* src) {
  for (int i = lane; i < D * D; i += 32) cp_async16(dst + (i % D) + (D + 1) * (i / D), src + i);
  cp_async_commit();
}

template <int D> __host__ __device__ constexpr size_t st_fwd_team_bytes(int np) {
  return (2 * (size_t)D * D + (size_t)np * D) * sizeof(float4);
}
template <int D> __host__ __device__ constexpr size_t st_bwd_team_bytes(int np) {
  return 2 * (size_t)D * (D + 1) * sizeof(float4) + (size_t)np * D * sizeof(float2);
}

// Forward in df: psi_s[k+1] = U_k psi_s[k], U_k the df propagator of the expm
// stage.  The states are stored in FP32 for the gradient; z_s = <t_s|psi_s[n]>,
// f(z_s) and kappa_s come from the df state in FP64, as the FP64 chain forms
// them.  Utot[m np + s] receives the propagation residual of the pair in
// FP64: |psi[n]|^2 - |psi[0]|^2 (Hermitian) or Tr rho[n] - Tr rho[0] (a
// vectorised density matrix, N^2 = D).
// Overlaps z_s, f, the chain-rule coefficients and the norm / trace residual
// of member m from its final df states Ps (one warp).
template <int D>
__device__ __forceinline__ void states_fwd_epilogue(int lane, const ProbDev& p, const WorkDev& w, int m,
                                                   const float4* Ps) {
  constexpr int T = 32;
  const int np = p.n_pairs;
  int N = (int)lrint(sqrt((double)p.D));
  if (p.gen != GEN_LIOUV || N * N != p.D) N = 0;
  double Fm = 0.0;
  for (int s = 0; s < np; ++s) {
    double2 acc = make_double2(0.0, 0.0), res = make_double2(0.0, 0.0);
    for (int r = lane; r < D; r += T) {
      const double2 v = dfc_to(dfc_load(Ps[s * D + r]));
      const double2 v0 = p.psi_init[s * D + r];
      acc = cmac_cj(acc, p.psi_targ[s * D + r], v);
      if (p.gen == GEN_HERM) {
        res.x += (v.x * v.x + v.y * v.y) - (v0.x * v0.x + v0.y * v0.y);
      } else if (N && r < N * N && r % (N + 1) == 0) {
        res.x += v.x - v0.x;
        res.y += v.y - v0.y;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
      res.x += __shfl_xor_sync(0xffffffffu, res.x, o);
      res.y += __shfl_xor_sync(0xffffffffu, res.y, o);
    }
    double f;
    double2 kap;
    fid_kappa(acc, p.fid, p.grad_mode, f, kap);
    Fm += f;
    if (lane == 0) {
      const double wgt = p.m_weight[m];
      w.z[(size_t)m * np + s] = acc;
      w.kap[(size_t)m * np + s] = make_double2(kap.x * wgt, kap.y * wgt);
      w.Utot[(size_t)m * np + s] = res;
    }
  }
  if (lane == 0) w.Fm[m] = Fm;
}

template <int D>
__global__ void __launch_bounds__(32 * StCfg<D>::TPC) k_chain_states_fwd_mx(ProbDev p, WorkDev w, int store) {
  constexpr int T = 32;
  constexpr int NO = (8 * D + T - 1) / T;  // outputs per lane: at most 8 pairs
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * StCfg<D>::TPC + team;
  if (m >= p.n_members) return;  // a whole warp: teams never share a barrier
  const int np = p.n_pairs, pan = np * D;
  float4* Ub = reinterpret_cast<float4*>(smem_raw + (size_t)team * st_fwd_team_bytes<D>(np));  // [2][D*D]
  float4* Ps = Ub + 2 * D * D;                                                                   // [np][D]
  float2* Pst = reinterpret_cast<float2*>(w.psi) + (size_t)m * (p.n_t + 1) * pan;
  const float4* Um = reinterpret_cast<const float4*>(w.U) + (size_t)m * p.n_t * D * D;
  constexpr size_t UB = (size_t)D * D * sizeof(float4);
  warp_copy_async(tm.lane, Ub, Um, UB);
  for (int e = tm.lane; e < pan; e += T) {
    Ps[e] = dfc_store(dfc_from(p.psi_init[e]));
    if (store) Pst[e] = make_float2(Ps[e].x, Ps[e].y);
  }
  cp_async_wait_all();
  tm.sync();
  for (int k = 0; k < p.n_t; ++k) {
    const float4* Uk = Ub + (size_t)(k & 1) * D * D;
    if (k + 1 < p.n_t)  // the other buffer was last read at slice k - 1
      warp_copy_async(tm.lane, Ub + (size_t)((k + 1) & 1) * D * D, Um + (size_t)(k + 1) * D * D, UB);
    float4 outv[NO];
#pragma unroll
    for (int i = 0; i < NO; ++i) {
      const int e = tm.lane + T * i;
      if (e < pan) {
        const int s = e / D, r = e % D;
        DfAcc acc;
        for (int q = 0; q < D; ++q) acc.mac(Uk[r + D * q], Ps[s * D + q]);
        outv[i] = dfc_store(acc.result());
      }
    }
    tm.sync();
#pragma unroll
    for (int i = 0; i < NO; ++i) {
      const int e = tm.lane + T * i;
      if (e < pan) {
        Ps[e] = outv[i];
        if (store) Pst[(size_t)(k + 1) * pan + e] = make_float2(outv[i].x, outv[i].y);
      }
    }
    cp_async_wait_all();
    tm.sync();
  }
  states_fwd_epilogue<D>(tm.lane, p, w, m, Ps);
}

// D >= 16: the same chain with each member's dot products split over kStW
// warps (k in [w D/kStW, (w+1) D/kStW) for warp w).  One member per CTA.  The
// partial df sums are merged in warp order after a barrier.  One warp per
// member leaves most SM sub-partitions idle (231 members, 608 of them), and a
// 16-term df dot product is a long dependent chain.
constexpr int kStW = 4;
template <int D> __host__ __device__ constexpr size_t st_fwd_split_bytes(int np) {
  return (2 * (size_t)D * D + (size_t)(1 + kStW) * np * D) * sizeof(float4);
}
template <int D>
__global__ void __launch_bounds__(32 * kStW) k_chain_states_fwd_split_mx(ProbDev p, WorkDev w, int store) {
  static_assert(D % kStW == 0, "k split");
  constexpr int NT = 32 * kStW, KQ = D / kStW;
  constexpr int NO = (8 * D + 31) / 32;  // outputs per lane: at most 8 pairs
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = blockIdx.x, tid = threadIdx.x, wp = tid / 32, lane = tid % 32;
  const int np = p.n_pairs, pan = np * D;
  float4* Ub = reinterpret_cast<float4*>(smem_raw);  // [2][D*D]
  float4* Ps = Ub + 2 * D * D;                        // [np][D]
  float4* part = Ps + pan;                            // [kStW][np * D] partial sums {sr, cr, si, ci}
  float2* Pst = reinterpret_cast<float2*>(w.psi) + (size_t)m * (p.n_t + 1) * pan;
  const float4* Um = reinterpret_cast<const float4*>(w.U) + (size_t)m * p.n_t * D * D;
  const auto copy_u = [&](float4* dst, const float4* src) {
    for (int i = tid; i < D * D; i += NT) cp_async16(dst + i, src + i);
    cp_async_commit();
  };
  copy_u(Ub, Um);
  for (int e = tid; e < pan; e += NT) {
    Ps[e] = dfc_store(dfc_from(p.psi_init[e]));
    if (store) Pst[e] = make_float2(Ps[e].x, Ps[e].y);
  }
  cp_async_wait_all();
  __syncthreads();
  for (int k = 0; k < p.n_t; ++k) {
    const float4* Uk = Ub + (size_t)(k & 1) * D * D;
    if (k + 1 < p.n_t)  // the other buffer was last read at slice k - 1
      copy_u(Ub + (size_t)((k + 1) & 1) * D * D, Um + (size_t)(k + 1) * D * D);
#pragma unroll
    for (int i = 0; i < NO; ++i) {
      const int e = lane + 32 * i;
      if (e < pan) {
        const int s = e / D, r = e % D;
        DfAcc acc;
#pragma unroll
        for (int q = wp * KQ; q < (wp + 1) * KQ; ++q) acc.mac(Uk[r + D * q], Ps[s * D + q]);
        part[(size_t)wp * pan + e] = make_float4(acc.sr, acc.cr, acc.si, acc.ci);
      }
    }
    __syncthreads();
    for (int e = tid; e < pan; e += NT) {
      const float4 v0 = part[e];
      DfAcc acc;
      acc.sr = v0.x; acc.cr = v0.y; acc.si = v0.z; acc.ci = v0.w;
#pragma unroll
      for (int q = 1; q < kStW; ++q) {
        const float4 v = part[(size_t)q * pan + e];
        float t, er;
        two_sum(acc.sr, v.x, t, er);
        acc.sr = t;
        acc.cr = (acc.cr + v.y) + er;
        two_sum(acc.si, v.z, t, er);
        acc.si = t;
        acc.ci = (acc.ci + v.w) + er;
      }
      const float4 o = dfc_store(acc.result());
      Ps[e] = o;
      if (store) Pst[(size_t)(k + 1) * pan + e] = make_float2(o.x, o.y);
    }
    cp_async_wait_all();
    __syncthreads();
  }
  if (wp == 0) states_fwd_epilogue<D>(lane, p, w, m, Ps);
}

// Backward in FP32: lambda_s[n] = conj(kappa_s) t_s, lambda_s[k] = U_k'
// lambda_s[k+1] with U_k rounded to FP32; every lambda[k] is stored (FP32)
// for the gradient kernel, which forms M_k = sum_s psi_s[k] lambda_s[k+1]'
// (lambda_s[k] for the first-order GRAPE formula) itself.
template <int D>
__global__ void __launch_bounds__(32 * StCfg<D>::TPC) k_chain_states_bwd_mx(ProbDev p, WorkDev w) {
  constexpr int T = 32;
  constexpr int NO = (8 * D + T - 1) / T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  const int m = blockIdx.x * StCfg<D>::TPC + team;
  if (m >= p.n_members) return;
  const int np = p.n_pairs, pan = np * D;
  // U_k in the padded layout: lane r reads column r of U (U' lambda), and a
  // leading dimension of D + 1 puts the lanes of one load in distinct banks
  constexpr int UP = D * (D + 1);
  unsigned char* base = smem_raw + (size_t)team * st_bwd_team_bytes<D>(np);
  float4* Ub = reinterpret_cast<float4*>(base);                                    // [2][D*(D+1)]
  float2* Ls = reinterpret_cast<float2*>(base + 2 * (size_t)UP * sizeof(float4));  // [np][D]
  const float4* Um = reinterpret_cast<const float4*>(w.U) + (size_t)m * p.n_t * D * D;
  float2* Lm = reinterpret_cast<float2*>(w.lam) + (size_t)m * (p.n_t + 1) * pan;
  const int k0 = p.n_t - 1;
  warp_copy_async_pad<D>(tm.lane, Ub, Um + (size_t)k0 * D * D);
  for (int e = tm.lane; e < pan; e += T) {
    const double2 kp = w.kap[(size_t)m * np + e / D];
    const double2 v = cmul(make_double2(kp.x, -kp.y), p.psi_targ[e]);
    Ls[e] = make_float2((float)v.x, (float)v.y);
    Lm[(size_t)p.n_t * pan + e] = Ls[e];
  }
  cp_async_wait_all();
  tm.sync();
  for (int k = k0; k >= 0; --k) {
    const int slot = (k0 - k) & 1;
    const float4* Uk = Ub + (size_t)slot * UP;
    if (k > 0)  // the other buffer was last read at slice k + 1
      warp_copy_async_pad<D>(tm.lane, Ub + (size_t)(slot ^ 1) * UP, Um + (size_t)(k - 1) * D * D);
    float2 outv[NO];
#pragma unroll
    for (int i = 0; i < NO; ++i) {
      const int e = tm.lane + T * i;
      if (e < pan) {
        const int s = e / D, r = e % D;
        float2 acc = make_float2(0.f, 0.f);
        for (int q = 0; q < D; ++q) {
          const float4 u = Uk[q + (D + 1) * r];
          acc = cmac_cj(acc, make_float2(u.x, u.y), Ls[s * D + q]);
        }
        outv[i] = acc;
      }
    }
    tm.sync();
#pragma unroll
    for (int i = 0; i < NO; ++i) {
      const int e = tm.lane + T * i;
      if (e < pan) {
        Ls[e] = outv[i];
        Lm[(size_t)k * pan + e] = outv[i];
      }
    }
    cp_async_wait_all();
    tm.sync();
  }
}

// ---- gradient in FP32 -----------------------------------------------------------
// g_j = Re(c dt scale Tr(X C_j)).  The team's first warp sums in a fixed order
// (stride-32 partial sums, then a fixed shuffle tree) so that the result does
// not depend on the team size the autotuner picks.
template <int D, int T, int SW>
__device__ __forceinline__ void trace_controls32(const Team<T>& tm, const ProbDev& p, const float2* X,
                                                 int m, int k, double* Gout, float2* red) {
  if constexpr (D >= 32) {
    // 256 fixed chunks (entries q = c, c + 256, ... summed in order), then a
    // fixed tree: warp-sized groups by xor shuffles, the 8 group sums in
    // order.  The order depends on D only, not on the team size; the scratch
    // holds the 256 chunk sums (2T >= 256).
    constexpr int NCH = 256, NGR = NCH / 32;
    static_assert(T >= 32 && 2 * T >= NCH, "trace scratch holds the 256 chunk sums");
    for (int j = 0; j < p.n_c; ++j) {
      const float2* Cj = p.ctrls_f32 + (size_t)j * D * D;
      for (int c = tm.lane; c < NCH; c += T) {
        float2 acc = make_float2(0.f, 0.f);
        for (int q = c; q < D * D; q += NCH) {
          const int r = q % D, cc = q / D;
          acc = cmac(acc, X[Lay<D, SW>::idx(r, cc)], Cj[cc + D * r]);
        }
        red[c] = acc;
      }
      tm.sync();
      for (int gl = tm.lane; gl < NGR * 32; gl += T) {  // whole warps: gl / 32 is uniform in a warp
        float2 v = red[gl];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
          v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (gl % 32 == 0) red[gl] = v;  // group sum over the group's first slot
      }
      tm.sync();
      if (tm.lane == 0) {
        float2 acc = red[0];
        for (int g = 1; g < NGR; ++g) acc = make_float2(acc.x + red[32 * g].x, acc.y + red[32 * g].y);
        Gout[j] = p.dt[k] * p.m_scale[m] * (double)(p.gen == GEN_HERM ? acc.y : acc.x);
      }
      tm.sync();
    }
    return;
  }
  if (tm.lane < 32) {
    for (int j = 0; j < p.n_c; ++j) {
      const float2* Cj = p.ctrls_f32 + (size_t)j * D * D;
      float2 acc = make_float2(0.f, 0.f);
      for (int q = tm.lane; q < D * D; q += 32) {
        const int r = q % D, c = q / D;
        acc = cmac(acc, X[Lay<D, SW>::idx(r, c)], Cj[c + D * r]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
      }
      if (tm.lane == 0) Gout[j] = p.dt[k] * p.m_scale[m] * (double)(p.gen == GEN_HERM ? acc.y : acc.x);
    }
  }
  tm.sync();
}

template <int D, int T>
__global__ void __launch_bounds__(CfgM<D, T>::THREADS) k_grad_gate_mx(ProbDev p, WorkDev w) {
  using G = CfgM<D, T>;
  using L = Lay<D, kSwzGrad>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int team = threadIdx.x / T;
  const Team<T> tm = team_of<D, T>();
  float2* base = reinterpret_cast<float2*>(smem_raw + (size_t)team * G::WSG);
  float2* red = reinterpret_cast<float2*>(smem_raw + G::TPC * G::WSG + (size_t)team * G::RED);
  using Wk = Work2<float2, D, L::SIZE>;
  const Wk W = Wk::at(base);
  const bool exact = (p.grad_mode == GRAD_EXACT);
  const long items = (long)p.n_members * p.n_t;
  for (long it = (long)blockIdx.x * G::TPC + team; it < items; it += (long)gridDim.x * G::TPC) {
    const int m = (int)(it / p.n_t), k = (int)(it % p.n_t);
    double* Gout = w.Gm + ((size_t)m * p.n_t + k) * p.n_c;
    if (p.target == TGT_GATE) {
      const float2* Mk = reinterpret_cast<const float2*>(w.P) + ((size_t)m * p.n_t + k) * D * D;
      if (!exact) {
        trace_controls32<D, T, 0>(tm, p, Mk, m, k, Gout, red);
        continue;
      }
      for (int e = tm.lane; e < D * D; e += T) W.dB[L::idx(e % D, e / D)] = Mk[e];
    } else {  // M_k = sum_s psi_s[k] lambda_s[li]'
      const int np = p.n_pairs, pan = np * D;
      const int li = (p.grad_mode == GRAD_REF_GRAPE) ? k : k + 1;
      const float2* ps = reinterpret_cast<const float2*>(w.psi) + ((size_t)m * (p.n_t + 1) + k) * pan;
      const float2* ls = reinterpret_cast<const float2*>(w.lam) + ((size_t)m * (p.n_t + 1) + li) * pan;
      for (int e = tm.lane; e < D * D; e += T) {
        const int r = e % D, c = e / D;
        float2 acc = make_float2(0.f, 0.f);
        for (int s = 0; s < np; ++s) {
          const float2 l = ls[s * D + c];
          acc = cmac(acc, ps[s * D + r], make_float2(l.x, -l.y));
        }
        W.dB[L::idx(r, c)] = acc;
      }
      if (!exact) {
        tm.sync();
        trace_controls32<D, T, kSwzGrad>(tm, p, W.dB, m, k, Gout, red);
        continue;
      }
    }
    build_A32<D, T, kSwzGrad>(tm, p, w, m, k, W.B);
    tm.sync();
    const float nrm = norm1f<D, T, kSwzGrad>(tm, W.B, reinterpret_cast<float*>(red));
    int deg, s;
    choose_degree_q2(nrm, c_theta32f, deg, s);
    const float sc = ldexpf(1.f, -s);
    for (int q = tm.lane; q < D * D; q += T) {
      const int e = L::idx(q % D, q / D);
      W.B[e] = cscale(W.B[e], sc);
      W.dB[e] = cscale(W.dB[e], sc);
    }
    tm.sync();
    taylor_exp_frechet2<D, T, kSwzGrad>(tm, W, deg, s, c_invf32);
    trace_controls32<D, T, kSwzGrad>(tm, p, W.dY, m, k, Gout, red);
    tm.sync();
  }
}

}  // namespace pgx

// the D = 64 tensor-core gradient (uses choose_degree_q2 and the tables above)
#include "pgx_grad_tc.cuh"
#include "pgx_fix_tc.cuh"
#include "pgx_expm_oz.cuh"

namespace pgx {

// ---- launchers ---------------------------------------------------------------------
template <class K>
static void ensure_smem_mx(K kernel, size_t bytes) {
  set_smem_once((const void*)kernel, bytes);
}

template <class K>
static int grid_for(K kernel, int threads, size_t smem, long teams, int tpc, int num_sms, int cap) {
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  if (per_sm < 1) per_sm = 1;
  long blocks = (teams + tpc - 1) / tpc;
  const long maxb = (long)num_sms * per_sm;
  if (blocks > maxb) blocks = maxb;
  if (cap > 0 && blocks > cap) blocks = cap;
  return blocks < 1 ? 1 : (int)blocks;
}

#define PGX_DISPATCH_MX(DP, CALL)                     \
  switch (DP) {                                       \
    case 2: { constexpr int D_ = 2; CALL; } break;    \
    case 4: { constexpr int D_ = 4; CALL; } break;    \
    case 8: { constexpr int D_ = 8; CALL; } break;    \
    case 16: { constexpr int D_ = 16; CALL; } break;  \
    case 32: { constexpr int D_ = 32; CALL; } break;  \
    case 64: { constexpr int D_ = 64; CALL; } break;  \
    default: return cudaErrorInvalidValue;            \
  }

// Team sizes each D admits (register budget of the blocked df products).  The
// D = 64 gradient also runs as one 512-thread team per SM: its six FP32
// matrices fill shared memory, so more threads per team is the only way to
// more warps.  For gate targets with the exact gradient the D = 64 gradient
// has a third form, the tensor-core engine (kTeamTensor): the default and the
// only one the autotuner times (its products are 3xTF32, not bit-identical
// to the CUDA-core teams, and several times faster); the CUDA-core teams stay
// selectable with pgx_problem_set_team.  The D = 64 df expm has a tensor-core
// form as well (every product by exact bf16 slicing, pgx_expm_oz.cuh) for every
// generator and target: the default and the autotuner's only candidate there,
// the CUDA-core team (256) selectable.
bool grad_tc_eligible(const ProbDev& p) {
  return p.Dp == 64 && p.target == TGT_GATE && p.grad_mode == GRAD_EXACT;
}
static bool expm_tc_eligible(const ProbDev& p) { return p.Dp == 64; }
static int variants_for(int Dp, int kernel, int* out) {
  int n = 0;
  if (Dp <= 8) out[n++] = 32;
  else if (Dp == 16) { out[n++] = 32; out[n++] = 64; out[n++] = 128; out[n++] = 256; }
  else if (Dp == 32) { out[n++] = 128; out[n++] = 256; }
  else {
    out[n++] = 256;
    if (kernel == kTuneGradMx) out[n++] = 512;
  }
  return n;
}
static bool tc_eligible(const ProbDev& p, int kernel) {
  return kernel == kTuneGradMx ? grad_tc_eligible(p) : expm_tc_eligible(p);
}
int mixed_variants(const ProbDev& p, int kernel, int* out) {
  if (tc_eligible(p, kernel)) {
    out[0] = kTeamTensor;
    return 1;
  }
  return variants_for(p.Dp, kernel, out);
}
int mixed_admitted(const ProbDev& p, int kernel, int* out) {
  int n = variants_for(p.Dp, kernel, out);
  if (tc_eligible(p, kernel)) out[n++] = kTeamTensor;
  return n;
}
// Defaults (problems that were never tuned: batches, served jobs) are the
// autotuner's usual choice on GB300 at each dimension.
int mixed_default_team(const ProbDev& p, int kernel) {
  const int Dp = p.Dp;
  if (Dp <= 8) return 32;
  if (Dp == 16) return kernel == kTuneExpmMx ? 128 : 32;
  if (Dp == 32) return kernel == kTuneExpmMx ? 256 : 128;
  if (tc_eligible(p, kernel)) return kTeamTensor;
  return kernel == kTuneExpmMx ? 256 : 512;
}

#define PGX_DISPATCH_MX_T(DP, TT, CALL)                                                        \
  switch (DP) {                                                                                \
    case 2: { constexpr int D_ = 2, T_ = 32; CALL; } break;                                   \
    case 4: { constexpr int D_ = 4, T_ = 32; CALL; } break;                                   \
    case 8: { constexpr int D_ = 8, T_ = 32; CALL; } break;                                   \
    case 16:                                                                                   \
      switch (TT) {                                                                            \
        case 32: { constexpr int D_ = 16, T_ = 32; CALL; } break;                             \
        case 64: { constexpr int D_ = 16, T_ = 64; CALL; } break;                             \
        case 128: { constexpr int D_ = 16, T_ = 128; CALL; } break;                           \
        default: { constexpr int D_ = 16, T_ = 256; CALL; } break;                            \
      }                                                                                        \
      break;                                                                                   \
    case 32:                                                                                   \
      if (TT == 128) { constexpr int D_ = 32, T_ = 128; CALL; }                               \
      else { constexpr int D_ = 32, T_ = 256; CALL; }                                         \
      break;                                                                                   \
    case 64: { constexpr int D_ = 64, T_ = 256; CALL; } break;                                \
    default: return cudaErrorInvalidValue;                                                     \
  }

template <int D, int T>
static cudaError_t do_expm_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  using G = CfgM<D, T>;
  const size_t smem = G::SMEM_E;
  // an instance per generator structure
  auto kern = (p.gen == GEN_HERM) ? k_expm_mx<D, T, kExpmHerm> : k_expm_mx<D, T, kExpmFull>;
  if constexpr (D == 64 && T == 256)
    if (p.lsym) kern = k_expm_mx<D, T, kExpmLSym>;
  ensure_smem_mx(kern, smem);
  const int grid = grid_for(kern, G::THREADS, smem, (long)p.n_members * p.n_t, G::TPC, li.num_sms,
                            G::SLAB ? w.slab_teams : 0);
  kern<<<grid, G::THREADS, smem, li.stream>>>(p, w);
  ++*li.launches;
  return cudaGetLastError();
}
// The tensor-core expm: one CTA per SM (its slice buffers and accumulators
// fill shared memory and TMEM), at most one per slab workspace.
static cudaError_t do_expm_oz64(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  if (!w.expm_plan) return cudaErrorInvalidValue;
  const long items = (long)p.n_members * p.n_t;
  ensure_smem_mx(k_expm_prep_oz64, kExpmPrepSmem);
  const int pgrid = grid_for(k_expm_prep_oz64, 256, kExpmPrepSmem, items, 1, li.num_sms, 0);
  k_expm_prep_oz64<<<pgrid, 256, kExpmPrepSmem, li.stream>>>(p, w);
  ++*li.launches;
  if (const cudaError_t e = cudaGetLastError(); e != cudaSuccess) return e;
  ensure_smem_mx(k_expm_oz64, oz::kExpmSmem);
  long grid = li.num_sms;
  if (grid > items) grid = items;
  if (grid > w.slab_teams) grid = w.slab_teams;
  k_expm_oz64<<<(int)grid, oz::kExpmThreads, oz::kExpmSmem, li.stream>>>(p, w);
  ++*li.launches;
  return cudaGetLastError();
}
// The register-resident expm (D <= 8): 256-thread blocks walking the items in
// warp-sized groups of slices, as many blocks as are resident at once.
template <int D, bool MULTI>
static cudaError_t do_expm_small(const sm::Set& set, const LaunchInfo& li) {
  constexpr long kPerBlock = (sm::kSmallThreads / 32) * sm::Grp<D>::SPW;
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sm::k_expm_small<D, MULTI>, sm::kSmallThreads, 0);
  long blocks = (set.items + kPerBlock - 1) / kPerBlock;
  const long cap = (long)li.num_sms * (per_sm < 1 ? 1 : per_sm);
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  sm::k_expm_small<D, MULTI><<<(int)blocks, sm::kSmallThreads, 0, li.stream>>>(set);
  ++*li.launches;
  return cudaGetLastError();
}
// The register-resident kernel runs at D = 2 only.  Measured on GB300 in the
// uneven batch's classes (one evaluation of all problems of a dimension):
//   - D = 2: 4.3 -> 2.8 ms, with one shared launch for the class;
//   - D = 4 and 8 lose: 5.7 -> 6.6 and 14.5 -> 85.7 ms.  A shuffle moves 4
//     bytes per lane and instruction where a shared-memory broadcast moves
//     16, and at D = 8 its 230 registers leave one block per SM.
// The shared-memory teams of D = 4 and 8 in one shared launch per class were
// slower as well (6.2 and 15.9 ms): the class's pipelines then wait for all
// of its propagators instead of overlapping on the batch's streams.  So
// batches share a launch only at D = 2.
int expm_small_align(int Dp) { return Dp == 2 ? sm::Grp<2>::SPW : 1; }
cudaError_t launch_expm_small_set(int Dp, const ProbDev* ps, const WorkDev* ws, const long* first, int n,
                                  long items, const LaunchInfo& li) {
  if (Dp != 2) return cudaErrorInvalidValue;
  sm::Set set{};
  set.ps = ps;
  set.ws = ws;
  set.first = first;
  set.n = n;
  set.items = items;
  return do_expm_small<2, true>(set, li);
}
cudaError_t launch_expm_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  if (p.Dp == 2) {
    sm::Set set{};
    set.p0 = p;
    set.w0 = w;
    set.items = (long)p.n_members * p.n_t;
    return do_expm_small<2, false>(set, li);
  }
  const int t = li.team[kTuneExpmMx] ? li.team[kTuneExpmMx] : mixed_default_team(p, kTuneExpmMx);
  if (t == kTeamTensor) {
    if (!expm_tc_eligible(p)) return cudaErrorInvalidValue;
    return do_expm_oz64(p, w, li);
  }
  PGX_DISPATCH_MX_T(p.Dp, t, return (do_expm_mx<D_, T_>(p, w, li)));
  return cudaSuccess;
}

template <int D>
static cudaError_t do_chain_fwd_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool store) {
  using G = Cfg<D>;
  if (p.target != TGT_GATE) {
    constexpr int TPC = StCfg<D>::TPC;
    if constexpr (D >= 16) {
      const size_t smem = st_fwd_split_bytes<D>(p.n_pairs);
      ensure_smem_mx(k_chain_states_fwd_split_mx<D>, smem);
      k_chain_states_fwd_split_mx<D><<<p.n_members, 32 * kStW, smem, li.stream>>>(p, w, store ? 1 : 0);
      ++*li.launches;
      return cudaGetLastError();
    }
    const size_t smem = (size_t)TPC * st_fwd_team_bytes<D>(p.n_pairs);
    ensure_smem_mx(k_chain_states_fwd_mx<D>, smem);
    k_chain_states_fwd_mx<D><<<(p.n_members + TPC - 1) / TPC, 32 * TPC, smem, li.stream>>>(p, w, store ? 1 : 0);
    ++*li.launches;
    return cudaGetLastError();
  }
  if (w.pit_blocks <= 1) {
    const size_t smem = (size_t)G::TPC * (2 * D * D + G::T) * sizeof(float4);
    ensure_smem_mx(k_chain_gate_fwd_mx<D>, smem);
    k_chain_gate_fwd_mx<D><<<(p.n_members + G::TPC - 1) / G::TPC, G::THREADS, smem, li.stream>>>(p, w, store);
    ++*li.launches;
    return cudaGetLastError();
  }
  const int expm_team = li.team[kTuneExpmMx] ? li.team[kTuneExpmMx] : mixed_default_team(p, kTuneExpmMx);
  if (D == 64 && expm_team == kTeamTensor) {
    // the in-block prefixes on the tensor-core expm's engine (pgx_expm_oz.cuh)
    ensure_smem_mx(k_chainf_local_oz64, oz::kExpmSmem);
    const long items = (long)p.n_members * w.pit_blocks;
    k_chainf_local_oz64<<<items < li.num_sms ? (int)items : li.num_sms, oz::kExpmThreads, oz::kExpmSmem,
                          li.stream>>>(p, w, store);
  } else {
    using PC = PreCfg<D>;
    const size_t smem_l = (size_t)PC::TPC * 2 * D * D * sizeof(float4);
    auto local = k_chainf_local_mx<D, false>;
    if constexpr (D == 64 && PC::T == 256)
      if (p.lsym) local = k_chainf_local_mx<D, true>;
    ensure_smem_mx(local, smem_l);
    const int grid_l = grid_for(local, PC::THREADS, smem_l, (long)p.n_members * w.pit_blocks, PC::TPC, li.num_sms, 0);
    local<<<grid_l, PC::THREADS, smem_l, li.stream>>>(p, w, store);
  }
  if (D == 64 && expm_team == kTeamTensor) {
    ensure_smem_mx(k_chainf_combine_oz64, oz::kExpmSmem);
    k_chainf_combine_oz64<<<p.n_members < li.num_sms ? p.n_members : li.num_sms, oz::kExpmThreads,
                            oz::kExpmSmem, li.stream>>>(p, w, store);
  } else {
    const size_t smem_c = (size_t)G::TPC * (2 * D * D + G::T) * sizeof(float4);
    auto combine = k_chainf_combine_mx<D, false>;
    if constexpr (D == 64 && G::T == 256)
      if (p.lsym) combine = k_chainf_combine_mx<D, true>;
    ensure_smem_mx(combine, smem_c);
    combine<<<(p.n_members + G::TPC - 1) / G::TPC, G::THREADS, smem_c, li.stream>>>(p, w, store);
  }
  *li.launches += 2;
  if (store && p.n_t > w.pit_len) {
    if constexpr (D == 64) {  // tensor cores (pgx_fix_tc.cuh)
      const size_t smem = 2 * tc::kBBytes + 3 * D * D * sizeof(float2) + tc::kSmemAlign;
      ensure_smem_mx(k_fix_tc64<0>, smem);
      const long items = (long)p.n_members * (p.n_t - w.pit_len);
      k_fix_tc64<0><<<items < li.num_sms ? (int)items : li.num_sms, tc::kThreads, smem, li.stream>>>(p, w);
      ++*li.launches;
      return cudaGetLastError();
    }
    using F = FixCfg<D>;
    const size_t smem_f = (size_t)F::TPC * 2 * Lay<D, 2>::SIZE * sizeof(float2);
    ensure_smem_mx(k_chainf_fix_mx<D>, smem_f);
    const int grid_f = grid_for(k_chainf_fix_mx<D>, F::THREADS, smem_f, (long)p.n_members * (p.n_t - w.pit_len),
                                F::TPC, li.num_sms, 0);
    k_chainf_fix_mx<D><<<grid_f, F::THREADS, smem_f, li.stream>>>(p, w);
    ++*li.launches;
  }
  return cudaGetLastError();
}
cudaError_t launch_chain_fwd_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool store) {
  PGX_DISPATCH_MX(p.Dp, return do_chain_fwd_mx<D_>(p, w, li, store));
  return cudaSuccess;
}

// Prefix teams one SM holds (queried once per dimension; the same on every
// device of one architecture).
template <int D>
static long prefix_teams_per_sm() {
  static std::atomic<int> cached{-1};
  int n = cached.load(std::memory_order_relaxed);
  if (n < 0) {
    using PC = PreCfg<D>;
    const size_t smem = (size_t)PC::TPC * 2 * D * D * sizeof(float4);  // <= 32 KB up to D = 32
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_chainf_local_mx<D, false>, PC::THREADS, smem) !=
        cudaSuccess)
      return 0;
    n = per_sm * PC::TPC;
    cached.store(n, std::memory_order_relaxed);
  }
  return n;
}
long chain_prefix_capacity(int Dp, int num_sms) {
  switch (Dp) {
    case 2: return prefix_teams_per_sm<2>() * num_sms;
    case 4: return prefix_teams_per_sm<4>() * num_sms;
    case 8: return prefix_teams_per_sm<8>() * num_sms;
    case 16: return prefix_teams_per_sm<16>() * num_sms;
    case 32: return prefix_teams_per_sm<32>() * num_sms;
    default: return 0;
  }
}

// In-block suffix products of the parallel-in-time backward chain.  They need
// only the U stack, so the pipeline may run them on a second stream while the
// forward chain runs.
template <int D>
static cudaError_t do_chain_bwd_local_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  using G = SufCfg<D>;
  const size_t smem_l = (size_t)G::TPC * 2 * D * D * sizeof(float2);
  ensure_smem_mx(k_chainb_local_mx<D>, smem_l);
  const int grid_l = grid_for(k_chainb_local_mx<D>, G::THREADS, smem_l, (long)p.n_members * w.pit_blocks, G::TPC,
                              li.num_sms, 0);
  k_chainb_local_mx<D><<<grid_l, G::THREADS, smem_l, li.stream>>>(p, w);
  ++*li.launches;
  return cudaGetLastError();
}

template <int D>
static cudaError_t do_chain_bwd_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool skip_local) {
  using G = Cfg<D>;
  if (p.target != TGT_GATE) {
    constexpr int TPC = StCfg<D>::TPC;
    const size_t smem = (size_t)TPC * st_bwd_team_bytes<D>(p.n_pairs);
    ensure_smem_mx(k_chain_states_bwd_mx<D>, smem);
    k_chain_states_bwd_mx<D><<<(p.n_members + TPC - 1) / TPC, 32 * TPC, smem, li.stream>>>(p, w);
    ++*li.launches;
    return cudaGetLastError();
  }
  if (w.pit_blocks <= 1) {
    const size_t smem = (size_t)G::TPC * 2 * D * D * sizeof(float2);
    ensure_smem_mx(k_chain_gate_bwd_mx<D>, smem);
    k_chain_gate_bwd_mx<D><<<(p.n_members + G::TPC - 1) / G::TPC, G::THREADS, smem, li.stream>>>(p, w);
    ++*li.launches;
    return cudaGetLastError();
  }
  if (!skip_local) {
    const cudaError_t e = do_chain_bwd_local_mx<D>(p, w, li);
    if (e != cudaSuccess) return e;
  }
  const size_t smem_c = (size_t)G::TPC * D * D * sizeof(float2);
  ensure_smem_mx(k_chainb_combine_mx<D>, smem_c);
  k_chainb_combine_mx<D><<<(p.n_members + G::TPC - 1) / G::TPC, G::THREADS, smem_c, li.stream>>>(p, w);
  if constexpr (D == 64) {  // tensor cores (pgx_fix_tc.cuh)
    const size_t smem = 2 * tc::kBBytes + 3 * D * D * sizeof(float2) + tc::kSmemAlign;
    ensure_smem_mx(k_fix_tc64<1>, smem);
    const long items = (long)p.n_members * p.n_t;
    k_fix_tc64<1><<<items < li.num_sms ? (int)items : li.num_sms, tc::kThreads, smem, li.stream>>>(p, w);
    *li.launches += 2;
    return cudaGetLastError();
  }
  using F = FixCfg<D>;
  const size_t smem_f = (size_t)F::TPC * 3 * Lay<D, 2>::SIZE * sizeof(float2);
  ensure_smem_mx(k_chainb_fix_mx<D>, smem_f);
  const int grid_f = grid_for(k_chainb_fix_mx<D>, F::THREADS, smem_f, (long)p.n_members * p.n_t, F::TPC,
                              li.num_sms, 0);
  k_chainb_fix_mx<D><<<grid_f, F::THREADS, smem_f, li.stream>>>(p, w);
  *li.launches += 2;
  return cudaGetLastError();
}
cudaError_t launch_chain_bwd_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li, bool skip_local) {
  PGX_DISPATCH_MX(p.Dp, return do_chain_bwd_mx<D_>(p, w, li, skip_local));
  return cudaSuccess;
}
cudaError_t launch_chain_bwd_local_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  if (p.target != TGT_GATE || w.pit_blocks <= 1) return cudaSuccess;
  PGX_DISPATCH_MX(p.Dp, return do_chain_bwd_local_mx<D_>(p, w, li));
  return cudaSuccess;
}

template <int D, int T>
static cudaError_t do_grad_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  using G = CfgM<D, T>;
  const size_t smem = G::SMEM_G;
  ensure_smem_mx(k_grad_gate_mx<D, T>, smem);
  const int grid = grid_for(k_grad_gate_mx<D, T>, G::THREADS, smem, (long)p.n_members * p.n_t, G::TPC,
                            li.num_sms, 0);
  k_grad_gate_mx<D, T><<<grid, G::THREADS, smem, li.stream>>>(p, w);
  ++*li.launches;
  return cudaGetLastError();
}
cudaError_t launch_prep_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  const int n = p.n_t * p.n_c;
  k_prep_mx<<<(n + 255) / 256, 256, 0, li.stream>>>(w.u, w.u_df, n);
  ++*li.launches;
  return cudaGetLastError();
}

static cudaError_t do_grad_tc64(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  const size_t smem = 4 * tc::kBBytesF16 + 3 * gtc::kMatBytes + gtc::kMkBytes + tc::kSmemAlign;
  ensure_smem_mx(k_grad_tc64, smem);
  const long items = (long)p.n_members * p.n_t;
  const int grid = items < li.num_sms ? (int)items : li.num_sms;  // one CTA per SM: TMEM and shared memory
  k_grad_tc64<<<grid, tc::kThreads, smem, li.stream>>>(p, w);
  ++*li.launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int nj = p.n_c < kTraceCtrls ? p.n_c : kTraceCtrls;
  const size_t tsmem = (size_t)nj * 64 * 64 * sizeof(float2);
  ensure_smem_mx(k_trace_tc64, tsmem);
  const long tgrid = (items + 7) / 8;
  k_trace_tc64<<<tgrid < li.num_sms ? (int)tgrid : li.num_sms, 256, tsmem, li.stream>>>(p, w);
  ++*li.launches;
  return cudaGetLastError();
}

int grad_tc_check() {
  int flag = 0, ex = 0;
  if (cudaMemcpyFromSymbol(&flag, g_grad_tc_timeout, sizeof(int)) != cudaSuccess ||
      cudaMemcpyFromSymbol(&ex, g_expm_tc_timeout, sizeof(int)) != cudaSuccess)
    return -1;
  const int zero = 0;
  if (flag) cudaMemcpyToSymbol(g_grad_tc_timeout, &zero, sizeof(int));
  if (ex) cudaMemcpyToSymbol(g_expm_tc_timeout, &zero, sizeof(int));
  return flag | (ex ? 1 : 0);
}

template <int D>
static cudaError_t do_refine_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  const size_t smem = (2 * (size_t)D * D + kRefThreads) * sizeof(double2);
  ensure_smem_mx(k_refine_unitary_mx<D>, smem);
  k_refine_unitary_mx<D><<<p.n_members, kRefThreads, smem, li.stream>>>(p, w);
  ++*li.launches;
  return cudaGetLastError();
}
bool refine_applies(const ProbDev& p) { return p.gen == GEN_HERM && p.target == TGT_GATE; }
bool tc_kernels_used(const ProbDev& p) { return p.Dp == 64; }
cudaError_t launch_refine_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  if (!refine_applies(p)) return cudaSuccess;
  PGX_DISPATCH_MX(p.Dp, return (do_refine_mx<D_>(p, w, li)));
  return cudaSuccess;
}

cudaError_t launch_grad_mx(const ProbDev& p, const WorkDev& w, const LaunchInfo& li) {
  const int t = li.team[kTuneGradMx] ? li.team[kTuneGradMx] : mixed_default_team(p, kTuneGradMx);
  if (t == kTeamTensor) {
    if (!grad_tc_eligible(p)) return cudaErrorInvalidValue;
    return do_grad_tc64(p, w, li);
  }
  if (p.Dp == 64 && t == 512) return do_grad_mx<64, 512>(p, w, li);
  PGX_DISPATCH_MX_T(p.Dp, t, return (do_grad_mx<D_, T_>(p, w, li)));
  return cudaSuccess;
}

}  // namespace pgx
