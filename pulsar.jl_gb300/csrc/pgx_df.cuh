// Double-float ("df") complex arithmetic on the FP32 pipe.
//
// A df number is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// giving ~44 significant bits.  GB300 issues FP32 FMAs at 64x its FP64 rate,
// so a df product (~12 FP32 operations per real multiply-add) is several times
// faster than an FP64 one while keeping the propagator chain accurate to
// ~1e-13.  The error-free transformations are the classical ones:
//   two_sum  (Knuth):  s = a + b exactly as s + e
//   two_prod (FMA):    p = a * b exactly as p + e with e = fma(a, b, -p)
// A df complex entry is stored as float4 {re.hi, im.hi, re.lo, im.lo}: the
// first two floats are the float2 rounding of the value, so FP32 consumers can
// read the leading half of a df stack directly.
#pragma once
#include <cuda_runtime.h>

#include "pgx_device.cuh"

namespace pgx {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}

struct df { float hi, lo; };

__device__ __forceinline__ df df_from(double x) {
  df r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}
__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df df_add(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  df r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  df r;
  fast_two_sum(p, e, r.hi, r.lo);
  return r;
}

// complex df in registers
struct dfc { df re, im; };

__device__ __forceinline__ dfc dfc_load(const float4& v) { return {{v.x, v.z}, {v.y, v.w}}; }
__device__ __forceinline__ float4 dfc_store(const dfc& a) { return make_float4(a.re.hi, a.im.hi, a.re.lo, a.im.lo); }
__device__ __forceinline__ dfc dfc_from(double2 v) { return {df_from(v.x), df_from(v.y)}; }
__device__ __forceinline__ double2 dfc_to(const dfc& a) { return make_double2(df_to(a.re), df_to(a.im)); }
__device__ __forceinline__ dfc dfc_add(const dfc& a, const dfc& b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ dfc dfc_scale(const dfc& a, df s) { return {df_mul(a.re, s), df_mul(a.im, s)}; }

// Accumulator of a complex df dot product: leading sums s (two_sum chain) and
// a float compensation c collecting every rounding error and the cross terms.
struct DfAcc {
  float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
  __device__ __forceinline__ void mac(const float4& a, const float4& b) {
    // leading products, exact as p + e
    const float p1 = a.x * b.x, p2 = -(a.y * b.y), p3 = a.x * b.y, p4 = a.y * b.x;
    const float e1 = fmaf(a.x, b.x, -p1), e2 = fmaf(-a.y, b.y, -p2);
    const float e3 = fmaf(a.x, b.y, -p3), e4 = fmaf(a.y, b.x, -p4);
    // cross terms hi*lo + lo*hi
    float xr = fmaf(a.x, b.z, e1 + e2);
    xr = fmaf(a.z, b.x, xr);
    xr = fmaf(-a.y, b.w, xr);
    xr = fmaf(-a.w, b.y, xr);
    float xi = fmaf(a.x, b.w, e3 + e4);
    xi = fmaf(a.z, b.y, xi);
    xi = fmaf(a.y, b.z, xi);
    xi = fmaf(a.w, b.x, xi);
    float t, e;
    two_sum(sr, p1, t, e);
    cr += e;
    two_sum(t, p2, sr, e);
    cr += e + xr;
    two_sum(si, p3, t, e);
    ci += e;
    two_sum(t, p4, si, e);
    ci += e + xi;
  }
  __device__ __forceinline__ dfc result() const {
    dfc r;
    two_sum(sr, cr, r.re.hi, r.re.lo);
    two_sum(si, ci, r.im.hi, r.im.lo);
    return r;
  }
};

struct DfEpiNone {
  __device__ __forceinline__ dfc operator()(int, int, int, dfc v) const { return v; }
};

// out = A1*B1 (+ A2*B2) in df, then epi(e, r, c, value); out may alias inputs.
template <int D, int T, bool TWO, int SW = 0, class Epi>
__device__ __forceinline__ void mm_df(const Team<T>& tm, float4* out, const float4* A1, const float4* B1,
                                      const float4* A2, const float4* B2, Epi epi) {
  using BK = Blocking<D, T>;
  using L = Lay<D, SW>;
  constexpr int RB = BK::RB, CB = BK::CB;
  const bool active = tm.lane < BK::ACTIVE;
  const int rb = tm.lane % BK::NR, cb = tm.lane / BK::NR;
  DfAcc acc[RB][CB];
  float4 res[RB][CB];
  // at D = 64 a lane owns 16 accumulators: an unrolled k-loop overflows the
  // instruction cache (ncu: "no instruction" stalls)
  constexpr int UNR = (D >= 64) ? 1 : 2;
  if (active) {
#pragma unroll UNR
    for (int k = 0; k < D; ++k) {
      float4 a[RB], b[CB];
#pragma unroll
      for (int i = 0; i < RB; ++i) a[i] = A1[L::idx(rb + BK::NR * i, k)];
#pragma unroll
      for (int j = 0; j < CB; ++j) b[j] = B1[L::idx(k, cb + BK::NCB * j)];
#pragma unroll
      for (int i = 0; i < RB; ++i)
#pragma unroll
        for (int j = 0; j < CB; ++j) acc[i][j].mac(a[i], b[j]);
    }
    if constexpr (TWO) {
#pragma unroll UNR
      for (int k = 0; k < D; ++k) {
        float4 a[RB], b[CB];
#pragma unroll
        for (int i = 0; i < RB; ++i) a[i] = A2[L::idx(rb + BK::NR * i, k)];
#pragma unroll
        for (int j = 0; j < CB; ++j) b[j] = B2[L::idx(k, cb + BK::NCB * j)];
#pragma unroll
        for (int i = 0; i < RB; ++i)
#pragma unroll
          for (int j = 0; j < CB; ++j) acc[i][j].mac(a[i], b[j]);
      }
    }
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const int r = rb + BK::NR * i, c = cb + BK::NCB * j;
        res[i][j] = dfc_store(epi(L::idx(r, c), r, c, acc[i][j].result()));
      }
  }
  tm.sync();
  if (active) {
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < CB; ++j) out[L::idx(rb + BK::NR * i, cb + BK::NCB * j)] = res[i][j];
  }
  tm.sync();
}

// out = A*B from the FP32 (leading) parts of df operands, plain FP32
// accumulation, then epi(e, r, c, value as df) -- for products whose
// contribution is small enough that FP32 rounding stays below df precision.
template <int D, int T, int SW = 0, class Epi>
__device__ __forceinline__ void mm_df_lo(const Team<T>& tm, float4* out, const float4* A, const float4* B,
                                         Epi epi) {
  using BK = Blocking<D, T>;
  using L = Lay<D, SW>;
  constexpr int RB = BK::RB, CB = BK::CB;
  const bool active = tm.lane < BK::ACTIVE;
  const int rb = tm.lane % BK::NR, cb = tm.lane / BK::NR;
  float2 acc[RB][CB];
#pragma unroll
  for (int i = 0; i < RB; ++i)
#pragma unroll
    for (int j = 0; j < CB; ++j) acc[i][j] = make_float2(0.f, 0.f);
  float4 res[RB][CB];
  if (active) {
#pragma unroll 4
    for (int k = 0; k < D; ++k) {
      float2 a[RB], b[CB];
#pragma unroll
      for (int i = 0; i < RB; ++i) {
        const float4 v = A[L::idx(rb + BK::NR * i, k)];
        a[i] = make_float2(v.x, v.y);
      }
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const float4 v = B[L::idx(k, cb + BK::NCB * j)];
        b[j] = make_float2(v.x, v.y);
      }
#pragma unroll
      for (int i = 0; i < RB; ++i)
#pragma unroll
        for (int j = 0; j < CB; ++j) acc[i][j] = cmac(acc[i][j], a[i], b[j]);
    }
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const int r = rb + BK::NR * i, c = cb + BK::NCB * j;
        const dfc v = {{acc[i][j].x, 0.f}, {acc[i][j].y, 0.f}};
        res[i][j] = dfc_store(epi(L::idx(r, c), r, c, v));
      }
  }
  tm.sync();
  if (active) {
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < CB; ++j) out[L::idx(rb + BK::NR * i, cb + BK::NCB * j)] = res[i][j];
  }
  tm.sync();
}

template <int D, int T, int SW = 0>
__device__ __forceinline__ void mm1_df(const Team<T>& tm, float4* out, const float4* A, const float4* B) {
  mm_df<D, T, false, SW>(tm, out, A, B, (const float4*)nullptr, (const float4*)nullptr, DfEpiNone{});
}

// Merge of two partial dot products held by lanes lane and lane ^ off of one
// warp (both lanes end with the same sums: two_sum is exact, so its error term
// does not depend on the operand order).
__device__ __forceinline__ void dfacc_merge_xor(DfAcc& a, int off) {
  const float sr = __shfl_xor_sync(0xffffffffu, a.sr, off), cr = __shfl_xor_sync(0xffffffffu, a.cr, off);
  const float si = __shfl_xor_sync(0xffffffffu, a.si, off), ci = __shfl_xor_sync(0xffffffffu, a.ci, off);
  float t, e;
  two_sum(a.sr, sr, t, e);
  a.sr = t;
  a.cr = (a.cr + cr) + e;
  two_sum(a.si, si, t, e);
  a.si = t;
  a.ci = (a.ci + ci) + e;
}

// Split of the k range of a triangular product: a power of two dividing D,
// fixed per D so that every team size sums each entry in the same order.
template <int D> struct TriSplit {
  static constexpr int KS = (D >= 64) ? 1 : (D >= 32) ? 2 : 4;
};

// out = A*B in df for a product known to be Hermitian (anti = false) or
// anti-Hermitian (anti = true) -- the powers of an anti-Hermitian matrix.
// Only the D(D+1)/2 entries of the lower triangle are computed; the upper
// triangle is written as their conjugates (negated when anti).
//  - Entries are enumerated by row pairs: pair p (0 <= p < D/2) holds row
//    D-1-p (columns 0..D-1-p) then row p (columns 0..p), D+1 entries each.
//  - Each entry's dot product is split over KS consecutive lanes: lane q
//    takes k = q, q + KS, ..., and the partial sums are merged by a fixed
//    xor-shuffle tree.
//  - Within each aligned block of 8 entries the groups are permuted so the
//    8 lanes of one 128-bit shared-memory phase read KS consecutive k of
//    columns KS apart: distinct banks for the B operand, a broadcast for A.
// out must not alias A or B, and no lane may still read out from an earlier
// step (each entry is stored as soon as its dot product completes).
// Column-major layouts only (SW != 1).
template <int D, int T, int SW = 0>
__device__ __forceinline__ void mm_df_tri(const Team<T>& tm, float4* out, const float4* A, const float4* B,
                                          bool anti) {
  static_assert(SW != 1, "mm_df_tri indexes k linearly");
  static_assert(T >= 32 && T % 32 == 0, "mm_df_tri shuffles within whole warps");
  static_assert(D % 2 == 0 && D >= 8, "mm_df_tri pairs rows");
  using L = Lay<D, SW>;
  constexpr int KS = TriSplit<D>::KS, G = 8 / KS, KK = D / KS;
  constexpr int NT = D * (D + 1) / 2, NTP = (NT + 7) / 8 * 8;
  constexpr int NO = (NTP * KS + T - 1) / T;
  constexpr int UNR = (D >= 64) ? 1 : 2;  // code size: the kernel is instruction-cache bound
  constexpr int PR = (NO < 2) ? NO : 2;
  // rounds whose entries all lie in full blocks of 8 need no bounds test
  constexpr int SAFE = (NT / 8) * 8 * KS / T;
  const int q = tm.lane % KS;
  const float sg = anti ? -1.f : 1.f;  // upper (c, r) = sg conj(lower (r, c))
  // PR rounds at a time: their accumulators, merged and stored before the
  // next ones start (out is not an operand, so no barrier is needed first)
#pragma unroll
  for (int i0 = 0; i0 < NO; i0 += PR) {
    int ia[PR], ib[PR];  // storage index of (r, q) and of (q, c); ia = -1: no entry
#pragma unroll
    for (int u = 0; u < PR; ++u) {
      const int i = i0 + u;
      const int g = (tm.lane + T * i) / KS, x = g % 8;
      const int e = (g - x) + x / G + KS * (x % G);
      const int pr = e / (D + 1), j = e % (D + 1);
      const bool lo_row = j < D - pr;
      const int r = lo_row ? D - 1 - pr : pr, c = lo_row ? j : j - (D - pr);
      const bool ok = i < NO && (i < SAFE || e < NT);
      ia[u] = ok ? L::idx(r, q) : -1;
      ib[u] = ok ? L::idx(q, c) : 0;
    }
    DfAcc acc[PR];
#pragma unroll UNR
    for (int j = 0; j < KK; ++j) {
#pragma unroll
      for (int u = 0; u < PR; ++u)
        if ((i0 + u < SAFE) || ia[u] >= 0) acc[u].mac(A[ia[u] + L::LD * KS * j], B[ib[u] + KS * j]);
    }
#pragma unroll
    for (int u = 0; u < PR; ++u) {
      if (i0 + u >= NO) continue;  // uniform over the team
#pragma unroll
      for (int off = 1; off < KS; off <<= 1) dfacc_merge_xor(acc[u], off);
      if (q != 0 || (i0 + u >= SAFE && ia[u] < 0)) continue;
      const int r = ia[u], c = ib[u] / L::LD;  // q = 0: ia = r, ib = LD c
      const float4 v = dfc_store(acc[u].result());
      out[L::idx(r, c)] = v;
      if (r != c)
        out[L::idx(c, r)] = make_float4(sg * v.x, -sg * v.y, sg * v.z, -sg * v.w);
    }
  }
  tm.sync();
}

// Hermiticity-preserving superoperators.  With vec(rho) indices a = i + d j
// (D = d^2) and the swap sigma(i + d j) = j + d i, a Lindblad generator and
// every polynomial in it satisfy X[a][b] = conj(X[sigma a][sigma b]).  So a
// product of two such matrices is determined by its d(d+1)/2 columns
// b = i + d j with i >= j; the other d(d-1)/2 columns are the conjugates of
// permuted entries.
template <int D> struct LSym {
  static constexpr int d = (D == 64) ? 8 : (D == 16) ? 4 : (D == 4) ? 2 : 0;
  static constexpr int NC = d * (d + 1) / 2;  // kept columns (i >= j)
  static constexpr int NM = d * (d - 1) / 2;  // mirrored columns (i < j)
};
// t -> (r, c), r >= c, in row-major order of the lower triangle (diagonal
// included when incl, else strictly below it).
__device__ __forceinline__ void lower_decode(int t, bool incl, int& r, int& c) {
  const int o = incl ? 0 : 1;  // strict: row r holds r entries
  r = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f) + o;
  while ((r + 1 - o) * (r + 2 - o) / 2 <= t) ++r;
  while ((r - o) * (r + 1 - o) / 2 > t) --r;
  c = t - (r - o) * (r + 1 - o) / 2;
}

// out = A*B for Hermiticity-preserving superoperators (LSym), df (LO =
// false) or plain FP32 from the leading halves (LO = true, as mm_df_lo), then
// epi(e, r, c, value) on the kept entries.  Lane (r, g) = (lane % D, lane / D)
// computes row r of the kept columns g, g + T/D, ...: the A reads of a warp
// are one column (consecutive rows), the B reads broadcast.  The mirrored
// columns are written after a barrier.  out may alias A or B.
template <int D, int T, bool LO, int SW, class Epi>
__device__ __forceinline__ void mm_df_lsym(const Team<T>& tm, float4* out, const float4* A, const float4* B,
                                           Epi epi) {
  using S = LSym<D>;
  using L = Lay<D, SW>;
  static_assert(S::d > 0 && T % D == 0 && S::NC % (T / D) == 0, "lsym blocking");
  constexpr int NG = T / D, CB = S::NC / NG;
  const int r = tm.lane % D, g = tm.lane / D;
  int col[CB];
#pragma unroll
  for (int u = 0; u < CB; ++u) {
    int i, j;
    lower_decode(g + NG * u, true, i, j);
    col[u] = i + S::d * j;
  }
  float4 res[CB];
  if constexpr (LO) {
    float2 acc[CB];
#pragma unroll
    for (int u = 0; u < CB; ++u) acc[u] = make_float2(0.f, 0.f);
#pragma unroll 2
    for (int k = 0; k < D; ++k) {
      const float4 a = A[L::idx(r, k)];
#pragma unroll
      for (int u = 0; u < CB; ++u) {
        const float4 b = B[L::idx(k, col[u])];
        acc[u] = cmac(acc[u], make_float2(a.x, a.y), make_float2(b.x, b.y));
      }
    }
#pragma unroll
    for (int u = 0; u < CB; ++u) {
      const dfc v = {{acc[u].x, 0.f}, {acc[u].y, 0.f}};
      res[u] = dfc_store(epi(L::idx(r, col[u]), r, col[u], v));
    }
  } else {
    DfAcc acc[CB];
#pragma unroll 1
    for (int k = 0; k < D; ++k) {
      const float4 a = A[L::idx(r, k)];
#pragma unroll
      for (int u = 0; u < CB; ++u) acc[u].mac(a, B[L::idx(k, col[u])]);
    }
#pragma unroll
    for (int u = 0; u < CB; ++u) res[u] = dfc_store(epi(L::idx(r, col[u]), r, col[u], acc[u].result()));
  }
  tm.sync();
#pragma unroll
  for (int u = 0; u < CB; ++u) out[L::idx(r, col[u])] = res[u];
  tm.sync();
  for (int e = tm.lane; e < S::NM * D; e += T) {  // column b = i + d j (i < j) from (sigma a, sigma b)
    const int a = e % D;
    int jj, ii;
    lower_decode(e / D, false, jj, ii);  // jj > ii
    const int b = ii + S::d * jj, sb = jj + S::d * ii, sa = a / S::d + S::d * (a % S::d);
    const float4 v = out[L::idx(sa, sb)];
    out[L::idx(a, b)] = make_float4(v.x, -v.y, v.z, -v.w);
  }
  tm.sync();
}

// Taylor block C_i = sum_{j<q} c_{qi+j} B^j in df at storage index e (B^0 =
// I; b1, b2, b3 hold B, B^2, B^3); coef[k] = 1/k! as df.
__device__ __forceinline__ dfc df_block(int i, int q, int r, int c, int e, const float4* b1, const float4* b2,
                                        const float4* b3, const df* coef) {
  const int o = q * i;
  dfc v = dfc_scale(dfc_load(b1[e]), coef[o + 1]);
  if (q >= 3) v = dfc_add(v, dfc_scale(dfc_load(b2[e]), coef[o + 2]));
  if (q >= 4) v = dfc_add(v, dfc_scale(dfc_load(b3[e]), coef[o + 3]));
  if (r == c) v.re = df_add(v.re, coef[o]);
  return v;
}

// Y = T_m(B)^(2^s) in df (B = A / 2^s on entry), Paterson-Stockmeyer with
// block size q in {2, 3, 4} and m = q L:
//   powers B^2 .. B^q (q - 1 products),
//   Y = C_{L-1} + c_m B^q,  Y <- B^q Y + C_i for i = L-2 .. 0,
// then s squarings.  Horner steps i >= lo_from multiply B^q by a tail of
// size <= e^a / (q(i+1))!; the caller sets lo_from where that step's FP32
// error, carried through i more factors B^q, stays below df precision, and
// those steps run in plain FP32.
// HERM (D >= 16, column-major layouts): B is anti-Hermitian, so B^2 and B^4
// are Hermitian and B^3 anti-Hermitian, and their products run as triangular
// ones.  The power products share one call site (one copy of the product's
// code: the kernel is instruction-cache bound otherwise).
// LSYM: B is a Hermiticity-preserving superoperator (LSym<D>, T a multiple of
// D): every product keeps d(d+1)/2 columns and mirrors the rest.
template <int D, int T, int SW = 0, bool HERM = false, bool LSYM = false>
__device__ void taylor_exp_df(const Team<T>& tm, float4* B, float4* B2, float4* B3, float4* B4, float4* Y,
                              int m, int q, int s, const df* coef, int lo_from = 1 << 30) {
  constexpr bool TRI = HERM && D >= 16 && SW != 1;
#pragma unroll 1
  for (int st = 0; st < q - 1; ++st) {  // B2 = B B, B3 = B2 B, B4 = B2 B2
    const float4* X = (st == 0) ? B : B2;
    const float4* Z = (st == 2) ? B2 : B;
    float4* out = (st == 0) ? B2 : (st == 1) ? B3 : B4;
    if constexpr (TRI)
      mm_df_tri<D, T, SW>(tm, out, X, Z, st == 1);
    else if constexpr (LSYM)
      mm_df_lsym<D, T, false, SW>(tm, out, X, Z, DfEpiNone{});
    else
      mm1_df<D, T, SW>(tm, out, X, Z);
  }
  const float4* Bq = (q == 2) ? B2 : (q == 3) ? B3 : B4;
  const int L = m / q;
  for (int t = tm.lane; t < D * D; t += T) {
    const int r = t % D, c = t / D, e = Lay<D, SW>::idx(r, c);
    dfc v = df_block(L - 1, q, r, c, e, B, B2, B3, coef);
    Y[e] = dfc_store(dfc_add(v, dfc_scale(dfc_load(Bq[e]), coef[m])));
  }
  tm.sync();
  for (int i = L - 2; i >= 0; --i) {
    const auto add_block = [=](int e, int r, int c, dfc v) {
      return dfc_add(v, df_block(i, q, r, c, e, B, B2, B3, coef));
    };
    if constexpr (LSYM) {
      if (i >= lo_from)
        mm_df_lsym<D, T, true, SW>(tm, Y, Bq, Y, add_block);
      else
        mm_df_lsym<D, T, false, SW>(tm, Y, Bq, Y, add_block);
    } else {
      if (i >= lo_from)
        mm_df_lo<D, T, SW>(tm, Y, Bq, Y, add_block);
      else
        mm_df<D, T, false, SW>(tm, Y, Bq, Y, (const float4*)nullptr, (const float4*)nullptr, add_block);
    }
  }
  for (int k = 0; k < s; ++k) {
    if constexpr (LSYM)
      mm_df_lsym<D, T, false, SW>(tm, Y, Y, Y, DfEpiNone{});
    else
      mm1_df<D, T, SW>(tm, Y, Y, Y);
  }
}

}  // namespace pgx
