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

// Taylor block C_i = c_{4i} I + c_{4i+1} B + c_{4i+2} B2 + c_{4i+3} B3 in df;
// coef[k] = 1/k! as df.
__device__ __forceinline__ dfc df_block(int i, int r, int c, const float4& b1, const float4& b2,
                                        const float4& b3, const df* coef) {
  dfc v = dfc_scale(dfc_load(b1), coef[4 * i + 1]);
  v = dfc_add(v, dfc_scale(dfc_load(b2), coef[4 * i + 2]));
  v = dfc_add(v, dfc_scale(dfc_load(b3), coef[4 * i + 3]));
  if (r == c) v.re = df_add(v.re, coef[4 * i]);
  return v;
}

// Y = T_m(B)^(2^s) in df (B = A / 2^s on entry).  Same Paterson-Stockmeyer
// schedule as taylor_exp: m = 4L costs 3 + (L - 1) products, then s squarings.
// Horner steps i >= lo_from multiply B4 by a tail of size <= 1/(4(i+1))!; the
// caller sets lo_from where D u32 ||B4||^(i+1) / (4(i+1))! is below df
// precision, and those steps run in plain FP32.
template <int D, int T, int SW = 0>
__device__ void taylor_exp_df(const Team<T>& tm, float4* B, float4* B2, float4* B3, float4* B4, float4* Y,
                              int m, int s, const df* coef, int lo_from = 1 << 30) {
  mm1_df<D, T, SW>(tm, B2, B, B);
  mm1_df<D, T, SW>(tm, B3, B2, B);
  mm1_df<D, T, SW>(tm, B4, B2, B2);
  const int L = m / 4;
  for (int q = tm.lane; q < D * D; q += T) {
    const int r = q % D, c = q / D, e = Lay<D, SW>::idx(r, c);
    dfc v = df_block(L - 1, r, c, B[e], B2[e], B3[e], coef);
    Y[e] = dfc_store(dfc_add(v, dfc_scale(dfc_load(B4[e]), coef[4 * L])));
  }
  tm.sync();
  for (int i = L - 2; i >= 0; --i) {
    const auto add_block = [=](int e, int r, int c, dfc v) {
      return dfc_add(v, df_block(i, r, c, B[e], B2[e], B3[e], coef));
    };
    if (i >= lo_from)
      mm_df_lo<D, T, SW>(tm, Y, B4, Y, add_block);
    else
      mm_df<D, T, false, SW>(tm, Y, B4, Y, (const float4*)nullptr, (const float4*)nullptr, add_block);
  }
  for (int k = 0; k < s; ++k) mm1_df<D, T, SW>(tm, Y, Y, Y);
}

}  // namespace pgx
