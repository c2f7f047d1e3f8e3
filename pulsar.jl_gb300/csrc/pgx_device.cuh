// Device building blocks for the GRAPE hot path on sm_103a.
//
// A "team" of T threads owns one D x D complex matrix problem.  T = 32 (one
// warp, __syncwarp) for D <= 8 and T = 256 (one CTA, __syncthreads) for
// D >= 16.  Matrices are column-major, element (r, c) at r + D*c, stored as
// interleaved complex (double2 / float2) -- the layout of Julia's
// Matrix{ComplexF64} and of the C-ABI buffers.
//
// Products stage every lane's outputs in registers before a team barrier and
// only then write, so an output may alias an input (Y = B4 * Y in place).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "taylor_table.h"

namespace pgx {

template <class R> struct CxOf;
template <> struct CxOf<double> { using type = double2; };
template <> struct CxOf<float> { using type = float2; };

template <class C> __device__ __forceinline__ C czero() { C z; z.x = 0; z.y = 0; return z; }
template <class C, class R> __device__ __forceinline__ C cmake(R x, R y) { C z; z.x = x; z.y = y; return z; }

// acc += a * b
template <class C> __device__ __forceinline__ C cmac(C acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
// acc += conj(a) * b
template <class C> __device__ __forceinline__ C cmac_cj(C acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
template <class C> __device__ __forceinline__ C cmul(C a, C b) { return cmac(czero<C>(), a, b); }
template <class C, class R> __device__ __forceinline__ C cscale(C a, R s) { a.x *= s; a.y *= s; return a; }
template <class C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }

// A team synchronises with __syncwarp (T <= 32) or with hardware barrier
// `bar` over its T threads (bar = 0 and T = blockDim is __syncthreads; several
// multi-warp teams in one CTA use barriers 1, 2, ...).
template <int T> struct Team {
  int lane;
  int bar = 0;
  __device__ __forceinline__ void sync() const {
    if constexpr (T <= 32) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(T) : "memory");
    }
  }
};

struct EpiNone {
  template <class C> __device__ __forceinline__ C operator()(int, int, int, C s) const { return s; }
};

// Storage of a D x D matrix in a team's shared memory.  SW = 0: column-major,
// (r, c) at r + D c.  SW = 1: XOR-swizzled column-major, (r, c) at
// (r ^ c) + D c (D a power of two): every column is still one contiguous
// block, but the same row of different columns lands in different banks, so
// the row-wise operand loads of a product are conflict-free.
template <int D, int SW> struct Lay {
  // SW = 0: column-major, leading dimension D.  SW = 1: rows XOR-swizzled by
  // the column.  SW = 2: column-major with leading dimension D + 1, so the
  // columns one warp reads at the same k fall in different shared-memory
  // banks; the inner-loop index stays one multiply-add.
  static constexpr int LD = (SW == 2) ? D + 1 : D;
  static constexpr int SIZE = LD * D;  // storage elements of one matrix
  __device__ __forceinline__ static int idx(int r, int c) { return (SW == 1 ? (r ^ (c & (D - 1))) : r) + LD * c; }
};

// Register blocking of a D x D product over T lanes: each lane owns an RB x CB
// block of outputs, interleaved (rows rb + NR*i, columns cb + NCB*j) so the
// lanes of one load instruction touch consecutive rows / columns.  With one
// output per lane (RB = CB = 1) lanes beyond D*D idle.
template <int D, int T> struct Blocking {
  static constexpr int NE = (D * D >= T) ? D * D / T : 1;
  static constexpr int RB = (NE >= 2 && D % 2 == 0) ? 2 : 1;
  static constexpr int CB = NE / RB;
  static constexpr int NR = D / RB;               // row blocks
  static constexpr int NCB = D / CB;              // column blocks
  static constexpr int ACTIVE = NR * NCB;         // lanes with work
  static_assert(RB * CB == NE, "blocking");
  static_assert(D * D >= T ? ACTIVE == T : ACTIVE == D * D, "blocking covers the matrix");
};

// out = A1*B1 (+ A2*B2 when TWO) then epi(e, r, c, value) with e the storage
// index of (r, c); out may alias any input (outputs are staged in registers
// across a team barrier).  Each output's dot product runs over k in order.
template <int D, int T, bool TWO, int SW = 0, class C, class Epi>
__device__ __forceinline__ void mm(const Team<T>& tm, C* out, const C* A1, const C* B1,
                                   const C* A2, const C* B2, Epi epi) {
  using BK = Blocking<D, T>;
  using L = Lay<D, SW>;
  constexpr int RB = BK::RB, CB = BK::CB;
  const bool active = tm.lane < BK::ACTIVE;
  const int rb = tm.lane % BK::NR, cb = tm.lane / BK::NR;
  C acc[RB][CB];
#pragma unroll
  for (int i = 0; i < RB; ++i)
#pragma unroll
    for (int j = 0; j < CB; ++j) acc[i][j] = czero<C>();
  if (active) {
#pragma unroll 4
    for (int k = 0; k < D; ++k) {
      C a[RB], b[CB];
#pragma unroll
      for (int i = 0; i < RB; ++i) a[i] = A1[L::idx(rb + BK::NR * i, k)];
#pragma unroll
      for (int j = 0; j < CB; ++j) b[j] = B1[L::idx(k, cb + BK::NCB * j)];
#pragma unroll
      for (int i = 0; i < RB; ++i)
#pragma unroll
        for (int j = 0; j < CB; ++j) acc[i][j] = cmac(acc[i][j], a[i], b[j]);
    }
    if constexpr (TWO) {
#pragma unroll 4
      for (int k = 0; k < D; ++k) {
        C a[RB], b[CB];
#pragma unroll
        for (int i = 0; i < RB; ++i) a[i] = A2[L::idx(rb + BK::NR * i, k)];
#pragma unroll
        for (int j = 0; j < CB; ++j) b[j] = B2[L::idx(k, cb + BK::NCB * j)];
#pragma unroll
        for (int i = 0; i < RB; ++i)
#pragma unroll
          for (int j = 0; j < CB; ++j) acc[i][j] = cmac(acc[i][j], a[i], b[j]);
      }
    }
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const int r = rb + BK::NR * i, c = cb + BK::NCB * j;
        acc[i][j] = epi(L::idx(r, c), r, c, acc[i][j]);
      }
  }
  tm.sync();
  if (active) {
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < CB; ++j) out[L::idx(rb + BK::NR * i, cb + BK::NCB * j)] = acc[i][j];
  }
  tm.sync();
}

template <int D, int T, int SW = 0, class C>
__device__ __forceinline__ void mm1(const Team<T>& tm, C* out, const C* A, const C* B) {
  mm<D, T, false, SW>(tm, out, A, B, (const C*)nullptr, (const C*)nullptr, EpiNone{});
}

// One pass over k of the product pair below: Q always, P when WITH_P.
template <int D, int T, int SW, bool WITH_P, class C, class EpiP, class EpiQ>
__device__ __forceinline__ void mm_pair_pass(const Team<T>& tm, C* outP, C* outQ, const C* A, const C* dA,
                                             const C* Bm, const C* dBm, EpiP epiP, EpiQ epiQ) {
  using BK = Blocking<D, T>;
  using L = Lay<D, SW>;
  constexpr int RB = BK::RB, CB = BK::CB;
  const bool active = tm.lane < BK::ACTIVE;
  const int rb = tm.lane % BK::NR, cb = tm.lane / BK::NR;
  C p[RB][CB], q[RB][CB];
#pragma unroll
  for (int i = 0; i < RB; ++i)
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      p[i][j] = czero<C>();
      q[i][j] = czero<C>();
    }
  if (active) {
#pragma unroll 1
    for (int k = 0; k < D; ++k) {
      C a[RB], da[RB], b[CB], db[CB];
#pragma unroll
      for (int i = 0; i < RB; ++i) {
        const int e = L::idx(rb + BK::NR * i, k);
        a[i] = A[e];
        da[i] = dA[e];
      }
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const int e = L::idx(k, cb + BK::NCB * j);
        b[j] = Bm[e];
        db[j] = dBm[e];
      }
#pragma unroll
      for (int i = 0; i < RB; ++i)
#pragma unroll
        for (int j = 0; j < CB; ++j) {
          q[i][j] = cmac(q[i][j], da[i], b[j]);
          q[i][j] = cmac(q[i][j], a[i], db[j]);
          if constexpr (WITH_P) p[i][j] = cmac(p[i][j], a[i], b[j]);
        }
    }
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const int r = rb + BK::NR * i, c = cb + BK::NCB * j, e = L::idx(r, c);
        if constexpr (WITH_P) p[i][j] = epiP(e, r, c, p[i][j]);
        q[i][j] = epiQ(e, r, c, q[i][j]);
      }
  }
  tm.sync();
  if (active) {
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < CB; ++j) {
        const int e = L::idx(rb + BK::NR * i, cb + BK::NCB * j);
        if constexpr (WITH_P) outP[e] = p[i][j];
        outQ[e] = q[i][j];
      }
  }
  tm.sync();
}

// The product pair of a Frechet step: P = A Bm and Q = dA Bm + A dBm (the
// derivative of A Bm along dA, dBm), then epiP / epiQ as in mm; outputs may
// alias inputs.  Q adds dA Bm before A dBm at every k, on every path, so the
// result does not depend on the team size.  With at most 8 outputs per lane
// both products run in one pass over k that loads A[., k] and Bm[k, .] once
// for both; beyond that the registers allow only Q's pass and then P's (outQ
// never aliases A or Bm, which are all that P reads).
template <int D, int T, int SW, class C, class EpiP, class EpiQ>
__device__ __forceinline__ void mm_frechet(const Team<T>& tm, C* outP, C* outQ, const C* A, const C* dA,
                                           const C* Bm, const C* dBm, EpiP epiP, EpiQ epiQ) {
  if constexpr (Blocking<D, T>::NE <= 8) {
    mm_pair_pass<D, T, SW, true>(tm, outP, outQ, A, dA, Bm, dBm, epiP, epiQ);
  } else {
    mm_pair_pass<D, T, SW, false>(tm, outP, outQ, A, dA, Bm, dBm, epiP, epiQ);
    mm<D, T, false, SW>(tm, outP, A, Bm, (const C*)nullptr, (const C*)nullptr, epiP);
  }
}

template <int D, int T, class C>
__device__ __forceinline__ void copy_mat(const Team<T>& tm, C* dst, const C* src) {
  for (int e = tm.lane; e < D * D; e += T) dst[e] = src[e];
}

// Team-wide sum of per-lane complex partials (scratch: T complex entries).
template <int T, class C>
__device__ __forceinline__ C team_sum(const Team<T>& tm, C v, C* scratch) {
  if constexpr (T <= 32) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
  } else {
    scratch[tm.lane] = v;
    tm.sync();
    for (int w = T / 2; w > 0; w >>= 1) {
      if (tm.lane < w) scratch[tm.lane] = cadd(scratch[tm.lane], scratch[tm.lane + w]);
      tm.sync();
    }
    C r = scratch[0];
    tm.sync();
    return r;
  }
}

template <int T>
__device__ __forceinline__ double team_max(const Team<T>& tm, double v, double* scratch) {
  if constexpr (T <= 32) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
  } else {
    scratch[tm.lane] = v;
    tm.sync();
    for (int w = T / 2; w > 0; w >>= 1) {
      if (tm.lane < w) scratch[tm.lane] = fmax(scratch[tm.lane], scratch[tm.lane + w]);
      tm.sync();
    }
    double r = scratch[0];
    tm.sync();
    return r;
  }
}

// 1-norm (max column abs sum) of a D x D matrix; computed in FP64 whatever the
// storage type, because it selects the Taylor degree and the squarings.
template <int D, int T, int SW = 0, class C>
__device__ __forceinline__ double norm1(const Team<T>& tm, const C* A, double* scratch) {
  double best = 0.0;
  for (int c = tm.lane; c < D; c += T) {
    double s = 0.0;
    for (int r = 0; r < D; ++r) {
      C a = A[Lay<D, SW>::idx(r, c)];
      s += hypot((double)a.x, (double)a.y);
    }
    best = fmax(best, s);
  }
  return team_max<T>(tm, best, scratch);
}

// Degree m in {4,...,20} and squarings s minimising products for ||A||_1.
__device__ __forceinline__ void choose_degree(double nrm, const double* theta, int& m, int& s) {
  int best_cost = 1 << 30;
  m = 4;
  s = 0;
#pragma unroll
  for (int i = 0; i < PGX_N_DEGREES; ++i) {
    int si = 0;
    double x = nrm;
    while (x > theta[i] && si < 60) { x *= 0.5; ++si; }
    const int mi = 4 * (i + 1);
    const int cost = (3 + mi / 4 - 1) + si;
    if (cost < best_cost) { best_cost = cost; m = mi; s = si; }
  }
}

// Taylor block C_i = c_{4i} I + c_{4i+1} B + c_{4i+2} B2 + c_{4i+3} B3 at element e.
template <class C, class R>
__device__ __forceinline__ C block_val(int i, int r, int c, C b1, C b2, C b3, const R* invf) {
  C v = cscale(b1, invf[4 * i + 1]);
  v = cadd(v, cscale(b2, invf[4 * i + 2]));
  v = cadd(v, cscale(b3, invf[4 * i + 3]));
  if (r == c) v.x += invf[4 * i];
  return v;
}
template <class C, class R>
__device__ __forceinline__ C block_der(int i, C d1, C d2, C d3, const R* invf) {
  C v = cscale(d1, invf[4 * i + 1]);
  v = cadd(v, cscale(d2, invf[4 * i + 2]));
  return cadd(v, cscale(d3, invf[4 * i + 3]));
}

// Workspace layout (10 matrices) used by the Taylor routines.
template <class C, int D, int S = D * D> struct Work {
  C* B; C* B2; C* B3; C* B4; C* Y;
  C* dB; C* dB2; C* dB3; C* dB4; C* dY;
  __device__ __forceinline__ static Work at(C* base) {
    Work w;
    w.B = base; w.B2 = base + S; w.B3 = base + 2 * S; w.B4 = base + 3 * S; w.Y = base + 4 * S;
    w.dB = base + 5 * S; w.dB2 = base + 6 * S; w.dB3 = base + 7 * S; w.dB4 = base + 8 * S;
    w.dY = base + 9 * S;
    return w;
  }
};

// Y = T_m(B)^(2^s).  B holds A / 2^s on entry (destroyed: B..B4 are scratch).
// Paterson-Stockmeyer with q = 4: powers B2, B3, B4, then Horner in B4 over
// blocks of four coefficients.  m = 4L costs 3 + (L - 1) products.
template <int D, int T, int SW = 0, class C, int S, class R>
__device__ void taylor_exp(const Team<T>& tm, const Work<C, D, S>& w, int m, int s, const R* invf) {
  mm1<D, T, SW>(tm, w.B2, w.B, w.B);
  mm1<D, T, SW>(tm, w.B3, w.B2, w.B);
  mm1<D, T, SW>(tm, w.B4, w.B2, w.B2);
  const int L = m / 4;
  for (int q = tm.lane; q < D * D; q += T) {
    const int r = q % D, c = q / D, e = Lay<D, SW>::idx(r, c);
    C v = block_val(L - 1, r, c, w.B[e], w.B2[e], w.B3[e], invf);
    w.Y[e] = cadd(v, cscale(w.B4[e], invf[4 * L]));
  }
  tm.sync();
  for (int i = L - 2; i >= 0; --i) {
    const C* B = w.B; const C* B2 = w.B2; const C* B3 = w.B3;
    mm<D, T, false, SW>(tm, w.Y, w.B4, w.Y, (const C*)nullptr, (const C*)nullptr,
                        [=](int e, int r, int c, C v) {
                          return cadd(v, block_val(i, r, c, B[e], B2[e], B3[e], invf));
                        });
  }
  for (int k = 0; k < s; ++k) mm1<D, T, SW>(tm, w.Y, w.Y, w.Y);
}

// (Y, dY) = (f(A), L_f(A, M)) for f(A) = T_m(A/2^s)^(2^s).  On entry B = A/2^s
// and dB = M/2^s.  The derivative is exact for the polynomial f actually
// evaluated, so Tr(L_f(A, M) E) equals Tr(M L_f(A, E)) to rounding.
template <int D, int T, int SW = 0, class C, int S, class R>
__device__ void taylor_exp_frechet(const Team<T>& tm, const Work<C, D, S>& w, int m, int s, const R* invf) {
  mm1<D, T, SW>(tm, w.B2, w.B, w.B);
  mm<D, T, true, SW>(tm, w.dB2, w.dB, w.B, w.B, w.dB, EpiNone{});
  mm1<D, T, SW>(tm, w.B3, w.B2, w.B);
  mm<D, T, true, SW>(tm, w.dB3, w.dB2, w.B, w.B2, w.dB, EpiNone{});
  mm1<D, T, SW>(tm, w.B4, w.B2, w.B2);
  mm<D, T, true, SW>(tm, w.dB4, w.dB2, w.B2, w.B2, w.dB2, EpiNone{});
  const int L = m / 4;
  for (int q = tm.lane; q < D * D; q += T) {
    const int r = q % D, c = q / D, e = Lay<D, SW>::idx(r, c);
    C v = block_val(L - 1, r, c, w.B[e], w.B2[e], w.B3[e], invf);
    w.Y[e] = cadd(v, cscale(w.B4[e], invf[4 * L]));
    C dv = block_der(L - 1, w.dB[e], w.dB2[e], w.dB3[e], invf);
    w.dY[e] = cadd(dv, cscale(w.dB4[e], invf[4 * L]));
  }
  tm.sync();
  for (int i = L - 2; i >= 0; --i) {
    const C* B = w.B; const C* B2 = w.B2; const C* B3 = w.B3;
    const C* dB = w.dB; const C* dB2 = w.dB2; const C* dB3 = w.dB3;
    // dY <- dB4*Y + B4*dY + dC_i   (uses the old Y)
    mm<D, T, true, SW>(tm, w.dY, w.dB4, w.Y, w.B4, w.dY,
                       [=](int e, int, int, C v) {
                         return cadd(v, block_der(i, dB[e], dB2[e], dB3[e], invf));
                       });
    // Y <- B4*Y + C_i
    mm<D, T, false, SW>(tm, w.Y, w.B4, w.Y, (const C*)nullptr, (const C*)nullptr,
                        [=](int e, int r, int c, C v) {
                          return cadd(v, block_val(i, r, c, B[e], B2[e], B3[e], invf));
                        });
  }
  for (int k = 0; k < s; ++k) {
    mm<D, T, true, SW>(tm, w.dY, w.Y, w.dY, w.dY, w.Y, EpiNone{});
    mm1<D, T, SW>(tm, w.Y, w.Y, w.Y);
  }
}

// Six-matrix workspace of the q = 2 Frechet evaluation (fits shared memory at
// D = 64, where the ten matrices of the q = 4 form do not).
template <class C, int D, int S = D * D> struct Work2 {
  C* B; C* X; C* Y; C* dB; C* dX; C* dY;
  __device__ __forceinline__ static Work2 at(C* base) {
    Work2 w;
    w.B = base; w.X = base + S; w.Y = base + 2 * S;
    w.dB = base + 3 * S; w.dX = base + 4 * S; w.dY = base + 5 * S;
    return w;
  }
};

// As taylor_exp_frechet with Paterson-Stockmeyer q = 2: X = B^2, then Horner
// in X over pairs of coefficients,
//   Y_{L-1} = c_{2L} X + c_{2L-1} B + c_{2L-2} I,  Y_i = X Y_{i+1} + c_{2i+1} B + c_{2i} I,
//   dY_{L-1} = c_{2L} dX + c_{2L-1} dB,          dY_i = dX Y_{i+1} + X dY_{i+1} + c_{2i+1} dB,
// m = 2L; then the s squarings.  1.5 m product units against 3 (m/4 + 2) for
// q = 4, in six matrices instead of ten.
template <int D, int T, int SW = 0, class C, int S, class R>
__device__ void taylor_exp_frechet2(const Team<T>& tm, const Work2<C, D, S>& w, int m, int s, const R* invf) {
  mm_frechet<D, T, SW>(tm, w.X, w.dX, w.B, w.dB, w.B, w.dB, EpiNone{}, EpiNone{});
  const int L = m / 2;
  for (int q = tm.lane; q < D * D; q += T) {
    const int r = q % D, c = q / D, e = Lay<D, SW>::idx(r, c);
    C y = cadd(cscale(w.X[e], invf[2 * L]), cscale(w.B[e], invf[2 * L - 1]));
    if (r == c) y.x += invf[2 * L - 2];
    w.Y[e] = y;
    w.dY[e] = cadd(cscale(w.dX[e], invf[2 * L]), cscale(w.dB[e], invf[2 * L - 1]));
  }
  tm.sync();
  for (int i = L - 2; i >= 0; --i) {
    const C* B = w.B;
    const C* dB = w.dB;
    // Y <- X Y + C_i and dY <- dX Y + X dY + dC_i (both from the old Y, dY)
    mm_frechet<D, T, SW>(
        tm, w.Y, w.dY, w.X, w.dX, w.Y, w.dY,
        [=](int e, int r, int c, C v) {
          C t = cadd(v, cscale(B[e], invf[2 * i + 1]));
          if (r == c) t.x += invf[2 * i];
          return t;
        },
        [=](int e, int, int, C v) { return cadd(v, cscale(dB[e], invf[2 * i + 1])); });
  }
  for (int k = 0; k < s; ++k) mm_frechet<D, T, SW>(tm, w.Y, w.dY, w.Y, w.dY, w.Y, w.dY, EpiNone{}, EpiNone{});
}

}  // namespace pgx
