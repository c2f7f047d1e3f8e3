// Register-resident df expm for small padded dimensions, and its
// multi-problem form for batches.  Written for D = 2, 4, 8; the library runs
// it at D = 2, where it beats the shared-memory teams (the launcher in
// pgx_mixed.cu records the measurement).
//
// A group of G lanes of one warp owns one slice: lane (j, h) holds rows
// h R .. h R + R - 1 of column j of every matrix in registers (H row chunks
// per column: H = 2 at D = 8, else 1; R = D / H; G = D H = 2, 4, 16 lanes),
// as float4 df complex values {re.hi, im.hi, re.lo, im.lo}.  A product
// C = X Z needs column k of X from the lanes that own it and, at D = 8, the
// other half of the lane's own column of Z: both arrive by warp shuffles
// inside the group, and each output sums its k terms in order with the df
// accumulator of the shared-memory kernels.  A warp holds 32 / G slices.
//
// The scheme is the CUDA-core kernel's (df Paterson-Stockmeyer Taylor with
// the df theta table, then squarings), with full products only and every
// Horner step in df.  The degree, block size and squarings are chosen once
// per warp from the largest 1-norm of its slices, so every group of the warp
// runs the same product sequence (no divergence between shuffling groups);
// a larger norm only ever selects a more accurate scheme.
//
// Items are (problem, member, slice) triples: one problem for a solo
// evaluation, every problem of a batch's D class for the batch's persistent
// launch.  The per-slice arithmetic does not depend on which, so batched and
// solo results are bit-identical.
#pragma once

namespace pgx {
namespace sm {

template <int D> struct Grp {
  static constexpr int H = (D == 8) ? 2 : 1;  // row chunks per column
  static constexpr int G = D * H;             // lanes per slice
  static constexpr int R = D / H;             // rows per lane
  static constexpr int SPW = 32 / G;          // slices per warp
};

template <int D> struct Part {
  float4 v[Grp<D>::R];
};

// Problems of one launch: one (p0, w0: n == 0), or n problems in device
// tables, problem i's items at [first[i], first[i] + members x slices), each
// range starting at a multiple of Grp<D>::SPW (items = first[n]).
struct Set {
  ProbDev p0;
  WorkDev w0;
  const ProbDev* ps;
  const WorkDev* ws;
  const long* first;  // [n + 1]
  int n;
  long items;
};

// C = X Z for this lane's part.  gbase: the group's first lane in the warp.
template <int D>
__device__ __forceinline__ void mm(Part<D>& C, const Part<D>& X, const Part<D>& Z, int gbase, int j, int h) {
  using Gp = Grp<D>;
  constexpr int R = Gp::R, H = Gp::H;
  float4 zc[D];  // column j of Z
#pragma unroll
  for (int hh = 0; hh < H; ++hh)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      float4 v = Z.v[r];
      if (H > 1) {
        const int src = gbase + j * H + hh;
        v.x = __shfl_sync(0xffffffffu, Z.v[r].x, src);
        v.y = __shfl_sync(0xffffffffu, Z.v[r].y, src);
        v.z = __shfl_sync(0xffffffffu, Z.v[r].z, src);
        v.w = __shfl_sync(0xffffffffu, Z.v[r].w, src);
      }
      zc[hh * R + r] = v;
    }
  DfAcc acc[R];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int src = gbase + k * H + h;  // owner of rows hR.. of column k
#pragma unroll
    for (int r = 0; r < R; ++r) {
      float4 x;
      x.x = __shfl_sync(0xffffffffu, X.v[r].x, src);
      x.y = __shfl_sync(0xffffffffu, X.v[r].y, src);
      x.z = __shfl_sync(0xffffffffu, X.v[r].z, src);
      x.w = __shfl_sync(0xffffffffu, X.v[r].w, src);
      acc[r].mac(x, zc[k]);
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r) C.v[r] = dfc_store(acc[r].result());
}

// The df degree choice of the CUDA-core kernel (choose_expm_df, full products)
// in one lane: m | q << 5 | s << 8.
__device__ __forceinline__ int choose_lane(float nrm, int D) {
  long long best = 0x7fffffffffffffffLL;
  int packed = 0;
#pragma unroll 1
  for (int t = 0; t < 21; ++t) {
    const int qq = (t < 5) ? 4 : (t < 11) ? 3 : 2;
    const int L = (t < 5) ? t + 1 : (t < 11) ? t - 4 : t - 10;
    const int mm = qq * L;
    int si = 0;
    float x = nrm;
    while (x > c_thetadf_all[mm - 1] && si < 60) {
      x *= 0.5f;
      ++si;
    }
    const int lo = lo_horner_from(x, L, D, qq);
    const int n_df = lo < L - 1 ? lo : L - 1;
    const int cost = (qq - 1) * kPowCost + 20 * n_df + kLoHornerCost * (L - 1 - n_df) + 20 * si;
    const long long key = (long long)cost * 32 + t;
    if (key < best) {
      best = key;
      packed = mm | (qq << 5) | (si << 8);
    }
  }
  return packed;
}

__device__ __forceinline__ float4 scale4(const float4& a, float s) {
  return make_float4(a.x * s, a.y * s, a.z * s, a.w * s);
}

// This lane's part of the Horner block C_i = sum_{j<q} c_{qi+j} B^j.
template <int D>
__device__ __forceinline__ float4 block_entry(int i, int q, bool diag, const float4& b1, const float4& b2,
                                              const float4& b3) {
  const int o = q * i;
  dfc v = dfc_scale(dfc_load(b1), c_dfcoef[o + 1]);
  if (q >= 3) v = dfc_add(v, dfc_scale(dfc_load(b2), c_dfcoef[o + 2]));
  if (q >= 4) v = dfc_add(v, dfc_scale(dfc_load(b3), c_dfcoef[o + 3]));
  if (diag) v.re = df_add(v.re, c_dfcoef[o]);
  return dfc_store(v);
}

constexpr int kSmallThreads = 256;

// One slice (item `loc` of problem p) for the group this lane belongs to;
// `live` false: a group past the last item, which still takes part in the
// warp's shuffles on zeros.
template <int D>
__device__ __forceinline__ void expm_item(const ProbDev& p, const WorkDev& w, long loc, bool live, int gbase, int j,
                                          int h) {
  using Gp = Grp<D>;
  constexpr int R = Gp::R, H = Gp::H;
  Part<D> B, B2, B3, B4, Q, Y, T;
  float colsum = 0.f;
  int m = 0, k = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    B.v[r] = make_float4(0.f, 0.f, 0.f, 0.f);
    B3.v[r] = B.v[r];
    B4.v[r] = B.v[r];
  }
  if (live) {
    m = (int)(loc / p.n_t);
    k = (int)(loc % p.n_t);
    const double* uk = w.u + (size_t)k * p.n_c;
    const auto u = [=](int c) { return df_from(uk[c]); };
#pragma unroll
    for (int r = 0; r < R; ++r) {
      B.v[r] = dfc_store(gen_entry_df<D>(p, m, k, h * R + r + D * j, u));
      colsum += sqrtf(fmaf(B.v[r].x, B.v[r].x, B.v[r].y * B.v[r].y));
    }
  }
  // 1-norm: column sums, then the largest over the warp's slices (x 1.00001
  // for the FP32 rounding, as the shared-memory kernels)
  if (H > 1) colsum += __shfl_xor_sync(0xffffffffu, colsum, 1);
  float nrm = colsum;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nrm = fmaxf(nrm, __shfl_xor_sync(0xffffffffu, nrm, o));
  const int pk = choose_lane(nrm * 1.00001f, D);
  const int deg = pk & 31, q = (pk >> 5) & 7, s = (pk >> 8) & 63, nL = deg / q;
  {
    const float sc = ldexpf(1.f, -s);  // B <- B / 2^s, exact in df
#pragma unroll
    for (int r = 0; r < R; ++r) B.v[r] = scale4(B.v[r], sc);
  }
  // powers B^2 = B B, B^3 = B^2 B, B^4 = B^2 B^2; Q = B^q
  mm<D>(B2, B, B, gbase, j, h);
  if (q >= 3) mm<D>(B3, B2, B, gbase, j, h);
  if (q >= 4) mm<D>(B4, B2, B2, gbase, j, h);
#pragma unroll
  for (int r = 0; r < R; ++r) Q.v[r] = (q == 2) ? B2.v[r] : (q == 3) ? B3.v[r] : B4.v[r];
  // Y = C_{L-1} + c_m B^q
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float4 c = block_entry<D>(nL - 1, q, h * R + r == j, B.v[r], B2.v[r], B3.v[r]);
    Y.v[r] = dfc_store(dfc_add(dfc_load(c), dfc_scale(dfc_load(Q.v[r]), c_dfcoef[deg])));
  }
  // Horner: Y <- B^q Y + C_i
#pragma unroll 1
  for (int i = nL - 2; i >= 0; --i) {
    mm<D>(T, Q, Y, gbase, j, h);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float4 c = block_entry<D>(i, q, h * R + r == j, B.v[r], B2.v[r], B3.v[r]);
      Y.v[r] = dfc_store(dfc_add(dfc_load(T.v[r]), dfc_load(c)));
    }
  }
  // squarings
#pragma unroll 1
  for (int r2 = 0; r2 < s; ++r2) {
    mm<D>(T, Y, Y, gbase, j, h);
    Y = T;
  }
  if (live) {
    float4* out = reinterpret_cast<float4*>(w.U) + ((size_t)m * p.n_t + k) * D * D;
#pragma unroll
    for (int r = 0; r < R; ++r) out[h * R + r + D * j] = Y.v[r];
  }
}

// MULTI = false: the items of set.p0 / set.w0; true: of the problem table.
template <int D, bool MULTI>
__global__ void __launch_bounds__(kSmallThreads) k_expm_small(Set set) {
  using Gp = Grp<D>;
  constexpr int H = Gp::H, G = Gp::G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane / G, gl = lane % G, gbase = grp * G;
  const int j = gl / H, h = gl % H;
  const long nw = (long)gridDim.x * (kSmallThreads / 32);
  // warp-uniform loop over groups of SPW items
  for (long base = ((long)blockIdx.x * (kSmallThreads / 32) + warp) * Gp::SPW; base < set.items;
       base += nw * Gp::SPW) {
    const long it = base + grp;
    if constexpr (MULTI) {
      // The item's problem: the last with first[pi] <= it.  Every problem's
      // range starts at a multiple of SPW, so a warp never mixes problems and
      // holds the same slices as in the problem's solo launch.
      int pi = 0;
      if (it < set.items) {
        int lo = 0, hi = set.n - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (set.first[mid] <= it) lo = mid;
          else hi = mid - 1;
        }
        pi = lo;
      }
      const ProbDev& p = set.ps[pi];
      const long loc = it - set.first[pi];
      const bool live = it < set.items && loc < (long)p.n_members * p.n_t;
      expm_item<D>(p, set.ws[pi], live ? loc : 0, live, gbase, j, h);
    } else {
      const bool live = it < set.items;
      expm_item<D>(set.p0, set.w0, it, live, gbase, j, h);
    }
  }
}

}  // namespace sm
}  // namespace pgx
