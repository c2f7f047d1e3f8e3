// The mixed-precision exact gradient at D = 64 on the tensor cores (tcgen05).
//
// Same mathematics as k_grad_gate_mx: per member-slice unit (m, k),
//   B = A_k / 2^s, dB = M_k / 2^s,
//   X = B^2, dX = dB B + B dB,
//   Y = c_2L X + c_2L-1 B + c_2L-2 I,  dY = c_2L dX + c_2L-1 dB,
//   Horner i = L-2 .. 0:  Y <- X Y + c_2i+1 B + c_2i I,
//                        dY <- dX Y + X dY + c_2i+1 dB,
//   s squarings:         dY <- Y dY + dY Y,  Y <- Y Y,
// then g_j = Re(c dt scale Tr(dY C_j)) (the q = 2 Paterson-Stockmeyer form of
// the Frechet derivative L(A_k, M_k) of the Taylor polynomial, degree and
// squarings from the FP32 theta table).  Here every product is a tcgen05 MMA
// in 3xFP16 (pgx_tc.cuh: fp16 hi/lo parts, FP32 accumulation, FP32-class
// accuracy) instead of FP32 CUDA-core FMAs.  FP16's range: the B family (B,
// X, Y: Taylor terms of a bounded exponential) is staged as is; the
// derivative family (dB, dX, dY) is scaled by a power of two per unit so that
// max|dB| lies in [1/2, 1) -- the Frechet derivative is linear in dB, so the
// traces divide the scale back out exactly.  A staged value beyond the FP16
// limit sets an error flag instead of overflowing silently.
//
// Layout: one persistent CTA per SM (256 threads, the whole 512-column TMEM).
//   TMEM: four 64-column slots in the stacked [re; im] layout that rotate
//   among Y, dY and the accumulators of the next Y and dY (columns 0..255),
//   and the expanded left factor [Pr -Pi; Pi Pr], hi and lo fp16 parts two
//   per column (256..383): the MMAs read A from TMEM and only B from shared
//   memory.
//   Shared memory (160 KB): the right factor staged hi/lo in the 128-byte
//   swizzled K-major layout; compact FP32 copies of B and dB (the additive
//   terms, and the left factors of the first products); a compact pair of
//   left factors (X and dX during Horner, Y and dY during the squarings),
//   from which any thread can read the partner rows of the expanded operand.
// A product restages a factor only when its staging area holds another one;
// the three products of a Horner step alternate their order, so that each
// step restages one left and two right factors.  Accumulators of a Horner
// step are initialised with the step's additive terms, so the MMAs accumulate
// onto them.  The traces sum each thread's 32 columns in order, then a fixed
// shuffle tree and the eight warps in order: results do not depend on timing.
//
// Included by pgx_mixed.cu after its FP32 Taylor tables and choose_degree_q2.
#pragma once
#include "pgx_tc.cuh"

namespace pgx {

// Set by k_grad_tc64: bit 0 when an MMA-completion wait gave up, bit 1 when a
// staged value was beyond the FP16 limit; read and cleared by the host after
// the evaluation (grad_tc_check).
__device__ int g_grad_tc_timeout = 0;

namespace gtc {

constexpr int kD = 64;
constexpr uint32_t kMatBytes = 64u * 64u * 8u;  // one compact complex FP32 matrix
// right-factor sources other than the TMEM slots 0..3, and left-factor sources
enum { R_B = 10, R_DB = 11, L_B = 20, L_DB = 21, L_C0 = 22, L_C1 = 23 };
constexpr uint32_t kAHi = 256, kALo = 256 + tc::kAColsF16;  // TMEM columns of the expanded left factor

struct State {
  uint8_t *b_hi, *b_lo;
  float2 *tB, *tdB, *c0, *c1;  // compact matrices in shared memory
  uint32_t tmem, mbar, phase;
  int staged_a, staged_b;      // source held by each staging area, -1 = none
};

__device__ __forceinline__ uint32_t slot_addr(const State& s, const tc::Lane& l, int slot) {
  return s.tmem + l.lane_addr + (uint32_t)(64 * slot + l.c0);
}
__device__ __forceinline__ const float2* left_src(const State& s, int id) {
  return id == L_B ? s.tB : id == L_DB ? s.tdB : id == L_C0 ? s.c0 : s.c1;
}
// this thread's 32 values (row l.i, part l.im, columns c0..c0+31) of a compact matrix
__device__ __forceinline__ void load_row(const float2* M, const tc::Lane& l, float (&v)[32]) {
  const float* f = reinterpret_cast<const float*>(M);
#pragma unroll
  for (int c = 0; c < 32; ++c) v[c] = f[2 * (l.i + 64 * (l.c0 + c)) + l.im];
}
__device__ __forceinline__ void store_row(float2* M, const tc::Lane& l, const float (&v)[32]) {
  float* f = reinterpret_cast<float*>(M);
#pragma unroll
  for (int c = 0; c < 32; ++c) f[2 * (l.i + 64 * (l.c0 + c)) + l.im] = v[c];
}

// A TMEM slot was rewritten: a right-factor staging that holds it is stale.
__device__ __forceinline__ void touch(State& s, int slot) {
  if (s.staged_b == slot) s.staged_b = -1;
}

// D(dst slot) = (acc ? D : 0) + left right, all threads; false when the wait
// gave up (*abort = 1) or a staged value was out of FP16 range (*range = 1).
__device__ __forceinline__ bool product(State& s, const tc::Lane& l, int left, int right, int dst, int acc,
                                        int* abort, int* range) {
  bool in_range = true;
  if (s.staged_a != left) {
    in_range &= tc::stage_A_tmem_f16(s.tmem + l.lane_addr + kAHi, s.tmem + l.lane_addr + kALo, left_src(s, left),
                                     l.L, l.c0 / 32);
    s.staged_a = left;
  }
  if (s.staged_b != right) {
    float v[32];
    if (right < 4) tc::tmem_ld32(slot_addr(s, l, right), v);
    else load_row(right == R_B ? s.tB : s.tdB, l, v);
    in_range &= tc::stage_B_f16(s.b_hi, s.b_lo, l, v);
    s.staged_b = right;
  }
  if (!in_range) *range = 1;
  tc::tmem_st_wait();
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::fence_after_sync();
    tc::issue_product_f16(s.tmem + (uint32_t)(64 * dst), s.tmem + kAHi, s.tmem + kALo, tc::smem_u32(s.b_hi),
                          tc::smem_u32(s.b_lo), (uint32_t)acc, s.mbar);
  }
  if (!tc::mbar_wait(s.mbar, s.phase)) *abort = 1;
  s.phase ^= 1;
  tc::fence_after_sync();
  __syncthreads();
  touch(s, dst);
  return *abort == 0 && *range == 0;
}

// slot dst = a x + b Y (+ c I), x given in registers, Y a compact matrix
__device__ __forceinline__ void combine(State& s, const tc::Lane& l, int dst, float a, const float (&x)[32],
                                        float b, const float2* Y, float c) {
  float y[32];
  load_row(Y, l, y);
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    y[k] = fmaf(a, x[k], b * y[k]);
    if (l.im == 0 && l.c0 + k == l.i) y[k] += c;
  }
  tc::tmem_st32(slot_addr(s, l, dst), y);
  touch(s, dst);
}

// slot dst = b Y (+ c I), Y a compact matrix
__device__ __forceinline__ void scaled(State& s, const tc::Lane& l, int dst, float b, const float2* Y, float c) {
  float y[32];
  load_row(Y, l, y);
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    y[k] *= b;
    if (l.im == 0 && l.c0 + k == l.i) y[k] += c;
  }
  tc::tmem_st32(slot_addr(s, l, dst), y);
  touch(s, dst);
}

// compact copies of two TMEM slots into the left-factor pair
__device__ __forceinline__ void slots_to_left(State& s, const tc::Lane& l, int s0, int s1) {
  float v[32];
  tc::tmem_ld32(slot_addr(s, l, s0), v);
  store_row(s.c0, l, v);
  tc::tmem_ld32(slot_addr(s, l, s1), v);
  store_row(s.c1, l, v);
  if (s.staged_a == L_C0 || s.staged_a == L_C1) s.staged_a = -1;
}

}  // namespace gtc

// Gate targets, exact gradient, Dp = 64.
__global__ void __launch_bounds__(tc::kThreads, 1) k_grad_tc64(ProbDev p, WorkDev w) {
  using namespace gtc;
  constexpr int D = kD;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int s_abort, s_range;
  __shared__ float s_nrm[2], s_mmax[8];
  __shared__ float s_part[4][64];
  __shared__ float2 s_red[8][8];
  const uint32_t pad = (tc::kSmemAlign - (tc::smem_u32(smem_raw) & (tc::kSmemAlign - 1))) & (tc::kSmemAlign - 1);
  State s;
  s.b_hi = smem_raw + pad;
  s.b_lo = s.b_hi + tc::kBBytesF16;
  s.tB = reinterpret_cast<float2*>(s.b_lo + tc::kBBytesF16);
  s.tdB = reinterpret_cast<float2*>(reinterpret_cast<uint8_t*>(s.tB) + kMatBytes);
  s.c0 = reinterpret_cast<float2*>(reinterpret_cast<uint8_t*>(s.tdB) + kMatBytes);
  s.c1 = reinterpret_cast<float2*>(reinterpret_cast<uint8_t*>(s.c0) + kMatBytes);
  s.mbar = tc::smem_u32(&s_bar);
  s.phase = 0;
  const tc::Lane l = tc::lane_of();
  if (threadIdx.x < 32) tc::tmem_alloc(&s_tmem, tc::kTmemCols);
  if (threadIdx.x == 0) {
    tc::mbar_init(s.mbar);
    s_abort = 0;
    s_range = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  s.tmem = s_tmem;
  float* nrm_scratch = reinterpret_cast<float*>(s.c0);  // [64 columns][65]: |A| for the column sums

  const long items = (long)p.n_members * p.n_t;
  for (long it = blockIdx.x; it < items; it += gridDim.x) {
    const int m = (int)(it / p.n_t), k = (int)(it % p.n_t);
    s.staged_a = s.staged_b = -1;
    // ---- A_k (FP32 assembly from the FP32 constant copies), this thread's row
    // l.i, 32 columns.  Each matrix is read as 32 independent warp-coalesced
    // loads (the columns unrolled), so their L2 latencies overlap.
    float ar[32], ai[32];
    {
      const float dt = p.dt_df[k].x, sc = p.m_scale_df[m].x, off = p.m_offset_df[m].x;
      const float2* Gd = p.drifts_f32 + (size_t)p.m_drift[m] * D * D + l.i + D * l.c0;
      const float2* Of = p.offset_f32 + l.i + D * l.c0;
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float2 g = Gd[D * c];
        const float2 o = Of[D * c];
        ar[c] = fmaf(off, o.x, g.x);
        ai[c] = fmaf(off, o.y, g.y);
      }
      const int ro = p.n_ramp ? p.m_ramp[m] : -1;
      if (ro >= 0) {
        const float4* Rm = p.ramp_ops_df + (size_t)ro * D * D + l.i + D * l.c0;
        const float tk = p.tau_df[k].x;
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          const float4 r = Rm[D * c];
          ar[c] = fmaf(tk, r.x, ar[c]);
          ai[c] = fmaf(tk, r.y, ai[c]);
        }
      }
      const float2* uk = w.u_df + (size_t)k * p.n_c;
      for (int j = 0; j < p.n_c; ++j) {
        const float a = sc * uk[j].x;
        const float2* Cj = p.ctrls_f32 + (size_t)j * D * D + l.i + D * l.c0;
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          const float2 cj = Cj[D * c];
          ar[c] = fmaf(a, cj.x, ar[c]);
          ai[c] = fmaf(a, cj.y, ai[c]);
        }
      }
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float vx = ar[c] * dt, vy = ai[c] * dt;
        if (p.gen == GEN_HERM) {  // times -i
          ar[c] = vy;
          ai[c] = -vx;
        } else {
          ar[c] = vx;
          ai[c] = vy;
        }
      }
    }
    // ---- 1-norm (FP32, enlarged by 1e-5 as norm1f): each column summed as
    // four 16-row partial sums (all 256 threads), then the four in order
    const float2* Mk = reinterpret_cast<const float2*>(w.P) + ((size_t)m * p.n_t + k) * D * D;
    if (l.im == 0) {
#pragma unroll
      for (int c = 0; c < 32; ++c) nrm_scratch[(l.c0 + c) * 65 + l.i] = sqrtf(fmaf(ar[c], ar[c], ai[c] * ai[c]));
    } else {  // the largest component of M_k, for the scale of the derivative family
      float mx = 0.f;
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float2 e = Mk[l.i + D * (l.c0 + c)];
        mx = fmaxf(mx, fmaxf(fabsf(e.x), fabsf(e.y)));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if ((threadIdx.x & 31) == 0) s_mmax[threadIdx.x >> 5] = mx;
    }
    if (l.im == 0 && (threadIdx.x & 31) == 0) s_mmax[threadIdx.x >> 5] = 0.f;
    __syncthreads();
    {
      const int col = threadIdx.x & 63, r0 = 16 * (threadIdx.x >> 6);
      float ps = 0.f;
#pragma unroll
      for (int r = 0; r < 16; ++r) ps += nrm_scratch[col * 65 + r0 + r];
      s_part[threadIdx.x >> 6][col] = ps;
    }
    __syncthreads();
    if (threadIdx.x < 64) {
      float cs = ((s_part[0][threadIdx.x] + s_part[1][threadIdx.x]) + s_part[2][threadIdx.x]) + s_part[3][threadIdx.x];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) cs = fmaxf(cs, __shfl_xor_sync(0xffffffffu, cs, o));
      if ((threadIdx.x & 31) == 0) s_nrm[threadIdx.x >> 5] = cs;
    }
    __syncthreads();
    const float nrm = fmaxf(s_nrm[0], s_nrm[1]) * 1.00001f;
    int deg, sq;
    choose_degree_q2(nrm, c_theta32f, deg, sq);
    const float scl = ldexpf(1.f, -sq);
    // derivative scale 2^-ed: max|dB| = max|M_k| 2^-s lands in [1/2, 1)
    int ed = 0;
    {
      float mmax = 0.f;
#pragma unroll
      for (int q = 0; q < 8; ++q) mmax = fmaxf(mmax, s_mmax[q]);
      if (mmax > 0.f) frexpf(mmax * scl, &ed);
    }
    const float dscl = ldexpf(scl, -ed);
    // ---- compact B (real-part threads) and dB = M_k / 2^s (imaginary-part threads)
    if (l.im == 0) {
#pragma unroll
      for (int c = 0; c < 32; ++c) s.tB[l.i + D * (l.c0 + c)] = make_float2(ar[c] * scl, ai[c] * scl);
    } else {
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float2 e = Mk[l.i + D * (l.c0 + c)];
        s.tdB[l.i + D * (l.c0 + c)] = make_float2(e.x * dscl, e.y * dscl);
      }
    }
    __syncthreads();
    int sy = 0, sdy = 1, ay = 2, ad = 3;
    // ---- X = B B (slot ay), dX = dB B + B dB (slot ad)
    if (!product(s, l, L_DB, R_B, ad, 0, &s_abort, &s_range)) break;
    if (!product(s, l, L_B, R_B, ay, 0, &s_abort, &s_range)) break;
    if (!product(s, l, L_B, R_DB, ad, 1, &s_abort, &s_range)) break;
    // ---- X, dX into the left-factor pair; Y, dY of the first Horner stage
    const int L = deg / 2;
    {
      float x[32];
      tc::tmem_ld32(slot_addr(s, l, ay), x);
      store_row(s.c0, l, x);
      combine(s, l, sy, c_invf32[2 * L], x, c_invf32[2 * L - 1], s.tB, c_invf32[2 * L - 2]);
      tc::tmem_ld32(slot_addr(s, l, ad), x);
      store_row(s.c1, l, x);
      combine(s, l, sdy, c_invf32[2 * L], x, c_invf32[2 * L - 1], s.tdB, 0.f);
    }
    __syncthreads();  // the left-factor pair is read across rows by the staging of the products
    bool ok = true;
    // ---- Horner in X
    for (int i = L - 2; i >= 0 && ok; --i) {
      scaled(s, l, ay, c_invf32[2 * i + 1], s.tB, c_invf32[2 * i]);
      scaled(s, l, ad, c_invf32[2 * i + 1], s.tdB, 0.f);
      if (((L - 2 - i) & 1) == 0) {
        ok = product(s, l, L_C0, sdy, ad, 1, &s_abort, &s_range) && product(s, l, L_C0, sy, ay, 1, &s_abort, &s_range) &&
             product(s, l, L_C1, sy, ad, 1, &s_abort, &s_range);
      } else {
        ok = product(s, l, L_C1, sy, ad, 1, &s_abort, &s_range) && product(s, l, L_C0, sy, ay, 1, &s_abort, &s_range) &&
             product(s, l, L_C0, sdy, ad, 1, &s_abort, &s_range);
      }
      int t = sy; sy = ay; ay = t;
      t = sdy; sdy = ad; ad = t;
    }
    if (!ok) break;
    // ---- squarings: Y, dY become the left-factor pair
    for (int r = 0; r < sq && ok; ++r) {
      slots_to_left(s, l, sy, sdy);
      __syncthreads();
      ok = product(s, l, L_C0, sdy, ad, 0, &s_abort, &s_range) && product(s, l, L_C0, sy, ay, 0, &s_abort, &s_range) &&
           product(s, l, L_C1, sy, ad, 1, &s_abort, &s_range);
      int t = sy; sy = ay; ay = t;
      t = sdy; sdy = ad; ad = t;
    }
    if (!ok) break;
    // ---- g_j = Re(c dt scale Tr(dY C_j))
    float v[32];
    tc::tmem_ld32(slot_addr(s, l, sdy), v);
    double* Gout = w.Gm + ((size_t)m * p.n_t + k) * p.n_c;
    const double gsc = ldexp(p.dt[k] * p.m_scale[m], ed);  // undoes the derivative scale
    // controls in groups of up to 8: each thread's partial sums (its 32
    // columns in order, 16 independent loads per control), a fixed shuffle
    // tree per warp, then the eight warps in order
    for (int j0 = 0; j0 < p.n_c; j0 += 8) {
      const int nj = p.n_c - j0 < 8 ? p.n_c - j0 : 8;
      for (int jj = 0; jj < nj; ++jj) {
        const float4* Cj =
            reinterpret_cast<const float4*>(p.ctrls_f32 + (size_t)(j0 + jj) * D * D + l.c0 + D * l.i);
        float4 cc[16];
#pragma unroll
        for (int h = 0; h < 16; ++h) cc[h] = Cj[h];  // C_j[c][i], C_j[c + 1][i] for c = c0 + 2h
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int h = 0; h < 16; ++h) {
          const float y0 = v[2 * h], y1 = v[2 * h + 1];
          if (l.im == 0) {
            re = fmaf(y0, cc[h].x, re); im = fmaf(y0, cc[h].y, im);
            re = fmaf(y1, cc[h].z, re); im = fmaf(y1, cc[h].w, im);
          } else {
            re = fmaf(-y0, cc[h].y, re); im = fmaf(y0, cc[h].x, im);
            re = fmaf(-y1, cc[h].w, re); im = fmaf(y1, cc[h].z, im);
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          re += __shfl_xor_sync(0xffffffffu, re, o);
          im += __shfl_xor_sync(0xffffffffu, im, o);
        }
        if ((threadIdx.x & 31) == 0) s_red[jj][threadIdx.x >> 5] = make_float2(re, im);
      }
      __syncthreads();
      if (threadIdx.x < nj) {
        const int jj = threadIdx.x;
        float2 acc = s_red[jj][0];
        for (int q = 1; q < 8; ++q) acc = make_float2(acc.x + s_red[jj][q].x, acc.y + s_red[jj][q].y);
        Gout[j0 + jj] = gsc * (double)(p.gen == GEN_HERM ? acc.y : acc.x);
      }
      __syncthreads();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (s_abort || s_range) {
    // units this CTA did not finish get NaN gradients, so no stale value
    // passes for a result even on paths that never read the flag
    for (long it = blockIdx.x + threadIdx.x * (long)gridDim.x; it < items; it += (long)gridDim.x * blockDim.x) {
      double* Gout = w.Gm + (size_t)it * p.n_c;
      for (int j = 0; j < p.n_c; ++j) Gout[j] = __longlong_as_double(0x7ff8000000000000LL);
    }
  }
  if (s_range && threadIdx.x == 0) atomicOr(&g_grad_tc_timeout, 2);
  if (s_abort && threadIdx.x == 0) {
    atomicOr(&g_grad_tc_timeout, 1);
    tc::mbar_wait(s.mbar, s.phase ^ 1);  // bounded: let a late group finish before TMEM is freed
  }
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(s.tmem, tc::kTmemCols);
  }
}

}  // namespace pgx
