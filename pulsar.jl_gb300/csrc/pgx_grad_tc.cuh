// The mixed-precision exact gradient at D = 64 on the tensor cores (tcgen05).
//
// Same mathematics as k_grad_gate_mx: per member-slice unit (m, k),
//   B = A_k / 2^s, dB = M_k / 2^s,
//   X = B^2, dX = dB B + B dB,
//   Y = c_2L X + c_2L-1 B + c_2L-2 I,  dY = c_2L dX + c_2L-1 dB,
//   Horner i = L-2 .. 0:  Y <- X Y + c_2i+1 B + c_2i I,
//                        dY <- dX Y + X dY + c_2i+1 dB,
//   s squarings:         dY <- Y dY + dY Y,  Y <- Y Y,
// the q = 2 Paterson-Stockmeyer form of the Frechet derivative L(A_k, M_k) of
// the Taylor polynomial, degree and squarings from the FP32 theta table.  Here
// every product is a tcgen05 MMA in 3xFP16 (pgx_tc.cuh: fp16 hi/lo parts,
// FP32 accumulation, FP32-class accuracy) instead of FP32 CUDA-core FMAs.
// FP16's range: the B family (B, X, Y: Taylor terms of a bounded exponential)
// is staged as is; the derivative family (dB, dX, dY) is scaled by a power of
// two per unit so that max|dB| lies in [1/2, 1) -- the Frechet derivative is
// linear in dB, so the result divides the scale back out exactly.  A staged
// value beyond the FP16 limit sets an error flag instead of overflowing.
//
// Each stage -- the first products, a Horner step, a squaring -- is three
// products that share their operands two by two, issued as one group:
//   first:    dB B -> dX,  B B -> X,  B dB -> dX (accumulating)
//   Horner:   X dY -> dY', X Y -> Y', dX Y -> dY'  (accumulators pre-set to
//             the step's additive terms)
//   squaring: Y dY -> dY', Y Y -> Y', dY Y -> dY'.
// Layout: one persistent CTA per SM (256 threads, the whole 512-column TMEM).
//   TMEM: four 64-column slots in the stacked [re; im] layout that rotate
//   among Y, dY and the accumulators of the next Y and dY (columns 0..255),
//   and two expanded left factors [Pr -Pi; Pi Pr], hi and lo fp16 parts two
//   per column (256..383 and 384..511): X and dX stay there through all of
//   Horner; B and dB before it, Y and dY in each squaring.
//   Shared memory (about 200 KB): two right factors staged hi/lo in the
//   128-byte swizzled MN-major layout; compact FP32 copies (planar, padded
//   rows) of B and dB (the additive terms and the first operands) and one
//   compact transit matrix through which a TMEM slot becomes an expanded left
//   factor (its partner rows belong to other warps); and the next unit's M_k,
//   fetched by a TMA bulk copy while the current unit's products run.
// The unit's result L(A_k, M_k) (scale undone) overwrites M_k in the P
// buffer, which nothing reads after the gradient, as two row-major planes, so
// that L[r][c] and C_j[c][r] share one index; k_trace_tc64 then forms
// g_j = Re(c dt scale Tr(L C_j)) for all units in a memory-bound pass with
// the controls in shared memory.  Both kernels sum in fixed orders: results
// do not depend on timing.
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
constexpr uint32_t kMatBytes = 2u * tc::kPlaneFloats * 4u;  // one compact complex matrix (two padded planes)
constexpr uint32_t kMkBytes = 64u * 64u * 8u;               // M_k as stored: column-major float2
constexpr uint32_t kA0 = 256, kA1 = 384;                    // TMEM columns of the two expanded left factors

struct State {
  uint8_t* b[2];               // right-factor buffers: hi part, lo part at + kBBytesF16
  float *tB, *tdB, *tr;        // compact matrices in shared memory (planar)
  uint32_t tmem, mbar, phase;
};

__device__ __forceinline__ uint32_t slot_addr(const State& s, const tc::Lane& l, int slot) {
  return s.tmem + l.lane_addr + (uint32_t)(64 * slot + l.c0);
}
// this thread's 32 values (row l.i, part l.im, columns c0..c0+31) of a compact matrix
__device__ __forceinline__ const float4* row_ptr(const float* M, const tc::Lane& l) {
  return reinterpret_cast<const float4*>(M + (l.im ? tc::kPlaneFloats : 0u) + (uint32_t)l.i * tc::kLdp + l.c0);
}
__device__ __forceinline__ void load_row(const float* M, const tc::Lane& l, float (&v)[32]) {
  const float4* r = row_ptr(M, l);
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float4 x = r[q];
    v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
  }
}
__device__ __forceinline__ void store_row(float* M, const tc::Lane& l, const float (&v)[32]) {
  float4* r = const_cast<float4*>(row_ptr(M, l));
#pragma unroll
  for (int q = 0; q < 8; ++q) r[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

// right-factor buffer `buf` <- a TMEM slot or a compact matrix
__device__ __forceinline__ bool stage_right_slot(State& s, const tc::Lane& l, int buf, int slot) {
  float v[32];
  tc::tmem_ld32(slot_addr(s, l, slot), v);
  return tc::stage_B_f16(s.b[buf], s.b[buf] + tc::kBBytesF16, l, v);
}
__device__ __forceinline__ bool stage_right_compact(State& s, const tc::Lane& l, int buf, const float* M) {
  float v[32];
  load_row(M, l, v);
  return tc::stage_B_f16(s.b[buf], s.b[buf] + tc::kBBytesF16, l, v);
}
// expanded left factor at TMEM column `a` <- a compact matrix (read across rows:
// the caller has synchronised after the matrix was written)
__device__ __forceinline__ bool stage_left(State& s, const tc::Lane& l, uint32_t a, const float* M) {
  return tc::stage_A_tmem_f16(s.tmem + l.lane_addr + a, s.tmem + l.lane_addr + a + tc::kAColsF16, M, l.L,
                              l.c0 / 32);
}
// expanded left factors <- two TMEM slots, through the compact transit matrix
__device__ __forceinline__ bool slots_to_left(State& s, const tc::Lane& l, int s0, int s1) {
  float v[32];
  bool ok = true;
  tc::tmem_ld32(slot_addr(s, l, s0), v);
  store_row(s.tr, l, v);
  __syncthreads();
  ok &= stage_left(s, l, kA0, s.tr);
  __syncthreads();
  tc::tmem_ld32(slot_addr(s, l, s1), v);
  store_row(s.tr, l, v);
  __syncthreads();
  ok &= stage_left(s, l, kA1, s.tr);
  return ok;
}

// One product of a group, by the elected thread.
struct Prod {
  uint32_t a;  // TMEM column of the expanded left factor
  int buf;     // right-factor buffer
  int dst;     // TMEM slot of the result
  int acc;     // accumulate onto the slot
};

// Issues the three products of a stage as one group and waits for them (all
// threads); false when the wait gave up (*abort) or a staged value was out of
// range (*range, set by the staging just before).
__device__ __forceinline__ bool run_group(State& s, Prod p0, Prod p1, Prod p2, bool in_range, int* abort,
                                          int* range) {
  if (!in_range) *range = 1;
  tc::tmem_st_wait();
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::fence_after_sync();
    const Prod ps[3] = {p0, p1, p2};
#pragma unroll
    for (int q = 0; q < 3; ++q)
      tc::mma_product_f16(s.tmem + (uint32_t)(64 * ps[q].dst), s.tmem + ps[q].a, s.tmem + ps[q].a + tc::kAColsF16,
                          tc::smem_u32(s.b[ps[q].buf]), tc::smem_u32(s.b[ps[q].buf] + tc::kBBytesF16),
                          (uint32_t)ps[q].acc);
    tc::commit(s.mbar);
  }
  if (!tc::mbar_wait(s.mbar, s.phase)) *abort = 1;
  s.phase ^= 1;
  tc::fence_after_sync();
  __syncthreads();
  return *abort == 0 && *range == 0;
}

// slot dst = a x + b Y (+ c I), x given in registers, Y a compact matrix
__device__ __forceinline__ void combine(State& s, const tc::Lane& l, int dst, float a, const float (&x)[32],
                                        float b, const float* Y, float c) {
  float y[32];
  load_row(Y, l, y);
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    y[k] = fmaf(a, x[k], b * y[k]);
    if (l.im == 0 && l.c0 + k == l.i) y[k] += c;
  }
  tc::tmem_st32(slot_addr(s, l, dst), y);
}

// slot dst = b Y (+ c I), Y a compact matrix
__device__ __forceinline__ void scaled(State& s, const tc::Lane& l, int dst, float b, const float* Y, float c) {
  float y[32];
  load_row(Y, l, y);
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    y[k] *= b;
    if (l.im == 0 && l.c0 + k == l.i) y[k] += c;
  }
  tc::tmem_st32(slot_addr(s, l, dst), y);
}

}  // namespace gtc

// Gate targets, exact gradient, Dp = 64.
__global__ void __launch_bounds__(tc::kThreads, 1) k_grad_tc64(ProbDev p, WorkDev w) {
  using namespace gtc;
  constexpr int D = kD;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar, s_mbar_mk;
  __shared__ int s_abort, s_range;
  __shared__ float s_nrm[2], s_mmax[8];
  __shared__ float s_part[4][64];
  const uint32_t pad = (tc::kSmemAlign - (tc::smem_u32(smem_raw) & (tc::kSmemAlign - 1))) & (tc::kSmemAlign - 1);
  State s;
  s.b[0] = smem_raw + pad;
  s.b[1] = s.b[0] + 2 * tc::kBBytesF16;
  s.tB = reinterpret_cast<float*>(s.b[1] + 2 * tc::kBBytesF16);
  s.tdB = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(s.tB) + kMatBytes);
  s.tr = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(s.tdB) + kMatBytes);
  const float2* Mbuf = reinterpret_cast<const float2*>(reinterpret_cast<uint8_t*>(s.tr) + kMatBytes);
  s.mbar = tc::smem_u32(&s_bar);
  s.phase = 0;
  const uint32_t mbar_mk = tc::smem_u32(&s_mbar_mk);
  uint32_t mk_phase = 0;
  bool mk_pending = false;  // a bulk copy into Mbuf is in flight
  const tc::Lane l = tc::lane_of();
  if (threadIdx.x < 32) tc::tmem_alloc(&s_tmem, tc::kTmemCols);
  if (threadIdx.x == 0) {
    tc::mbar_init(s.mbar);
    tc::mbar_init(mbar_mk);
    s_abort = 0;
    s_range = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  s.tmem = s_tmem;
  float* nrm_scratch = s.tr;  // [64 columns][65]: |A| for the column sums

  const long items = (long)p.n_members * p.n_t;
  const float2* Pslots = reinterpret_cast<const float2*>(w.P);
  if (threadIdx.x == 0 && (long)blockIdx.x < items)
    tc::tma_bulk_g2s(tc::smem_u32(Mbuf), Pslots + (size_t)blockIdx.x * D * D, kMkBytes, mbar_mk);
  mk_pending = (long)blockIdx.x < items;
  for (long it = blockIdx.x; it < items; it += gridDim.x) {
    const int m = (int)(it / p.n_t), k = (int)(it % p.n_t);
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
    if (!tc::mbar_wait(mbar_mk, mk_phase)) s_abort = 1;  // M_k of this unit in Mbuf
    else mk_pending = false;
    mk_phase ^= 1;
    const float2* Mk = Mbuf;
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
    // ---- compact B (real-part threads) and dB = M_k 2^-s 2^-ed (imaginary-part threads)
    if (l.im == 0) {
      float4* re = reinterpret_cast<float4*>(s.tB + (uint32_t)l.i * tc::kLdp + l.c0);
      float4* im = reinterpret_cast<float4*>(s.tB + tc::kPlaneFloats + (uint32_t)l.i * tc::kLdp + l.c0);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        re[q] = make_float4(ar[4 * q] * scl, ar[4 * q + 1] * scl, ar[4 * q + 2] * scl, ar[4 * q + 3] * scl);
        im[q] = make_float4(ai[4 * q] * scl, ai[4 * q + 1] * scl, ai[4 * q + 2] * scl, ai[4 * q + 3] * scl);
      }
    } else {
      float4* re = reinterpret_cast<float4*>(s.tdB + (uint32_t)l.i * tc::kLdp + l.c0);
      float4* im = reinterpret_cast<float4*>(s.tdB + tc::kPlaneFloats + (uint32_t)l.i * tc::kLdp + l.c0);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float2 e0 = Mk[l.i + D * (l.c0 + 4 * q)], e1 = Mk[l.i + D * (l.c0 + 4 * q + 1)];
        const float2 e2 = Mk[l.i + D * (l.c0 + 4 * q + 2)], e3 = Mk[l.i + D * (l.c0 + 4 * q + 3)];
        re[q] = make_float4(e0.x * dscl, e1.x * dscl, e2.x * dscl, e3.x * dscl);
        im[q] = make_float4(e0.y * dscl, e1.y * dscl, e2.y * dscl, e3.y * dscl);
      }
    }
    __syncthreads();
    if (s_abort) break;  // the wait for M_k gave up
    // the next unit's M_k into Mbuf while this unit's products run (Mbuf is
    // free: every thread passed the barrier after its last read)
    if (it + gridDim.x < items) {
      if (threadIdx.x == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc::tma_bulk_g2s(tc::smem_u32(Mbuf), Pslots + (size_t)(it + gridDim.x) * D * D, kMkBytes, mbar_mk);
      }
      mk_pending = true;
    }
    int sy = 0, sdy = 1, ay = 2, ad = 3;
    // ---- X = B B (slot ay), dX = dB B + B dB (slot ad)
    bool in_range = stage_left(s, l, kA0, s.tB) & stage_left(s, l, kA1, s.tdB);
    in_range &= stage_right_compact(s, l, 0, s.tB) & stage_right_compact(s, l, 1, s.tdB);
    if (!run_group(s, {kA1, 0, ad, 0}, {kA0, 0, ay, 0}, {kA0, 1, ad, 1}, in_range, &s_abort, &s_range)) break;
    // ---- X, dX as the resident left factors; Y, dY of the first Horner stage
    const int L = deg / 2;
    in_range = slots_to_left(s, l, ay, ad);
    {
      float x[32];
      tc::tmem_ld32(slot_addr(s, l, ay), x);
      combine(s, l, sy, c_invf32[2 * L], x, c_invf32[2 * L - 1], s.tB, c_invf32[2 * L - 2]);
      tc::tmem_ld32(slot_addr(s, l, ad), x);
      combine(s, l, sdy, c_invf32[2 * L], x, c_invf32[2 * L - 1], s.tdB, 0.f);
    }
    tc::tmem_st_wait();
    bool ok = true;
    // ---- Horner in X: dY' = X dY + dX Y + c dB, Y' = X Y + c B + c' I
    for (int i = L - 2; i >= 0 && ok; --i) {
      scaled(s, l, ay, c_invf32[2 * i + 1], s.tB, c_invf32[2 * i]);
      scaled(s, l, ad, c_invf32[2 * i + 1], s.tdB, 0.f);
      in_range &= stage_right_slot(s, l, 0, sdy) & stage_right_slot(s, l, 1, sy);
      ok = run_group(s, {kA0, 0, ad, 1}, {kA0, 1, ay, 1}, {kA1, 1, ad, 1}, in_range, &s_abort, &s_range);
      int t = sy; sy = ay; ay = t;
      t = sdy; sdy = ad; ad = t;
    }
    if (!ok) break;
    // ---- squarings: dY' = Y dY + dY Y, Y' = Y Y
    for (int r = 0; r < sq && ok; ++r) {
      __syncthreads();  // the transit matrix is free
      in_range = slots_to_left(s, l, sy, sdy);
      in_range &= stage_right_slot(s, l, 0, sdy) & stage_right_slot(s, l, 1, sy);
      ok = run_group(s, {kA0, 0, ad, 0}, {kA0, 1, ay, 0}, {kA1, 1, ad, 1}, in_range, &s_abort, &s_range);
      int t = sy; sy = ay; ay = t;
      t = sdy; sdy = ad; ad = t;
    }
    if (!ok) break;
    // ---- L(A_k, M_k) = 2^ed dY over M_k in the P buffer: two row-major planes
    // (coalesced through shared memory)
    {
      float v[32];
      tc::tmem_ld32(slot_addr(s, l, sdy), v);
#pragma unroll
      for (int c = 0; c < 32; ++c) v[c] = ldexpf(v[c], ed);
      store_row(s.tr, l, v);
      __syncthreads();
      float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float2*>(w.P) + ((size_t)m * p.n_t + k) * D * D);
      for (int e = threadIdx.x; e < 2 * D * D / 4; e += tc::kThreads) {
        const int plane = e >> 10, r = (e >> 4) & 63, c4 = e & 15;
        dst[e] = *reinterpret_cast<const float4*>(s.tr + plane * tc::kPlaneFloats + r * tc::kLdp + 4 * c4);
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (s_abort || s_range) {
    // units this CTA did not finish get a NaN entry in their P slot, so the
    // trace pass gives them NaN gradients: no stale value passes for a result
    // even on paths that never read the flag
    for (long it = blockIdx.x + threadIdx.x * (long)gridDim.x; it < items; it += (long)gridDim.x * blockDim.x)
      reinterpret_cast<float2*>(w.P)[(size_t)it * D * D] = make_float2(__int_as_float(0x7fc00000), 0.f);
  }
  if (mk_pending && threadIdx.x == 0) tc::mbar_wait(mbar_mk, mk_phase);  // a copy into Mbuf is in flight (bounded)
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

// g_j of every unit from L = L(A_k, M_k) stored in the P buffer as two
// row-major planes: g_j = Re(c dt_k scale_m Tr(L C_j))
// = dt scale (Im or Re) sum_q L[q] C_j[q], q = c + 64 r pairing L[r][c] with
// C_j[c][r] (C_j column-major).  The controls sit in shared memory, up to
// kTraceCtrls at a time; one warp per unit, each lane summing the entries
// q = 4 lane + 128 t, t = 0..31 in order, then a fixed shuffle tree.
constexpr int kTraceCtrls = 6;
__global__ void __launch_bounds__(256) k_trace_tc64(ProbDev p, WorkDev w) {
  constexpr int D = 64;
  extern __shared__ __align__(16) float2 cT[];  // [nj][D * D] the controls, column-major
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long items = (long)p.n_members * p.n_t;
  for (int j0 = 0; j0 < p.n_c; j0 += kTraceCtrls) {
    const int nj = p.n_c - j0 < kTraceCtrls ? p.n_c - j0 : kTraceCtrls;
    __syncthreads();
    for (int e = threadIdx.x; e < nj * D * D; e += blockDim.x) cT[e] = p.ctrls_f32[(size_t)j0 * D * D + e];
    __syncthreads();
    for (long it = (long)blockIdx.x * 8 + warp; it < items; it += (long)gridDim.x * 8) {
      const float4* Lre = reinterpret_cast<const float4*>(reinterpret_cast<const float2*>(w.P) + (size_t)it * D * D);
      const float4* Lim = Lre + D * D / 4;
      float re[kTraceCtrls], im[kTraceCtrls];
#pragma unroll
      for (int j = 0; j < kTraceCtrls; ++j) re[j] = im[j] = 0.f;
#pragma unroll 4
      for (int t = 0; t < 32; ++t) {
        const int q4 = lane + 32 * t;  // entries 4 q4 .. 4 q4 + 3
        const float4 a = Lre[q4], b = Lim[q4];
#pragma unroll
        for (int j = 0; j < kTraceCtrls; ++j) {
          if (j < nj) {
            const float4* cj = reinterpret_cast<const float4*>(cT + (size_t)j * D * D);
            const float4 c01 = cj[2 * q4], c23 = cj[2 * q4 + 1];  // C[4 q4 + 0..3] as re, im pairs
            re[j] = fmaf(a.x, c01.x, re[j]); re[j] = fmaf(-b.x, c01.y, re[j]);
            im[j] = fmaf(a.x, c01.y, im[j]); im[j] = fmaf(b.x, c01.x, im[j]);
            re[j] = fmaf(a.y, c01.z, re[j]); re[j] = fmaf(-b.y, c01.w, re[j]);
            im[j] = fmaf(a.y, c01.w, im[j]); im[j] = fmaf(b.y, c01.z, im[j]);
            re[j] = fmaf(a.z, c23.x, re[j]); re[j] = fmaf(-b.z, c23.y, re[j]);
            im[j] = fmaf(a.z, c23.y, im[j]); im[j] = fmaf(b.z, c23.x, im[j]);
            re[j] = fmaf(a.w, c23.z, re[j]); re[j] = fmaf(-b.w, c23.w, re[j]);
            im[j] = fmaf(a.w, c23.w, im[j]); im[j] = fmaf(b.w, c23.z, im[j]);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < kTraceCtrls; ++j) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          re[j] += __shfl_xor_sync(0xffffffffu, re[j], o);
          im[j] += __shfl_xor_sync(0xffffffffu, im[j], o);
        }
      }
      if (lane == 0) {
        const int m = (int)(it / p.n_t), k = (int)(it % p.n_t);
        const double gsc = p.dt[k] * p.m_scale[m];
        double* Gout = w.Gm + (size_t)it * p.n_c + j0;
#pragma unroll
        for (int j = 0; j < kTraceCtrls; ++j)
          if (j < nj) Gout[j] = gsc * (double)(p.gen == GEN_HERM ? im[j] : re[j]);
      }
    }
  }
}

}  // namespace pgx
