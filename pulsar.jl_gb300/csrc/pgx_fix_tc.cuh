// The fix-up products of the parallel-in-time gate chains at D = 64 on the
// tensor cores (tcgen05, 3xTF32: FP32-class, like the CUDA-core kernels they
// replace, and FP32's exponent range, so the small costates need no scaling).
//   forward (BWD = 0):  P_k <- P_k T_b          for every slice past the first block;
//   backward (BWD = 1): Lambda = Lambda_b R_kk (when kk is not the block end),
//                       M_k = P_k Lambda        for every slice;
// the same products, operands and outputs as k_chainf_fix_mx /
// k_chainb_fix_mx.  Each unit is independent: its operands (32 KB each,
// contiguous) arrive by TMA bulk copies on one mbarrier, the left factor is
// expanded into TMEM, the right one staged in shared memory, and the result
// leaves through shared memory as coalesced stores.  One persistent CTA per SM
// (the whole TMEM: the expanded left factor takes 256 columns).  Waits are
// clock-bounded; a CTA that gives up flags the evaluation, writes NaN into its
// unfinished outputs, waits (bounded) for its copies and frees its TMEM.
//
// Included by pgx_mixed.cu after pgx_grad_tc.cuh (g_grad_tc_timeout).
#pragma once
#include "pgx_tc.cuh"

namespace pgx {

template <int BWD>
__global__ void __launch_bounds__(tc::kThreads, 1) k_fix_tc64(ProbDev p, WorkDev w) {
  constexpr int D = 64;
  constexpr uint32_t kMat = D * D * sizeof(float2);  // 32 KB
  constexpr uint32_t kAHi = 256, kALo = 384, kSlotLam = 0, kSlotOut = 64;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar, s_ld;
  __shared__ int s_abort;
  const uint32_t pad = (tc::kSmemAlign - (tc::smem_u32(smem_raw) & (tc::kSmemAlign - 1))) & (tc::kSmemAlign - 1);
  uint8_t* b_hi = smem_raw + pad;
  uint8_t* b_lo = b_hi + tc::kBBytes;
  float2* cA = reinterpret_cast<float2*>(b_lo + tc::kBBytes);  // left operand P_k (column-major)
  float2* cB = cA + D * D;                                      // T_b / Lambda_b
  float2* cR = cB + D * D;                                      // R_kk
  const tc::Lane l = tc::lane_of();
  const uint32_t mbar = tc::smem_u32(&s_bar), mld = tc::smem_u32(&s_ld);
  uint32_t phase = 0, ld_phase = 0;
  if (threadIdx.x < 32) tc::tmem_alloc(&s_tmem, tc::kTmemCols);
  if (threadIdx.x == 0) {
    tc::mbar_init(mbar);
    tc::mbar_init(mld);
    s_abort = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  const uint32_t lane_base = tmem + l.lane_addr;
  const int Lb = w.pit_len;
  const int nk = BWD ? p.n_t : p.n_t - Lb;
  const long items = (long)p.n_members * (nk > 0 ? nk : 0);
  const bool grape = (p.grad_mode == GRAD_REF_GRAPE);
  float2* Pst = reinterpret_cast<float2*>(w.P);
  long it = blockIdx.x;
  for (; it < items; it += gridDim.x) {
    const int m = (int)(it / nk), k = (BWD ? 0 : Lb) + (int)(it % nk), b = k / Lb;
    const int k1 = min(p.n_t, (b + 1) * Lb);
    const int kk = grape ? k : k + 1;
    const bool with_r = BWD && kk != k1;
    float2* Pk = Pst + ((size_t)m * p.n_t + k) * D * D;
    const float2* Xb = (BWD ? w.pit_lam : w.pit_pre) + ((size_t)m * w.pit_blocks + b) * D * D;
    if (threadIdx.x == 0) {
      tc::mbar_expect_tx(mld, (with_r ? 3u : 2u) * kMat);
      tc::tma_bulk_copy(tc::smem_u32(cA), Pk, kMat, mld);
      tc::tma_bulk_copy(tc::smem_u32(cB), Xb, kMat, mld);
      if (with_r) tc::tma_bulk_copy(tc::smem_u32(cR), w.pit_r + ((size_t)m * p.n_t + kk) * D * D, kMat, mld);
    }
    if (!tc::mbar_wait(mld, ld_phase)) s_abort = 1;
    ld_phase ^= 1;
    __syncthreads();
    if (s_abort) break;
    float v[32];
    if (with_r) {  // Lambda = Lambda_b R_kk into TMEM slot kSlotLam
      tc::stage_A_tmem(lane_base + kAHi, lane_base + kALo, cB, l.L, l.c0 / 32);
#pragma unroll
      for (int c = 0; c < 32; ++c) v[c] = reinterpret_cast<const float*>(cR)[2 * (l.i + D * (l.c0 + c)) + l.im];
      tc::stage_B(b_hi, b_lo, l, v);
      tc::tmem_st_wait();
      tc::fence_smem_to_async();
      tc::fence_before_sync();
      __syncthreads();
      if (threadIdx.x == 0) {
        tc::fence_after_sync();
        tc::issue_product_ta(tmem + kSlotLam, tmem + kAHi, tmem + kALo, tc::smem_u32(b_hi), tc::smem_u32(b_lo), 0,
                             mbar);
      }
      if (!tc::mbar_wait(mbar, phase)) s_abort = 1;
      phase ^= 1;
      tc::fence_after_sync();
      __syncthreads();
      if (s_abort) break;
      tc::tmem_ld32(lane_base + kSlotLam + l.c0, v);  // the right factor of the next product
    } else {
#pragma unroll
      for (int c = 0; c < 32; ++c) v[c] = reinterpret_cast<const float*>(cB)[2 * (l.i + D * (l.c0 + c)) + l.im];
    }
    // result = P_k X into TMEM slot kSlotOut
    tc::stage_A_tmem(lane_base + kAHi, lane_base + kALo, cA, l.L, l.c0 / 32);
    tc::stage_B(b_hi, b_lo, l, v);
    tc::tmem_st_wait();
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::fence_after_sync();
      tc::issue_product_ta(tmem + kSlotOut, tmem + kAHi, tmem + kALo, tc::smem_u32(b_hi), tc::smem_u32(b_lo), 0,
                           mbar);
    }
    if (!tc::mbar_wait(mbar, phase)) s_abort = 1;
    phase ^= 1;
    tc::fence_after_sync();
    __syncthreads();
    if (s_abort) break;
    tc::tmem_ld32(lane_base + kSlotOut + l.c0, v);
#pragma unroll
    for (int c = 0; c < 32; ++c) reinterpret_cast<float*>(cA)[2 * (l.i + D * (l.c0 + c)) + l.im] = v[c];
    __syncthreads();
    float4* dst = reinterpret_cast<float4*>(Pk);
    const float4* src = reinterpret_cast<const float4*>(cA);
    for (int e = threadIdx.x; e < D * D / 2; e += tc::kThreads) dst[e] = src[e];
    // cA is reloaded by the next unit's copy: every store above must have read it
    __syncthreads();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (s_abort) {
    for (long u = it + threadIdx.x * (long)gridDim.x; u < items; u += (long)gridDim.x * blockDim.x) {
      const int m = (int)(u / nk), k = (BWD ? 0 : Lb) + (int)(u % nk);
      Pst[((size_t)m * p.n_t + k) * D * D] = make_float2(__int_as_float(0x7fc00000), 0.f);
    }
    if (threadIdx.x == 0) {
      atomicOr(&g_grad_tc_timeout, 1);
      tc::mbar_wait(mld, ld_phase ^ 1);  // bounded: copies in flight
      tc::mbar_wait(mbar, phase ^ 1);    // bounded: a late product group
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, tc::kTmemCols);
  }
}

}  // namespace pgx
