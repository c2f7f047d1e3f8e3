// pgx_diag_tc_cmatmul64: batched complex 64 x 64 products C_i = P_i Q_i
// through the tcgen05 product engine of pgx_tc.cuh (the engine the D = 64
// mixed gradient runs on), for tests and profiling of the engine alone.
#include <cuda_runtime.h>

#include <vector>

#include "pgx.h"
#include "pgx_tc.cuh"

namespace pgx {
namespace tc {

// One persistent CTA per SM.  Per item: Q is loaded into TMEM in the stacked
// layout (columns 64..127), read back and staged as the B operand; P is
// loaded into TMEM (columns 0..63) and staged as the expanded A operand in
// shared memory, or (a_tmem) copied into shared memory compact and expanded
// into TMEM columns 256..511.  The product lands in columns 128..191 and is
// written out.  mode 2 runs the 3xFP16 form (fp16 parts, A in TMEM), the
// gradient's path; passes is then 3.
__global__ void __launch_bounds__(kThreads, 1)
k_tc_cmm64(const float2* __restrict__ P, const float2* __restrict__ Q, float2* __restrict__ C, int n, int passes,
           int a_tmem, int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int s_abort;
  const uint32_t pad = (kSmemAlign - (smem_u32(smem_raw) & (kSmemAlign - 1))) & (kSmemAlign - 1);
  uint8_t* a_hi = smem_raw + pad;
  uint8_t* a_lo = a_hi + kABytes;
  uint8_t* b_hi = a_lo + kABytes;
  uint8_t* b_lo = b_hi + kBBytes;
  const Lane l = lane_of();
  const uint32_t mbar = smem_u32(&s_bar);
  if (threadIdx.x < 32) tmem_alloc(&s_tmem, kTmemCols);
  if (threadIdx.x == 0) {
    mbar_init(mbar);
    s_abort = 0;
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_tmem;
  const uint32_t my = tmem + l.lane_addr + (uint32_t)l.c0;
  uint32_t phase = 0;
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const float* Pf = reinterpret_cast<const float*>(P + (size_t)it * 4096);
    const float* Qf = reinterpret_cast<const float*>(Q + (size_t)it * 4096);
    float v[32];
    if (a_tmem == 2) {  // planar, row-padded compact copy of P
      float* Pc = reinterpret_cast<float*>(a_hi);
      for (int e = threadIdx.x; e < 4096; e += kThreads) {
        const float2 x = P[(size_t)it * 4096 + e];  // column-major: row e % 64, column e / 64
        Pc[(e % 64) * kLdp + e / 64] = x.x;
        Pc[kPlaneFloats + (e % 64) * kLdp + e / 64] = x.y;
      }
    } else if (a_tmem) {
      float2* Pc = reinterpret_cast<float2*>(a_hi);  // compact copy of P
      for (int e = threadIdx.x; e < 4096; e += kThreads) Pc[e] = P[(size_t)it * 4096 + e];
    }
#pragma unroll
    for (int c = 0; c < 32; ++c) v[c] = Pf[2 * (l.i + 64 * (l.c0 + c)) + l.im];
    tmem_st32(my + 0, v);
#pragma unroll
    for (int c = 0; c < 32; ++c) v[c] = Qf[2 * (l.i + 64 * (l.c0 + c)) + l.im];
    tmem_st32(my + 64, v);
    tmem_st_wait();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (a_tmem == 2) {
      __syncthreads();  // the compact copy of P is complete
      stage_A_tmem_f16(tmem + l.lane_addr + 256, tmem + l.lane_addr + 256 + kAColsF16,
                       reinterpret_cast<const float*>(a_hi), l.L, l.c0 / 32);
      tmem_st_wait();
    } else if (a_tmem) {
      __syncthreads();  // the compact copy of P is complete
      stage_A_tmem(tmem + l.lane_addr + 256, tmem + l.lane_addr + 384, reinterpret_cast<const float2*>(a_hi), l.L,
                   l.c0 / 32);
      tmem_st_wait();
    } else {
      tmem_ld32(my + 0, v);
      stage_A(a_hi, a_lo, l, v);
    }
    tmem_ld32(my + 64, v);
    if (a_tmem == 2) stage_B_f16(b_hi, b_hi + kBBytesF16, l, v);
    else stage_B(b_hi, b_lo, l, v);
    fence_smem_to_async();
    fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
      fence_after_sync();
      if (a_tmem == 2)
        issue_product_f16(tmem + 128, tmem + 256, tmem + 256 + kAColsF16, smem_u32(b_hi),
                          smem_u32(b_hi + kBBytesF16), 0, mbar);
      else if (a_tmem)
        issue_product_ta(tmem + 128, tmem + 256, tmem + 384, smem_u32(b_hi), smem_u32(b_lo), 0, mbar, passes);
      else
        issue_product(tmem + 128, smem_u32(a_hi), smem_u32(a_lo), smem_u32(b_hi), smem_u32(b_lo), 0, mbar, passes);
    }
    if (!mbar_wait(mbar, phase)) s_abort = 1;
    phase ^= 1;
    fence_after_sync();
    __syncthreads();
    if (s_abort) break;
    tmem_ld32(my + 128, v);
    float* Cf = reinterpret_cast<float*>(C + (size_t)it * 4096);
#pragma unroll
    for (int c = 0; c < 32; ++c) Cf[2 * (l.i + 64 * (l.c0 + c)) + l.im] = v[c];
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
  }
  if (s_abort && threadIdx.x == 0) {
    atomicExch(err, 1);
    mbar_wait(mbar, phase ^ 1);  // bounded: let a late group finish before TMEM is freed
  }
  fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    fence_after_sync();
    tmem_dealloc(tmem, kTmemCols);
  }
}

}  // namespace tc
}  // namespace pgx

extern "C" int pgx_diag_tc_cmatmul64(const double* P, const double* Q, double* C, int32_t n, int32_t passes,
                                     int32_t mode) {
  using namespace pgx::tc;
  if (!P || !Q || !C || n < 1 || (passes != 1 && passes != 3) || mode < 0 || mode > 2 || (mode == 2 && passes != 3))
    return PGX_ERR_INVALID;
  const size_t elems = (size_t)n * 4096;
  std::vector<float> hP(2 * elems), hQ(2 * elems), hC(2 * elems);
  for (size_t e = 0; e < 2 * elems; ++e) {
    hP[e] = (float)P[e];
    hQ[e] = (float)Q[e];
  }
  float2 *dP = nullptr, *dQ = nullptr, *dC = nullptr;
  int* dErr = nullptr;
  int st = PGX_OK;
  int dev = 0, sms = 0, herr = 0;
  const size_t smem = kStageBytes + kSmemAlign;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMalloc(&dP, elems * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&dQ, elems * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&dC, elems * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&dErr, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dP, hP.data(), elems * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dQ, hQ.data(), elems * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dErr, 0, sizeof(int));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_tc_cmm64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    const int grid = n < sms ? n : sms;
    k_tc_cmm64<<<grid, kThreads, smem>>>(dP, dQ, dC, n, passes, mode, dErr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&herr, dErr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hC.data(), dC, elems * sizeof(float2), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) st = e == cudaErrorMemoryAllocation ? PGX_ERR_NOMEM : PGX_ERR_CUDA;
  else if (herr) st = PGX_ERR_TIMEOUT;
  if (st == PGX_OK)
    for (size_t k = 0; k < 2 * elems; ++k) C[k] = (double)hC[k];
  cudaFree(dP);
  cudaFree(dQ);
  cudaFree(dC);
  cudaFree(dErr);
  return st;
}
