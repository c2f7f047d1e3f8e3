// tcgen05 building blocks: 64 x 64 complex FP32 products on the tensor cores
// with 3xTF32 splitting.
//
// A complex product C = P Q (64 x 64) is one real MMA of M = 128, N = 64,
// K = 128:
//     [Cr; Ci] = [Pr -Pi; Pi Pr] [Qr; Qi].
// The accumulator [Cr; Ci] sits in tensor memory (TMEM) with lane L = row L
// of the stack: lanes 0..63 hold the real rows, 64..127 the imaginary rows.
// The same "stacked" layout stores every complex 64 x 64 matrix a kernel
// keeps in TMEM (64 columns per matrix).  A thread that owns lane L and 32
// columns can stage its values straight into either operand:
//   - A (the left factor, expanded): its own row and the partner row of
//     [Pr -Pi; Pi Pr];
//   - B (the right factor): row k = L of [Qr; Qi].
// Both operands are K-major with the 128-byte swizzle in shared memory:
// 8-row groups of 128-byte rows (32 tf32 values) at 1024-byte stride, the
// 16-byte chunks of a row XOR-permuted by the row index mod 8, and K beyond
// 32 values in further 128-byte-wide column blocks.  Every staging store of a
// warp lands in distinct banks.
//
// 3xTF32: each operand x is split into hi = tf32(x) (round to nearest) and
// lo = x - hi (exact in FP32), and P Q = P_lo Q_hi + P_hi Q_lo + P_hi Q_hi is
// accumulated in FP32: about 2^-22 relative per product, FP32 class.
//
// CTA shape: 256 threads.  Warp w serves TMEM lanes 32 (w % 4) .. +31 (a warp
// may only access its own lane quarter) and columns 32 (w / 4) .. +31 of every
// 64-column matrix.  One elected thread issues the MMAs; completion is tracked
// by an mbarrier that all threads wait on with a clock bound.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pgx {
namespace tc {

constexpr int kThreads = 256;
constexpr uint32_t kTmemCols = 512;                       // 8 matrices of 64 columns
constexpr uint32_t kABytes = 128u * 128u * 4u;            // one part (hi or lo) of the expanded A
constexpr uint32_t kBBytes = 64u * 128u * 4u;             // one part of B
constexpr uint32_t kStageBytes = 2u * kABytes + 2u * kBBytes;  // 192 KB
constexpr uint32_t kSmemAlign = 1024;                     // the 128-byte swizzle repeats every 1024 bytes
// Instruction descriptor of tcgen05.mma kind::tf32: D FP32 (bits 4-5 = 1),
// A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
// Clock cycles an MMA-completion wait may take before the kernel gives up
// (about 2 s at 2 GHz; one product group takes a few microseconds).
constexpr long long kWaitCycles = 4000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) in a K-major, 128-byte-swizzled tile with
// `rows` rows of 32-bit elements (k blocks of 32 values, rows x 128 bytes each).
__device__ __forceinline__ uint32_t sw128_off(int row, int k, int rows) {
  const int blk = k >> 5, kk = k & 31;
  return (uint32_t)(blk * rows * 128 + (row >> 3) * 1024 + (row & 7) * 128 + (((kk >> 2) ^ (row & 7)) << 4) +
                    ((kk & 3) << 2));
}

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset (unused by swizzled K-major tiles; 16 bytes) >> 4 (bits 16-29),
// stride byte offset between 8-row groups >> 4 (bits 32-45), the fixed
// version 0b001 (bits 46-48), base offset 0 (the tiles are 1024-byte
// aligned), swizzle mode 2 = 128-byte swizzle (bits 61-63).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d_tmem), "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes this thread's shared-memory stores visible to the tensor cores.
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// TMEM allocation by one whole warp; the base address lands in *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// TMA bulk copy (cp.async.bulk) of `bytes` (a multiple of 16, both addresses
// 16-byte aligned) from global to this CTA's shared memory, completing on
// `mbar`, whose expected transaction count the same thread raises first.
__device__ __forceinline__ void tma_bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

// The same in two steps, for several copies completing on one barrier: the
// issuing thread arms the barrier once with the total byte count, then issues
// each copy.
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

// Waits for the barrier phase `parity` to complete, at most kWaitCycles.
// Returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  const long long t0 = clock64();
  uint32_t ok = 0;
  while (true) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > kWaitCycles) return false;
  }
}

// Loads 32 consecutive columns of this thread's TMEM lane (the warp's lane
// quarter, `taddr` = base | lane quarter << 16 | column).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  // the load and its completion wait in one statement, so no use of r[] can be
  // scheduled between them
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// Stores 32 consecutive columns of this thread's TMEM lane; completion is
// awaited by tmem_st_wait() before the values are read by an MMA or a load.
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float (&v)[32]) {
  uint32_t r[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) r[k] = __float_as_uint(v[k]);
  asm volatile("tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};"
               :: "r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
               : "memory");
}

// tf32 rounding (to nearest, ties away) of x, returned as FP32 with the low
// 13 mantissa bits zero.
__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// This thread's place in the 256-thread CTA.
struct Lane {
  int L;               // TMEM lane: row L of the stacked [re; im] matrix
  int i;               // matrix row 0..63
  int im;              // 0: real-part rows, 1: imaginary-part rows
  int c0;              // first of the 32 columns this thread handles
  uint32_t lane_addr;  // the warp's lane quarter in a TMEM address (lane << 16)
};
__device__ __forceinline__ Lane lane_of() {
  const int w = threadIdx.x >> 5;
  Lane l;
  l.L = 32 * (w & 3) + (threadIdx.x & 31);
  l.i = l.L & 63;
  l.im = l.L >> 6;
  l.c0 = 32 * (w >> 2);
  l.lane_addr = (uint32_t)(32 * (w & 3)) << 16;
  return l;
}

// Stages this thread's 32 values (row l.i of the real or imaginary part,
// columns c0..c0+31) into the expanded left operand [Pr -Pi; Pi Pr]: its own
// row and the partner row, hi and lo parts, 16-byte stores.
__device__ __forceinline__ void stage_A(uint8_t* a_hi, uint8_t* a_lo, const Lane& l, const float (&v)[32]) {
  const int r1 = l.im ? 64 + l.i : l.i;   // [Pr | .] or [Pi | .]
  const int r2 = l.im ? l.i : 64 + l.i;   // [. | -Pi] or [. | Pr]
  const float sg = l.im ? -1.f : 1.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float h[4], o[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      h[e] = tf32_hi(v[4 * j + e]);
      o[e] = v[4 * j + e] - h[e];
    }
    const int k1 = l.c0 + 4 * j, k2 = 64 + l.c0 + 4 * j;
    *reinterpret_cast<float4*>(a_hi + sw128_off(r1, k1, 128)) = make_float4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<float4*>(a_lo + sw128_off(r1, k1, 128)) = make_float4(o[0], o[1], o[2], o[3]);
    *reinterpret_cast<float4*>(a_hi + sw128_off(r2, k2, 128)) =
        make_float4(sg * h[0], sg * h[1], sg * h[2], sg * h[3]);
    *reinterpret_cast<float4*>(a_lo + sw128_off(r2, k2, 128)) =
        make_float4(sg * o[0], sg * o[1], sg * o[2], sg * o[3]);
  }
}

// Stages this thread's 32 values into the right operand [Qr; Qi]: k = l.L,
// n = c0..c0+31, hi and lo parts.  A warp's 32 lanes fill one 128-byte row.
__device__ __forceinline__ void stage_B(uint8_t* b_hi, uint8_t* b_lo, const Lane& l, const float (&v)[32]) {
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    const uint32_t off = sw128_off(l.c0 + c, l.L, 64);
    const float h = tf32_hi(v[c]);
    *reinterpret_cast<float*>(b_hi + off) = h;
    *reinterpret_cast<float*>(b_lo + off) = v[c] - h;
  }
}

// tcgen05.mma with the A operand in tensor memory: A (M = 128 rows, one
// per lane; K = 8 tf32 values in 8 consecutive 32-bit columns from a_tmem).
__device__ __forceinline__ void mma_tf32_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}"
      ::"r"(d_tmem), "r"(a_tmem), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

// Expanded left operand in TMEM: 128 lanes x 128 columns per part (hi at
// a_hi, lo at a_lo = a_hi + 128).  Thread (lane L, column half h) writes
// columns 64 h .. 64 h + 63 of its lane from the compact complex matrix P
// (64 x 64 float2, column-major, anywhere in shared memory):
//   lane i < 64:  [Pr | -Pi],   lane 64 + i:  [Pi | Pr]   (row i).
__device__ __forceinline__ void stage_A_tmem(uint32_t a_hi_lane, uint32_t a_lo_lane, const float2* P, int L,
                                             int h) {
  const int i = L & 63, im = L >> 6;
  const bool take_im = (h == 0) ? (im == 1) : (im == 0);  // h = 0: own part; h = 1: the other part
  const float sg = (h == 1 && im == 0) ? -1.f : 1.f;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float hv[32], lv[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) {
      const float2 e = P[i + 64 * (32 * half + c)];
      const float x = sg * (take_im ? e.y : e.x);
      hv[c] = tf32_hi(x);
      lv[c] = x - hv[c];
    }
    tmem_st32(a_hi_lane + (uint32_t)(64 * h + 32 * half), hv);
    tmem_st32(a_lo_lane + (uint32_t)(64 * h + 32 * half), lv);
  }
}

// One elected thread: D = (accumulate ? D : 0) + A B in 3xTF32 with A in TMEM
// (hi at a_hi, lo at a_lo: 128 columns each) and B in shared memory.
__device__ __forceinline__ void issue_product_ta(uint32_t d_tmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi,
                                                 uint32_t b_lo, uint32_t accumulate, uint32_t mbar, int passes = 3) {
  const uint32_t pa[3] = {a_lo, a_hi, a_hi};
  const uint32_t pb[3] = {b_hi, b_lo, b_hi};
  uint32_t acc = accumulate;
  for (int ps = 3 - passes; ps < 3; ++ps) {
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const uint64_t db = make_desc(pb[ps] + (uint32_t)((t >> 2) * (64 * 128) + (t & 3) * 32));
      mma_tf32_ta(d_tmem, pa[ps] + (uint32_t)(8 * t), db, acc);
      acc = 1;
    }
  }
  commit(mbar);
}

// One elected thread: D (64 TMEM columns at d_tmem) = (accumulate ? D : 0) +
// A B in 3xTF32 (passes = 3: lo*hi, hi*lo, hi*hi) or plain TF32 (passes = 1),
// K = 128 in 16 steps of 8; then commits the group to the mbarrier.
__device__ __forceinline__ void issue_product(uint32_t d_tmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi,
                                              uint32_t b_lo, uint32_t accumulate, uint32_t mbar, int passes = 3) {
  const uint32_t pa[3] = {a_lo, a_hi, a_hi};
  const uint32_t pb[3] = {b_hi, b_lo, b_hi};
  uint32_t acc = accumulate;
  for (int ps = 3 - passes; ps < 3; ++ps) {
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const uint64_t da = make_desc(pa[ps] + (uint32_t)((t >> 2) * (128 * 128) + (t & 3) * 32));
      const uint64_t db = make_desc(pb[ps] + (uint32_t)((t >> 2) * (64 * 128) + (t & 3) * 32));
      mma_tf32(d_tmem, da, db, acc);
      acc = 1;
    }
  }
  commit(mbar);
}

// ---- 3xFP16 variant: the same products with fp16 operand parts -------------
// FP16 has TF32's 11-bit significand, and kind::f16 MMAs take K = 16 per
// instruction at the same issue cost (measured on GB300: an M = 128, N = 64
// MMA takes 48 cycles in either kind), so a product needs half the
// instructions and half the staging bytes.  Its exponent range is narrow:
// callers keep every staged value below kF16Limit in magnitude (the gradient
// scales the derivative family by a power of two per unit); values whose lo
// part falls below FP16's normal range keep an absolute error of 2^-25.
// F32 += F16 x F16, A K-major (from TMEM), B MN-major (bit 16)
constexpr uint32_t kIdescF16 = (1u << 4) | (1u << 16) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
constexpr uint32_t kBBytesF16 = 64u * 128u * 2u;  // one part of B: 64 n-rows x 128 k fp16
constexpr uint32_t kAColsF16 = 64;                // TMEM columns of one part of the expanded A (2 fp16 each)
constexpr float kF16Limit = 32768.f;

// Byte offset of fp16 element (k, n) of the right operand in an MN-major,
// 128-byte-swizzled tile: one 128-byte row of 64 n values per k, 8-row
// groups of 1024 bytes along k, the 16-byte chunks of a row XOR-permuted by
// k mod 8.  An MMA step (K = 16) reads two groups: 2048 bytes.
__device__ __forceinline__ uint32_t sw128_mn16(int k, int n) {
  return (uint32_t)((k >> 3) * 1024 + (k & 7) * 128 + (((n >> 3) ^ (k & 7)) << 4) + ((n & 7) << 1));
}
// Descriptor of an MN-major 128-byte-swizzled tile: the 8-row groups along K
// are 1024 bytes apart; N = 64 fits one swizzle atom, so the atom stride along
// N is never used (both byte offsets are set to 1024).
__device__ __forceinline__ uint64_t make_desc_mn(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(1024u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// x = hi + lo to about 2^-22 relative: hi = fp16(x), lo = fp16(x - hi).
// Returns false when x is beyond kF16Limit.
__device__ __forceinline__ bool split_f16(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(x - __half2float(hi));
  return fabsf(x) < kF16Limit;
}

// Two values at once: hi = fp16x2(x), lo = fp16x2(x - hi), packed as the MMA
// reads them (the first value in the low half).  Returns false when a value
// is beyond kF16Limit.
__device__ __forceinline__ bool split_f16x2(float x0, float x1, uint32_t& hw, uint32_t& lw) {
  const __half2 h = __floats2half2_rn(x0, x1);
  const float2 hf = __half22float2(h);
  const __half2 o = __floats2half2_rn(x0 - hf.x, x1 - hf.y);
  hw = *reinterpret_cast<const uint32_t*>(&h);
  lw = *reinterpret_cast<const uint32_t*>(&o);
  return fmaxf(fabsf(x0), fabsf(x1)) < kF16Limit;
}

// As stage_B: this thread's 32 values into the right operand [Qr; Qi] (k = l.L,
// n = c0..c0+31), hi and lo fp16 parts, MN-major: eight consecutive n per
// 16-byte store.  Returns false if a value is out of range.
__device__ __forceinline__ bool stage_B_f16(uint8_t* b_hi, uint8_t* b_lo, const Lane& l, const float (&v)[32]) {
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) ok &= split_f16x2(v[8 * j + 2 * e], v[8 * j + 2 * e + 1], hw[e], lw[e]);
    const uint32_t off = sw128_mn16(l.L, l.c0 + 8 * j);
    *reinterpret_cast<uint4*>(b_hi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(b_lo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
  return ok;
}

// Compact complex 64 x 64 matrices in shared memory as two row-major planes
// (real, then imaginary) with rows padded to kLdp floats: a warp's 16-byte
// row accesses (lanes = consecutive rows) fall in distinct banks.
constexpr int kLdp = 68;
constexpr uint32_t kPlaneFloats = 64u * kLdp;

// As stage_A_tmem with fp16 parts, from a planar compact matrix P: TMEM
// columns hold two consecutive k values each (the lower k in the low half),
// so one part of the expanded operand is 128 lanes x 64 columns; thread
// (L, h) writes columns 32 h .. 32 h + 31 (k = 64 h .. 64 h + 63): row i of
// one plane, read as 16-byte vectors.  Returns false if out of range.
__device__ __forceinline__ bool stage_A_tmem_f16(uint32_t a_hi_lane, uint32_t a_lo_lane, const float* P, int L,
                                                 int h) {
  const int i = L & 63, im = L >> 6;
  const bool take_im = (h == 0) ? (im == 1) : (im == 0);
  const float sg = (h == 1 && im == 0) ? -1.f : 1.f;
  const float4* row = reinterpret_cast<const float4*>(P + (take_im ? kPlaneFloats : 0u) + (uint32_t)i * kLdp);
  float hv[32], lv[32];
  bool ok = true;
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const float4 r = row[q];
    const float x[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      uint32_t hw, lw;
      ok &= split_f16x2(sg * x[2 * e], sg * x[2 * e + 1], hw, lw);
      hv[2 * q + e] = __uint_as_float(hw);
      lv[2 * q + e] = __uint_as_float(lw);
    }
  }
  tmem_st32(a_hi_lane + (uint32_t)(32 * h), hv);
  tmem_st32(a_lo_lane + (uint32_t)(32 * h), lv);
  return ok;
}

__device__ __forceinline__ void mma_f16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}"
      ::"r"(d_tmem), "r"(a_tmem), "l"(b), "r"(kIdescF16), "r"(accumulate)
      : "memory");
}

// One elected thread: D = (accumulate ? D : 0) + A B in 3xFP16 (lo*hi, hi*lo,
// hi*hi), A in TMEM (kAColsF16 columns per part), B MN-major in shared
// memory, K = 128 in 8 steps of 16.  Not committed: several products are
// issued back to back and committed together.
__device__ __forceinline__ void mma_product_f16(uint32_t d_tmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi,
                                                uint32_t b_lo, uint32_t accumulate) {
  const uint32_t pa[3] = {a_lo, a_hi, a_hi};
  const uint32_t pb[3] = {b_hi, b_lo, b_hi};
  uint32_t acc = accumulate;
#pragma unroll
  for (int ps = 0; ps < 3; ++ps) {
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      mma_f16_ta(d_tmem, pa[ps] + (uint32_t)(8 * t), make_desc_mn(pb[ps] + (uint32_t)(2048 * t)), acc);
      acc = 1;
    }
  }
}

// As mma_product_f16, then commits the group to the mbarrier.
__device__ __forceinline__ void issue_product_f16(uint32_t d_tmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi,
                                                  uint32_t b_lo, uint32_t accumulate, uint32_t mbar) {
  const uint32_t pa[3] = {a_lo, a_hi, a_hi};
  const uint32_t pb[3] = {b_hi, b_lo, b_hi};
  uint32_t acc = accumulate;
#pragma unroll
  for (int ps = 0; ps < 3; ++ps) {
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const uint64_t db = make_desc_mn(pb[ps] + (uint32_t)(2048 * t));
      mma_f16_ta(d_tmem, pa[ps] + (uint32_t)(8 * t), db, acc);
      acc = 1;
    }
  }
  commit(mbar);
}

}  // namespace tc
}  // namespace pgx
