// df-class complex 64 x 64 products on the tcgen05 tensor cores by exact
// integer slicing (the Ozaki scheme, with bf16 slices and FP32 accumulation).
//
// A df operand (hi + lo, ~48 significant bits) is scaled by a power of two 2^e
// so that every entry lies in [-1/2, 1/2], then cut into six slices of 8 bits:
//     x = 2^e sum_i s_i 2^(-8 (i + 1)),   s_i integers,
//     |s_0|, |s_1|, |s_2|, |s_4|, |s_5| <= 128,   |s_3| <= 256.
// s_0..s_2 come from hi alone; lo joins the remainder before s_3 (one FP32
// rounding at 2^-49 of the scale).  Every slice is exact in bf16 (8
// significant bits).
//
// A complex product is the real MMA [Cr; Ci] = [Pr -Pi; Pi Pr] [Qr; Qi]
// (M = 128, N = 64, K = 128).  With S_i, T_j the slices of the two real
// operands,
//     C = 2^(eA + eB) sum_l 2^(-8 (l + 2)) L_l,   L_l = sum_{i + j = l} S_i T_j.
// Each level L_l is accumulated in its own FP32 TMEM accumulator.  Slice
// products are integers, and with K = 128 the bounds above keep every level's
// partial sums at most 2^24 in magnitude (level 5: 2 pairs with s_3 at 2^22
// plus 4 pairs at 2^21), so the FP32 accumulation is exact.  Levels 0..5 take
// 21 slice pairs; level 6 (5 more pairs, also exact) is optional.  The levels
// are summed in df on the CUDA cores, smallest first.  What is dropped (levels
// beyond the last, the slicing remainder) stays below 2^-44 of K max|A| max|B|
// in the worst case of aligned signs.
//
// Measured on GB300: an M = 128 MMA of K = 16 takes 46-48 cycles at N = 64
// and 64 at N = 128; pairs that share a left slice go two at a time, so the 26
// pairs of levels 0..6 (12 MMA groups of N = 128, 2 of N = 64, K = 128 each)
// take ~7,000 cycles of one SM's tensor pipe, against ~48,000 FP32-pipe
// cycles for the same product in df arithmetic (~23 FP32 instructions per
// complex multiply-add).
//
// Layouts (128-byte swizzle, 1024-byte aligned tiles):
//   - the expanded left operand of one slice, K-major: 128 rows x 128 k bf16,
//     two 64-k column blocks of 16 KB (the 3xTF32 engine's byte layout, with
//     64 bf16 instead of 32 tf32 per 128-byte row);
//   - the right operand of one slice, MN-major: 128 k x 64 n bf16 (the 3xFP16
//     engine's layout).
#pragma once
#include <cuda_bf16.h>

#include "pgx_df.cuh"
#include "pgx_tc.cuh"

namespace pgx {
namespace oz {

using tc::Lane;

constexpr int kSlices = 6;
constexpr uint32_t kASlice = 128u * 128u * 2u;  // 32 KB
constexpr uint32_t kBSlice = 128u * 64u * 2u;   // 16 KB
// F32 += BF16 x BF16: D F32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 =
// 1), A K-major, B MN-major (bit 16), N = 64, M = 128.
constexpr uint32_t kIdescBF16 =
    (1u << 4) | (1u << 7) | (1u << 10) | (1u << 16) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

// Byte offset of bf16 element (row, k) of a K-major, 128-byte-swizzled tile of
// 128 rows: k blocks of 64 values (128 rows x 128 bytes each), 8-row groups at
// 1024 bytes, the 16-byte chunks of a row XOR-permuted by the row mod 8.
__device__ __forceinline__ uint32_t sw128_k16(int row, int k) {
  const int blk = k >> 6, kk = k & 63;
  return (uint32_t)(blk * 16384 + (row >> 3) * 1024 + (row & 7) * 128 + (((kk >> 3) ^ (row & 7)) << 4) +
                    ((kk & 7) << 1));
}

// The exponent e of the operand scale: the smallest power of two with
// 2^e >= 2 max|x| (entries of x 2^-e then lie in [-1/2, 1/2]; lo adds at most
// a relative 2^-24, which the rounding of slice 0 absorbs).  0 for a zero
// operand.
__device__ __forceinline__ int scale_exp(float maxabs) {
  if (!(maxabs > 0.f)) return 0;
  int ex;
  frexpf(maxabs, &ex);  // maxabs = f 2^ex, f in [1/2, 1)
  return ex + 1;
}

// Slice i of a scaled df value: h holds the remainder (hi's part, from slice 3
// on with lo joined), l the scaled lo.  Returns s_i and advances h.
__device__ __forceinline__ float next_slice(float& h, float l, int i) {
  if (i == 3) h = fmaf(l, 16777216.f, h);  // lo in units of slice 2's remainder (2^-24)
  const float s = rintf(h * 256.f);
  h = fmaf(h, 256.f, -s);  // exact: s is the integer nearest to 256 h
  return s;
}

// 32 slice values of this thread (row l.i of the real or imaginary part,
// columns c0..c0+31) into the expanded left operand: its own row and the
// partner row of [Pr -Pi; Pi Pr], 16-byte stores.
__device__ __forceinline__ void stage_A(uint8_t* a, const Lane& l, const float (&s)[32]) {
  const int r1 = l.im ? 64 + l.i : l.i;
  const int r2 = l.im ? l.i : 64 + l.i;
  const float sg = l.im ? -1.f : 1.f;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t w1[4], w2[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const __nv_bfloat162 p = __floats2bfloat162_rn(s[8 * q + 2 * e], s[8 * q + 2 * e + 1]);
      const __nv_bfloat162 m = __floats2bfloat162_rn(sg * s[8 * q + 2 * e], sg * s[8 * q + 2 * e + 1]);
      w1[e] = *reinterpret_cast<const uint32_t*>(&p);
      w2[e] = *reinterpret_cast<const uint32_t*>(&m);
    }
    *reinterpret_cast<uint4*>(a + sw128_k16(r1, l.c0 + 8 * q)) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
    *reinterpret_cast<uint4*>(a + sw128_k16(r2, 64 + l.c0 + 8 * q)) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
  }
}

// 32 slice values of this thread (k = l.L, n = c0..c0+31) into the right
// operand, MN-major.
__device__ __forceinline__ void stage_B(uint8_t* b, const Lane& l, const float (&s)[32]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const __nv_bfloat162 p = __floats2bfloat162_rn(s[8 * q + 2 * e], s[8 * q + 2 * e + 1]);
      w[e] = *reinterpret_cast<const uint32_t*>(&p);
    }
    *reinterpret_cast<uint4*>(b + tc::sw128_mn16(l.L, l.c0 + 8 * q)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Right-operand descriptor of two adjacent slices read as one N = 128
// operand: the second 64-wide swizzle atom along N is the next slice, kBSlice
// bytes on (the leading byte offset of an MN-major layout); 8-row groups along
// K at 1024 bytes.
__device__ __forceinline__ uint64_t make_desc_mn2(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(kBSlice >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
constexpr uint32_t kIdescBF16N128 =
    (1u << 4) | (1u << 7) | (1u << 10) | (1u << 16) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_bf16_n(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                           uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// One elected thread: the slice pairs (I, j) of left slice I (in shared
// memory at a) with every right slice j (at b + j kBSlice) whose level I + j
// is below LEVELS, into the level accumulators (64 TMEM columns each at
// acc + 64 level).  Adjacent right slices j, j + 1 go as one N = 128 MMA
// (its two halves land in the accumulators of levels I + j and I + j + 1):
// an M = 128 MMA takes 46-48 cycles at N = 64 and 64 at N = 128 (measured on
// GB300), so a pair costs 32 cycles instead of 48.  Slice 0's MMAs overwrite
// (at the first K step); every later one accumulates, so a level first
// reached after slice 0 (level 6, from slice 1 on) must be zeroed by the
// caller.  Straight-line code: the descriptors of the K steps are the base
// descriptors plus immediate offsets (a start address below 256 KB keeps the
// 14-bit address field from carrying).
template <int LEVELS, int I>
__device__ __forceinline__ void issue_slice_i(uint32_t acc, uint32_t a, uint32_t b) {
  constexpr int NJ = (LEVELS - I < kSlices) ? LEVELS - I : kSlices;  // right slices j = 0 .. NJ-1
  const uint64_t da0 = tc::make_desc(a);
#pragma unroll
  for (int j = 0; j < NJ; j += 2) {
    const bool two = j + 1 < NJ;
    const uint64_t db0 = two ? make_desc_mn2(b + (uint32_t)j * kBSlice) : tc::make_desc_mn(b + (uint32_t)j * kBSlice);
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const uint64_t da = da0 + (uint64_t)(((t >> 2) * 16384 + (t & 3) * 32) >> 4);
      const uint64_t db = db0 + (uint64_t)((2048u * t) >> 4);
      mma_bf16_n(acc + 64u * (uint32_t)(I + j), da, db, two ? kIdescBF16N128 : kIdescBF16,
                 (I != 0 || t != 0) ? 1u : 0u);
    }
  }
}
template <int LEVELS>
__device__ __forceinline__ void issue_slice(uint32_t acc, uint32_t a, uint32_t b, int i) {
  switch (i) {
    case 0: issue_slice_i<LEVELS, 0>(acc, a, b); break;
    case 1: issue_slice_i<LEVELS, 1>(acc, a, b); break;
    case 2: issue_slice_i<LEVELS, 2>(acc, a, b); break;
    case 3: issue_slice_i<LEVELS, 3>(acc, a, b); break;
    case 4: issue_slice_i<LEVELS, 4>(acc, a, b); break;
    default: issue_slice_i<LEVELS, 5>(acc, a, b); break;
  }
}

// Zeroes this thread's 32 columns (c0 ..) of the level-6 accumulator in its
// TMEM lane (levels beyond slice 0's reach start from zero).
__device__ __forceinline__ void zero_level6(uint32_t tmem, const Lane& l) {
  float z[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) z[c] = 0.f;
  tc::tmem_st32(tmem + l.lane_addr + (uint32_t)(64 * 6 + l.c0), z);
  tc::tmem_st_wait();
}

// Loads 8 consecutive columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

// Seven 8-column loads of this thread's TMEM lane (the seven level
// accumulators at 64-column steps from taddr) and one completion wait: one
// round trip instead of seven.
__device__ __forceinline__ void tmem_ld8x7(uint32_t taddr, float (&v)[7][8]) {
  uint32_t r[56];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%56];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8, %9, %10, %11, %12, %13, %14, %15}, [%57];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16, %17, %18, %19, %20, %21, %22, %23}, [%58];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%24, %25, %26, %27, %28, %29, %30, %31}, [%59];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%32, %33, %34, %35, %36, %37, %38, %39}, [%60];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%40, %41, %42, %43, %44, %45, %46, %47}, [%61];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%48, %49, %50, %51, %52, %53, %54, %55}, [%62];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55])
      : "r"(taddr), "r"(taddr + 64u), "r"(taddr + 128u), "r"(taddr + 192u), "r"(taddr + 256u), "r"(taddr + 320u),
        "r"(taddr + 384u)
      : "memory");
#pragma unroll
  for (int k = 0; k < 7; ++k)
#pragma unroll
    for (int j = 0; j < 8; ++j) v[k][j] = __uint_as_float(r[8 * k + j]);
}

// sum_l 2^(-8 l) L_l (levels exact FP32 integers) as df, smallest levels
// first: levels 4.. in FP32 (their rounding is below 2^-56 of level 0's
// scale), levels 3, 2, 1, 0 joined by error-free sums.  (Rounding level 3 in
// FP32 as well would cost 2^-24 of its size, ~2^-43 of the product.)
template <int LEVELS>
__device__ __forceinline__ void combine_levels(const float (&L)[LEVELS], float& hi, float& lo) {
  float t = 0.f;
#pragma unroll
  for (int lv = LEVELS - 1; lv >= 4; --lv) t = fmaf(L[lv], ldexpf(1.f, -8 * lv), t);
  float s, e;
  two_sum(L[3] * 0x1p-24f, t, s, lo);
  two_sum(L[2] * 0x1p-16f, s, s, e);
  lo += e;
  two_sum(L[1] * 0x1p-8f, s, s, e);
  lo += e;
  two_sum(L[0], s, s, e);
  lo += e;
  fast_two_sum(s, lo, hi, lo);
}

}  // namespace oz
}  // namespace pgx
