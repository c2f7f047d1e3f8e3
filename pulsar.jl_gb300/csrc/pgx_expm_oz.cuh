// The D = 64 df expm with every product on the tensor cores (the sliced bf16
// engine of pgx_oz.cuh, levels 0..6).
//
// The scheme is the CUDA-core kernel's: A_k = c dt_k (...) in df, the degree
// m = q L, block size q and squarings s from the FP32 1-norm and the df theta
// table, B = A / 2^s, the powers B^2 .. B^q, the Paterson-Stockmeyer Horner
// steps Y <- Y B^q + C_i (Y and B^q are polynomials in B and commute), then s
// squarings.  Every product is a full one (no triangular or half-column
// forms: the tensor-core product costs the same either way).
//
// One CTA per SM: 256 worker threads and one issuing warp.
//   - Worker (TMEM lane L, column half) owns entries (L mod 64, c0 .. c0+31)
//     of the real (L < 64) or imaginary part of every matrix: exactly the
//     values it stages into both operands of a sliced product and the values
//     it reads back from the accumulators.  So a product's result feeds the
//     next product from registers.
//   - The workers cut the left factor's six slices into two alternating
//     buffers; after each slice one worker arrives on the buffer's "full"
//     barrier with the slice index.  The issuing thread waits there, issues
//     the slice's pairs and commits them to the buffer's "empty" barrier,
//     which the workers wait on before they reuse the buffer.  The workers
//     never wait for the issue itself, so the Horner block of a step is
//     formed while its MMAs run.
//   - A prologue kernel assembles every unit's generator, takes its 1-norm
//     and degree, and leaves B = A / 2^s in the unit's U slot.
//   - The slab (the per-CTA global workspace of the CUDA-core kernel) keeps
//     B, B^2, B^3 as every worker's own values, thread-major, for the Horner
//     blocks C_i = sum_j c_{qi+j} B^j: each worker reads back only what it
//     wrote.
#pragma once
#include "pgx_oz.cuh"

namespace pgx {
namespace oz {

constexpr int kExpmLevels = 7;
constexpr int kWorkers = 256;
constexpr int kExpmThreads = kWorkers + 32;
constexpr uint32_t kCiBytes = kWorkers * 32u * 8u;  // 32 df values per worker
constexpr size_t kExpmSmem = (size_t)kSlices * kBSlice + 2 * kASlice + kCiBytes + tc::kSmemAlign;

// Barrier 1 of the 256 workers (the issuing warp never joins it).
__device__ __forceinline__ void wsync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
// The same, returning whether any worker's pred was true.
__device__ __forceinline__ bool wsync_or(bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred pi, po;\n\tsetp.ne.u32 pi, %1, 0;\n\t"
      "bar.red.or.pred po, 1, 256, pi;\n\tselp.u32 %0, 1, 0, po;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)pred)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

struct Engine {
  uint8_t* bsl;       // kSlices right-operand slices
  uint8_t* abuf;      // two left-operand slice buffers
  float2* ci;         // [32][256] the next Horner block, every worker's values {hi, lo}
  float* red;         // [2][8] block-maximum scratch, used alternately
  volatile int* cmd;  // [2] the slice index behind each "full" arrival (-1: stop)
  uint32_t tmem;
  uint32_t full[2], empty[2];
  uint32_t eph[2];  // parity of the next "empty" phase to wait for
  int pend[2];      // slices committed on each buffer and not yet waited for
  int par;
  int seq;  // slices handed to the issuer so far (their buffer alternates)
  bool abort;
};

// Exponent of the scale of a matrix given by every worker's 32 leading parts.
__device__ __forceinline__ int block_exp(Engine& g, const float (&h)[32]) {
  float mx = 0.f;
#pragma unroll
  for (int c = 0; c < 32; ++c) mx = fmaxf(mx, fabsf(h[c]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  float* r = g.red + 8 * g.par;  // alternate: a slow reader of the previous call is past a barrier
  g.par ^= 1;
  if ((threadIdx.x & 31) == 0) r[threadIdx.x >> 5] = mx;
  wsync();
  mx = 0.f;
#pragma unroll
  for (int w = 0; w < 8; ++w) mx = fmaxf(mx, r[w]);
  return scale_exp(mx);
}

// Stages the six right-operand slices of the matrix whose values this worker
// holds in (h, lo) (unchanged); returns its scale exponent.  No MMA may be
// reading the slices (every product waits for its MMAs before it returns).
__device__ __forceinline__ int stage_right(Engine& g, const Lane& l, const float (&h)[32], const float (&lo)[32]) {
  const int e = block_exp(g, h);
  const float sc = ldexpf(1.f, -e);
  float hh[32], ll[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    hh[c] = h[c] * sc;
    ll[c] = lo[c] * sc;
  }
#pragma unroll 1
  for (int j = 0; j < kSlices; ++j) {
    float s[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) s[c] = next_slice(hh[c], ll[c], j);
    stage_B(g.bsl + j * kBSlice, l, s);
  }
  return e;
}

// Waits for the MMAs still reading buffer b.  Returns false on timeout.
__device__ __forceinline__ bool drain(Engine& g, int b) {
  if (g.pend[b] == 0) return true;
  if (!tc::mbar_wait(g.empty[b], g.eph[b])) return false;
  g.eph[b] ^= 1;
  --g.pend[b];
  return true;
}

// Hands a command (a staged slice index, or -1 to stop) to the issuing warp
// on the next buffer.  Called by worker 0 after a workers' barrier.
__device__ __forceinline__ void hand_over(Engine& g, int cmd) {
  const int b = g.seq & 1;
  g.cmd[b] = cmd;
  mbar_arrive(g.full[b]);
}

// (h, lo) <- this worker's values of X R in df: X given by this worker's
// values (h, lo), R by the staged right-operand slices (exponent eR).
// `during()` runs while the MMAs execute; with `add` the Horner block parked
// in g.ci is added.  Returns false (g.abort set) when a wait gave up.
template <class During>
__device__ __forceinline__ bool product(Engine& g, const Lane& l, float (&h)[32], float (&lo)[32], int eR, bool add,
                                        During during) {
  const int eX = block_exp(g, h);
  {
    const float sc = ldexpf(1.f, -eX);
#pragma unroll
    for (int c = 0; c < 32; ++c) {
      h[c] *= sc;
      lo[c] *= sc;
    }
  }
  zero_level6(g.tmem, l);  // this worker read it in the previous product's combine
#pragma unroll 1
  for (int i = 0; i < kSlices; ++i) {
    const int b = g.seq & 1;
    const bool ok = drain(g, b);  // the pairs of slice i - 2 have read buffer b
    if (ok) {
      float s[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) s[c] = next_slice(h[c], lo[c], i);
      stage_A(g.abuf + b * kASlice, l, s);
      tc::fence_smem_to_async();
      tc::fence_before_sync();
    }
    if (wsync_or(!ok)) {
      g.abort = true;
      return false;
    }
    if (threadIdx.x == 0) hand_over(g, i);
    ++g.pend[b];
    ++g.seq;
  }
  during();
  const bool ok = drain(g, 0) & drain(g, 1);
  if (wsync_or(!ok)) {
    g.abort = true;
    return false;
  }
  tc::fence_after_sync();
  const float sc = ldexpf(1.f, eX + eR - 16);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float Lv[kExpmLevels][8];
    static_assert(kExpmLevels == 7, "one load batch per level set");
    tmem_ld8x7(g.tmem + l.lane_addr + (uint32_t)(l.c0 + 8 * q), Lv);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      float L[kExpmLevels];
#pragma unroll
      for (int lv = 0; lv < kExpmLevels; ++lv) L[lv] = Lv[lv][c];
      float hi, lw;
      combine_levels<kExpmLevels>(L, hi, lw);
      df v{hi * sc, lw * sc};
      if (add) {
        const float2 a = g.ci[(8 * q + c) * kWorkers + threadIdx.x];
        v = df_add(v, df{a.x, a.y});
      }
      h[8 * q + c] = v.hi;
      lo[8 * q + c] = v.lo;
    }
  }
  tc::fence_before_sync();  // accumulators read before the next product's MMAs
  return true;
}

// The issuing thread: waits for each staged slice in turn, issues its pairs
// and commits them to the buffer's "empty" barrier, until a stop command.
// Every wait is bounded; a timeout stops it (the workers' own bounded waits
// then fail too).
__device__ __forceinline__ void issue_loop(Engine& g) {
  uint32_t fph[2] = {0, 0};
  for (int n = 0;; ++n) {
    const int b = n & 1;
    if (!tc::mbar_wait(g.full[b], fph[b])) return;
    fph[b] ^= 1;
    const int cmd = g.cmd[b];
    if (cmd < 0) return;
    tc::fence_after_sync();
    issue_slice<kExpmLevels>(g.tmem, tc::smem_u32(g.abuf + b * kASlice), tc::smem_u32(g.bsl), cmd);
    tc::commit(g.empty[b]);
  }
}

// This worker's part of the Horner block C_i = sum_{j<q} c_{qi+j} B^j at two
// of its entries (columns c0 + 2 cp, + 1; B^0 = I), from the own-value copies
// of B, B^2, B^3 (float4 {hi, lo, hi, lo} per entry pair): v0, v1.
__device__ __forceinline__ void block_pair(int i, int q, int row, int c0, bool real, const float4* own, int cp,
                                           const df* coef, df& v0, df& v1) {
  const int o = q * i;
  const float4 b1 = __ldcg(own + cp * kWorkers + threadIdx.x);
  const float4 b2 = q >= 3 ? __ldcg(own + (16 + cp) * kWorkers + threadIdx.x) : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 b3 = q >= 4 ? __ldcg(own + (32 + cp) * kWorkers + threadIdx.x) : make_float4(0.f, 0.f, 0.f, 0.f);
  v0 = df_mul(df{b1.x, b1.y}, coef[o + 1]);
  v1 = df_mul(df{b1.z, b1.w}, coef[o + 1]);
  if (q >= 3) {
    v0 = df_add(v0, df_mul(df{b2.x, b2.y}, coef[o + 2]));
    v1 = df_add(v1, df_mul(df{b2.z, b2.w}, coef[o + 2]));
  }
  if (q >= 4) {
    v0 = df_add(v0, df_mul(df{b3.x, b3.y}, coef[o + 3]));
    v1 = df_add(v1, df_mul(df{b3.z, b3.w}, coef[o + 3]));
  }
  if (real && row == c0 + 2 * cp) v0 = df_add(v0, coef[o]);
  if (real && row == c0 + 2 * cp + 1) v1 = df_add(v1, coef[o]);
}

// Writes this worker's values as matrix `mat` (0: B, 1: B^2, 2: B^3) of the
// own-value copies: thread-major float4 {hi, lo, hi, lo} per entry pair, so a
// warp's loads are 512 contiguous bytes.
__device__ __forceinline__ void store_own(float4* own, int mat, const float (&h)[32], const float (&lo)[32]) {
#pragma unroll
  for (int cp = 0; cp < 16; ++cp)
    own[(16 * mat + cp) * kWorkers + threadIdx.x] = make_float4(h[2 * cp], lo[2 * cp], h[2 * cp + 1], lo[2 * cp + 1]);
}

// Shared-memory carve-up, TMEM, barriers and the engine state of a CTA of the
// sliced engine's kernels (kExpmThreads threads, kExpmSmem dynamic bytes).
struct CtaStatic {
  uint32_t tmem;
  uint64_t bar[5];  // full[2], empty[2], and the chain kernels' operand copies
  float red[16];
  int cmd[2];
};
__device__ __forceinline__ void engine_setup(Engine& g, uint8_t* smem_raw, CtaStatic& st) {
  const uint32_t pad = (tc::kSmemAlign - (tc::smem_u32(smem_raw) & (tc::kSmemAlign - 1))) & (tc::kSmemAlign - 1);
  g.bsl = smem_raw + pad;
  g.abuf = g.bsl + kSlices * kBSlice;
  g.ci = reinterpret_cast<float2*>(g.abuf + 2 * kASlice);
  g.red = st.red;
  g.cmd = st.cmd;
  g.par = 0;
  g.seq = 0;
  g.abort = false;
  g.eph[0] = g.eph[1] = 0;
  g.pend[0] = g.pend[1] = 0;
  for (int b = 0; b < 2; ++b) {
    g.full[b] = tc::smem_u32(&st.bar[b]);
    g.empty[b] = tc::smem_u32(&st.bar[2 + b]);
  }
  if (threadIdx.x < 32) tc::tmem_alloc(&st.tmem, tc::kTmemCols);
  if (threadIdx.x == 0)
    for (int b = 0; b < 5; ++b) tc::mbar_init(tc::smem_u32(&st.bar[b]));
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  g.tmem = st.tmem;
}

// The chain kernels' next left factor (one 64 KB df matrix, contiguous in
// HBM) into g.ci by two bulk copies (TMA) on barrier `mbar`; issued by worker
// 0 once every worker has read the previous one.
__device__ __forceinline__ void fetch_left(Engine& g, uint32_t mbar, const float4* src) {
  tc::mbar_expect_tx(mbar, 65536u);
  tc::tma_bulk_copy(tc::smem_u32(g.ci), src, 32768u, mbar);
  tc::tma_bulk_copy(tc::smem_u32(g.ci) + 32768u, reinterpret_cast<const uint8_t*>(src) + 32768, 32768u, mbar);
}
// This worker's values of the fetched matrix (after waiting for the copy).
__device__ __forceinline__ void read_left(const Engine& g, const Lane& l, float (&h)[32], float (&lo)[32]) {
  const float4* M = reinterpret_cast<const float4*>(g.ci);
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    const float4 v = M[l.i + 64 * (l.c0 + c)];
    h[c] = l.im ? v.y : v.x;
    lo[c] = l.im ? v.w : v.z;
  }
}
// Workers: stop the issuer, then (bounded) let the groups in flight finish.
__device__ __forceinline__ void workers_finish(Engine& g) {
  wsync();
  if (threadIdx.x == 0) hand_over(g, -1);
  drain(g, 0);
  drain(g, 1);
}
// Every thread: frees TMEM once workers and issuer are done.
__device__ __forceinline__ void engine_teardown(Engine& g) {
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(g.tmem, tc::kTmemCols);
  }
}

}  // namespace oz

// Flag of the tensor-core expm: a completion wait gave up (its units are
// NaN-poisoned).
__device__ int g_expm_tc_timeout;

// Prologue of the tensor-core expm, per unit (member, slice): the generator
// A_k in df (the CUDA-core kernel's assembly), its FP32 1-norm and the
// degree, block size and squarings (the CUDA-core kernel's choice, without
// the triangular costs), then B = A_k / 2^s as planar df {hi, lo} (real part,
// then imaginary part, column-major) in the unit's U slot, which the expm
// overwrites with exp(A_k) at the end.  Memory-bound work at full occupancy,
// kept out of the one-CTA-per-SM tensor-core kernel.
// FP32 1-norm of the prologue's 64 x 64 df matrix by all 256 threads (x
// 1.00001, as norm1f): thread t sums rows 16 (t % 4) .. + 15 of column t / 4,
// the four partial sums of a column meet by two xor shuffles (every lane of
// the four ends with the same sum), and the largest column comes from warp
// and block maxima.  red: 8 floats.
__device__ __forceinline__ float prep_norm1_64(const float4* A, float* red) {
  using L = Lay<64, kSwzExpm>;
  const int t = threadIdx.x, c = t >> 2, r0 = (t & 3) * 16;
  float s = 0.f;
#pragma unroll 4
  for (int r = r0; r < r0 + 16; ++r) {
    const float4 a = A[L::idx(r, c)];
    s += sqrtf(fmaf(a.x, a.x, a.y * a.y));
  }
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, o));
  if ((t & 31) == 0) red[t >> 5] = s;
  __syncthreads();
  float best = red[0];
#pragma unroll
  for (int i = 1; i < 8; ++i) best = fmaxf(best, red[i]);
  __syncthreads();  // red is the degree choice's scratch next
  return best * 1.00001f;
}

__global__ void __launch_bounds__(256) k_expm_prep_oz64(ProbDev p, WorkDev w) {
  using L = Lay<64, kSwzExpm>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* A = reinterpret_cast<float4*>(smem_raw);
  float* red = reinterpret_cast<float*>(A + L::SIZE);
  const Team<256> tm{(int)threadIdx.x};
  const long items = (long)p.n_members * p.n_t;
  for (long it = blockIdx.x; it < items; it += gridDim.x) {
    const int m = (int)(it / p.n_t), k = (int)(it % p.n_t);
    build_A_df<64, 256, kSwzExpm>(tm, p, w, m, k, A);
    tm.sync();
    const float nrm = prep_norm1_64(A, red);
    const int pk = choose_expm_df<256>(tm, nrm, 64, false, reinterpret_cast<int*>(red));
    const float sc = ldexpf(1.f, -((pk >> 8) & 63));
    float2* out = reinterpret_cast<float2*>(w.U) + (size_t)it * 8192;
    for (int e = tm.lane; e < 4096; e += 256) {
      const float4 v = A[L::idx(e % 64, e / 64)];
      __stcs(out + e, make_float2(v.x * sc, v.z * sc));  // read once, by the expm
      __stcs(out + 4096 + e, make_float2(v.y * sc, v.w * sc));
    }
    if (tm.lane == 0) w.expm_plan[it] = pk;
    tm.sync();  // A is rebuilt by the next unit
  }
}
constexpr size_t kExpmPrepSmem = (size_t)Lay<64, kSwzExpm>::SIZE * sizeof(float4) + 256;

// 288 threads: an SM sub-partition hosts three of the nine warps, so at most
// 168 registers per thread.
__global__ void __launch_bounds__(oz::kExpmThreads, 1) k_expm_oz64(ProbDev p, WorkDev w) {
  using namespace oz;
  extern __shared__ uint8_t smem_raw[];
  __shared__ CtaStatic st;
  Engine g;
  engine_setup(g, smem_raw, st);
  if (threadIdx.x >= kWorkers) {  // the issuing warp
    if (threadIdx.x == kWorkers) issue_loop(g);
    __syncwarp();
  } else {
    const Lane l = tc::lane_of();
    float4* own = reinterpret_cast<float4*>(w.slab) + (size_t)blockIdx.x * 3 * 16 * kWorkers;  // B, B^2, B^3
    const auto nop = [] {};
    const long items = (long)p.n_members * p.n_t;
    long it = blockIdx.x;
    for (; it < items; it += gridDim.x) {
      const int m = (int)(it / p.n_t), k = (int)(it % p.n_t);
      const int pk = w.expm_plan[it];
      const int deg = pk & 31, q = (pk >> 5) & 7, s = (pk >> 8) & 63, nL = deg / q;
      // x: the values this worker holds of the matrix in hand, first B (the
      // prologue's planar copy in the U slot)
      float xh[32], xl[32];
      {
        const float2* Bp = reinterpret_cast<const float2*>(w.U) + (size_t)it * 8192 + l.im * 4096 + l.i;
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          const float2 v = __ldcs(Bp + 64 * (l.c0 + c));
          xh[c] = v.x;
          xl[c] = v.y;
        }
        store_own(own, 0, xh, xl);
      }
      // The products of the unit, at one call site (one copy of the
      // product's code), in place on x:
      //   powers:  B^2 = B B (st 0), B^3 = B^2 B (st 1), B^4 = B^2 B^2 (st 2);
      //   then x = B^q becomes the right factor and Y = C_{L-1} + c_m B^q
      //   (C_{L-1} parked during the last power product);
      //   Horner:  Y <- Y B^q + C_i, i = L-2 .. 0;
      //   squarings: Y <- Y Y.
      const int n_pow = q - 1, n_hor = nL - 1, n_steps = n_pow + n_hor + s;
      int eR = 0;
      bool ok = true;
#pragma unroll 1
      for (int st = 0; st <= n_steps && ok; ++st) {
        if (st == 1 && q >= 3) store_own(own, 1, xh, xl);
        if (st == 2 && q == 4) {  // B^4 = B^2 B^2
          store_own(own, 2, xh, xl);
#pragma unroll
          for (int cp = 0; cp < 16; ++cp) {
            const float4 v = own[(16 + cp) * kWorkers + threadIdx.x];
            xh[2 * cp] = v.x;
            xl[2 * cp] = v.y;
            xh[2 * cp + 1] = v.z;
            xl[2 * cp + 1] = v.w;
          }
          eR = stage_right(g, l, xh, xl);
        }
        if (st == n_pow) {  // x = B^q
          if (q == 2) store_own(own, 1, xh, xl);
          if (q == 3) store_own(own, 2, xh, xl);
          eR = stage_right(g, l, xh, xl);
#pragma unroll
          for (int c = 0; c < 32; ++c) {  // C_{L-1} was parked during the last power product
            const float2 a = g.ci[c * kWorkers + threadIdx.x];
            const df v = df_add(df{a.x, a.y}, df_mul(df{xh[c], xl[c]}, c_dfcoef[deg]));
            xh[c] = v.hi;
            xl[c] = v.lo;
          }
        }
        if (st == n_steps) break;
        if (st == 0 || st >= n_pow + n_hor) eR = stage_right(g, l, xh, xl);  // B; or a squaring's Y
        // the last power product parks C_{L-1} (B^1 .. B^{q-1} are known), each
        // Horner step the next block
        if ((st >= n_pow && st < n_pow + n_hor) || st == n_pow - 1) {
          const int i = st == n_pow - 1 ? nL - 1 : n_pow + n_hor - 1 - st;
          const auto park = [&] {  // C_i into shared memory while the MMAs run
#pragma unroll 4
            for (int cp = 0; cp < 16; ++cp) {
              df v0, v1;
              block_pair(i, q, l.i, l.c0, l.im == 0, own, cp, c_dfcoef, v0, v1);
              g.ci[(2 * cp) * kWorkers + threadIdx.x] = make_float2(v0.hi, v0.lo);
              g.ci[(2 * cp + 1) * kWorkers + threadIdx.x] = make_float2(v1.hi, v1.lo);
            }
          };
          ok = product(g, l, xh, xl, eR, st != n_pow - 1, park);
        } else {
          ok = product(g, l, xh, xl, eR, false, nop);
        }
      }
      if (!ok) break;
      // U: the stack streams out (gigabytes, read back from DRAM by the chains)
      float* out = reinterpret_cast<float*>(w.U) + ((size_t)m * p.n_t + k) * 64 * 64 * 4;
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const size_t e = (size_t)(l.i + 64 * (l.c0 + c)) * 4;
        __stcs(out + e + l.im, xh[c]);
        __stcs(out + e + 2 + l.im, xl[c]);
      }
    }
    if (g.abort) {
      // units from the one that failed on: NaN, so no stale propagator is used
      const float nan = __int_as_float(0x7fffffff);
      for (; it < items; it += gridDim.x) {
        float* out = reinterpret_cast<float*>(w.U) + (size_t)it * 64 * 64 * 4;
        for (int e = threadIdx.x; e < 64 * 64 * 4; e += kWorkers) out[e] = nan;
      }
      if (threadIdx.x == 0) atomicOr(&g_expm_tc_timeout, 1);
    }
    workers_finish(g);
  }
  engine_teardown(g);
}

// The parallel-in-time forward chain's in-block prefix products at D = 64 on
// the same engine: per (member m, block b of slices k0 .. k1-1) P_k0 = I,
// P_{k+1} = U_k P_k in df; with `store` the FP32 rounding of every P_k
// (k0 <= k < k1) for the gradient; the block product P_k1 into pit_tot.
// P_{k0+1} = U_k0 is taken as is.  Each step stages P_k as the right factor
// and multiplies U_k (left, this worker's values) into it; U_{k+1} arrives in
// shared memory by TMA bulk copies while the step's MMAs run.  Same CTA shape, barriers and
// bounded waits as k_expm_oz64; a CTA that gives up NaN-poisons the block
// products of its remaining items.
__global__ void __launch_bounds__(oz::kExpmThreads, 1) k_chainf_local_oz64(ProbDev p, WorkDev w, int store) {
  using namespace oz;
  extern __shared__ uint8_t smem_raw[];
  __shared__ CtaStatic st;
  Engine g;
  engine_setup(g, smem_raw, st);  // g.ci receives U_{k+1}
  if (threadIdx.x >= kWorkers) {
    if (threadIdx.x == kWorkers) issue_loop(g);
    __syncwarp();
  } else {
    const Lane l = tc::lane_of();
    const long items = (long)p.n_members * w.pit_blocks;
    const uint32_t tbar = tc::smem_u32(&st.bar[4]);
    uint32_t tph = 0;
    int tpend = 0;  // operand copies issued and not yet waited for
    // this worker's entries e = i + 64 c of a 4096-entry matrix
    const auto entry = [&](int c) { return (size_t)(l.i + 64 * (l.c0 + c)); };
    long it = blockIdx.x;
    for (; it < items; it += gridDim.x) {
      const int m = (int)(it / w.pit_blocks), b = (int)(it % w.pit_blocks);
      const int k0 = b * w.pit_len, k1 = min(p.n_t, k0 + w.pit_len);
      const float4* Um = reinterpret_cast<const float4*>(w.U) + (size_t)m * p.n_t * 4096;
      float* Pst = reinterpret_cast<float*>(w.P) + (size_t)m * p.n_t * 4096 * 2;  // float2 {re, im} per entry
      float xh[32], xl[32], uh[32], ul[32];
      if (store) {  // P_k0 = I
#pragma unroll
        for (int c = 0; c < 32; ++c)
          Pst[((size_t)k0 * 4096 + entry(c)) * 2 + l.im] = (l.im == 0 && l.i == l.c0 + c) ? 1.f : 0.f;
      }
#pragma unroll
      for (int c = 0; c < 32; ++c) {  // x = P_{k0+1} = U_k0
        const float4 v = Um[(size_t)k0 * 4096 + entry(c)];
        xh[c] = l.im ? v.y : v.x;
        xl[c] = l.im ? v.w : v.z;
      }
      bool ok = true;
      if (k0 + 1 < k1) {  // U_{k0+1} by TMA
        if (threadIdx.x == 0) fetch_left(g, tbar, Um + (size_t)(k0 + 1) * 4096);
        ++tpend;
      }
#pragma unroll 1
      for (int k = k0 + 1; k <= k1 && ok; ++k) {  // x holds P_k
        if (store && k < k1)
#pragma unroll
          for (int c = 0; c < 32; ++c) Pst[((size_t)k * 4096 + entry(c)) * 2 + l.im] = xh[c];
        if (k == k1) break;
        const int eR = stage_right(g, l, xh, xl);  // P_k
        const bool got = tc::mbar_wait(tbar, tph);  // U_k in shared memory
        if (wsync_or(!got)) {
          g.abort = true;
          ok = false;
          break;
        }
        tph ^= 1;
        --tpend;
        read_left(g, l, uh, ul);
        const auto prefetch = [&] {  // U_{k+1} while the MMAs run: every worker has read U_k
          if (k + 1 < k1) {
            if (threadIdx.x == 0) fetch_left(g, tbar, Um + (size_t)(k + 1) * 4096);
            ++tpend;
          }
        };
        ok = product(g, l, uh, ul, eR, false, prefetch);  // U_k P_k
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          xh[c] = uh[c];
          xl[c] = ul[c];
        }
      }
      if (!ok) break;
      float* tot = reinterpret_cast<float*>(w.pit_tot + ((size_t)m * w.pit_blocks + b) * 4096);
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        tot[entry(c) * 4 + l.im] = xh[c];
        tot[entry(c) * 4 + 2 + l.im] = xl[c];
      }
    }
    if (g.abort) {
      const float nan = __int_as_float(0x7fffffff);
      for (; it < items; it += gridDim.x) {
        float* tot = reinterpret_cast<float*>(w.pit_tot + (size_t)it * 4096);
        for (int e = threadIdx.x; e < 4096 * 4; e += kWorkers) tot[e] = nan;
      }
      if (threadIdx.x == 0) atomicOr(&g_expm_tc_timeout, 1);
      if (tpend > 0) tc::mbar_wait(tbar, tph);  // bounded: the copy in flight lands before the CTA ends
    }
    workers_finish(g);
  }
  engine_teardown(g);
}

// The parallel-in-time forward chain's combine at D = 64 on the same engine:
// per member P = I, then for each block b in order pit_pre[b] = P (FP32, when
// `store`) and P <- T_b P in df (T_0 I = T_0 as is; T_{b+1} arrives by TMA
// bulk copies while step b's MMAs run); then the CUDA-core
// kernel's epilogue (U_total in FP64, the overlap, f and the chain-rule
// coefficient) on P copied into shared memory.  A CTA that gives up
// NaN-poisons the objective of its remaining members.
__global__ void __launch_bounds__(oz::kExpmThreads, 1) k_chainf_combine_oz64(ProbDev p, WorkDev w, int store) {
  using namespace oz;
  extern __shared__ uint8_t smem_raw[];
  __shared__ CtaStatic st;
  Engine g;
  engine_setup(g, smem_raw, st);
  if (threadIdx.x >= kWorkers) {
    if (threadIdx.x == kWorkers) issue_loop(g);
    __syncwarp();
  } else {
    const Lane l = tc::lane_of();
    const Team<256> tm{(int)threadIdx.x, 1};           // the workers' barrier
    float4* Pc = reinterpret_cast<float4*>(g.ci);       // 64 KB: P for the epilogue
    double2* red = reinterpret_cast<double2*>(g.abuf);  // the epilogue's scratch (idle slice buffers)
    const auto entry = [&](int c) { return (size_t)(l.i + 64 * (l.c0 + c)); };
    const uint32_t tbar = tc::smem_u32(&st.bar[4]);
    uint32_t tph = 0;
    int tpend = 0;  // operand copies issued and not yet waited for
    int m = blockIdx.x;
    for (; m < p.n_members; m += gridDim.x) {
      float xh[32], xl[32], uh[32], ul[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) {  // P = I
        xh[c] = (l.im == 0 && l.i == l.c0 + c) ? 1.f : 0.f;
        xl[c] = 0.f;
      }
      bool ok = true;
      const float4* Tm = w.pit_tot + (size_t)m * w.pit_blocks * 4096;
      if (store) {  // pit_pre[0] = I
        float* pre = reinterpret_cast<float*>(w.pit_pre + (size_t)m * w.pit_blocks * 4096);
#pragma unroll
        for (int c = 0; c < 32; ++c) pre[entry(c) * 2 + l.im] = xh[c];
      }
#pragma unroll
      for (int c = 0; c < 32; ++c) {  // P = T_0 I = T_0
        const float4 v = Tm[entry(c)];
        xh[c] = l.im ? v.y : v.x;
        xl[c] = l.im ? v.w : v.z;
      }
      if (w.pit_blocks > 1) {  // T_1 by TMA
        if (threadIdx.x == 0) fetch_left(g, tbar, Tm + 4096);
        ++tpend;
      }
#pragma unroll 1
      for (int b = 1; b < w.pit_blocks && ok; ++b) {
        if (store) {
          float* pre = reinterpret_cast<float*>(w.pit_pre + ((size_t)m * w.pit_blocks + b) * 4096);
#pragma unroll
          for (int c = 0; c < 32; ++c) pre[entry(c) * 2 + l.im] = xh[c];
        }
        const int eR = stage_right(g, l, xh, xl);  // P
        const bool got = tc::mbar_wait(tbar, tph);  // T_b in shared memory
        if (wsync_or(!got)) {
          g.abort = true;
          ok = false;
          break;
        }
        tph ^= 1;
        --tpend;
        read_left(g, l, uh, ul);
        const auto prefetch = [&] {  // T_{b+1} while the MMAs run: every worker has read T_b
          if (b + 1 < w.pit_blocks) {
            if (threadIdx.x == 0) fetch_left(g, tbar, Tm + (size_t)(b + 1) * 4096);
            ++tpend;
          }
        };
        ok = product(g, l, uh, ul, eR, false, prefetch);  // T_b P
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          xh[c] = uh[c];
          xl[c] = ul[c];
        }
      }
      if (!ok) break;
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        float* f = reinterpret_cast<float*>(Pc + entry(c));
        f[l.im] = xh[c];
        f[2 + l.im] = xl[c];
      }
      wsync();
      chain_epilogue_mx<64, 256>(tm, p, w, m, Pc, red);
      tc::fence_smem_to_async();  // these writes to g.ci before the next member's copies into it
      wsync();  // P and the scratch are read before the next member reuses them
    }
    if (g.abort && threadIdx.x == 0) {
      for (; m < p.n_members; m += gridDim.x) w.Fm[m] = __longlong_as_double(0x7ff8000000000000LL);
      atomicOr(&g_expm_tc_timeout, 1);
    }
    if (g.abort && tpend > 0) tc::mbar_wait(tbar, tph);  // bounded: the copy in flight lands first
    workers_finish(g);
  }
  engine_teardown(g);
}

}  // namespace pgx
