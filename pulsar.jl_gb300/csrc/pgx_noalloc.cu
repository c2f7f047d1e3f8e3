// pgx_total_propagator_noalloc: the total-propagator computation for callers
// that may not allocate device memory.
//
// Some hosts cannot call cudaMalloc at the point where they need a propagator:
// real-time control loops that forbid allocation once they have started, and
// plugin hosts whose device memory all belongs to their own pool allocator (a
// cudaMalloc there fails or takes memory the host has promised elsewhere).
// For them this entry point keeps all of its working memory -- the stack of
// slice propagators and, for 64 x 64 generators, the Taylor workspace -- in
// one file-scope device array of fixed size.  The caller passes the
// generators, the slice durations and the output in device memory it already
// owns.
//
// Set-up: the first call on a device (with that device current) resolves the
// array's device address with cudaGetSymbolAddress, sets the kernels'
// shared-memory limits and queries every kernel instantiation, so that under
// lazy module loading all of them are loaded then rather than at a later
// first launch; make that first call before any stream capture.  Every GPU
// that loads the library holds the array until the process exits.  All calls
// share the array: calls whose GPU work overlaps (other streams, other
// threads) race on it and must be serialised by the caller.  Each call writes
// every scratch element it reads before reading it, so stale contents from an
// earlier call never reach a result and nothing needs clearing.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "pgx.h"
#include "pgx_device.cuh"

namespace pgx_noalloc {

using namespace pgx;

constexpr size_t kScratchBytes = PGX_NOALLOC_SCRATCH_BYTES;
constexpr int kSlabTeams64 = 8;  // concurrent 64 x 64 Taylor workspaces

// The scratch.  In host code this name is only a stand-in for the device
// array: host code must use the address from cudaGetSymbolAddress.
static __device__ __align__(256) double2 g_scratch[kScratchBytes / sizeof(double2)];

__constant__ double c_invf_na[PGX_N_INVFACT] = PGX_INVFACT_INIT;
__constant__ double c_theta_na[PGX_N_DEGREES] = PGX_THETA64_INIT;

template <int D> struct NaCfg {
  static constexpr int T = (D <= 8) ? 32 : 256;
  static constexpr int TPC = (D <= 8) ? 4 : 1;
  static constexpr bool SLAB = (D >= 64);
  static constexpr int THREADS = T * TPC;
  static constexpr size_t SMEM = (SLAB ? 0 : (size_t)TPC * 10 * D * D * sizeof(double2)) +
                                 (size_t)TPC * T * sizeof(double2);
};

// U_k = exp(c dt_k G_k) for k < n, generators read unpadded (dim x dim) and
// zero-padded to D on the fly; U stack and (D = 64) workspace in scratch.
template <int D>
__global__ void __launch_bounds__(NaCfg<D>::THREADS)
k_na_expm(int gen, int dim, int n, const double2* __restrict__ G, const double* __restrict__ dt,
          double2* Ustack, double2* slab) {
  using Cf = NaCfg<D>;
  constexpr int T = Cf::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int team = threadIdx.x / T;
  const Team<T> tm{(int)(threadIdx.x % T)};
  double2 *base, *red;
  if constexpr (Cf::SLAB) {
    base = slab + (size_t)blockIdx.x * 10 * D * D;
    red = smem + (size_t)team * T;
  } else {
    base = smem + (size_t)team * 10 * D * D;
    red = smem + (size_t)Cf::TPC * 10 * D * D + (size_t)team * T;
  }
  const Work<double2, D> W = Work<double2, D>::at(base);
  for (long it = (long)blockIdx.x * Cf::TPC + team; it < n; it += (long)gridDim.x * Cf::TPC) {
    const int k = (int)it;
    const double h = dt[k];
    const double2* Gk = G + (size_t)k * dim * dim;
    for (int e = tm.lane; e < D * D; e += T) {
      const int r = e % D, c = e / D;
      double2 v = make_double2(0.0, 0.0);
      if (r < dim && c < dim) v = Gk[r + (size_t)dim * c];
      v.x *= h;
      v.y *= h;
      W.B[e] = gen == PGX_GEN_HERMITIAN ? make_double2(v.y, -v.x) : v;  // c = -i or 1
    }
    tm.sync();
    const double nrm = norm1<D, T>(tm, W.B, reinterpret_cast<double*>(red));
    int deg, s;
    choose_degree(nrm, c_theta_na, deg, s);
    const double sc = ldexp(1.0, -s);
    for (int e = tm.lane; e < D * D; e += T) W.B[e] = cscale(W.B[e], sc);
    tm.sync();
    taylor_exp<D, T>(tm, W, deg, s, c_invf_na);
    double2* out = Ustack + (size_t)k * D * D;
    for (int e = tm.lane; e < D * D; e += T) out[e] = W.Y[e];
    tm.sync();
  }
}

// U_total = U_{n-1} ... U_0 by one team; written unpadded.
template <int D>
__global__ void __launch_bounds__(NaCfg<D>::THREADS)
k_na_chain(int dim, int n, const double2* Ustack, double2* Utot) {
  using Cf = NaCfg<D>;
  constexpr int T = Cf::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  if (threadIdx.x >= T) return;  // one team
  const Team<T> tm{(int)threadIdx.x};
  double2* P = smem;
  double2* Ub = smem + D * D;
  for (int e = tm.lane; e < D * D; e += T) P[e] = make_double2((e % D) == (e / D) ? 1.0 : 0.0, 0.0);
  tm.sync();
  for (int k = 0; k < n; ++k) {
    for (int e = tm.lane; e < D * D; e += T) Ub[e] = Ustack[(size_t)k * D * D + e];
    tm.sync();
    mm1<D, T>(tm, P, Ub, P);
  }
  for (int e = tm.lane; e < D * D; e += T) {
    const int r = e % D, c = e / D;
    if (r < dim && c < dim) Utot[r + (size_t)dim * c] = P[e];
  }
}

struct DeviceSetup {
  bool done = false;
  double2* scratch = nullptr;
};
static std::mutex g_mu;
static DeviceSetup g_setup[64];

template <int D>
constexpr size_t chain_smem() { return 2 * (size_t)D * D * sizeof(double2); }

// Sets the shared-memory limit of the instantiations that need more than the
// default 48 KB and queries the attributes of both kernels of dimension D,
// which loads their code now (lazy module loading would otherwise load it at
// the first launch).  Return codes are checked directly, so an error the
// caller left pending is neither taken for this call's nor cleared.
template <int D>
static cudaError_t prepare_kernels() {
  cudaFuncAttributes attr;
  cudaError_t e = cudaFuncGetAttributes(&attr, k_na_expm<D>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, k_na_chain<D>);
  if (e == cudaSuccess && NaCfg<D>::SMEM > 48 * 1024)
    e = cudaFuncSetAttribute(k_na_expm<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)NaCfg<D>::SMEM);
  if (e == cudaSuccess && chain_smem<D>() > 48 * 1024)
    e = cudaFuncSetAttribute(k_na_chain<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chain_smem<D>());
  return e;
}

static cudaError_t setup_current_device(double2** scratch) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_setup[dev].done) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e == cudaSuccess) e = prepare_kernels<2>();
    if (e == cudaSuccess) e = prepare_kernels<4>();
    if (e == cudaSuccess) e = prepare_kernels<8>();
    if (e == cudaSuccess) e = prepare_kernels<16>();
    if (e == cudaSuccess) e = prepare_kernels<32>();
    if (e == cudaSuccess) e = prepare_kernels<64>();
    if (e != cudaSuccess) return e;
    g_setup[dev].scratch = static_cast<double2*>(p);
    g_setup[dev].done = true;
  }
  *scratch = g_setup[dev].scratch;
  return cudaSuccess;
}

template <int D>
static cudaError_t run(int gen, int dim, int n, const double2* G, const double* dt, double2* Utot,
                       double2* scratch, cudaStream_t st) {
  using Cf = NaCfg<D>;
  double2* Ustack = scratch;
  double2* slab = scratch + (size_t)n * D * D;
  int grid = (n + Cf::TPC - 1) / Cf::TPC;
  if (Cf::SLAB && grid > kSlabTeams64) grid = kSlabTeams64;
  if (grid > 4096) grid = 4096;
  // A launch-configuration error is reported by cudaPeekAtLastError without
  // clearing it; the arguments here are validated, so any error seen is a
  // real failure of this call (or one the caller left pending and still owns).
  k_na_expm<D><<<grid, Cf::THREADS, Cf::SMEM, st>>>(gen, dim, n, G, dt, Ustack, slab);
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) return e;
  k_na_chain<D><<<1, Cf::THREADS, chain_smem<D>(), st>>>(dim, n, Ustack, Utot);
  return cudaPeekAtLastError();
}

size_t scratch_needed(int Dp, int n) {
  return ((size_t)n * Dp * Dp + (Dp >= 64 ? (size_t)kSlabTeams64 * 10 * Dp * Dp : 0)) * sizeof(double2);
}

}  // namespace pgx_noalloc

static int na_fail(char* err, size_t len, int status, const char* msg) {
  if (err && len) std::snprintf(err, len, "%s", msg);
  return status;
}

extern "C" int pgx_total_propagator_noalloc(int32_t dim, int32_t generator, int32_t n_slices,
                                            const double* d_gens, const double* d_dt,
                                            double* d_U_total, void* stream, char* err, size_t err_len) {
  using namespace pgx_noalloc;
  if (err && err_len) err[0] = '\0';
  if (dim < 1 || dim > 64) return na_fail(err, err_len, PGX_ERR_DIMS, "dim must be in [1, 64]");
  if (n_slices < 1) return na_fail(err, err_len, PGX_ERR_DIMS, "n_slices must be >= 1");
  if (generator != PGX_GEN_HERMITIAN && generator != PGX_GEN_LIOUVILLIAN)
    return na_fail(err, err_len, PGX_ERR_INVALID, "unknown generator kind");
  if (!d_gens || !d_dt || !d_U_total)
    return na_fail(err, err_len, PGX_ERR_INVALID, "d_gens, d_dt and d_U_total are required");
  int Dp = 2;
  while (Dp < dim) Dp *= 2;
  if (scratch_needed(Dp, n_slices) > kScratchBytes) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "n_slices=%d with dim=%d needs %zu bytes of scratch; the static scratch holds %zu "
                  "(PGX_NOALLOC_SCRATCH_BYTES)",
                  n_slices, dim, scratch_needed(Dp, n_slices), kScratchBytes);
    return na_fail(err, err_len, PGX_ERR_BUDGET, msg);
  }
  double2* scratch = nullptr;
  cudaError_t e = setup_current_device(&scratch);
  if (e == cudaSuccess) {
    const auto* G = reinterpret_cast<const double2*>(d_gens);
    auto* U = reinterpret_cast<double2*>(d_U_total);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (Dp) {
      case 2: e = run<2>(generator, dim, n_slices, G, d_dt, U, scratch, st); break;
      case 4: e = run<4>(generator, dim, n_slices, G, d_dt, U, scratch, st); break;
      case 8: e = run<8>(generator, dim, n_slices, G, d_dt, U, scratch, st); break;
      case 16: e = run<16>(generator, dim, n_slices, G, d_dt, U, scratch, st); break;
      case 32: e = run<32>(generator, dim, n_slices, G, d_dt, U, scratch, st); break;
      default: e = run<64>(generator, dim, n_slices, G, d_dt, U, scratch, st); break;
    }
  }
  if (e != cudaSuccess) {
    char msg[200];
    std::snprintf(msg, sizeof msg, "CUDA error: %s", cudaGetErrorString(e));
    return na_fail(err, err_len, e == cudaErrorMemoryAllocation ? PGX_ERR_NOMEM : PGX_ERR_CUDA, msg);
  }
  return PGX_OK;
}
