/* cpu_baseline.c -- FP64 multi-core C restatement of Pulsar.jl's CPU GRAPE
 * evaluation, used as the timed CPU baseline and as a second checker.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle.  The product (libpulsar_gb300.so)
 * never links or calls this file.
 *
 * It consumes the same pgx_problem_desc as the GPU library and follows the
 * reference's CPU algorithm:
 *   - per slice H_k = drift + offset*O + scale*sum_j u_jk C_j
 *     (Propagators.jl:520-544, GRAPEState.jl:187-191);
 *   - U_k = V diag(exp(-i lambda dt)) V' from a Hermitian eigendecomposition
 *     (Propagators.jl:659-674: eigen(Hermitian(H)), which Julia's
 *     LinearAlgebra runs as LAPACK zheevr, then mul!(out, tmp, V') = zgemm);
 *     with pgx_cpu_set_lapack the same LAPACK zheevr and BLAS zgemm run here
 *     (function pointers handed in by the caller, e.g. the OpenBLAS/LAPACK
 *     that SciPy bundles), otherwise a cyclic complex Jacobi and plain loops;
 *   - forward chain, overlap, backward chain (Propagators.jl:309-406,
 *     GRAPEState.jl:201-217);
 *   - first-order gradients of Gradients.jl:254-291,357-399 ("ref_grape") and
 *     GRAPEState.jl:220-230 ("ref_mr"), or the exact gradient from the
 *     spectral Frechet derivative V (Gamma o (V' M V)) V' (divided
 *     differences of exp), with the adjoint identity Tr(M L(A,E)) = Tr(L(A,M) E);
 *   - members in parallel with OpenMP static scheduling and one thread per
 *     member, as Threads.@threads :static with BLAS pinned to one thread
 *     (GRAPEState.jl:168-174, EnsembleObjective.jl:297-302); the member sum
 *     is reduced in member order.
 * Hermitian generators only (the Liouvillian path is checked by the numpy
 * oracle).
 */
#include <complex.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "pgx.h"

typedef double complex cd;

#define IDX(r, c, D) ((r) + (size_t)(D) * (c)) /* column-major */

static cd ld(const double* buf, size_t i) { return buf[2 * i] + I * buf[2 * i + 1]; }

/* Optional LAPACK/BLAS backend (Fortran calling convention, column-major). */
typedef void (*zheevr_fn)(char* jobz, char* range, char* uplo, int* n, cd* a, int* lda, double* vl,
                          double* vu, int* il, int* iu, double* abstol, int* m, double* w, cd* z,
                          int* ldz, int* isuppz, cd* work, int* lwork, double* rwork, int* lrwork,
                          int* iwork, int* liwork, int* info);
typedef void (*zgemm_fn)(char* ta, char* tb, int* m, int* n, int* k, cd* alpha, cd* a, int* lda, cd* b,
                         int* ldb, cd* beta, cd* c, int* ldc);
static zheevr_fn g_zheevr = NULL;
static zgemm_fn g_zgemm = NULL;

/* Hands in LAPACK zheevr and BLAS zgemm; a NULL pointer selects the built-in
 * routine instead (the Jacobi eigensolver, plain product loops). */
int pgx_cpu_set_lapack(void* zheevr, void* zgemm) {
  g_zheevr = (zheevr_fn)zheevr;
  g_zgemm = (zgemm_fn)zgemm;
  return PGX_OK;
}
/* Bit 0: LAPACK zheevr in use; bit 1: BLAS zgemm in use. */
int pgx_cpu_backend(void) { return (g_zheevr != NULL) | ((g_zgemm != NULL) << 1); }

/* Per-thread LAPACK workspace sizes for an n x n zheevr (JOBZ='V', RANGE='A'):
 * generous fixed multiples of n, above the routine's documented minima. */
#define EV_LWORK(n) (66 * (n) + 64)
#define EV_LRWORK(n) (24 * (n) + 64)
#define EV_LIWORK(n) (10 * (n) + 64)
typedef struct {
  cd* work;
  double* rwork;
  int* iwork;
  int* isuppz;
} EvWork;

static void gemm(char ta, char tb, int n, const cd* A, const cd* B, cd* C) {
  cd one = 1.0, zero = 0.0;
  g_zgemm(&ta, &tb, &n, &n, &n, &one, (cd*)A, &n, (cd*)B, &n, &zero, C, &n);
}

/* Cyclic complex Jacobi: A (Hermitian, column-major, destroyed) -> eigenvalues
 * w and eigenvectors V (columns). */
static void jacobi_eigh(int n, cd* A, double* w, cd* V) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[IDX(i, j, n)] = (i == j) ? 1.0 : 0.0;
  double tot = 0.0;
  for (size_t i = 0; i < (size_t)n * n; ++i) tot += creal(A[i] * conj(A[i]));
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int q = 0; q < n; ++q)
      for (int p = 0; p < q; ++p) off += creal(A[IDX(p, q, n)] * conj(A[IDX(p, q, n)]));
    if (off <= 1e-34 * tot || off == 0.0) break;
    for (int q = 1; q < n; ++q)
      for (int p = 0; p < q; ++p) {
        const cd apq = A[IDX(p, q, n)];
        const double r = cabs(apq);
        if (r <= 1e-300) continue;
        const cd e = apq / r; /* e^{i phi} */
        const double app = creal(A[IDX(p, p, n)]), aqq = creal(A[IDX(q, q, n)]);
        const double th = (aqq - app) / (2.0 * r);
        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        const cd ec = conj(e);
        /* A <- A U with U_sub = [[c, s], [-s e^{-i phi}, c e^{-i phi}]] */
        for (int k = 0; k < n; ++k) {
          const cd akp = A[IDX(k, p, n)], akq = A[IDX(k, q, n)];
          A[IDX(k, p, n)] = c * akp - s * ec * akq;
          A[IDX(k, q, n)] = s * akp + c * ec * akq;
          const cd vkp = V[IDX(k, p, n)], vkq = V[IDX(k, q, n)];
          V[IDX(k, p, n)] = c * vkp - s * ec * vkq;
          V[IDX(k, q, n)] = s * vkp + c * ec * vkq;
        }
        /* A <- U' A */
        for (int k = 0; k < n; ++k) {
          const cd apk = A[IDX(p, k, n)], aqk = A[IDX(q, k, n)];
          A[IDX(p, k, n)] = c * apk - s * e * aqk;
          A[IDX(q, k, n)] = s * apk + c * e * aqk;
        }
        A[IDX(p, q, n)] = 0.0;
        A[IDX(q, p, n)] = 0.0;
      }
  }
  for (int i = 0; i < n; ++i) w[i] = creal(A[IDX(i, i, n)]);
}

static void matmul(int n, const cd* A, const cd* B, cd* C) { /* C = A B */
  if (g_zgemm) { gemm('N', 'N', n, A, B, C); return; }
  for (int c = 0; c < n; ++c) {
    for (int r = 0; r < n; ++r) C[IDX(r, c, n)] = 0.0;
    for (int k = 0; k < n; ++k) {
      const cd b = B[IDX(k, c, n)];
      for (int r = 0; r < n; ++r) C[IDX(r, c, n)] += A[IDX(r, k, n)] * b;
    }
  }
}

/* C = A B' */
static void matmul_nh(int n, const cd* A, const cd* B, cd* C) {
  if (g_zgemm) { gemm('N', 'C', n, A, B, C); return; }
  for (int c = 0; c < n; ++c) {
    for (int r = 0; r < n; ++r) C[IDX(r, c, n)] = 0.0;
    for (int k = 0; k < n; ++k) {
      const cd b = conj(B[IDX(c, k, n)]);
      for (int r = 0; r < n; ++r) C[IDX(r, c, n)] += A[IDX(r, k, n)] * b;
    }
  }
}

/* C = A' B */
static void matmul_hn(int n, const cd* A, const cd* B, cd* C) {
  if (g_zgemm) { gemm('C', 'N', n, A, B, C); return; }
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < n; ++r) {
      cd s = 0.0;
      for (int k = 0; k < n; ++k) s += conj(A[IDX(k, r, n)]) * B[IDX(k, c, n)];
      C[IDX(r, c, n)] = s;
    }
}

/* Hermitian eigendecomposition of A (column-major, destroyed): zheevr with
 * JOBZ='V', RANGE='A', UPLO='U', ABSTOL=-1 (the call Julia's
 * eigen(Hermitian(A)) makes), or the Jacobi sweep without the backend. */
static int eigh(int n, cd* A, double* w, cd* V, const EvWork* ew) {
  if (!g_zheevr) {
    jacobi_eigh(n, A, w, V);
    return 0;
  }
  char jobz = 'V', range = 'A', uplo = 'U';
  double vl = 0.0, vu = 0.0, abstol = -1.0;
  int il = 0, iu = 0, m = 0, info = 0;
  int lwork = EV_LWORK(n), lrwork = EV_LRWORK(n), liwork = EV_LIWORK(n);
  g_zheevr(&jobz, &range, &uplo, &n, A, &n, &vl, &vu, &il, &iu, &abstol, &m, w, V, &n, ew->isuppz, ew->work,
           &lwork, ew->rwork, &lrwork, ew->iwork, &liwork, &info);
  return info;
}

/* H <- Gamma o H with Gamma_pq = e^{-i (t_p + t_q)/2} sinc((t_p - t_q)/2),
 * t_p = lambda_p dt: the divided differences of exp(-i t) in the eigenbasis
 * (the spectral Frechet derivative).  The phases and half-angle sines and
 * cosines are formed once per eigenvalue: e^{-i(t_p+t_q)/2} = h_p h_q and
 * sin((t_p - t_q)/2) = s_p c_q - c_p s_q; below |y| = 1/4 the sinc is its
 * Taylor series to y^10 (truncation below 1e-17), which also avoids the
 * cancellation of the difference formula. */
static void apply_gamma(int D, const double* lam, double dt, cd* H) {
  cd h[64];
  double sn[64], cs[64], t[64];
  for (int p = 0; p < D; ++p) {
    t[p] = lam[p] * dt;
    sn[p] = sin(0.5 * t[p]);
    cs[p] = cos(0.5 * t[p]);
    h[p] = cs[p] - I * sn[p];
  }
  for (int c = 0; c < D; ++c)
    for (int r = 0; r < D; ++r) {
      const double y = 0.5 * (t[r] - t[c]);
      double sinc;
      if (fabs(y) < 0.25) {
        const double y2 = y * y;
        sinc = 1.0 + y2 * (-1.0 / 6 + y2 * (1.0 / 120 + y2 * (-1.0 / 5040 + y2 * (1.0 / 362880 - y2 / 39916800.0))));
      } else {
        sinc = (sn[r] * cs[c] - cs[r] * sn[c]) / y;
      }
      H[IDX(r, c, D)] *= h[r] * h[c] * sinc;
    }
}

typedef struct {
  const pgx_problem_desc* d;
  const double* u;
  int D, nc, nt, np;
  int exact;
} Ctx;

static double member_eval(const Ctx* X, int m, double* Gm, cd* work, const EvWork* ew, int* err) {
  const pgx_problem_desc* d = X->d;
  const int D = X->D, nc = X->nc, nt = X->nt, np = X->np;
  const size_t DD = (size_t)D * D;
  const int di = d->member_drift ? d->member_drift[m] : 0;
  const double sc = d->member_scale ? d->member_scale[m] : 1.0;
  const double of = d->member_offset ? d->member_offset[m] : 0.0;
  const double wm = d->member_weight ? d->member_weight[m] : 1.0 / ((double)d->n_members * (np > 0 ? np : 1));
  cd* U = work;                       /* [nt][DD]   */
  cd* V = U + nt * DD;                /* [nt][DD]   eigenvectors (exact) */
  double* lam = (double*)(V + nt * DD); /* [nt][D] */
  cd* P = (cd*)(lam + (size_t)nt * D + (nt * D) % 2); /* [nt+1][DD] or states */
  const size_t pst = (np > 0 && (size_t)np * D > DD) ? (size_t)np * D : DD;
  cd* T1 = P + (size_t)(nt + 1) * pst;
  cd* T2 = T1 + DD;
  cd* T3 = T2 + DD;
  cd* H = T3 + DD;
  double* wv = (double*)(H + DD);
  /* ---- propagators ---- */
  for (int k = 0; k < nt; ++k) {
    for (size_t e = 0; e < DD; ++e) {
      cd h = ld(d->drifts, (size_t)di * DD + e);
      if (d->offset_op) h += of * ld(d->offset_op, e);
      for (int j = 0; j < nc; ++j) h += sc * X->u[j + (size_t)nc * k] * ld(d->controls, (size_t)j * DD + e);
      H[e] = h;
    }
    cd* Vk = V + k * DD;
    if (eigh(D, H, wv, Vk, ew) != 0) *err = 1;
    const double dt = d->dt[k];
    for (int c = 0; c < D; ++c) {
      lam[(size_t)k * D + c] = wv[c];
      const cd ph = cexp(-I * wv[c] * dt);
      for (int r = 0; r < D; ++r) T1[IDX(r, c, D)] = Vk[IDX(r, c, D)] * ph;
    }
    matmul_nh(D, T1, Vk, U + k * DD);
  }
  double Fm = 0.0;
  const int grape = d->grad_mode == PGX_GRAD_REF_GRAPE;
  const cd cfac = -I;
  if (d->target == PGX_TARGET_GATE) {
    /* forward chain P_k (state before slice k) */
    for (size_t e = 0; e < DD; ++e) P[e] = 0.0;
    for (int i = 0; i < D; ++i) P[IDX(i, i, D)] = 1.0;
    for (int k = 0; k < nt; ++k) matmul(D, U + k * DD, P + k * DD, P + (k + 1) * DD);
    cd z = 0.0;
    for (size_t e = 0; e < DD; ++e) z += conj(ld(d->target_op, e)) * P[nt * DD + e];
    z /= D;
    double f;
    cd kap;
    if (d->fidelity == PGX_FID_SQUARE) { f = creal(z * conj(z)); kap = 2.0 * conj(z); }
    else if (d->fidelity == PGX_FID_REAL) { f = creal(z); kap = 1.0; }
    else {
      f = cabs(z);
      kap = f < 1e-14 ? 0.0 : (X->exact ? conj(z) / f : 1.0 / f);
    }
    Fm = f;
    if (Gm) {
      const cd ks = kap * wm / D;
      cd* Lam = T2; /* Lambda = kappa T' U_{n-1}...U_{k+1} */
      for (int r = 0; r < D; ++r)
        for (int c = 0; c < D; ++c) Lam[IDX(r, c, D)] = ks * conj(ld(d->target_op, IDX(c, r, D)));
      for (int k = nt - 1; k >= 0; --k) {
        if (grape) { matmul(D, Lam, U + k * DD, T1); memcpy(Lam, T1, DD * sizeof(cd)); }
        matmul(D, P + k * DD, Lam, T1); /* M_k */
        cd* Xk = T1;
        if (X->exact) {
          /* X = V (Gamma o (V' M V)) V', a_p = -i lambda_p dt */
          const cd* Vk = V + k * DD;
          const double dt = d->dt[k];
          matmul_hn(D, Vk, T1, T3);
          matmul(D, T3, Vk, H);
          apply_gamma(D, lam + (size_t)k * D, dt, H);
          matmul(D, Vk, H, T3);
          matmul_nh(D, T3, Vk, T1);
          Xk = T1;
        }
        const double cds = d->dt[k] * sc;
        for (int j = 0; j < nc; ++j) {
          cd t = 0.0;
          for (int c = 0; c < D; ++c)
            for (int r = 0; r < D; ++r) t += Xk[IDX(r, c, D)] * ld(d->controls, (size_t)j * DD + IDX(c, r, D));
          Gm[j + (size_t)nc * k] += creal(cfac * cds * t);
        }
        if (!grape) { matmul(D, Lam, U + k * DD, T1); memcpy(Lam, T1, DD * sizeof(cd)); }
      }
    }
  } else {
    /* states: psi stack [nt+1][np][D], lambda computed backwards */
    cd* psi = P;
    cd* lamv = (cd*)malloc(sizeof(cd) * (size_t)(nt + 1) * np * D);
    for (int s = 0; s < np; ++s)
      for (int r = 0; r < D; ++r) psi[(size_t)s * D + r] = ld(d->states_init, (size_t)s * D + r);
    for (int k = 0; k < nt; ++k)
      for (int s = 0; s < np; ++s)
        for (int r = 0; r < D; ++r) {
          cd acc = 0.0;
          for (int q = 0; q < D; ++q) acc += U[k * DD + IDX(r, q, D)] * psi[((size_t)k * np + s) * D + q];
          psi[((size_t)(k + 1) * np + s) * D + r] = acc;
        }
    cd kaps[8];
    for (int s = 0; s < np; ++s) {
      cd z = 0.0;
      for (int r = 0; r < D; ++r) z += conj(ld(d->states_target, (size_t)s * D + r)) * psi[((size_t)nt * np + s) * D + r];
      double f;
      cd kap;
      if (d->fidelity == PGX_FID_SQUARE) { f = creal(z * conj(z)); kap = 2.0 * conj(z); }
      else if (d->fidelity == PGX_FID_REAL) { f = creal(z); kap = 1.0; }
      else { f = cabs(z); kap = f < 1e-14 ? 0.0 : (X->exact ? conj(z) / f : 1.0 / f); }
      Fm += f;
      kaps[s] = kap * wm;
    }
    if (Gm) {
      for (int s = 0; s < np; ++s)
        for (int r = 0; r < D; ++r)
          lamv[((size_t)nt * np + s) * D + r] = conj(kaps[s]) * ld(d->states_target, (size_t)s * D + r);
      for (int k = nt - 1; k >= 0; --k)
        for (int s = 0; s < np; ++s)
          for (int r = 0; r < D; ++r) {
            cd acc = 0.0;
            for (int q = 0; q < D; ++q) acc += conj(U[k * DD + IDX(q, r, D)]) * lamv[((size_t)(k + 1) * np + s) * D + q];
            lamv[((size_t)k * np + s) * D + r] = acc;
          }
      for (int k = 0; k < nt; ++k) {
        const cd* ps = psi + (size_t)k * np * D;
        const cd* la = lamv + (size_t)(grape ? k : k + 1) * np * D;
        const double cds = d->dt[k] * sc;
        if (!X->exact) {
          for (int j = 0; j < nc; ++j) {
            cd t = 0.0;
            for (int s = 0; s < np; ++s)
              for (int c = 0; c < D; ++c) {
                cd cp = 0.0;
                for (int r = 0; r < D; ++r) cp += conj(la[(size_t)s * D + r]) * ld(d->controls, (size_t)j * DD + IDX(r, c, D));
                t += cp * ps[(size_t)s * D + c];
              }
            Gm[j + (size_t)nc * k] += creal(cfac * cds * t);
          }
        } else {
          for (int c = 0; c < D; ++c)
            for (int r = 0; r < D; ++r) {
              cd acc = 0.0;
              for (int s = 0; s < np; ++s) acc += ps[(size_t)s * D + r] * conj(la[(size_t)s * D + c]);
              T1[IDX(r, c, D)] = acc;
            }
          const cd* Vk = V + k * DD;
          const double dt = d->dt[k];
          matmul_hn(D, Vk, T1, T3);
          matmul(D, T3, Vk, H);
          apply_gamma(D, lam + (size_t)k * D, dt, H);
          matmul(D, Vk, H, T3);
          matmul_nh(D, T3, Vk, T1);
          for (int j = 0; j < nc; ++j) {
            cd t = 0.0;
            for (int c = 0; c < D; ++c)
              for (int r = 0; r < D; ++r) t += T1[IDX(r, c, D)] * ld(d->controls, (size_t)j * DD + IDX(c, r, D));
            Gm[j + (size_t)nc * k] += creal(cfac * cds * t);
          }
        }
      }
    }
    free(lamv);
  }
  return Fm;
}

static size_t work_elems(int D, int nt, int np) {
  const size_t DD = (size_t)D * D;
  size_t n = 2 * (size_t)nt * DD + ((size_t)nt * D + 2) / 2 + 1;
  size_t pst = (size_t)(nt + 1) * (np > 0 ? ((size_t)np * D > DD ? (size_t)np * D : DD) : DD);
  return n + pst + 4 * DD + D + 16;
}

/* (F, G) of a pgx_problem_desc at controls u ([n_c x n_t] column-major),
 * member-parallel on n_threads OpenMP threads (<= 0: all).  G may be NULL.
 * Returns 0 on success, PGX_ERR_UNSUPPORTED for Liouvillian generators,
 * PGX_ERR_INVALID when zheevr reports a failure.                           */
int pgx_cpu_eval(const pgx_problem_desc* d, const double* u, double* F, double* G, int n_threads) {
  if (!d || !u || !F) return PGX_ERR_INVALID;
  if (d->generator != PGX_GEN_HERMITIAN) return PGX_ERR_UNSUPPORTED;
  if (d->dim < 1 || d->dim > 64) return PGX_ERR_DIMS;
  Ctx X = {d, u, d->dim, d->n_controls, d->n_slices, d->target == PGX_TARGET_STATES ? d->n_pairs : 0,
           d->grad_mode == PGX_GRAD_EXACT};
  const int nm = d->n_members;
  const size_t ng = (size_t)X.nc * X.nt;
  double* Fm = (double*)calloc(nm, sizeof(double));
  double* Gms = G ? (double*)calloc((size_t)nm * ng, sizeof(double)) : NULL;
  const size_t we = work_elems(X.D, X.nt, X.np);
  if (n_threads <= 0) n_threads = omp_get_max_threads();
  int err = 0;
#pragma omp parallel num_threads(n_threads)
  {
    cd* work = (cd*)malloc(sizeof(cd) * we);
    EvWork ew;
    ew.work = (cd*)malloc(sizeof(cd) * EV_LWORK(X.D));
    ew.rwork = (double*)malloc(sizeof(double) * EV_LRWORK(X.D));
    ew.iwork = (int*)malloc(sizeof(int) * EV_LIWORK(X.D));
    ew.isuppz = (int*)malloc(sizeof(int) * 2 * X.D);
    int terr = 0;
#pragma omp for schedule(static)
    for (int m = 0; m < nm; ++m) Fm[m] = member_eval(&X, m, Gms ? Gms + (size_t)m * ng : NULL, work, &ew, &terr);
    if (terr) {
#pragma omp atomic write
      err = 1;
    }
    free(ew.work);
    free(ew.rwork);
    free(ew.iwork);
    free(ew.isuppz);
    free(work);
  }
  double f = 0.0;
  for (int m = 0; m < nm; ++m)
    f += (d->member_weight ? d->member_weight[m] : 1.0 / ((double)nm * (X.np > 0 ? X.np : 1))) * Fm[m];
  *F = f;
  if (G) {
    for (size_t i = 0; i < ng; ++i) {
      double s = 0.0;
      for (int m = 0; m < nm; ++m) s += Gms[(size_t)m * ng + i];
      G[i] = s;
    }
  }
  free(Fm);
  free(Gms);
  return err ? PGX_ERR_INVALID : PGX_OK;
}

int pgx_cpu_max_threads(void) { return omp_get_max_threads(); }
