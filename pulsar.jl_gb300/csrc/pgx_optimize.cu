// Optimiser loops over the device-resident problem (pgx_optimize).
//
// Each loop restates the reference's control flow, step rules and convergence
// tests; only the physics call is replaced by the GPU evaluation.
//   PGX_OPT_GRAPE           grape_optimize              GRAPE.jl:469-643
//   PGX_OPT_ENSEMBLE_LBFGS  grape_optimize_ensemble     GRAPE.jl:1012-1230
//   PGX_OPT_MR_LBFGS        _optimcon_lbfgs             OptControl.jl:380-482,565-611
//   PGX_OPT_MR_GRAPE        _optimcon_grape             OptControl.jl:486-561
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "pgx.h"
#include "pgx_runtime.h"

namespace {

using Vec = std::vector<double>;

double dot(const Vec& a, const Vec& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}
double nrm2(const Vec& a) { return std::sqrt(dot(a, a)); }
double maxabs(const Vec& a) {
  double m = 0.0;
  for (double x : a) m = std::max(m, std::fabs(x));
  return m;
}

struct Runner {
  pgx_problem* p;
  int status = PGX_OK;
  int nf = 0, ng = 0;
  Vec fh, gh;
  double F(const Vec& u) {
    double f = 0.0;
    if (status == PGX_OK) status = eval_host(p, u.data(), &f, nullptr, nullptr);
    return f;
  }
  double FG(const Vec& u, Vec& g) {
    double f = 0.0;
    g.resize(u.size());
    if (status == PGX_OK) status = eval_host(p, u.data(), &f, g.data(), nullptr);
    return f;
  }
};

// adapt_grape_step_size (GRAPE.jl:309-334)
double adapt_step(const Vec& fh, double step, double lo, double hi) {
  if (fh.size() < 2) return step;
  const double d = fh[fh.size() - 1] - fh[fh.size() - 2];
  double s = step;
  if (d > 0.0) s = step * 1.05;
  else if (d < -1e-14) s = step * 0.5;
  return std::min(std::max(s, lo), hi);
}

// Two-loop recursion.  guarded = true: the ensemble form with 1e-14 floors
// (GRAPE.jl:1064-1084); false: the MR form without them (OptControl.jl:565-590).
Vec lbfgs_dir(const Vec& g, const std::deque<Vec>& S, const std::deque<Vec>& Y, bool guarded) {
  const size_t k = S.size();
  if (k == 0) return g;
  Vec q = g;
  Vec al(k), rho(k);
  for (size_t i = 0; i < k; ++i) {
    const double ys = dot(Y[i], S[i]);
    rho[i] = 1.0 / (guarded ? std::max(ys, 1e-14) : ys);
  }
  for (size_t ii = k; ii-- > 0;) {
    al[ii] = rho[ii] * dot(S[ii], q);
    for (size_t t = 0; t < q.size(); ++t) q[t] -= al[ii] * Y[ii][t];
  }
  const double yy = dot(Y[k - 1], Y[k - 1]);
  const double gam = dot(S[k - 1], Y[k - 1]) / (guarded ? std::max(yy, 1e-14) : yy);
  for (double& x : q) x *= gam;
  for (size_t i = 0; i < k; ++i) {
    const double b = rho[i] * dot(Y[i], q);
    for (size_t t = 0; t < q.size(); ++t) q[t] += (al[i] - b) * S[i][t];
  }
  return q;
}

void clampv(Vec& v, double lo, double hi) {
  for (double& x : v) x = std::min(std::max(x, lo), hi);
}

void set_reason(pgx_opt_result* r, const std::string& s) {
  std::snprintf(r->reason, sizeof(r->reason), "%s", s.c_str());
}

int finish(Runner& R, pgx_opt_result* res, double* fhist, double* ghist, int cap, double t0s) {
  (void)t0s;
  const int nh = (int)std::min<size_t>(R.fh.size(), (size_t)std::max(cap, 0));
  if (fhist) std::copy(R.fh.begin(), R.fh.begin() + nh, fhist);
  if (ghist) {
    const int ng = (int)std::min<size_t>(R.gh.size(), (size_t)std::max(cap, 0));
    std::copy(R.gh.begin(), R.gh.begin() + ng, ghist);
  }
  res->history_len = (int)R.fh.size();
  res->gnorm_history_len = (int)R.gh.size();
  res->n_fidelity_evals = R.nf;
  res->n_gradient_evals = R.ng;
  return R.status;
}

int opt_grape(Runner& R, const pgx_opt_desc* o, Vec& u, pgx_opt_result* res) {
  double step = o->step_size;
  Vec best = u, G;
  double F = R.F(u);
  R.nf++;
  R.fh.push_back(F);
  double bestF = F;
  bool conv = false;
  std::string reason = "maximum iterations reached";
  int n_iter = 0;
  for (int it = 1; it <= o->max_iter && R.status == PGX_OK; ++it) {
    n_iter = it;
    F = R.FG(u, G);
    R.nf++;
    R.ng++;
    const double gn = nrm2(G);
    R.fh.push_back(F);
    R.gh.push_back(gn);
    if (F > bestF) { bestF = F; best = u; }
    if (o->adapt_step_size && R.fh.size() >= 2)
      step = adapt_step(R.fh, step, o->min_step_size, o->max_step_size);
    for (size_t i = 0; i < u.size(); ++i) u[i] += step * G[i];
    // check_grape_convergence (GRAPE.jl:371-402)
    const size_t n = R.fh.size();
    bool c = false;
    if (R.fh.back() >= 1.0 - 1e-12) { c = true; reason = "perfect fidelity (F >= 1 - 1e-12)"; }
    else if (gn < o->gradient_norm_tol) { c = true; reason = "gradient norm below tolerance"; }
    else if (n >= 3 && std::fabs(R.fh[n - 1] - R.fh[n - 2]) < o->convergence_tol) {
      c = true;
      reason = "fidelity change below tolerance";
    }
    if (c) {
      conv = true;
      const double Fp = R.F(u);
      R.nf++;
      R.fh.push_back(Fp);
      if (Fp > bestF) { bestF = Fp; best = u; }
      break;
    }
  }
  const double Ff = R.F(best);
  R.nf++;
  u = best;
  res->fidelity = Ff;
  res->n_iterations = n_iter;
  res->converged = conv;
  res->step_size_final = step;
  set_reason(res, reason);
  return R.status;
}

int opt_ensemble_lbfgs(Runner& R, const pgx_opt_desc* o, Vec& u, pgx_opt_result* res) {
  const double lim = o->amplitude_limit;
  const bool clip = std::isfinite(lim);
  std::deque<Vec> S, Y;
  double F = R.F(u);
  R.nf++;
  R.fh.push_back(F);
  double bestF = F;
  Vec best = u, g, gn;
  bool conv = false;
  std::string reason = "maximum iterations reached";
  for (int it = 1; it <= o->max_iter && R.status == PGX_OK; ++it) {
    R.FG(u, g);
    R.ng++;
    const double gnorm = nrm2(g);
    R.gh.push_back(gnorm);
    Vec d = lbfgs_dir(g, S, Y, true);
    const double dmax = maxabs(d);
    if (dmax < 1e-14) { conv = true; reason = "zero gradient direction"; break; }
    for (double& x : d) x /= dmax;
    const double a0 = clip ? o->step_size * lim : o->step_size;
    // backtracking: accept F_new >= F0, halve up to 20 times (GRAPE.jl:1088-1104)
    double a = a0, Fn = 0.0;
    Vec un(u.size());
    bool accepted = false;
    for (int bt = 0; bt < 20 && R.status == PGX_OK; ++bt) {
      for (size_t i = 0; i < u.size(); ++i) un[i] = u[i] + a * d[i];
      if (clip) clampv(un, -lim, lim);
      Fn = R.F(un);
      R.nf++;
      if (Fn >= F) { accepted = true; break; }
      a *= 0.5;
    }
    if (!accepted) {
      for (size_t i = 0; i < u.size(); ++i) un[i] = u[i] + a * d[i];
      if (clip) clampv(un, -lim, lim);
      Fn = R.F(un);
      R.nf++;
    }
    R.FG(un, gn);
    R.ng++;
    Vec s(u.size()), y(u.size());
    for (size_t i = 0; i < u.size(); ++i) { s[i] = a * d[i]; y[i] = gn[i] - g[i]; }
    const double sn = nrm2(s);
    if (dot(y, s) > 1e-14 * sn * sn) {
      S.push_back(s);
      Y.push_back(y);
      if ((int)S.size() > o->lbfgs_memory) { S.pop_front(); Y.pop_front(); }
    }
    u = un;
    F = Fn;
    R.fh.push_back(F);
    if (F > bestF) { bestF = F; best = u; }
    if (gnorm < o->gradient_norm_tol) { conv = true; reason = "gradient norm below tolerance"; break; }
    if (F >= 1.0 - 1e-8) { conv = true; reason = "near-perfect fidelity"; break; }
    const size_t n = R.fh.size();
    if (n >= 2 && std::fabs(R.fh[n - 1] - R.fh[n - 2]) < o->convergence_tol) {
      conv = true;
      reason = "fidelity change below tolerance";
      break;
    }
  }
  u = best;
  res->fidelity = bestF;
  res->n_iterations = (int)R.fh.size();
  res->converged = conv;
  res->step_size_final = o->step_size;
  set_reason(res, reason);
  return R.status;
}

int opt_mr_lbfgs(Runner& R, const pgx_opt_desc* o, Vec& u, pgx_opt_result* res) {
  const double lo = o->l_bound, hi = o->u_bound;
  clampv(u, lo, hi);
  Vec G, Gn;
  double F = R.FG(u, G);
  R.nf++;
  R.ng++;
  Vec best = u;
  double bestF = F;
  R.fh.push_back(F);
  R.gh.push_back(nrm2(G));
  std::deque<Vec> S, Y;
  bool conv = false;
  std::string reason = "max iterations reached";
  for (int it = 1; it <= o->max_iter && R.status == PGX_OK; ++it) {
    Vec d = lbfgs_dir(G, S, Y, false);
    const double dmax = maxabs(d);
    if (dmax < 1e-14) { conv = true; reason = "zero gradient direction"; break; }
    for (double& x : d) x /= dmax;
    // _line_search (OptControl.jl:594-611): F_new >= F0 - 1e-4 |alpha|
    double a = 0.05 * (hi - lo), Fn = 0.0;
    Vec wn(u.size());
    bool accepted = false;
    for (int h = 1; h <= 20 && R.status == PGX_OK; ++h) {
      for (size_t i = 0; i < u.size(); ++i) wn[i] = u[i] + a * d[i];
      clampv(wn, lo, hi);
      Fn = R.F(wn);
      if (Fn >= F - 1e-4 * std::fabs(a)) { R.nf += h + 1; accepted = true; break; }
      a *= 0.5;
    }
    if (!accepted) {
      for (size_t i = 0; i < u.size(); ++i) wn[i] = u[i] + a * d[i];
      clampv(wn, lo, hi);
      Fn = R.F(wn);
      if (!(Fn > F)) wn = u;
      R.nf += 21;
    }
    const double F2 = R.FG(wn, Gn);
    R.nf++;
    R.ng++;
    Vec s(u.size()), y(u.size());
    for (size_t i = 0; i < u.size(); ++i) { s[i] = wn[i] - u[i]; y[i] = Gn[i] - G[i]; }
    const double sn = nrm2(s);
    if (dot(y, s) > 1e-14 * sn * sn) {
      S.push_back(s);
      Y.push_back(y);
      if ((int)S.size() > o->lbfgs_memory) { S.pop_front(); Y.pop_front(); }
    }
    u = wn;
    G = Gn;
    const double Fprev = F;
    F = F2;
    R.fh.push_back(F);
    const double gnorm = nrm2(G);
    R.gh.push_back(gnorm);
    if (F > bestF) { bestF = F; best = u; }
    if (F >= 1.0 - 1e-8) { conv = true; reason = "near-perfect fidelity"; break; }
    if (gnorm < o->gradient_norm_tol) { conv = true; reason = "gradient norm below tolerance"; break; }
    if (R.fh.size() >= 2 && std::fabs(F - Fprev) < 1e-9) { conv = true; reason = "fidelity stalled"; break; }
  }
  u = best;
  res->fidelity = bestF;
  res->n_iterations = (int)R.fh.size() - 1;
  res->converged = conv;
  res->step_size_final = 0.0;
  set_reason(res, reason);
  return R.status;
}

int opt_mr_grape(Runner& R, const pgx_opt_desc* o, Vec& u, pgx_opt_result* res) {
  const double lo = o->l_bound, hi = o->u_bound;
  clampv(u, lo, hi);
  Vec G;
  double F = R.FG(u, G);
  R.nf++;
  R.ng++;
  Vec best = u;
  double bestF = F;
  R.fh.push_back(F);
  R.gh.push_back(nrm2(G));
  bool conv = false;
  std::string reason = "max iterations reached";
  for (int it = 1; it <= o->max_iter && R.status == PGX_OK; ++it) {
    const double gmax = maxabs(G);
    if (gmax > 1e-14) {
      const double st = 0.05 * (hi - lo) / gmax;
      for (size_t i = 0; i < u.size(); ++i) u[i] += st * G[i];
      clampv(u, lo, hi);
    }
    F = R.FG(u, G);
    R.nf++;
    R.ng++;
    R.fh.push_back(F);
    const double gnorm = nrm2(G);
    R.gh.push_back(gnorm);
    if (F > bestF) { bestF = F; best = u; }
    if (F >= 1.0 - 1e-8) { conv = true; reason = "near-perfect fidelity"; break; }
    if (gnorm < o->gradient_norm_tol) { conv = true; reason = "gradient norm below tolerance"; break; }
  }
  u = best;
  res->fidelity = bestF;
  res->n_iterations = (int)R.fh.size() - 1;
  res->converged = conv;
  res->step_size_final = 0.05;
  set_reason(res, reason);
  return R.status;
}

}  // namespace

extern "C" int pgx_optimize(pgx_problem* p, const pgx_opt_desc* o, double* u_inout, double* fhist,
                            double* ghist, int32_t cap, pgx_opt_result* res) {
  if (!p || !o || !u_inout || !res) return PGX_ERR_INVALID;
  if (o->struct_size < sizeof(pgx_opt_desc)) return ctx_fail(p->ctx, PGX_ERR_INVALID, "opt struct_size");
  if (o->max_iter < 1 || o->step_size <= 0.0 || o->lbfgs_memory < 1 || o->min_step_size <= 0.0 ||
      o->max_step_size < o->step_size || o->gradient_norm_tol <= 0.0 || o->convergence_tol <= 0.0)
    return ctx_fail(p->ctx, PGX_ERR_INVALID, "invalid optimiser settings (GRAPE.jl:108-119)");
  if ((o->method == PGX_OPT_MR_LBFGS || o->method == PGX_OPT_MR_GRAPE) && !(o->l_bound < o->u_bound))
    return ctx_fail(p->ctx, PGX_ERR_INVALID, "l_bound must be < u_bound");
  std::memset(res, 0, sizeof(*res));
  const auto t0 = std::chrono::steady_clock::now();
  Runner R{p};
  Vec u(u_inout, u_inout + (size_t)p->desc.n_controls * p->desc.n_slices);
  int st;
  switch (o->method) {
    case PGX_OPT_GRAPE: st = opt_grape(R, o, u, res); break;
    case PGX_OPT_ENSEMBLE_LBFGS: st = opt_ensemble_lbfgs(R, o, u, res); break;
    case PGX_OPT_MR_LBFGS: st = opt_mr_lbfgs(R, o, u, res); break;
    case PGX_OPT_MR_GRAPE: st = opt_mr_grape(R, o, u, res); break;
    default: return ctx_fail(p->ctx, PGX_ERR_INVALID, "unknown optimiser method");
  }
  res->total_time_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  finish(R, res, fhist, ghist, cap, 0.0);
  if (st) return st;
  std::copy(u.begin(), u.end(), u_inout);
  return PGX_OK;
}
