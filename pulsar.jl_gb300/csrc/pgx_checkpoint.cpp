// Checkpoint blobs (host code only): encoding, verification, the warm-start
// constructor and the problem fingerprint.
//
// The reference writes its Checkpoint struct (IO/Checkpoint.jl:64-131) with
// Julia Serialization behind a temp-file rename (:166-177); the payload is a
// Julia-version-specific object graph.  Here a checkpoint is a flat byte blob
// with the same fields plus the device state an exact continuation needs.
// Every field is written byte by byte in little-endian order, so a blob is
// the same on x86-64 and AArch64 hosts.
//
// Layout (offsets in bytes):
//     0  "PGXCKPT\0"          8  u32 version        12  u32 header bytes (208)
//    16  i32 flags           20  i32 system_dim     24  i32 n_controls
//    28  i32 n_timesteps     32  i32 n_members      36  i32 iteration
//    40  i32 history_len     44  i32 gnorm_len      48  i32 prior_iteration
//    52  i32 prior_hist_len  56  i32 prior_gnorm    60  i32 lbfgs_pairs
//    64  i32 round           68  i32 step_iter      72  f64 F_opt
//    80  f64 F               88  f64 timestamp      96  u64 fingerprint
//   104  i32 opt method, max_iter, adapt_step_size, lbfgs_memory
//   120  f64 opt convergence_tol, step_size, min_step_size, max_step_size,
//            gradient_norm_tol, amplitude_limit, l_bound, u_bound
//   184  f64 step           192  f64 F_prev        200  u64 payload bytes
//   208  payload (f64): w_opt[n], fidelity history, gradient-norm history;
//        exact snapshots add u[n], g[n] and, for L-BFGS, rho[c], S[c n], Y[c n]
//        then u64 metadata bytes m and m bytes of metadata (UTF-8 text, JSON
//        by convention: the reference's domain tags and metadata dict)
//   end  u64 FNV-1a-64 of every preceding byte
// with n = n_controls * n_timesteps and c = lbfgs_pairs.
#include <chrono>
#include <cmath>
#include <cstring>

#include "pgx.h"
#include "pgx_ckpt.h"

namespace pgx {

constexpr uint64_t kMaxMeta = 1ull << 20;  // metadata bytes a blob may carry

namespace {

constexpr char kMagic[8] = {'P', 'G', 'X', 'C', 'K', 'P', 'T', '\0'};
constexpr uint64_t kFnvOffset = 0xcbf29ce484222325ull;
constexpr uint64_t kFnvPrime = 0x100000001b3ull;
constexpr int32_t kMaxPairs = 64;

uint64_t fnv1a(const uint8_t* p, size_t n, uint64_t h = kFnvOffset) {
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= kFnvPrime;
  }
  return h;
}

uint64_t bits_of(double x) {
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
}

double double_of(uint64_t b) {
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
}

struct Writer {
  std::vector<uint8_t> out;
  void u64(uint64_t v) {
    for (int i = 0; i < 8; ++i) out.push_back((uint8_t)(v >> (8 * i)));
  }
  void u32(uint32_t v) {
    for (int i = 0; i < 4; ++i) out.push_back((uint8_t)(v >> (8 * i)));
  }
  void i32(int32_t v) { u32((uint32_t)v); }
  void f64(double v) { u64(bits_of(v)); }
  void vec(const std::vector<double>& v) {
    for (double x : v) f64(x);
  }
};

struct Reader {
  const uint8_t* p;
  size_t pos = 0;
  uint64_t u64() {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)p[pos + i] << (8 * i);
    pos += 8;
    return v;
  }
  uint32_t u32() {
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)p[pos + i] << (8 * i);
    pos += 4;
    return v;
  }
  int32_t i32() { return (int32_t)u32(); }
  double f64() { return double_of(u64()); }
  void vec(std::vector<double>* v, size_t n) {
    v->resize(n);
    for (size_t i = 0; i < n; ++i) (*v)[i] = f64();
  }
};

// Hash input for the fingerprint: every value in little-endian bytes.
struct Hasher {
  uint64_t h = kFnvOffset;
  void bytes(const uint8_t* p, size_t n) { h = fnv1a(p, n, h); }
  void i32(int32_t v) {
    uint8_t b[4];
    for (int i = 0; i < 4; ++i) b[i] = (uint8_t)((uint32_t)v >> (8 * i));
    bytes(b, 4);
  }
  void f64s(const double* x, size_t n) {
    const uint8_t present = x ? 1 : 0;
    bytes(&present, 1);
    for (size_t i = 0; x && i < n; ++i) {
      uint8_t b[8];
      const uint64_t v = bits_of(x[i]);
      for (int k = 0; k < 8; ++k) b[k] = (uint8_t)(v >> (8 * k));
      bytes(b, 8);
    }
  }
  void i32s(const int32_t* x, size_t n) {
    const uint8_t present = x ? 1 : 0;
    bytes(&present, 1);
    for (size_t i = 0; x && i < n; ++i) i32(x[i]);
  }
};

bool exact_of(const Ckpt& c) { return (c.info.flags & PGX_CKPT_EXACT) != 0; }
bool lbfgs_of(const Ckpt& c) {
  return c.info.opt.method == PGX_OPT_ENSEMBLE_LBFGS || c.info.opt.method == PGX_OPT_MR_LBFGS;
}

}  // namespace

double unix_now() {
  return std::chrono::duration<double>(std::chrono::system_clock::now().time_since_epoch()).count();
}

std::vector<uint8_t> ckpt_encode(const Ckpt& c) {
  const pgx_checkpoint_info& I = c.info;
  const pgx_opt_desc& o = I.opt;
  const int32_t pairs = exact_of(c) && lbfgs_of(c) ? (int32_t)c.rho.size() : 0;
  Writer w;
  w.out.reserve(PGX_CHECKPOINT_HEADER_BYTES + 8 * (c.w.size() + c.fh.size() + c.gh.size() + c.u.size() +
                                                  c.g.size() + c.rho.size() + c.S.size() + c.Y.size()) + 8);
  w.out.insert(w.out.end(), kMagic, kMagic + 8);
  w.u32(PGX_CHECKPOINT_VERSION);
  w.u32(PGX_CHECKPOINT_HEADER_BYTES);
  w.i32(I.flags);
  w.i32(I.system_dim);
  w.i32(I.n_controls);
  w.i32(I.n_timesteps);
  w.i32(I.n_members);
  w.i32(I.iteration);
  w.i32((int32_t)c.fh.size());
  w.i32((int32_t)c.gh.size());
  w.i32(c.prior_iteration);
  w.i32(c.prior_history_len);
  w.i32(c.prior_gnorm_len);
  w.i32(pairs);
  w.i32(c.round);
  w.i32(c.step_iter);
  w.f64(I.F_opt);
  w.f64(I.F);
  w.f64(I.timestamp);
  w.u64(I.fingerprint);
  w.i32(o.method);
  w.i32(o.max_iter);
  w.i32(o.adapt_step_size);
  w.i32(o.lbfgs_memory);
  for (double x : {o.convergence_tol, o.step_size, o.min_step_size, o.max_step_size, o.gradient_norm_tol,
                   o.amplitude_limit, o.l_bound, o.u_bound})
    w.f64(x);
  w.f64(c.step);
  w.f64(c.F_prev);
  const size_t at_payload = w.out.size();
  w.u64(0);  // payload bytes, patched below
  w.vec(c.w);
  w.vec(c.fh);
  w.vec(c.gh);
  if (exact_of(c)) {
    w.vec(c.u);
    w.vec(c.g);
    if (lbfgs_of(c)) {
      w.vec(c.rho);
      w.vec(c.S);
      w.vec(c.Y);
    }
  }
  const uint64_t payload = w.out.size() - PGX_CHECKPOINT_HEADER_BYTES;
  for (int i = 0; i < 8; ++i) w.out[at_payload + i] = (uint8_t)(payload >> (8 * i));
  w.u64(c.meta.size());
  w.out.insert(w.out.end(), c.meta.begin(), c.meta.end());
  w.u64(fnv1a(w.out.data(), w.out.size()));
  return std::move(w.out);
}

int ckpt_decode(const void* blob, uint64_t len, Ckpt* out, std::string* why) {
  auto bad = [&](const char* m) {
    *why = m;
    return PGX_ERR_INVALID;
  };
  if (!blob) return bad("checkpoint blob is NULL");
  if (len < PGX_CHECKPOINT_HEADER_BYTES + 16) return bad("checkpoint blob is truncated");
  const uint8_t* p = static_cast<const uint8_t*>(blob);
  if (std::memcmp(p, kMagic, 8) != 0) return bad("not a checkpoint blob (magic)");
  Reader r{p, 8};
  if (r.u32() != PGX_CHECKPOINT_VERSION) return bad("unsupported checkpoint version");
  if (r.u32() != PGX_CHECKPOINT_HEADER_BYTES) return bad("unexpected checkpoint header size");
  Ckpt c;
  pgx_checkpoint_info& I = c.info;
  I.struct_size = sizeof(pgx_checkpoint_info);
  I.version = PGX_CHECKPOINT_VERSION;
  I.flags = r.i32();
  I.system_dim = r.i32();
  I.n_controls = r.i32();
  I.n_timesteps = r.i32();
  I.n_members = r.i32();
  I.iteration = r.i32();
  I.history_len = r.i32();
  I.gnorm_history_len = r.i32();
  c.prior_iteration = r.i32();
  c.prior_history_len = r.i32();
  c.prior_gnorm_len = r.i32();
  I.lbfgs_pairs = r.i32();
  c.round = r.i32();
  c.step_iter = r.i32();
  I.F_opt = r.f64();
  I.F = r.f64();
  I.timestamp = r.f64();
  I.fingerprint = r.u64();
  pgx_opt_desc& o = I.opt;
  o.struct_size = sizeof(pgx_opt_desc);
  o.method = r.i32();
  o.max_iter = r.i32();
  o.adapt_step_size = r.i32();
  o.lbfgs_memory = r.i32();
  o.convergence_tol = r.f64();
  o.step_size = r.f64();
  o.min_step_size = r.f64();
  o.max_step_size = r.f64();
  o.gradient_norm_tol = r.f64();
  o.amplitude_limit = r.f64();
  o.l_bound = r.f64();
  o.u_bound = r.f64();
  c.step = r.f64();
  c.F_prev = r.f64();
  const uint64_t payload = r.u64();
  if (I.flags & ~(PGX_CKPT_EXACT | PGX_CKPT_CONVERGED)) return bad("unknown checkpoint flags");
  if (I.system_dim < 0 || I.n_controls < 1 || I.n_timesteps < 1 || I.n_members < 0 || I.iteration < 0 ||
      I.history_len < 0 || I.gnorm_history_len < 0 || c.prior_iteration < 0 || c.prior_iteration > I.iteration ||
      c.prior_history_len < 0 || c.prior_history_len > I.history_len || c.prior_gnorm_len < 0 ||
      c.prior_gnorm_len > I.gnorm_history_len || I.lbfgs_pairs < 0 || I.lbfgs_pairs > kMaxPairs ||
      o.method < PGX_OPT_GRAPE || o.method > PGX_OPT_MR_GRAPE)
    return bad("checkpoint header fields out of range");
  const bool exact = (I.flags & PGX_CKPT_EXACT) != 0;
  const bool lb = o.method == PGX_OPT_ENSEMBLE_LBFGS || o.method == PGX_OPT_MR_LBFGS;
  if (I.lbfgs_pairs > 0 && !(exact && lb)) return bad("L-BFGS pairs in a checkpoint that cannot hold them");
  const uint64_t n = (uint64_t)I.n_controls * (uint64_t)I.n_timesteps;
  if (n > (1ull << 31)) return bad("checkpoint waveform too large");
  const uint64_t np = (uint64_t)I.lbfgs_pairs;
  const uint64_t doubles = n + (uint64_t)I.history_len + (uint64_t)I.gnorm_history_len +
                           (exact ? 2 * n + (lb ? np + 2 * np * n : 0) : 0);
  if (payload != 8 * doubles || len < PGX_CHECKPOINT_HEADER_BYTES + payload + 16)
    return bad("checkpoint blob length does not match its header");
  const uint64_t meta = Reader{p, (size_t)(PGX_CHECKPOINT_HEADER_BYTES + payload)}.u64();
  if (meta > kMaxMeta || len != PGX_CHECKPOINT_HEADER_BYTES + payload + 16 + meta)
    return bad("checkpoint blob length does not match its header");
  Reader tail{p, (size_t)(len - 8)};
  if (tail.u64() != fnv1a(p, (size_t)(len - 8))) return bad("checkpoint checksum mismatch (corrupted blob)");
  r.vec(&c.w, n);
  r.vec(&c.fh, (size_t)I.history_len);
  r.vec(&c.gh, (size_t)I.gnorm_history_len);
  if (exact) {
    r.vec(&c.u, n);
    r.vec(&c.g, n);
    if (lb) {
      r.vec(&c.rho, np);
      r.vec(&c.S, np * n);
      r.vec(&c.Y, np * n);
    }
  }
  r.pos += 8;
  c.meta.assign(reinterpret_cast<const char*>(p + r.pos), (size_t)meta);
  I.metadata_len = (int32_t)meta;
  *out = std::move(c);
  return PGX_OK;
}

uint64_t problem_fingerprint(const pgx_problem_desc* d, const pgx_job_extras* x) {
  const size_t D = (size_t)d->dim, DD = D * D, nc = (size_t)d->n_controls, nt = (size_t)d->n_slices;
  const size_t nm = (size_t)d->n_members, nd = (size_t)d->n_drifts;
  const size_t np = d->target == PGX_TARGET_STATES ? (size_t)d->n_pairs : 0;
  Hasher h;
  const uint8_t tag[4] = {'P', 'G', 'X', 'P'};
  h.bytes(tag, 4);
  for (int32_t v : {d->dim, d->n_controls, d->n_slices, d->generator, d->target, d->fidelity, d->grad_mode,
                    d->precision, d->n_drifts, d->n_members, d->n_pairs})
    h.i32(v);
  h.f64s(d->dt, nt);
  h.f64s(d->drifts, 2 * DD * nd);
  h.f64s(d->controls, 2 * DD * nc);
  h.f64s(d->offset_op, 2 * DD);
  h.i32s(d->member_drift, nm);
  h.f64s(d->member_scale, nm);
  h.f64s(d->member_offset, nm);
  h.f64s(d->member_weight, nm);
  h.f64s(d->target == PGX_TARGET_GATE ? d->target_op : nullptr, 2 * DD);
  h.f64s(np ? d->states_init : nullptr, 2 * np * D);
  h.f64s(np ? d->states_target : nullptr, 2 * np * D);
  h.f64s(np ? d->grad_states_init : nullptr, 2 * np * D);
  if (x && (x->n_penalties > 0 || x->n_tracking > 0 || x->n_ramp_ops > 0)) {
    const uint8_t xt[4] = {'P', 'G', 'X', 'X'};
    h.bytes(xt, 4);
    h.i32(x->n_penalties);
    for (int i = 0; i < x->n_penalties; ++i) {
      h.i32(x->penalties[i].type);
      h.f64s(&x->penalties[i].weight, 3);  // weight, l_bound, u_bound
    }
    h.i32(x->n_tracking);
    if (x->n_tracking > 0) {
      h.i32s(x->tracking_steps, (size_t)x->n_tracking);
      h.f64s(x->tracking_weights, (size_t)x->n_tracking);
      h.f64s(x->tracking_targets, 2 * DD * (size_t)x->n_tracking);
    }
    h.i32(x->n_ramp_ops);
    if (x->n_ramp_ops > 0) {
      h.f64s(x->ramp_ops, 2 * DD * (size_t)x->n_ramp_ops);
      h.i32s(x->ramp_member_op, nm);
      h.f64s(x->ramp_tau, nt);
    }
  }
  return h.h;
}

}  // namespace pgx

extern "C" int pgx_checkpoint_parse(const void* blob, uint64_t blob_len, pgx_checkpoint_info* info, double* w_opt,
                                    double* fidelity_history, double* gnorm_history) {
  if (!blob || !info) return PGX_ERR_INVALID;
  pgx::Ckpt c;
  std::string why;
  const int st = pgx::ckpt_decode(blob, blob_len, &c, &why);
  if (st) return st;
  *info = c.info;
  if (w_opt) std::copy(c.w.begin(), c.w.end(), w_opt);
  if (fidelity_history) std::copy(c.fh.begin(), c.fh.end(), fidelity_history);
  if (gnorm_history) std::copy(c.gh.begin(), c.gh.end(), gnorm_history);
  return PGX_OK;
}

extern "C" int pgx_checkpoint_metadata(const void* blob, uint64_t blob_len, char* metadata, uint64_t cap) {
  if (!blob || (!metadata && cap)) return PGX_ERR_INVALID;
  pgx::Ckpt c;
  std::string why;
  const int st = pgx::ckpt_decode(blob, blob_len, &c, &why);
  if (st) return st;
  if (cap < c.meta.size()) return PGX_ERR_DIMS;
  std::memcpy(metadata, c.meta.data(), c.meta.size());
  return PGX_OK;
}

extern "C" int pgx_checkpoint_create(const pgx_checkpoint_info* info, const double* w_opt,
                                     const double* fidelity_history, const double* gnorm_history,
                                     const char* metadata, void* blob, uint64_t cap, uint64_t* blob_len) {
  if (!info || !w_opt || !blob_len) return PGX_ERR_INVALID;
  if (info->struct_size < sizeof(pgx_checkpoint_info) || info->n_controls < 1 || info->n_timesteps < 1 ||
      info->system_dim < 0 || info->n_members < 0 || info->iteration < 0 || info->history_len < 0 ||
      info->gnorm_history_len < 0 || (info->history_len > 0 && !fidelity_history) ||
      (info->gnorm_history_len > 0 && !gnorm_history) || (info->flags & PGX_CKPT_EXACT) ||
      (info->flags & ~PGX_CKPT_CONVERGED) || info->opt.method < PGX_OPT_GRAPE ||
      info->opt.method > PGX_OPT_MR_GRAPE || info->metadata_len < 0 ||
      (uint64_t)info->metadata_len > pgx::kMaxMeta || (info->metadata_len > 0 && !metadata))
    return PGX_ERR_INVALID;
  const uint64_t n = (uint64_t)info->n_controls * (uint64_t)info->n_timesteps;
  if (n > (1ull << 31)) return PGX_ERR_DIMS;
  pgx::Ckpt c;
  c.info = *info;
  c.info.lbfgs_pairs = 0;
  if (c.info.timestamp == 0.0) c.info.timestamp = pgx::unix_now();
  c.w.assign(w_opt, w_opt + n);
  c.fh.assign(fidelity_history, fidelity_history + info->history_len);
  c.gh.assign(gnorm_history, gnorm_history + info->gnorm_history_len);
  if (info->metadata_len > 0) c.meta.assign(metadata, (size_t)info->metadata_len);
  const std::vector<uint8_t> b = pgx::ckpt_encode(c);
  *blob_len = b.size();
  if (!blob) return PGX_OK;
  if (cap < b.size()) return PGX_ERR_DIMS;
  std::memcpy(blob, b.data(), b.size());
  return PGX_OK;
}

extern "C" int pgx_checkpoint_set_metadata(const void* blob, uint64_t blob_len, const char* metadata,
                                           uint64_t metadata_len, void* out, uint64_t cap, uint64_t* out_len) {
  if (!blob || !out_len || (metadata_len && !metadata) || metadata_len > pgx::kMaxMeta) return PGX_ERR_INVALID;
  pgx::Ckpt c;
  std::string why;
  const int st = pgx::ckpt_decode(blob, blob_len, &c, &why);
  if (st) return st;
  c.meta.assign(metadata ? metadata : "", (size_t)metadata_len);
  const std::vector<uint8_t> b = pgx::ckpt_encode(c);
  *out_len = b.size();
  if (!out) return PGX_OK;
  if (cap < b.size()) return PGX_ERR_DIMS;
  std::memcpy(out, b.data(), b.size());
  return PGX_OK;
}

extern "C" int pgx_problem_fingerprint(const pgx_problem_desc* d, uint64_t* fingerprint) {
  if (!d || !fingerprint || d->struct_size < sizeof(pgx_problem_desc) || d->dim < 1 || d->n_controls < 1 ||
      d->n_slices < 1 || d->n_drifts < 1 || d->n_members < 1 || d->n_pairs < 0 || !d->dt || !d->drifts ||
      !d->controls)
    return PGX_ERR_INVALID;
  *fingerprint = pgx::problem_fingerprint(d);
  return PGX_OK;
}
