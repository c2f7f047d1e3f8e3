// Checkpoint blobs of served jobs: the host-side state a checkpoint carries
// and its byte encoding (pgx_checkpoint.cpp).  The blob replaces the Julia
// Serialization of Checkpoint (IO/Checkpoint.jl:64-131, 166-208).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "pgx.h"

namespace pgx {

struct Ckpt {
  pgx_checkpoint_info info{};     // dims, counters, F_opt, F, timestamp, fingerprint, settings
  int32_t prior_iteration = 0;    // iterations of the runs before the snapshotted one
  int32_t prior_history_len = 0;  // leading fidelity-history entries from those runs
  int32_t prior_gnorm_len = 0;    // leading gradient-norm entries from those runs
  int32_t round = 0;              // GRAPE: steps applied; L-BFGS: the iteration counter
  int32_t step_iter = 0;          // GRAPE step state: steps the step rule has seen
  double step = 0.0, F_prev = 0.0;  // GRAPE step state: step size, previous objective
  std::vector<double> w;          // best controls [n_c x n_t]
  std::vector<double> fh, gh;     // fidelity / gradient-norm histories
  // exact snapshots
  std::vector<double> u, g;       // current controls and the gradient there
  std::vector<double> rho, S, Y;  // L-BFGS pairs, oldest first: rho[c], S[c][n], Y[c][n]
  std::string meta;               // opaque metadata bytes (UTF-8 JSON by convention)
};

// Encodes c (info.history_len etc. are taken from the vectors).
std::vector<uint8_t> ckpt_encode(const Ckpt& c);
// Decodes and verifies a blob; on failure returns PGX_ERR_INVALID and *why.
int ckpt_decode(const void* blob, uint64_t len, Ckpt* out, std::string* why);
// FNV-1a-64 of a descriptor and, when any part is set, of the job extras.
uint64_t problem_fingerprint(const pgx_problem_desc* d, const pgx_job_extras* x = nullptr);
double unix_now();

}  // namespace pgx
