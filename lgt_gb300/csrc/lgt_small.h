// lgt_small.h -- persistent per-CTA Lanczos for small sectors.
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "lgt_internal.h"

namespace lgt {

// Largest sector the per-CTA solver takes (rows held in registers:
// 16 per thread x 512 threads).
constexpr int kSmallMaxN = 8192;

// Result of the lookup pass: neighbour ranks of every row (index << 2 |
// kind) in CSR order, and the integer parts of the diagonal.
struct Pattern {
  int N = 0;
  int nnz = 0;
  uint32_t model = 0;
  int* rowptr = nullptr;
  uint32_t* nbr = nullptr;
  int16_t* e2 = nullptr;
  int16_t* stag = nullptr;
  void* block = nullptr;  // the one allocation the arrays above are carved from
};

struct SmallProblem {
  int N;
  const int* rowptr;
  const uint32_t* nbr;
  const int16_t* e2;
  const int16_t* stag;
};

struct SmallUnit {
  int prob;        // index into the problem table
  int k;           // coupling point (start-vector stream)
  double cE, cm, ch, cp;
  double* psi;     // output (and start vector when given), stride psi_stride
  int psi_stride;
  void* V;         // (m + 1) x N Krylov basis, storage precision
  double* x;       // N doubles
  double* out;     // 8 doubles: E0, residual, steps, restarts, converged, estimate
};

struct SmallParams {
  int m;
  int maxiter;
  double tol;
  int reorth;
  int check_every;
  uint64_t seed;
  int start_given;
  int rows_per_thread = 0;  // launch shape: 0 the smallest R with N <= 512 R
  int v_smem = 0;           // set by the launcher: Krylov basis in shared memory
};

// One Hamiltonian's share of a batched launch.
struct SmallJob {
  const Pattern* pattern;
  int K;
  const double *cE, *cm, *ch, *cp;  // host arrays [K]
  double* psi;                      // device panel [N][K]
  double* E0;                       // host [K]
  double* resid;                    // host [K] or null
  int* steps;                       // host [K] or null
  int* restarts;                    // host [K] or null
  bool* converged;                  // host [K] or null
};

// Per-Hamiltonian workspace of the per-CTA solver: device memory for the
// unit tables, bases and outputs; a pinned host buffer that stages the
// tables (kept as the copy last uploaded, so that an unchanged batch skips
// the upload) and the outputs; and the timing events.
struct SmallWork {
  void* base = nullptr;
  size_t bytes = 0;
  void* host = nullptr;      // pinned: [uploaded tables][outputs]
  size_t host_bytes = 0;
  size_t up_bytes = 0;       // bytes of tables the device buffer holds (0: none)
  cudaEvent_t ev[2] = {nullptr, nullptr};
};
void free_small_work(SmallWork* w, cudaStream_t s);

std::string build_pattern(const BasisDev& B, uint32_t model, Pattern* P, cudaStream_t s);
void free_pattern(Pattern* P, cudaStream_t s);

// All (job, point) units in one launch, largest sectors first.
// dev_err (may be null): a device error word copied back with the results
// into *err_out (or'd into it).
// before_sync (may be empty): enqueued work of the caller's (e.g. the
// observables of the solution) run after the solve's output copies and
// before the one synchronisation.
std::string small_ground_states(const std::vector<SmallJob>& jobs, const SmallParams& prm,
                                int mixed, SmallWork* ws, cudaStream_t s, double* seconds,
                                const int* dev_err = nullptr, int* err_out = nullptr,
                                const std::function<cudaError_t()>& before_sync = {});

}  // namespace lgt
