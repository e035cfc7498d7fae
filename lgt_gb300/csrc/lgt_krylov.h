// lgt_krylov.h -- batched Krylov drivers (Lanczos ground state and Krylov
// exp(-iHt) steps) on K-interleaved panels.
#pragma once

#include <string>

#include "lgt_hpsi.h"

namespace lgt {

// Host-side description of the operator the drivers apply: the basis, the
// model and per-point coefficient arrays on the device in both precisions.
struct OpDev {
  Geom G;
  RankView R;
  int* err;
  uint32_t model;
  int K;
  int seg_smem;
  const double *cE_d, *cm_d, *ch_d, *cp_d;
  const float *cE_f, *cm_f, *ch_f, *cp_f;
  int force_generic = 0;  // H*psi through the run-time-geometry kernel only
  int vpl = 0;            // fixed-shape H*psi: vector loads per lane (0: by width)
  NbrTable* table = nullptr;  // the Hamiltonian's neighbour table (built on demand)
  int use_table = 0;          // H*psi from the stored table
  // The table renumbered to its breadth-first row order (order.cu), built
  // with the table; the Krylov drivers keep their basis vectors in that
  // order (krylov_order = 1) when the table kernel is chosen.
  NbrTable* table_ord = nullptr;
  int krylov_order = 0;
};

struct KrylovParams {
  int krylovdim;
  int maxiter;
  double tol;
  int mixed;        // FP32 storage + H*psi, FP64 dots
  int reorth;       // Gram-Schmidt passes
  int check_every;
  int refine;       // FP64 Lanczos correction steps after a mixed solve
  uint64_t seed;
  int use_graph;
  int start_given;
};

struct KrylovCache;

// Autotuner choice for one operator shape (see krylov.cu).
enum HpsiVariant : int {
  kHpsiDefault = 0,   // built-in rule
  kHpsiGeneric = 1,   // run-time geometry
  kHpsiFixed1 = 2,    // fixed shape, one 16-byte vector per lane
  kHpsiFixed2 = 3,    // fixed shape, two 16-byte vectors per lane
  kHpsiFixed2w = 4,   // fixed shape, two vectors as one 32-byte access
  kHpsiTable1 = 5,    // stored neighbour table, one 16-byte vector per lane
  kHpsiTable2 = 6,    // stored neighbour table, two 16-byte vectors per lane
  kHpsiTable2w = 7,   // stored neighbour table, one 32-byte access per lane
  kHpsiTableBulk = 8, // stored neighbour table, rows gathered by the copy engine
};
struct TuneChoice {
  int hpsi_variant = kHpsiDefault;
  int red_blocks = 0;
  int red_nblk = 0;
  double hpsi_ms = 0.0;  // one H*psi of the chosen variant
  double red_ms = 0.0;   // one 8-vector Gram-Schmidt pass (dots + update), chosen blocks
  int measured = 0;      // 0: built-in rules (tuning disabled)
};

// Runs (or looks up) the autotuner for the Krylov panels of this operator:
// ncomp = 1 the ground-state shape, 2 the exponential's (two real columns
// per point); mixed = FP32 storage.
std::string krylov_autotune(const OpDev& op, KrylovCache* cache, int ncomp, int mixed,
                            cudaStream_t s, TuneChoice* out);

// H*psi variant for this operator and panel width, timed on (x, y) at the
// first call of each shape (x is only read; y is overwritten); sets op's
// kernel selection.  No timing while `s` is capturing or LGT_AUTOTUNE=0.
// The table variants are candidates when op's neighbour table is built or
// can be: the basis fits the format and the table's size bound is within
// min(free device memory / 4, LGT_NBR_TABLE_MB, default 16384 MB);
// LGT_NBR_TABLE=0 disables it.
std::string hpsi_choose_d(OpDev* op, const double* x, double* y, int ncomp, cudaStream_t s);
std::string hpsi_choose_f(OpDev* op, const float* x, float* y, int ncomp, cudaStream_t s);

struct KrylovReport {
  int64_t matvecs = 0;
  int restarts = 0;
  int converged = 0;
  double max_residual = 0.0;
  double seconds = 0.0;
};

// Workspaces and captured graphs of the drivers, kept per Hamiltonian.
struct KrylovCache;
KrylovCache* krylov_cache_new();
void krylov_cache_free(KrylovCache* c);

// Lowest eigenpair of each of the K operators.  X (device, double, [N][K])
// receives the normalised eigenvectors; when start_given, X holds the start
// vectors on entry.  E0, resid: host arrays of K.
std::string lanczos_ground_state(const OpDev& op, const KrylovParams& p, KrylovCache* cache,
                                 double* X, double* E0, double* resid, cudaStream_t s,
                                 KrylovReport* rep);

// n_steps steps psi <- exp(-i H dt) psi (renormalised) on the complex panel
// X (device, double, [N][K][2]).  After each step (and before the first)
// `observe_cb(step)` is called with X holding the current state.
struct StepObserver {
  virtual ~StepObserver() {}
  virtual std::string on_step(int step, const double* X) = 0;
};
std::string krylov_expm(const OpDev& op, const KrylovParams& p, KrylovCache* cache, double dt,
                        int n_steps, double* X, double* norm_drift, StepObserver* obs,
                        cudaStream_t s, KrylovReport* rep);

// Builds (on first use) the stored neighbour table and its renumbered copy
// and sets op to apply H in that row order (table kernel, krylov_order).
// Returns an empty string, or why the order is not available.
std::string ensure_row_order(OpDev* op, cudaStream_t s);

// y = H x on a double or float panel (C = K * ncomp columns).
cudaError_t apply_h_d(const OpDev& op, const double* x, double* y, int ncomp, cudaStream_t s);
cudaError_t apply_h_f(const OpDev& op, const float* x, float* y, int ncomp, cudaStream_t s);

// Per-point Re <x|y> (FP64) of two double panels: out[K] on host.
std::string panel_dots(KrylovCache* cache, const double* x, const double* y, int64_t N, int K,
                       int ncomp, double* out, cudaStream_t s);

}  // namespace lgt
