/*
 * lgt_ed.h -- C ABI of the GB300 exact-diagonalisation library (liblgted.so).
 *
 * Drop-in boundary for the exact-diagonalisation path of NoaFeldman/LGT
 * (finite_ed.jl with the local-operator conventions of u1_lgt_hamiltonian.jl
 * and, for the plaquette + Jordan-Wigner model, the term list of
 * matter_gauge_entanglement_pjw.jl).  Each entry point names the reference
 * function it replaces.  A Julia `ccall` shim binds these symbols one to one
 * (lgt_gb300/julia/LGTED.jl).
 *
 * Conventions
 *  - Every function returns an lgt_status; 0 is success.  lgt_last_error()
 *    gives a message for the calling thread's last failure.  Nothing aborts
 *    the process: the reference's @assert failures become status codes.
 *  - The library owns all device memory behind opaque handles.  Host buffers
 *    are caller-owned.  Arrays that mirror Julia matrices are column-major.
 *  - Basis indices returned to the caller are 1-based where they replace a
 *    reference index (key_dict values), 0-based elsewhere, as documented.
 *  - Amplitude panels are "K-interleaved": element (row, k, comp) of K
 *    vectors of length N lives at ((row * K) + k) * ncomp + comp, ncomp = 1
 *    for real and 2 for complex (re, im).  For K = 1, ncomp = 2 this is
 *    exactly a Julia Vector{ComplexF64}.
 *  - A handle is used by one host thread at a time.  Each basis handle owns
 *    a CUDA stream; calls return when results are in the caller's buffers.
 *  - Flags LGT_DEVICE_PTRS: the amplitude pointers given to lgt_matvec,
 *    lgt_observe, lgt_ground_state and lgt_expm_steps are device pointers on
 *    the basis's device (no host<->device copies are made).
 */
#ifndef LGT_ED_H
#define LGT_ED_H

#include <stdint.h>

#if defined(__GNUC__)
#define LGT_API __attribute__((visibility("default")))
#else
#define LGT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t lgt_status;

enum {
  LGT_OK = 0,
  LGT_ERR_ARG = 1,        /* invalid argument (sizes, pointers, flags)          */
  LGT_ERR_SECTOR = 2,     /* inconsistent charge sector (finite_ed.jl:127)      */
  LGT_ERR_KEYWIDTH = 3,   /* lattice/dg beyond the key width                    */
  LGT_ERR_MEMORY = 4,     /* device allocation failed                           */
  LGT_ERR_CUDA = 5,       /* a CUDA call failed                                 */
  LGT_ERR_NOCONV = 6,     /* Krylov solver did not converge (finite_ed.jl:339)  */
  LGT_ERR_DEVICE = 7,     /* a kernel self-check failed (rank/bounds/NaN)       */
  LGT_ERR_NOTFOUND = 8,   /* state not in the basis (finite_ed.jl:530)          */
  LGT_ERR_UNSUPPORTED = 9 /* feature not available for these arguments          */
};

/* Model flags (bit set) for lgt_ham_create. */
enum {
  LGT_MODEL_REF = 0,   /* finite_ed.jl:252-322: on-site + bare hopping          */
  LGT_MODEL_JW = 1,    /* Jordan-Wigner strings on the column snake             */
  LGT_MODEL_PLAQ = 2,  /* magnetic plaquette -(1/2g^2)(W + W^dag)              */
  LGT_MODEL_PJW = 3    /* matter_gauge_entanglement_pjw.jl:82-147               */
};

/* Arithmetic of the amplitude panels. */
enum {
  LGT_FP64 = 0,        /* FP64 amplitudes, coefficients and accumulation       */
  LGT_FP32 = 1,        /* FP32 amplitudes, coefficients and accumulation       */
  LGT_FP32_MIXED = 2   /* Krylov drivers: FP32 H*psi and storage, FP64 dots,
                          reorthogonalisation, tridiagonal solve, residual and
                          refinement                                           */
};

enum {
  LGT_DEVICE_PTRS = 1, /* amplitude pointers are device pointers                  */
  LGT_ASYNC = 2,       /* with LGT_DEVICE_PTRS: lgt_matvec returns without waiting
                          for the kernel (stream-ordered; no self-check read)   */
  LGT_GENERIC_KERNELS = 4, /* lgt_matvec: use the run-time-geometry H*psi kernel
                          even where a fixed-shape one exists (cross-checks)    */
  LGT_ROW_ORDER = 8       /* lgt_matvec with LGT_DEVICE_PTRS: x and y are in the
                          row order of lgt_ham_row_order (stored-table kernel) */
};

typedef struct lgt_basis lgt_basis;
typedef struct lgt_ham lgt_ham;

/* Krylov solver options.  lgt_krylov_defaults() fills the reference's values
   (finite_ed.jl:336-338 for eigsolve, :417-419 for exponentiate). */
typedef struct lgt_krylov_opts {
  int32_t krylovdim;     /* Krylov dimension (eigsolve: 50, exponentiate: 30) */
  int32_t maxiter;       /* restarts (eigsolve: 300, exponentiate: 100)        */
  double tol;            /* absolute residual / error tolerance (1e-10)        */
  int32_t precision;     /* LGT_FP64 or LGT_FP32_MIXED                         */
  int32_t reorth_passes; /* Gram-Schmidt passes against the whole basis (2)    */
  int32_t check_every;   /* steps between convergence checks                   */
  int32_t refine_steps;  /* FP64 correction steps after an FP32 solve          */
  uint64_t seed;         /* start vector of point k: normal(seed, k)           */
  int32_t use_graph;     /* replay the step sequence as a CUDA graph           */
  int32_t start_given;   /* ground state: 1 = psi holds the start vectors      */
  int32_t solver;        /* ground state: LGT_SOLVER_*                          */
} lgt_krylov_opts;

/* Ground-state solver selection. */
enum {
  LGT_SOLVER_AUTO = 0,   /* per-CTA for sectors up to 8192 states, else panel   */
  LGT_SOLVER_PANEL = 1,  /* K-interleaved panels, CUDA-graph Lanczos steps      */
  LGT_SOLVER_CTA = 2     /* one CTA per coupling point, whole solve in a kernel */
};

/* Per-call solver report. */
typedef struct lgt_info {
  int64_t matvecs;       /* H*psi panel applications                           */
  int32_t restarts;      /* Krylov restarts                                    */
  int32_t converged;     /* points that met tol                                */
  double max_residual;   /* largest final residual / error estimate            */
  double seconds;        /* device time of the call (CUDA events)              */
} lgt_info;

/* Observables of one state (one coupling point), measure_ED
   (finite_ed.jl:369-393) plus the plaquette.  Grids are column-major. */
typedef struct lgt_obs {
  double t;              /* time stamp passed by the caller                    */
  double nf_mean, nf_even, nf_odd, E2_mean;
  double plaq_mean;      /* (1/N_P) sum_p <W_p + W_p^dag>                       */
  double n_stag;         /* (1/N_s) sum (-1)^(ix+iy) <n_f>                     */
  double norm2;          /* <psi|psi>                                          */
} lgt_obs;

LGT_API void lgt_krylov_defaults(lgt_krylov_opts* o, int for_exponentiate);
LGT_API const char* lgt_last_error(void);
LGT_API const char* lgt_version(void);

/* ---- basis -------------------------------------------------------------- */

/* build_basis (finite_ed.jl:125-162).  g_charges: nx*ny, column-major
   (g[ix,iy] at (ix-1) + (iy-1)*nx).  Enumerates the Gauss-law sector on the
   GPU as sorted order keys.  device < 0 uses the current device. */
LGT_API lgt_status lgt_basis_create(int32_t nx, int32_t ny, int32_t dg, const int32_t* g_charges,
                            int32_t device, lgt_basis** out);

/* length(states) (finite_ed.jl:133,227-231). */
LGT_API lgt_status lgt_basis_dim(const lgt_basis* b, int64_t* dim);

/* Keys of states [first, first+count): the order key (mask << w*N_U | e_U
   digits, strictly increasing in reference index order) and/or the
   reference _encode key (finite_ed.jl:80-97, dg == 1 only; bit pattern of
   the Int64).  Either pointer may be NULL. */
LGT_API lgt_status lgt_basis_keys(const lgt_basis* b, int64_t first, int64_t count, uint64_t* order_keys,
                          int64_t* ref_keys);

/* Contents of `states` (finite_ed.jl:229) for [first, first+count): per
   state the column-major n_f (nx*ny), e_R ((nx-1)*ny), e_U (nx*(ny-1))
   blocks, states one after the other.  Any pointer may be NULL. */
LGT_API lgt_status lgt_basis_states(const lgt_basis* b, int64_t first, int64_t count, int8_t* n_f,
                            int8_t* e_R, int8_t* e_U);

/* key_dict lookup (finite_ed.jl:291-292,527-531): for each reference
   _encode key, its 1-based index, or 0 when the configuration is not in the
   basis.  dg == 1 only. */
LGT_API lgt_status lgt_basis_lookup(const lgt_basis* b, const int64_t* ref_keys, int64_t n,
                            int64_t* index1);

/* Same for order keys: 0-based index or -1. */
LGT_API lgt_status lgt_basis_rank(const lgt_basis* b, const uint64_t* order_keys, int64_t n,
                          int64_t* index0);

/* Releases the caller's handle.  Hamiltonians made from the basis keep it
   alive: handles may be destroyed in any order (the basis is freed with the
   last of them). */
LGT_API void lgt_basis_destroy(lgt_basis* b);

/* Run this basis' work (and that of its Hamiltonians) on a caller-owned
   cudaStream_t (passed as void*), e.g. a CUDA.jl or PyTorch stream; NULL
   restores the basis' own stream.  No reference counterpart (the reference
   has no device). */
LGT_API lgt_status lgt_basis_set_stream(lgt_basis* b, void* stream);

/* Number of kernels this process has launched through the library so far
   (graph replays count their kernel nodes).  No reference counterpart. */
LGT_API lgt_status lgt_launch_count(uint64_t* count);

/* ---- Hamiltonian -------------------------------------------------------- */

/* build_hamiltonian (finite_ed.jl:252-322) for K coupling points that share
   the basis: point k has couplings g[k], t[k], m[k].  Matrix-free: nothing
   of size nnz is stored.  model: LGT_MODEL_* flags. */
LGT_API lgt_status lgt_ham_create(const lgt_basis* b, int32_t K, const double* g, const double* t,
                          const double* m, uint32_t model, lgt_ham** out);

/* Replace the couplings of all K points (quench: build_hamiltonian at the
   final couplings, finite_ed.jl:582,632). */
LGT_API lgt_status lgt_ham_set_couplings(lgt_ham* h, const double* g, const double* t, const double* m);

/* nnz(H) as SparseArrays counts it (finite_ed.jl:355): stored diagonal
   entries plus the off-diagonal entries. */
LGT_API lgt_status lgt_ham_nnz(const lgt_ham* h, int64_t* nnz);

/* The sparse matrix of point k as CSR (host buffers; rowptr has N+1 entries,
   colidx/values nnz).  H is symmetric, so these are also the colptr/rowval/
   nzval arrays of the reference's SparseMatrixCSC.  Indices are 0-based.
   Values are computed in the reference's own summation order. */
LGT_API lgt_status lgt_ham_export_csr(const lgt_ham* h, int32_t k, int64_t* rowptr, int32_t* colidx,
                              double* values);

/* y = H x for all K points (the SparseMatrixCSC * Vector product inside
   KrylovKit).  x, y: K-interleaved panels of N rows; ncomp 1 or 2;
   precision LGT_FP64 (double) or LGT_FP32 (float). */
LGT_API lgt_status lgt_matvec(const lgt_ham* h, const void* x, void* y, int32_t ncomp, int32_t precision,
                      uint32_t flags);

/* The locality row order of the stored-table H*psi (no counterpart in the
   reference): the rows in breadth-first order of the Hamiltonian's hop
   graph, which the Krylov drivers use internally for their basis vectors
   (the x gathers of a product then mostly hit L2).  Builds the neighbour
   table and its renumbered copy on first use (LGT_ERR_UNSUPPORTED where the
   table is not available).  perm: N int32 (may be NULL), perm[n] = the
   0-based basis index of row n of that order.  lgt_matvec with
   LGT_ROW_ORDER applies H to device panels kept in this order. */
LGT_API lgt_status lgt_ham_row_order(lgt_ham* h, int32_t* perm);

/* find_ground_state (finite_ed.jl:333-341) for all K points: lowest
   eigenpair by Lanczos with full reorthogonalisation.  E0: K doubles.  psi:
   real panel [N][K] (double; float for LGT_FP32_MIXED with device pointers
   is not accepted -- the output is always double), may be NULL.  residual:
   K doubles (final FP64 residual norm ||H psi - E0 psi||), may be NULL. */
LGT_API lgt_status lgt_ground_state(lgt_ham* h, const lgt_krylov_opts* opts, double* E0, void* psi,
                            double* residual, uint32_t flags, lgt_info* info);

/* find_ground_state then measure_ED of the ground states in one call
   (gs_benchmark.jl:116-125 runs the two per point): as lgt_ground_state
   followed by lgt_observe(h, psi, 1, LGT_FP64, flags, 0, nf_grid, E2_grid,
   plaq_grid, summary), with the observables launched on the device result
   before the one synchronisation that returns both.  Replaces the pair
   find_ground_state (finite_ed.jl:333-341) + measure_ED (:369-393). */
LGT_API lgt_status lgt_ground_state_observe(lgt_ham* h, const lgt_krylov_opts* opts, double* E0,
                                            void* psi, double* residual, uint32_t flags,
                                            lgt_info* info, double* nf_grid, double* E2_grid,
                                            double* plaq_grid, lgt_obs* summary);

/* find_ground_state over several Hamiltonians at once (the GS benchmark
   grid, gs_benchmark.jl:36-52,86-175, and lattices / sectors of uneven
   dimension): every (Hamiltonian, point) pair of a sector up to 8192 states
   runs in ONE persistent launch, one CTA each, largest sectors first;
   larger sectors go through the panel solver.  E0[i], psi[i], residual[i]
   are the per-Hamiltonian arrays of lgt_ground_state (psi[i] and
   residual[i] may be NULL; psi must be device pointers with
   LGT_DEVICE_PTRS).  All Hamiltonians must live on one device. */
LGT_API lgt_status lgt_ground_state_batch(int32_t nham, lgt_ham* const* hams,
                                          const lgt_krylov_opts* opts, double* const* E0,
                                          void* const* psi, double* const* residual,
                                          uint32_t flags, lgt_info* info);

/* evolve_ED! (finite_ed.jl:405-431): n_steps Krylov steps
   psi <- exp(-i H dt) psi, each followed by renormalisation, for all K
   points.  psi: complex double panel [N][K][2], updated in place.  obs:
   (n_steps + 1) * K records (t = step * dt), filled every step, or NULL.
   norm_drift: K doubles (max |1 - ||psi||| before renormalisation), may be
   NULL. */
LGT_API lgt_status lgt_expm_steps(lgt_ham* h, const lgt_krylov_opts* opts, double dt, int32_t n_steps,
                          void* psi, lgt_obs* obs, double* norm_drift, uint32_t flags,
                          lgt_info* info);

/* lgt_expm_steps that also returns the site grids of every step's
   measure_ED record (evolve_ED! keeps the whole record, nf_grid and
   E2_grid included, for each step: finite_ed.jl:380-386,409,421-422).
   nf_grid, E2_grid: (n_steps + 1) * K * nx*ny doubles; plaq_grid:
   (n_steps + 1) * K * (nx-1)*(ny-1) doubles; record (step, k) starts at
   (step * K + k) times the grid size, each grid column-major.  Any grid
   pointer may be NULL; with all of them and obs NULL nothing is measured. */
LGT_API lgt_status lgt_expm_steps_grids(lgt_ham* h, const lgt_krylov_opts* opts, double dt,
                                        int32_t n_steps, void* psi, lgt_obs* obs,
                                        double* nf_grid, double* E2_grid, double* plaq_grid,
                                        double* norm_drift, uint32_t flags, lgt_info* info);

/* measure_ED (finite_ed.jl:369-393) of K states: per point the nx*ny grids
   <n_f> and <E^2> (column-major, point after point) and the (nx-1)*(ny-1)
   plaquette grid <W + W^dag>; any grid pointer may be NULL.  summary: K
   records, may be NULL.  psi: panel [N][K][ncomp] in `precision`. */
LGT_API lgt_status lgt_observe(const lgt_ham* h, const void* psi, int32_t ncomp, int32_t precision,
                       uint32_t flags, double t_now, double* nf_grid, double* E2_grid,
                       double* plaq_grid, lgt_obs* summary);

/* lgt_observe without any device allocation.  No counterpart in the
   reference (finite_ed.jl measures on the host); it exists for callers that
   cannot call cudaMalloc: applications that reserve all device memory for
   their own pool, and loops that must not trigger the device
   synchronisation an allocation can cause.  psi must be a device panel
   [N][K][ncomp] on the basis' device (the LGT_DEVICE_PTRS form of
   lgt_observe); outputs are host arrays as in lgt_observe.  Its scratch is a
   fixed 2 MiB static device array per GPU: calls whose K * (2 nx ny +
   (nx-1)(ny-1) + 1) doubles per block do not fit are rejected with
   LGT_ERR_ARG.  All calls share that array, so calls that overlap on the GPU
   race.  The first call on a device looks up the array's address (make it
   before any stream capture on that device). */
LGT_API lgt_status lgt_observe_noalloc(const lgt_ham* h, const void* psi, int32_t ncomp,
                                       int32_t precision, double t_now, double* nf_grid,
                                       double* E2_grid, double* plaq_grid, lgt_obs* summary);

/* Energy <psi|H|psi> / <psi|psi> per point, FP64 (finite_ed.jl has no
   counterpart; used for energy-drift reports of evolve_ED!). */
LGT_API lgt_status lgt_energy(const lgt_ham* h, const void* psi, int32_t ncomp, uint32_t flags,
                      double* energy);

/* Autotuner report (no counterpart in the reference).  The Krylov drivers
   time their kernel candidates at the first solve of each operator shape
   (lattice, model, storage precision, panel width) and keep the fastest for
   the process: the H*psi kernel (run-time geometry, the fixed-shape kernel
   or the stored-neighbour-table kernel, each with its load modes;
   lgt_matvec uses and, on its first call for a shape, makes the same
   choice) and the block count of the Gram-Schmidt reductions.  The table
   kernel reads the neighbour ranks of every row from a table built once per
   Hamiltonian (4 bytes per off-diagonal entry and per row; no matrix values)
   when its size bound fits min(free device memory / 4, LGT_NBR_TABLE_MB,
   default 16384 MB); LGT_NBR_TABLE=0 disables it.  LGT_AUTOTUNE=0 in the
   environment keeps the built-in rules; LGT_HPSI_VARIANT=1..8 forces one
   H*psi kernel (the hpsi_kernel codes below) for cross-checks. */
typedef struct lgt_tuning {
  int32_t hpsi_kernel;    /* 0 built-in rule, 1 run-time geometry, fixed
                             shape with 2 one / 3 two 16-byte vectors per
                             lane, 4 two vectors as one 32-byte access;
                             5, 6, 7 the same load modes from the stored
                             neighbour table; 8 the stored table with the
                             neighbour rows gathered by the copy engine
                             (FP32 panels of 16 columns)                    */
  int32_t reduce_blocks;  /* block-count cap of the panel reductions         */
  double hpsi_ms;         /* one H*psi with the chosen kernel                */
  double reduce_ms;       /* one 8-vector Gram-Schmidt pass, chosen blocks   */
  int32_t measured;       /* 1 timed on this device, 0 built-in rules        */
} lgt_tuning;

/* Runs (or looks up) the autotuner for h's Krylov panels: ncomp 1 is the
   ground-state shape (K real columns), 2 the exponential's (2K real
   columns); precision LGT_FP64, or LGT_FP32 / LGT_FP32_MIXED (FP32
   storage).  Tuning allocates a temporary workspace and synchronises. */
LGT_API lgt_status lgt_autotune(lgt_ham* h, int32_t ncomp, int32_t precision, lgt_tuning* out);

LGT_API void lgt_ham_destroy(lgt_ham* h);

#ifdef __cplusplus
}
#endif

#endif /* LGT_ED_H */
