// capi.cu -- the extern "C" boundary (include/lgt_ed.h): handles, argument
// checks, host<->device staging and error reporting around the kernels.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <memory>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lgt_ed.h"
#include "lgt_hpsi.h"
#include "lgt_internal.h"
#include "lgt_krylov.h"
#include "lgt_observe.h"
#include "lgt_small.h"
#include "lgt_handles.h"

using namespace lgt;

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
thread_local bool g_capturing = false;

lgt_status fail(lgt_status code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

lgt_status cuda_fail(cudaError_t e, const char* where) {
  return fail(e == cudaErrorMemoryAllocation ? LGT_ERR_MEMORY : LGT_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

lgt_status from_msg(const std::string& m) {
  if (m.empty()) return LGT_OK;
  if (m.rfind("NOCONV", 0) == 0) return fail(LGT_ERR_NOCONV, m);
  if (m.find("out of memory") != std::string::npos) return fail(LGT_ERR_MEMORY, m);
  return fail(LGT_ERR_CUDA, m);
}

#define CUDA_OR_FAIL(call)                            \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

}  // namespace

namespace lgt {
void note_launch(int n) {
  if (!g_capturing) g_launches.fetch_add(uint64_t(n), std::memory_order_relaxed);
}
void set_capturing(bool on) { g_capturing = on; }
}  // namespace lgt


namespace {

lgt_status set_device(const lgt_basis* b) {
  CUDA_OR_FAIL(cudaSetDevice(b->device));
  return LGT_OK;
}

// Reads and clears the basis' device error word.
// The device error word: a fast path copies it into pinned memory next to
// its results so that it rides on the same synchronisation; err_status
// interprets a value (and resets the device word).
lgt_status err_status(const lgt_basis* b, int err) {
  if (err) {
    cudaMemsetAsync(b->B.err, 0, sizeof(int), b->B.stream);
    std::string m = "device self-check failed:";
    if (err & kDevErrRank) m += " neighbour key not in basis;";
    if (err & kDevErrBounds) m += " index out of bounds;";
    if (err & kDevErrNaN) m += " non-finite value;";
    if (err & kDevErrSpin) m += " bounded wait expired;";
    return fail(LGT_ERR_DEVICE, m);
  }
  return LGT_OK;
}

lgt_status check_device_errors(const lgt_basis* b) {
  int err = 0;
  CUDA_OR_FAIL(cudaMemcpyAsync(&err, b->B.err, sizeof(int), cudaMemcpyDeviceToHost, b->B.stream));
  CUDA_OR_FAIL(cudaStreamSynchronize(b->B.stream));
  return err_status(b, err);
}

// measure_ED's outputs from the features [K][nfeat] of observe_dev.
void fill_observables(const lgt_ham* h, const double* feat, double t_now, double* nf_grid,
                      double* E2_grid, double* plaq_grid, lgt_obs* summary) {
  const Geom& G = h->b->B.G;
  const int nf = observe_nfeat(G);
  for (int k = 0; k < h->K; ++k) {
    const double* f = feat + size_t(k) * nf;
    if (nf_grid) std::memcpy(nf_grid + size_t(k) * G.ns, f, sizeof(double) * G.ns);
    if (E2_grid) std::memcpy(E2_grid + size_t(k) * G.ns, f + G.ns, sizeof(double) * G.ns);
    if (plaq_grid && G.nP)
      std::memcpy(plaq_grid + size_t(k) * G.nP, f + 2 * G.ns, sizeof(double) * G.nP);
    if (summary) summarize_obs(G, f, t_now, summary + k);
  }
}

// The pinned staging of K feature rows and an error word (observe_dev and
// the fused ground state + observables call).
lgt_status ensure_hfeat(lgt_ham* h, size_t n) {
  if (h->hfeat_n >= n + 1) return LGT_OK;
  cudaStream_t s = h->b->B.stream;
  if (h->hfeat) {
    CUDA_OR_FAIL(cudaStreamSynchronize(s));
    pinned_put(h->hfeat, h->hfeat_n * sizeof(double));
  }
  h->hfeat = nullptr;
  h->hfeat_n = 0;
  void* p = nullptr;
  size_t cap = 0;
  CUDA_OR_FAIL(pinned_get(sizeof(double) * (n + 1), &p, &cap));
  h->hfeat = static_cast<double*>(p);
  h->hfeat_n = cap / sizeof(double);
  return LGT_OK;
}

lgt_status upload_couplings(lgt_ham* h) {
  const int K = h->K;
  // [4][K] FP64 coefficients followed by their FP32 copies, as on the device
  std::vector<double> stage(4 * size_t(K) + 2 * size_t(K));
  double* cd = stage.data();
  float* cf = reinterpret_cast<float*>(stage.data() + 4 * size_t(K));
  for (int k = 0; k < K; ++k) {
    const double g = h->g[k], t = h->t[k], m = h->m[k];
    if (!std::isfinite(g) || !std::isfinite(t) || !std::isfinite(m))
      return fail(LGT_ERR_ARG, "couplings must be finite");
    // g = 0 is a valid reference-model point (no electric energy); only the
    // plaquette's 1/(2 g^2) needs g != 0
    const bool plaq = (h->model & LGT_MODEL_PLAQ) != 0;
    if (plaq && g == 0.0) return fail(LGT_ERR_ARG, "the plaquette term needs g != 0");
    cd[k] = (g * g) / 2;             // finite_ed.jl:268,271
    cd[K + k] = m;                   // finite_ed.jl:274
    cd[2 * K + k] = -t;              // finite_ed.jl:293-294,312-313
    cd[3 * K + k] = plaq ? -(1.0 / (2.0 * (g * g))) : 0.0;  // matter_gauge_entanglement_pjw.jl:131,142-143
  }
  for (size_t i = 0; i < 4 * size_t(K); ++i) cf[i] = float(cd[i]);
  // A copy from pageable memory stages the host data before it returns, and
  // every kernel that reads the coefficients runs later on the same stream:
  // no synchronisation needed here.
  CUDA_OR_FAIL(cudaMemcpyAsync(h->coef_d, stage.data(), sizeof(double) * stage.size(),
                               cudaMemcpyHostToDevice, h->b->B.stream));
  return LGT_OK;
}

bool on_device(uint32_t flags) { return (flags & LGT_DEVICE_PTRS) != 0; }

}  // namespace

extern "C" {

void lgt_krylov_defaults(lgt_krylov_opts* o, int for_exponentiate) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->krylovdim = for_exponentiate ? 30 : 50;   // finite_ed.jl:337,418
  o->maxiter = for_exponentiate ? 100 : 300;   // finite_ed.jl:338,418
  o->tol = 1e-10;                              // finite_ed.jl:338,419
  o->precision = LGT_FP64;
  o->reorth_passes = 2;
  o->check_every = 5;
  o->refine_steps = 0;
  o->seed = 0;
  o->use_graph = 1;
  o->start_given = 0;
}

const char* lgt_last_error(void) { return g_last_error.c_str(); }

const char* lgt_version(void) { return "lgted 0.1 (sm_103a)"; }

lgt_status lgt_basis_create(int32_t nx, int32_t ny, int32_t dg, const int32_t* g_charges,
                            int32_t device, lgt_basis** out) {
  if (!out || !g_charges) return fail(LGT_ERR_ARG, "null argument");
  *out = nullptr;
  Geom G;
  std::string m = make_geom(nx, ny, dg, g_charges, &G);
  if (!m.empty()) {
    if (m.rfind("Inconsistent sector", 0) == 0) return fail(LGT_ERR_SECTOR, m);
    if (m.find("bits") != std::string::npos || m.find("31 sites") != std::string::npos)
      return fail(LGT_ERR_KEYWIDTH, m);
    return fail(LGT_ERR_ARG, m);
  }
  lgt_basis* b = new (std::nothrow) lgt_basis();
  if (!b) return fail(LGT_ERR_MEMORY, "host allocation failed");
  if (device < 0) {
    if (cudaGetDevice(&b->device) != cudaSuccess) b->device = 0;
  } else {
    b->device = device;
  }
  cudaError_t e = cudaSetDevice(b->device);
  if (e == cudaSuccess) e = stream_get(b->device, &b->B.stream);
  b->own_stream = b->B.stream;
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "lgt_basis_create");
  }
  b->B.G = G;
  m = build_basis_device(&b->B);
  if (!m.empty()) {
    free_basis_device(&b->B);
    stream_put(b->device, b->own_stream);
    delete b;
    if (m.find("memory") != std::string::npos) return fail(LGT_ERR_MEMORY, m);
    return fail(LGT_ERR_CUDA, m);
  }
  *out = b;
  return LGT_OK;
}

lgt_status lgt_basis_dim(const lgt_basis* b, int64_t* dim) {
  if (!b || !dim) return fail(LGT_ERR_ARG, "null argument");
  *dim = b->B.dim;
  return LGT_OK;
}

lgt_status lgt_basis_keys(const lgt_basis* b, int64_t first, int64_t count, uint64_t* order_keys,
                          int64_t* ref_keys) {
  if (!b) return fail(LGT_ERR_ARG, "null basis");
  if (first < 0 || count < 0 || first + count > b->B.dim) return fail(LGT_ERR_ARG, "range");
  if (ref_keys && b->B.G.dg != 1)
    return fail(LGT_ERR_UNSUPPORTED, "_encode keys exist only for dg == 1 (finite_ed.jl:89,93)");
  lgt_status st = set_device(b);
  if (st) return st;
  if (count == 0) return LGT_OK;
  cudaStream_t s = b->B.stream;
  if (order_keys)
    CUDA_OR_FAIL(cudaMemcpyAsync(order_keys, b->B.keys + first, sizeof(uint64_t) * count,
                                 cudaMemcpyDeviceToHost, s));
  if (ref_keys) {
    uint64_t* d = nullptr;
    CUDA_OR_FAIL(dev_alloc_n(&d, size_t(count), s));
    launch_ref_keys(b->B, first, count, d, s);
    CUDA_OR_FAIL(cudaGetLastError());
    CUDA_OR_FAIL(cudaMemcpyAsync(ref_keys, d, sizeof(uint64_t) * count, cudaMemcpyDeviceToHost, s));
    CUDA_OR_FAIL(dev_free(d, s));
  }
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  return LGT_OK;
}

lgt_status lgt_basis_states(const lgt_basis* b, int64_t first, int64_t count, int8_t* n_f,
                            int8_t* e_R, int8_t* e_U) {
  if (!b) return fail(LGT_ERR_ARG, "null basis");
  if (first < 0 || count < 0 || first + count > b->B.dim) return fail(LGT_ERR_ARG, "range");
  lgt_status st = set_device(b);
  if (st) return st;
  if (count == 0) return LGT_OK;
  const Geom& G = b->B.G;
  cudaStream_t s = b->B.stream;
  const size_t a = size_t(count) * G.ns, r = size_t(count) * G.nR, u = size_t(count) * G.nU;
  int8_t* d = nullptr;
  CUDA_OR_FAIL(dev_alloc_n(&d, a + r + u + 3, s));
  launch_decode_states(b->B, first, count, d, d + a, d + a + r, s);
  CUDA_OR_FAIL(cudaGetLastError());
  if (n_f) CUDA_OR_FAIL(cudaMemcpyAsync(n_f, d, a, cudaMemcpyDeviceToHost, s));
  if (e_R && r) CUDA_OR_FAIL(cudaMemcpyAsync(e_R, d + a, r, cudaMemcpyDeviceToHost, s));
  if (e_U && u) CUDA_OR_FAIL(cudaMemcpyAsync(e_U, d + a + r, u, cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(dev_free(d, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  return LGT_OK;
}

static lgt_status rank_common(const lgt_basis* b, const void* keys, int64_t n, int64_t* out,
                              bool ref) {
  if (!b || (n > 0 && (!keys || !out))) return fail(LGT_ERR_ARG, "null argument");
  if (n < 0) return fail(LGT_ERR_ARG, "negative count");
  if (ref && b->B.G.dg != 1)
    return fail(LGT_ERR_UNSUPPORTED, "_encode keys exist only for dg == 1");
  lgt_status st = set_device(b);
  if (st) return st;
  if (n == 0) return LGT_OK;
  cudaStream_t s = b->B.stream;
  uint64_t* din = nullptr;
  int64_t* dout = nullptr;
  CUDA_OR_FAIL(dev_alloc_n(&din, size_t(n), s));
  CUDA_OR_FAIL(dev_alloc_n(&dout, size_t(n), s));
  CUDA_OR_FAIL(cudaMemcpyAsync(din, keys, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, s));
  if (ref) launch_rank_ref_keys(b->B, din, n, dout, s);
  else launch_rank_order_keys(b->B, din, n, dout, s);
  CUDA_OR_FAIL(cudaGetLastError());
  CUDA_OR_FAIL(cudaMemcpyAsync(out, dout, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(dev_free(din, s));
  CUDA_OR_FAIL(dev_free(dout, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  return LGT_OK;
}

lgt_status lgt_basis_lookup(const lgt_basis* b, const int64_t* ref_keys, int64_t n,
                            int64_t* index1) {
  return rank_common(b, ref_keys, n, index1, true);
}

lgt_status lgt_basis_rank(const lgt_basis* b, const uint64_t* order_keys, int64_t n,
                          int64_t* index0) {
  return rank_common(b, order_keys, n, index0, false);
}

}  // extern "C"

namespace {
void release_basis(lgt_basis* b) {
  if (!b || b->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(b->device);
  // stream-ordered frees; the basis' own stream goes back to the device's
  // list with them queued
  free_basis_device(&b->B);
  stream_put(b->device, b->own_stream);
  delete b;
}
}  // namespace

extern "C" {

void lgt_basis_destroy(lgt_basis* b) { release_basis(b); }

lgt_status lgt_basis_set_stream(lgt_basis* b, void* stream) {
  if (!b) return fail(LGT_ERR_ARG, "null basis");
  lgt_status st = set_device(b);
  if (st) return st;
  CUDA_OR_FAIL(cudaStreamSynchronize(b->B.stream));
  b->B.stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  return LGT_OK;
}

lgt_status lgt_launch_count(uint64_t* count) {
  if (!count) return fail(LGT_ERR_ARG, "null argument");
  *count = g_launches.load();
  return LGT_OK;
}

lgt_status lgt_ham_create(const lgt_basis* b, int32_t K, const double* g, const double* t,
                          const double* m, uint32_t model, lgt_ham** out) {
  if (!b || !g || !t || !m || !out) return fail(LGT_ERR_ARG, "null argument");
  *out = nullptr;
  if (K < 1 || K > 256) return fail(LGT_ERR_ARG, "K must be in 1..256");
  if (model > LGT_MODEL_PJW) return fail(LGT_ERR_ARG, "unknown model flags");
  if (b->B.dim >= (int64_t(1) << 30))
    return fail(LGT_ERR_UNSUPPORTED, "sector dimension must be below 2^30");
  lgt_status st = set_device(b);
  if (st) return st;
  lgt_ham* h = new (std::nothrow) lgt_ham();
  if (!h) return fail(LGT_ERR_MEMORY, "host allocation failed");
  h->b = b;
  const_cast<lgt_basis*>(b)->refs.fetch_add(1);
  h->K = K;
  h->model = model;
  h->g.assign(g, g + K);
  h->t.assign(t, t + K);
  h->m.assign(m, m + K);
  h->seg_smem = hpsi_seg_smem_default(b->B.nmasks);
  // the FP64 coefficients and their FP32 copies in one allocation
  cudaError_t e = dev_alloc_n(&h->coef_d, 6 * size_t(K), b->B.stream);
  if (e == cudaSuccess) h->coef_f = reinterpret_cast<float*>(h->coef_d + 4 * size_t(K));
  if (e != cudaSuccess) {
    lgt_ham_destroy(h);
    return cuda_fail(e, "lgt_ham_create");
  }
  st = upload_couplings(h);
  if (st) {
    lgt_ham_destroy(h);
    return st;
  }
  h->cache = krylov_cache_new();
  *out = h;
  return LGT_OK;
}

lgt_status lgt_ham_set_couplings(lgt_ham* h, const double* g, const double* t, const double* m) {
  if (!h || !g || !t || !m) return fail(LGT_ERR_ARG, "null argument");
  lgt_status st = set_device(h->b);
  if (st) return st;
  std::vector<double> og = h->g, ot = h->t, om = h->m;
  h->g.assign(g, g + h->K);
  h->t.assign(t, t + h->K);
  h->m.assign(m, m + h->K);
  st = upload_couplings(h);
  if (st) {
    h->g = og;
    h->t = ot;
    h->m = om;
  }
  return st;
}

lgt_status lgt_ham_nnz(const lgt_ham* h, int64_t* nnz) {
  if (!h || !nnz) return fail(LGT_ERR_ARG, "null argument");
  lgt_status st = set_device(h->b);
  if (st) return st;
  const int64_t N = h->b->B.dim;
  cudaStream_t s = h->b->B.stream;
  int64_t* d = nullptr;
  CUDA_OR_FAIL(dev_alloc_n(&d, size_t(N) + 1, s));
  CUDA_OR_FAIL(launch_row_nnz(h->b->B.G, h->b->B.view(), h->model, d, s));
  std::vector<int64_t> c(N);
  if (N) CUDA_OR_FAIL(cudaMemcpyAsync(c.data(), d, sizeof(int64_t) * N, cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(dev_free(d, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  int64_t tot = 0;
  for (int64_t v : c) tot += v;
  *nnz = tot;
  return LGT_OK;
}

lgt_status lgt_ham_export_csr(const lgt_ham* h, int32_t k, int64_t* rowptr, int32_t* colidx,
                              double* values) {
  if (!h || !rowptr || !colidx || !values) return fail(LGT_ERR_ARG, "null argument");
  if (k < 0 || k >= h->K) return fail(LGT_ERR_ARG, "point index out of range");
  lgt_status st = set_device(h->b);
  if (st) return st;
  const int64_t N = h->b->B.dim;
  cudaStream_t s = h->b->B.stream;
  int64_t* dcnt = nullptr;
  CUDA_OR_FAIL(dev_alloc_n(&dcnt, size_t(N) + 1, s));
  CUDA_OR_FAIL(launch_row_nnz(h->b->B.G, h->b->B.view(), h->model, dcnt, s));
  std::vector<int64_t> c(N + 1, 0);
  if (N) CUDA_OR_FAIL(cudaMemcpyAsync(c.data(), dcnt, sizeof(int64_t) * N, cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  rowptr[0] = 0;
  for (int64_t i = 0; i < N; ++i) rowptr[i + 1] = rowptr[i] + c[i];
  const int64_t nnz = rowptr[N];
  int32_t* dcol = nullptr;
  double* dval = nullptr;
  CUDA_OR_FAIL(cudaMemcpyAsync(dcnt, rowptr, sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice, s));
  CUDA_OR_FAIL(dev_alloc_n(&dcol, size_t(nnz) + 1, s));
  CUDA_OR_FAIL(dev_alloc_n(&dval, size_t(nnz) + 1, s));
  CUDA_OR_FAIL(launch_row_fill(h->b->B.G, h->b->B.view(), h->model, dcnt, h->g[k], h->t[k],
                               h->m[k], dcol, dval, h->b->B.err, s));
  if (nnz) {
    CUDA_OR_FAIL(cudaMemcpyAsync(colidx, dcol, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost, s));
    CUDA_OR_FAIL(cudaMemcpyAsync(values, dval, sizeof(double) * nnz, cudaMemcpyDeviceToHost, s));
  }
  CUDA_OR_FAIL(dev_free(dcnt, s));
  CUDA_OR_FAIL(dev_free(dcol, s));
  CUDA_OR_FAIL(dev_free(dval, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  return check_device_errors(h->b);
}

lgt_status lgt_matvec(const lgt_ham* hc, const void* x, void* y, int32_t ncomp, int32_t precision,
                      uint32_t flags) {
  lgt_ham* h = const_cast<lgt_ham*>(hc);
  if (!h || !x || !y) return fail(LGT_ERR_ARG, "null argument");
  if (ncomp != 1 && ncomp != 2) return fail(LGT_ERR_ARG, "ncomp must be 1 or 2");
  if (precision != LGT_FP64 && precision != LGT_FP32)
    return fail(LGT_ERR_ARG, "matvec precision must be LGT_FP64 or LGT_FP32");
  lgt_status st = set_device(h->b);
  if (st) return st;
  const int64_t N = h->b->B.dim;
  const size_t es = precision == LGT_FP64 ? 8 : 4;
  const size_t bytes = size_t(N) * h->K * ncomp * es;
  cudaStream_t s = h->b->B.stream;
  const void* dx = x;
  void* dy = y;
  if (!on_device(flags)) {
    CUDA_OR_FAIL(h->x.need(bytes, h->b->B.stream));
    CUDA_OR_FAIL(h->y.need(bytes, h->b->B.stream));
    CUDA_OR_FAIL(cudaMemcpyAsync(h->x.p, x, bytes, cudaMemcpyHostToDevice, s));
    dx = h->x.p;
    dy = h->y.p;
  }
  OpDev op = h->op();
  op.force_generic = (flags & LGT_GENERIC_KERNELS) ? 1 : 0;
  if (flags & LGT_ROW_ORDER) {
    if (!on_device(flags) || op.force_generic)
      return fail(LGT_ERR_ARG, "LGT_ROW_ORDER needs LGT_DEVICE_PTRS and the table kernel");
    // the tuner's load mode when it chose the table kernel, else the built-in one
    std::string m =
        (precision == LGT_FP64)
            ? hpsi_choose_d(&op, static_cast<const double*>(dx), static_cast<double*>(dy), ncomp, s)
            : hpsi_choose_f(&op, static_cast<const float*>(dx), static_cast<float*>(dy), ncomp, s);
    if (!m.empty()) return from_msg(m);
    if (!op.use_table) op.vpl = 0;
    m = ensure_row_order(&op, s);
    if (!m.empty()) return fail(LGT_ERR_UNSUPPORTED, m);
  } else if (!op.force_generic) {  // the autotuner's kernel for this shape (timed on first use)
    std::string m =
        (precision == LGT_FP64)
            ? hpsi_choose_d(&op, static_cast<const double*>(dx), static_cast<double*>(dy), ncomp, s)
            : hpsi_choose_f(&op, static_cast<const float*>(dx), static_cast<float*>(dy), ncomp, s);
    if (!m.empty()) return from_msg(m);
  }
  cudaError_t e = (precision == LGT_FP64)
                      ? apply_h_d(op, static_cast<const double*>(dx), static_cast<double*>(dy), ncomp, s)
                      : apply_h_f(op, static_cast<const float*>(dx), static_cast<float*>(dy), ncomp, s);
  if (e != cudaSuccess) return cuda_fail(e, "lgt_matvec");
  if (on_device(flags) && (flags & LGT_ASYNC)) return LGT_OK;
  if (!on_device(flags)) CUDA_OR_FAIL(cudaMemcpyAsync(y, dy, bytes, cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  return check_device_errors(h->b);
}

lgt_status lgt_ham_row_order(lgt_ham* h, int32_t* perm) {
  if (!h) return fail(LGT_ERR_ARG, "null argument");
  lgt_status st = set_device(h->b);
  if (st) return st;
  OpDev op = h->op();
  cudaStream_t s = h->b->B.stream;
  std::string m = ensure_row_order(&op, s);
  if (!m.empty()) return fail(LGT_ERR_UNSUPPORTED, m);
  if (perm) {
    CUDA_OR_FAIL(cudaMemcpyAsync(perm, h->table_ord.perm, sizeof(int32_t) * h->b->B.dim,
                                 cudaMemcpyDeviceToHost, s));
    CUDA_OR_FAIL(cudaStreamSynchronize(s));
  }
  return check_device_errors(h->b);
}

static KrylovParams to_params(const lgt_krylov_opts* o, int for_exp) {
  lgt_krylov_opts d;
  lgt_krylov_defaults(&d, for_exp);
  if (!o) o = &d;
  KrylovParams p;
  p.krylovdim = o->krylovdim > 0 ? o->krylovdim : d.krylovdim;
  p.maxiter = o->maxiter >= 0 ? o->maxiter : d.maxiter;
  p.tol = o->tol > 0 ? o->tol : d.tol;
  p.mixed = (o->precision == LGT_FP32_MIXED || o->precision == LGT_FP32) ? 1 : 0;
  p.reorth = o->reorth_passes > 0 ? o->reorth_passes : d.reorth_passes;
  p.check_every = o->check_every > 0 ? o->check_every : d.check_every;
  p.refine = o->refine_steps > 0 ? o->refine_steps : 0;
  p.seed = o->seed;
  p.use_graph = o->use_graph;
  p.start_given = o->start_given;
  return p;
}

}  // extern "C"

namespace {

bool use_cta(const lgt_ham* h, const lgt_krylov_opts* opts, const KrylovParams& p) {
  const int solver = opts ? opts->solver : LGT_SOLVER_AUTO;
  if (solver == LGT_SOLVER_PANEL) return false;
  const bool fits = h->b->B.dim <= kSmallMaxN && p.krylovdim <= 63;
  return fits && (solver == LGT_SOLVER_CTA || solver == LGT_SOLVER_AUTO);
}

lgt_status ensure_pattern(lgt_ham* h) {
  if (h->pattern.rowptr) return LGT_OK;
  std::string m = build_pattern(h->b->B, h->model, &h->pattern, h->b->B.stream);
  if (!m.empty()) {
    free_pattern(&h->pattern, h->b->B.stream);
    return from_msg(m);
  }
  return LGT_OK;
}

SmallParams small_params(const KrylovParams& p) {
  SmallParams q;
  q.m = p.krylovdim;
  q.maxiter = p.maxiter;
  q.tol = p.tol;
  q.reorth = p.reorth;
  q.check_every = p.check_every;
  q.seed = p.seed;
  q.start_given = p.start_given;
  // launch shape of the per-CTA solver: rows held per thread (LGT_CTA_ROWS
  // overrides the built-in choice, the smallest that fits 512 threads)
  if (const char* e = getenv("LGT_CTA_ROWS")) q.rows_per_thread = atoi(e);
  return q;
}

// Per-CTA solves of several Hamiltonians (device panels X[i]).
lgt_status cta_solve(const std::vector<lgt_ham*>& hams, const KrylovParams& p,
                     const std::vector<double*>& X, double* const* E0, double* const* residual,
                     lgt_info* info, const std::function<cudaError_t()>& before_sync = {}) {
  std::vector<SmallJob> jobs;
  std::vector<std::vector<double>> coef(hams.size());
  std::vector<std::vector<int>> steps(hams.size()), rest(hams.size());
  std::vector<std::unique_ptr<bool[]>> conv(hams.size());
  for (size_t i = 0; i < hams.size(); ++i) {
    lgt_ham* h = hams[i];
    lgt_status st = ensure_pattern(h);
    if (st) return st;
    const int K = h->K;
    coef[i].resize(4 * size_t(K));
    for (int k = 0; k < K; ++k) {
      const double g = h->g[k], t = h->t[k], m = h->m[k];
      coef[i][k] = (g * g) / 2;
      coef[i][K + k] = m;
      coef[i][2 * K + k] = -t;
      coef[i][3 * K + k] = (h->model & LGT_MODEL_PLAQ) ? -(1.0 / (2.0 * (g * g))) : 0.0;
    }
    steps[i].assign(K, 0);
    rest[i].assign(K, 0);
    conv[i].reset(new bool[K]);
    SmallJob J;
    J.pattern = &h->pattern;
    J.K = K;
    J.cE = coef[i].data();
    J.cm = coef[i].data() + K;
    J.ch = coef[i].data() + 2 * K;
    J.cp = coef[i].data() + 3 * K;
    J.psi = X[i];
    J.E0 = E0[i];
    J.resid = residual ? residual[i] : nullptr;
    J.steps = steps[i].data();
    J.restarts = rest[i].data();
    J.converged = conv[i].get();
    jobs.push_back(J);
  }
  lgt_ham* h0 = hams[0];
  double secs = 0.0;
  // one basis for all jobs: its error word rides on the solve's own
  // synchronisation
  bool one_basis = true;
  for (lgt_ham* hh : hams) one_basis = one_basis && hh->b == h0->b;
  int dev_err = 0;
  const bool refine = p.mixed && p.refine > 0;
  std::string m = small_ground_states(jobs, small_params(p), p.mixed, &h0->small,
                                      h0->b->B.stream, &secs,
                                      one_basis ? h0->b->B.err : nullptr, &dev_err,
                                      refine ? std::function<cudaError_t()>() : before_sync);
  if (!m.empty()) return from_msg(m);
  if (p.mixed && p.refine > 0) {
    // FP64 correction: a short FP64 Lanczos per point (Krylov dimension
    // refine_steps, restarted up to maxiter) started from the FP32-mixed
    // solution, which the first launch left normalised in the panels; the
    // energy becomes the FP64 Ritz value and the state FP64-accurate.
    std::vector<std::vector<int>> steps2(hams.size()), rest2(hams.size());
    for (size_t i = 0; i < hams.size(); ++i) {
      steps2[i].assign(hams[i]->K, 0);
      rest2[i].assign(hams[i]->K, 0);
      jobs[i].steps = steps2[i].data();
      jobs[i].restarts = rest2[i].data();
    }
    SmallParams q = small_params(p);
    q.m = p.refine;
    if (q.check_every > q.m) q.check_every = q.m;
    q.start_given = 1;
    q.rows_per_thread = 0;
    double secs2 = 0.0;
    m = small_ground_states(jobs, q, 0, &h0->small, h0->b->B.stream, &secs2,
                            one_basis ? h0->b->B.err : nullptr, &dev_err, before_sync);
    if (!m.empty()) return from_msg(m);
    secs += secs2;
    for (size_t i = 0; i < hams.size(); ++i)
      for (int k = 0; k < hams[i]->K; ++k) {
        steps[i][k] += steps2[i][k];
        rest[i][k] += rest2[i][k];
      }
  }
  int nconv = 0, maxsteps = 0, maxrest = 0;
  double maxr = 0.0;
  bool all = true;
  for (size_t i = 0; i < hams.size(); ++i)
    for (int k = 0; k < hams[i]->K; ++k) {
      nconv += conv[i][k] ? 1 : 0;
      all = all && conv[i][k];
      maxsteps = std::max(maxsteps, steps[i][k]);
      maxrest = std::max(maxrest, rest[i][k]);
      if (residual) maxr = std::max(maxr, residual[i][k]);
    }
  if (info) {
    info->matvecs = maxsteps + 1;
    info->restarts = maxrest;
    info->converged = nconv;
    info->max_residual = maxr;
    info->seconds = secs;
  }
  if (one_basis) {
    lgt_status de = err_status(h0->b, dev_err);
    if (de) return de;
  } else {
    for (lgt_ham* h : hams) {
      lgt_status de = check_device_errors(h->b);
      if (de) return de;
    }
  }
  if (!all) return fail(LGT_ERR_NOCONV, "NOCONV: Lanczos did not converge within maxiter restarts");
  return LGT_OK;
}

}  // namespace

extern "C" {

lgt_status lgt_ground_state(lgt_ham* h, const lgt_krylov_opts* opts, double* E0, void* psi,
                            double* residual, uint32_t flags, lgt_info* info) {
  if (!h || !E0) return fail(LGT_ERR_ARG, "null argument");
  KrylovParams p = to_params(opts, 0);
  if (p.check_every > p.krylovdim) p.check_every = p.krylovdim;
  if (p.start_given && !psi) return fail(LGT_ERR_ARG, "start_given needs psi");
  lgt_status st = set_device(h->b);
  if (st) return st;
  const int64_t N = h->b->B.dim;
  if (N == 0) return fail(LGT_ERR_ARG, "empty basis");
  const size_t bytes = size_t(N) * h->K * sizeof(double);
  cudaStream_t s = h->b->B.stream;
  double* X = nullptr;
  if (psi && on_device(flags)) {
    X = static_cast<double*>(psi);
  } else {
    CUDA_OR_FAIL(h->x.need(bytes, h->b->B.stream));
    X = static_cast<double*>(h->x.p);
    if (p.start_given) CUDA_OR_FAIL(cudaMemcpyAsync(X, psi, bytes, cudaMemcpyHostToDevice, s));
  }
  std::vector<double> res(h->K);
  if (use_cta(h, opts, p)) {
    double* r = res.data();
    // a host psi is copied back behind the solve, before its one
    // synchronisation (on an error status its contents are unspecified)
    const bool host_psi = psi && !on_device(flags);
    auto copy_back = [&]() -> cudaError_t {
      return host_psi ? cudaMemcpyAsync(psi, X, bytes, cudaMemcpyDeviceToHost, s) : cudaSuccess;
    };
    lgt_status rc = cta_solve({h}, p, {X}, &E0, &r, info, copy_back);
    if (residual) std::memcpy(residual, res.data(), sizeof(double) * h->K);
    return rc;
  }
  KrylovReport rep;
  std::string m = lanczos_ground_state(h->op(), p, h->cache, X, E0, res.data(), s, &rep);
  if (residual) std::memcpy(residual, res.data(), sizeof(double) * h->K);
  if (info) {
    info->matvecs = rep.matvecs;
    info->restarts = rep.restarts;
    info->converged = rep.converged;
    info->max_residual = rep.max_residual;
    info->seconds = rep.seconds;
  }
  lgt_status rc = from_msg(m);
  if (rc != LGT_OK && rc != LGT_ERR_NOCONV) return rc;
  if (psi && !on_device(flags))
    CUDA_OR_FAIL(cudaMemcpyAsync(psi, X, bytes, cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  lgt_status de = check_device_errors(h->b);
  if (de) return de;
  if (rc == LGT_ERR_NOCONV) return fail(LGT_ERR_NOCONV, m);
  return LGT_OK;
}

lgt_status lgt_ground_state_observe(lgt_ham* h, const lgt_krylov_opts* opts, double* E0,
                                    void* psi, double* residual, uint32_t flags, lgt_info* info,
                                    double* nf_grid, double* E2_grid, double* plaq_grid,
                                    lgt_obs* summary) {
  if (!h || !E0) return fail(LGT_ERR_ARG, "null argument");
  KrylovParams p = to_params(opts, 0);
  if (p.check_every > p.krylovdim) p.check_every = p.krylovdim;
  if (p.start_given && !psi) return fail(LGT_ERR_ARG, "start_given needs psi");
  lgt_status st = set_device(h->b);
  if (st) return st;
  if (!use_cta(h, opts, p)) {
    // the panel solver: the two calls in turn (the state stays where it is)
    lgt_status rc = lgt_ground_state(h, opts, E0, psi, residual, flags, info);
    if (rc != LGT_OK && rc != LGT_ERR_NOCONV) return rc;
    if (!psi) return rc;
    lgt_status ro = lgt_observe(h, psi, 1, LGT_FP64, flags, 0.0, nf_grid, E2_grid, plaq_grid,
                                summary);
    return ro ? ro : rc;
  }
  const int64_t N = h->b->B.dim;
  if (N == 0) return fail(LGT_ERR_ARG, "empty basis");
  const size_t bytes = size_t(N) * h->K * sizeof(double);
  cudaStream_t s = h->b->B.stream;
  double* X = nullptr;
  if (psi && on_device(flags)) {
    X = static_cast<double*>(psi);
  } else {
    CUDA_OR_FAIL(h->x.need(bytes, h->b->B.stream));
    X = static_cast<double*>(h->x.p);
    if (p.start_given) CUDA_OR_FAIL(cudaMemcpyAsync(X, psi, bytes, cudaMemcpyHostToDevice, s));
  }
  const Geom& G = h->b->B.G;
  const int nf = observe_nfeat(G);
  int nblk;
  int64_t rpb;
  observe_plan(N, &nblk, &rpb);
  CUDA_OR_FAIL(h->part.need(sizeof(double) * size_t(nblk) * h->K * nf, s));
  CUDA_OR_FAIL(h->out.need(sizeof(double) * size_t(h->K) * nf, s));
  const size_t n = size_t(h->K) * nf;
  st = ensure_hfeat(h, n);
  if (st) return st;
  int* herr = reinterpret_cast<int*>(h->hfeat + n);
  // the observables of the solution, launched before the solve's one
  // synchronisation
  auto observe = [&]() -> cudaError_t {
    cudaError_t e = launch_observe_planned<double>(G, h->b->B.view(), X, h->K, 1, nblk, rpb,
                                                   static_cast<double*>(h->part.p),
                                                   static_cast<double*>(h->out.p), h->b->B.err, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->hfeat, h->out.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(herr, h->b->B.err, sizeof(int), cudaMemcpyDeviceToHost, s);
    return e;
  };
  std::vector<double> res(h->K);
  double* r = res.data();
  lgt_status rc = cta_solve({h}, p, {X}, &E0, &r, info, observe);
  if (residual) std::memcpy(residual, res.data(), sizeof(double) * h->K);
  if (rc != LGT_OK && rc != LGT_ERR_NOCONV) return rc;
  lgt_status de = err_status(h->b, *herr);
  if (de) return de;
  fill_observables(h, h->hfeat, 0.0, nf_grid, E2_grid, plaq_grid, summary);
  if (psi && !on_device(flags)) {
    CUDA_OR_FAIL(cudaMemcpyAsync(psi, X, bytes, cudaMemcpyDeviceToHost, s));
    CUDA_OR_FAIL(cudaStreamSynchronize(s));
  }
  return rc;
}

lgt_status lgt_ground_state_batch(int32_t nham, lgt_ham* const* hams, const lgt_krylov_opts* opts,
                                  double* const* E0, void* const* psi, double* const* residual,
                                  uint32_t flags, lgt_info* info) {
  if (nham < 1 || !hams || !E0) return fail(LGT_ERR_ARG, "null argument");
  for (int i = 0; i < nham; ++i) {
    if (!hams[i] || !E0[i]) return fail(LGT_ERR_ARG, "null Hamiltonian or E0");
    if (hams[i]->b->device != hams[0]->b->device)
      return fail(LGT_ERR_ARG, "all Hamiltonians must live on one device");
    if (psi && psi[i] && !on_device(flags))
      return fail(LGT_ERR_ARG, "lgt_ground_state_batch takes device psi panels");
  }
  KrylovParams p = to_params(opts, 0);
  if (p.check_every > p.krylovdim) p.check_every = p.krylovdim;
  lgt_status st = set_device(hams[0]->b);
  if (st) return st;
  std::vector<lgt_ham*> small;
  std::vector<double*> xs;
  std::vector<double*> e0s, rs;
  std::vector<int> large;
  for (int i = 0; i < nham; ++i) {
    lgt_ham* h = hams[i];
    const size_t bytes = size_t(h->b->B.dim) * h->K * sizeof(double);
    if (use_cta(h, opts, p)) {
      double* X = (psi && psi[i]) ? static_cast<double*>(psi[i]) : nullptr;
      if (!X) {
        CUDA_OR_FAIL(h->x.need(bytes, h->b->B.stream));
        X = static_cast<double*>(h->x.p);
      }
      small.push_back(h);
      xs.push_back(X);
      e0s.push_back(E0[i]);
      rs.push_back(residual ? residual[i] : nullptr);
    } else {
      large.push_back(i);
    }
  }
  lgt_info tot;
  std::memset(&tot, 0, sizeof(tot));
  lgt_status worst = LGT_OK;
  // The one-CTA-per-point launch of the small sectors runs on its own host
  // thread (and its basis' stream) while the large sectors' panel solves
  // run here, so the two overlap on the GPU.
  std::vector<std::vector<double>> rbuf(small.size());
  std::vector<double*> rp(small.size());
  for (size_t i = 0; i < small.size(); ++i) {
    rbuf[i].resize(small[i]->K);
    rp[i] = rs[i] ? rs[i] : rbuf[i].data();
  }
  lgt_info small_info;
  std::memset(&small_info, 0, sizeof(small_info));
  lgt_status small_rc = LGT_OK;
  std::string small_err;
  auto run_small = [&]() {
    if (set_device(small[0]->b) != LGT_OK) {
      small_rc = LGT_ERR_CUDA;
      small_err = lgt_last_error();
      return;
    }
    small_rc = cta_solve(small, p, xs, e0s.data(), rp.data(), &small_info);
    if (small_rc != LGT_OK) small_err = lgt_last_error();
  };
  std::thread small_thread;
  if (!small.empty()) {
    if (large.empty())
      run_small();
    else
      small_thread = std::thread(run_small);
  }
  lgt_status large_rc = LGT_OK;
  for (int i : large) {
    lgt_info one;
    std::memset(&one, 0, sizeof(one));
    lgt_status rc = lgt_ground_state(hams[i], opts, E0[i], psi ? psi[i] : nullptr,
                                     residual ? residual[i] : nullptr, flags, &one);
    if (rc != LGT_OK && rc != LGT_ERR_NOCONV) {
      large_rc = rc;
      break;
    }
    if (rc) worst = rc;
    tot.matvecs = std::max(tot.matvecs, one.matvecs);
    tot.restarts = std::max(tot.restarts, one.restarts);
    tot.converged += one.converged;
    tot.max_residual = std::max(tot.max_residual, one.max_residual);
    tot.seconds += one.seconds;
  }
  const std::string large_err = large_rc ? std::string(lgt_last_error()) : std::string();
  if (small_thread.joinable()) small_thread.join();
  if (small_rc != LGT_OK && small_rc != LGT_ERR_NOCONV) return fail(small_rc, small_err);
  if (large_rc) return fail(large_rc, large_err);
  if (small_rc) worst = small_rc;
  if (!small.empty()) {
    tot.matvecs = std::max(tot.matvecs, small_info.matvecs);
    tot.restarts = std::max(tot.restarts, small_info.restarts);
    tot.converged += small_info.converged;
    tot.max_residual = std::max(tot.max_residual, small_info.max_residual);
    tot.seconds = std::max(tot.seconds, small_info.seconds);
  }
  if (info) *info = tot;
  if (worst) return fail(worst, "NOCONV: some points did not converge within maxiter restarts");
  return LGT_OK;
}

}  // extern "C"

void lgt::set_last_error(const std::string& msg) { g_last_error = msg; }


namespace {

template <typename T>
lgt_status observe_dev(lgt_ham* h, const T* x, int ncomp, std::vector<double>* feat) {
  const Geom& G = h->b->B.G;
  const int nf = observe_nfeat(G);
  int nblk;
  int64_t rpb;
  observe_plan(h->b->B.dim, &nblk, &rpb);
  CUDA_OR_FAIL(h->part.need(sizeof(double) * size_t(nblk) * h->K * nf, h->b->B.stream));
  CUDA_OR_FAIL(h->out.need(sizeof(double) * size_t(h->K) * nf, h->b->B.stream));
  cudaStream_t s = h->b->B.stream;
  cudaError_t e = launch_observe<T>(G, h->b->B.view(), x, h->K, ncomp,
                                    static_cast<double*>(h->part.p), static_cast<double*>(h->out.p),
                                    h->b->B.err, s);
  if (e != cudaSuccess) return cuda_fail(e, "observe");
  // features and the device error word back through pinned memory, one
  // synchronisation
  const size_t n = size_t(h->K) * nf;
  {
    lgt_status hs = ensure_hfeat(h, n);  // the features, then the error word
    if (hs) return hs;
  }
  int* herr = reinterpret_cast<int*>(h->hfeat + n);
  CUDA_OR_FAIL(cudaMemcpyAsync(h->hfeat, h->out.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(cudaMemcpyAsync(herr, h->b->B.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  feat->assign(h->hfeat, h->hfeat + n);
  return err_status(h->b, *herr);
}

// Observables after every step: the summaries and, where asked for, the
// site grids of that step (finite_ed.jl:409,421-422 keep measure_ED's whole
// record, grids included, for every step).
struct ObsRecorder : StepObserver {
  lgt_ham* h = nullptr;
  lgt_obs* obs = nullptr;
  double* nf_grid = nullptr;
  double* E2_grid = nullptr;
  double* plaq_grid = nullptr;
  double dt = 0.0;
  bool wanted() const { return obs || nf_grid || E2_grid || plaq_grid; }
  std::string on_step(int step, const double* X) override {
    if (!wanted()) return std::string();
    std::vector<double> feat;
    if (observe_dev<double>(h, X, 2, &feat) != LGT_OK) return std::string(lgt_last_error());
    const Geom& G = h->b->B.G;
    const int nf = observe_nfeat(G);
    for (int k = 0; k < h->K; ++k) {
      const double* f = feat.data() + size_t(k) * nf;
      const size_t rec = size_t(step) * h->K + k;
      if (obs) summarize_obs(G, f, step * dt, obs + rec);
      if (nf_grid) std::memcpy(nf_grid + rec * G.ns, f, sizeof(double) * G.ns);
      if (E2_grid) std::memcpy(E2_grid + rec * G.ns, f + G.ns, sizeof(double) * G.ns);
      if (plaq_grid && G.nP) std::memcpy(plaq_grid + rec * G.nP, f + 2 * G.ns, sizeof(double) * G.nP);
    }
    return std::string();
  }
};

}  // namespace

extern "C" {

lgt_status lgt_expm_steps(lgt_ham* h, const lgt_krylov_opts* opts, double dt, int32_t n_steps,
                          void* psi, lgt_obs* obs, double* norm_drift, uint32_t flags,
                          lgt_info* info) {
  return lgt_expm_steps_grids(h, opts, dt, n_steps, psi, obs, nullptr, nullptr, nullptr,
                              norm_drift, flags, info);
}

lgt_status lgt_expm_steps_grids(lgt_ham* h, const lgt_krylov_opts* opts, double dt,
                                int32_t n_steps, void* psi, lgt_obs* obs, double* nf_grid,
                                double* E2_grid, double* plaq_grid, double* norm_drift,
                                uint32_t flags, lgt_info* info) {
  if (!h || !psi) return fail(LGT_ERR_ARG, "null argument");
  if (n_steps < 0 || !std::isfinite(dt)) return fail(LGT_ERR_ARG, "bad dt or n_steps");
  KrylovParams p = to_params(opts, 1);
  if (p.check_every > p.krylovdim) p.check_every = p.krylovdim;
  lgt_status st = set_device(h->b);
  if (st) return st;
  const int64_t N = h->b->B.dim;
  const size_t bytes = size_t(N) * h->K * 2 * sizeof(double);
  cudaStream_t s = h->b->B.stream;
  double* X = nullptr;
  if (on_device(flags)) {
    X = static_cast<double*>(psi);
  } else {
    CUDA_OR_FAIL(h->y.need(bytes, h->b->B.stream));
    X = static_cast<double*>(h->y.p);
    CUDA_OR_FAIL(cudaMemcpyAsync(X, psi, bytes, cudaMemcpyHostToDevice, s));
  }
  ObsRecorder rec;
  rec.h = h;
  rec.obs = obs;
  rec.nf_grid = nf_grid;
  rec.E2_grid = E2_grid;
  rec.plaq_grid = plaq_grid;
  rec.dt = dt;
  KrylovReport rep;
  std::string m = krylov_expm(h->op(), p, h->cache, dt, n_steps, X, norm_drift,
                              rec.wanted() ? &rec : nullptr, s, &rep);
  if (info) {
    info->matvecs = rep.matvecs;
    info->restarts = rep.restarts;
    info->converged = rep.converged;
    info->max_residual = rep.max_residual;
    info->seconds = rep.seconds;
  }
  lgt_status rc = from_msg(m);
  if (rc) return rc;
  if (!on_device(flags)) CUDA_OR_FAIL(cudaMemcpyAsync(psi, X, bytes, cudaMemcpyDeviceToHost, s));
  CUDA_OR_FAIL(cudaStreamSynchronize(s));
  return check_device_errors(h->b);
}

lgt_status lgt_observe(const lgt_ham* hc, const void* psi, int32_t ncomp, int32_t precision,
                       uint32_t flags, double t_now, double* nf_grid, double* E2_grid,
                       double* plaq_grid, lgt_obs* summary) {
  lgt_ham* h = const_cast<lgt_ham*>(hc);
  if (!h || !psi) return fail(LGT_ERR_ARG, "null argument");
  if (ncomp != 1 && ncomp != 2) return fail(LGT_ERR_ARG, "ncomp must be 1 or 2");
  if (precision != LGT_FP64 && precision != LGT_FP32)
    return fail(LGT_ERR_ARG, "precision must be LGT_FP64 or LGT_FP32");
  lgt_status st = set_device(h->b);
  if (st) return st;
  const Geom& G = h->b->B.G;
  const int64_t N = h->b->B.dim;
  const size_t es = precision == LGT_FP64 ? 8 : 4;
  const size_t bytes = size_t(N) * h->K * ncomp * es;
  cudaStream_t s = h->b->B.stream;
  const void* dx = psi;
  if (!on_device(flags)) {
    CUDA_OR_FAIL(h->x.need(bytes, h->b->B.stream));
    CUDA_OR_FAIL(cudaMemcpyAsync(h->x.p, psi, bytes, cudaMemcpyHostToDevice, s));
    dx = h->x.p;
  }
  std::vector<double> feat;
  st = (precision == LGT_FP64) ? observe_dev<double>(h, static_cast<const double*>(dx), ncomp, &feat)
                               : observe_dev<float>(h, static_cast<const float*>(dx), ncomp, &feat);
  if (st) return st;
  fill_observables(h, feat.data(), t_now, nf_grid, E2_grid, plaq_grid, summary);
  return LGT_OK;  // observe_dev read the device error word
}

lgt_status lgt_energy(const lgt_ham* hc, const void* psi, int32_t ncomp, uint32_t flags,
                      double* energy) {
  lgt_ham* h = const_cast<lgt_ham*>(hc);
  if (!h || !psi || !energy) return fail(LGT_ERR_ARG, "null argument");
  if (ncomp != 1 && ncomp != 2) return fail(LGT_ERR_ARG, "ncomp must be 1 or 2");
  lgt_status st = set_device(h->b);
  if (st) return st;
  const int64_t N = h->b->B.dim;
  const size_t bytes = size_t(N) * h->K * ncomp * sizeof(double);
  cudaStream_t s = h->b->B.stream;
  CUDA_OR_FAIL(h->y.need(bytes, h->b->B.stream));
  const double* dx = static_cast<const double*>(psi);
  if (!on_device(flags)) {
    CUDA_OR_FAIL(h->x.need(bytes, h->b->B.stream));
    CUDA_OR_FAIL(cudaMemcpyAsync(h->x.p, psi, bytes, cudaMemcpyHostToDevice, s));
    dx = static_cast<const double*>(h->x.p);
  }
  double* dy = static_cast<double*>(h->y.p);
  cudaError_t e = apply_h_d(h->op(), dx, dy, ncomp, s);
  if (e != cudaSuccess) return cuda_fail(e, "lgt_energy");
  std::vector<double> num(h->K), den(h->K);
  std::string m = panel_dots(h->cache, dx, dy, N, h->K, ncomp, num.data(), s);
  if (m.empty()) m = panel_dots(h->cache, dx, dx, N, h->K, ncomp, den.data(), s);
  if (!m.empty()) return from_msg(m);
  for (int k = 0; k < h->K; ++k) energy[k] = num[k] / den[k];
  return check_device_errors(h->b);
}

lgt_status lgt_autotune(lgt_ham* h, int32_t ncomp, int32_t precision, lgt_tuning* out) {
  if (!h || !out) return fail(LGT_ERR_ARG, "null argument");
  if (ncomp != 1 && ncomp != 2) return fail(LGT_ERR_ARG, "ncomp must be 1 or 2");
  if (precision != LGT_FP64 && precision != LGT_FP32 && precision != LGT_FP32_MIXED)
    return fail(LGT_ERR_ARG, "unknown precision");
  lgt_status st = set_device(h->b);
  if (st) return st;
  TuneChoice c;
  std::string m = krylov_autotune(h->op(), h->cache, ncomp, precision != LGT_FP64 ? 1 : 0,
                                  h->b->B.stream, &c);
  if (!m.empty()) return from_msg(m);
  out->hpsi_kernel = c.hpsi_variant;
  out->reduce_blocks = c.red_blocks;
  out->hpsi_ms = c.hpsi_ms;
  out->reduce_ms = c.red_ms;
  out->measured = c.measured;
  return check_device_errors(h->b);
}

void lgt_ham_destroy(lgt_ham* h) {
  if (!h) return;
  // pool buffers are freed in stream order on the basis' stream; the Krylov
  // workspaces and the neighbour tables (plain device allocations) are freed
  // by cudaFree, which waits for the device
  cudaStream_t s = h->b ? h->b->B.stream : nullptr;
  if (h->b) cudaSetDevice(h->b->device);
  krylov_cache_free(h->cache);
  h->x.release(s);
  h->y.release(s);
  h->part.release(s);
  h->out.release(s);
  free_pattern(&h->pattern, s);
  free_nbr_table(&h->table);
  free_nbr_table(&h->table_ord);
  free_small_work(&h->small, s);
  if (h->hfeat) {
    if (s) cudaStreamSynchronize(s);
    pinned_put(h->hfeat, h->hfeat_n * sizeof(double));
  }
  dev_free(h->coef_d, s);  // coef_f lives in the same allocation
  lgt_basis* b = const_cast<lgt_basis*>(h->b);
  delete h;
  release_basis(b);
}

}  // extern "C"
