// noalloc.cu -- lgt_observe_noalloc: the observables reduction of
// lgt_observe without any device allocation.
//
// Some callers of this library cannot call cudaMalloc: applications that
// reserve the whole device memory up front for their own pool or arena (a
// framework's caching allocator, a Julia CUDA.jl memory pool) and leave no
// room for a library to allocate behind their back, and time-critical loops
// that must not trigger the implicit device synchronisation an allocation
// or a free may cause.  lgt_observe needs per-block partial sums and a
// result buffer on the device and takes them from a growable buffer owned
// by the Hamiltonian handle (allocated on first use).  This entry point
// computes the same observables with its scratch held in a file-scope
// static __device__ array instead, so it never allocates: the caller passes
// the state (a device panel) and the host output arrays.
//
// Limits and rules of use:
//  * Scratch size is fixed at kScratchDoubles doubles (2 MiB) per device.
//    The block partition of the reduction is shrunk to fit it; a call whose
//    per-block share alone does not fit ((K * nfeat) * 2 + 8 K doubles, with
//    nfeat = 2 nx ny + (nx-1)(ny-1) + 1) is rejected with LGT_ERR_ARG.  Every
//    GPU that loads the library holds this array until the process exits.
//  * The scratch is shared by every call on a device and keeps the last
//    call's contents.  Nothing in it needs to start at zero: every partial
//    sum and every result is written before it is read.  Calls that overlap
//    on the GPU (two host threads, or two streams) race on it.
//  * The first call on a device looks up the array's device address once
//    (cudaGetSymbolAddress with that device current); make that first call
//    before any stream capture on the device.
#include <cmath>
#include <mutex>

#include "lgt_handles.h"
#include "lgt_observe.h"

namespace {

constexpr size_t kScratchDoubles = size_t(1) << 18;  // 2 MiB of doubles
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current).
cudaError_t scratch_address(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

// Per-point summaries (lgt::summarize_obs, shared with lgt_observe), one
// thread per point, straight into the scratch.
__global__ void k_summarize(lgt::Geom G, const double* feat, int K, int nfeat, double t_now,
                            lgt_obs* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  lgt::summarize_obs(G, feat + size_t(k) * nfeat, t_now, out + k);
}

lgt_status fail_na(lgt_status code, const std::string& msg) {
  lgt::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" {

lgt_status lgt_observe_noalloc(const lgt_ham* h, const void* psi, int32_t ncomp,
                               int32_t precision, double t_now, double* nf_grid, double* E2_grid,
                               double* plaq_grid, lgt_obs* summary) {
  if (!h || !psi) return fail_na(LGT_ERR_ARG, "null argument");
  if (ncomp != 1 && ncomp != 2) return fail_na(LGT_ERR_ARG, "ncomp must be 1 or 2");
  if (precision != LGT_FP64 && precision != LGT_FP32)
    return fail_na(LGT_ERR_ARG, "precision must be LGT_FP64 or LGT_FP32");
  const lgt_basis* b = h->b;
  cudaError_t e = cudaSetDevice(b->device);
  if (e != cudaSuccess) return fail_na(LGT_ERR_CUDA, cudaGetErrorString(e));
  cudaPointerAttributes attr;
  e = cudaPointerGetAttributes(&attr, psi);
  if (e != cudaSuccess || attr.type != cudaMemoryTypeDevice || attr.device != b->device)
    return fail_na(LGT_ERR_ARG, "psi must be a device pointer on the basis' device");
  const lgt::Geom& G = b->B.G;
  const int K = h->K;
  const int nfeat = lgt::observe_nfeat(G);
  const size_t per_block = size_t(K) * nfeat;
  const size_t fixed = per_block + 8 * size_t(K);  // results + summaries
  if (per_block + fixed > kScratchDoubles)
    return fail_na(LGT_ERR_ARG, "K * features exceeds the 2 MiB scratch of lgt_observe_noalloc");
  double* scratch = nullptr;
  e = scratch_address(b->device, &scratch);
  if (e != cudaSuccess) return fail_na(LGT_ERR_CUDA, std::string("scratch set-up: ") + cudaGetErrorString(e));
  int nblk;
  int64_t rpb;
  lgt::observe_plan(b->B.dim, &nblk, &rpb);
  const int fit = int((kScratchDoubles - fixed) / per_block);
  if (nblk > fit) {
    nblk = fit;
    rpb = (b->B.dim + nblk - 1) / nblk;
    nblk = int((b->B.dim + rpb - 1) / rpb);
  }
  double* part = scratch;
  double* feat = scratch + size_t(nblk) * per_block;
  lgt_obs* obs = reinterpret_cast<lgt_obs*>(feat + per_block);
  cudaStream_t s = b->B.stream;
  e = (precision == LGT_FP64)
          ? lgt::launch_observe_planned<double>(G, b->B.view(), static_cast<const double*>(psi), K,
                                                ncomp, nblk, rpb, part, feat, b->B.err, s)
          : lgt::launch_observe_planned<float>(G, b->B.view(), static_cast<const float*>(psi), K,
                                               ncomp, nblk, rpb, part, feat, b->B.err, s);
  if (e != cudaSuccess) return fail_na(LGT_ERR_CUDA, cudaGetErrorString(e));
  k_summarize<<<(K + 63) / 64, 64, 0, s>>>(G, feat, K, nfeat, t_now, obs), lgt::note_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail_na(LGT_ERR_CUDA, std::string("k_summarize: ") + cudaGetErrorString(e));
  const size_t pitch = size_t(nfeat) * sizeof(double);
  if (nf_grid)
    e = cudaMemcpy2DAsync(nf_grid, sizeof(double) * G.ns, feat, pitch, sizeof(double) * G.ns, K,
                          cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && E2_grid)
    e = cudaMemcpy2DAsync(E2_grid, sizeof(double) * G.ns, feat + G.ns, pitch,
                          sizeof(double) * G.ns, K, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && plaq_grid && G.nP)
    e = cudaMemcpy2DAsync(plaq_grid, sizeof(double) * G.nP, feat + 2 * G.ns, pitch,
                          sizeof(double) * G.nP, K, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && summary)
    e = cudaMemcpyAsync(summary, obs, sizeof(lgt_obs) * K, cudaMemcpyDeviceToHost, s);
  int derr = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&derr, b->B.err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail_na(LGT_ERR_CUDA, cudaGetErrorString(e));
  if (derr) {
    cudaMemsetAsync(b->B.err, 0, sizeof(int), s);
    return fail_na(LGT_ERR_DEVICE, "device self-check failed in the observables kernel");
  }
  return LGT_OK;
}

}  // extern "C"
