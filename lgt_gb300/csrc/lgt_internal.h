// lgt_internal.h -- internal host-side structures of the library (not part of
// the C-ABI).
#pragma once

#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "lgt_common.cuh"

namespace lgt {

// Raises `func`'s dynamic shared-memory limit to at least `bytes` on the
// current device.  The attribute belongs to the (function, device) pair, so
// the raised limit is remembered per device, under a lock (host threads of
// different handles launch concurrently).  The first launch of a
// configuration is eager, so the attribute call never falls inside a graph
// capture.
inline cudaError_t raise_smem_limit(const void* func, int bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> raised;
  std::lock_guard<std::mutex> lock(mu);
  int& have = raised[std::make_pair(func, dev)];
  if (bytes <= have) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) have = bytes;
  return e;
}

// The FP32-mixed Krylov reductions (Gram-Schmidt dots and updates, norms)
// run in double-float arithmetic on the FP32 pipe; LGT_DF_REDUCTIONS=0 in
// the environment runs the panel drivers' reductions in FP64 instead
// (cross-checks).  Read at every launch configuration.
inline bool df_reductions_enabled() {
  const char* e = getenv("LGT_DF_REDUCTIONS");
  return !(e && e[0] == '0');
}

// Stream-ordered device memory from the library's per-device pool
// (devmem.cu): the allocation is usable by work enqueued on `s` after the
// call; a free takes effect after the work enqueued on `s` before it.
cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s);
cudaError_t dev_free(void* p, cudaStream_t s);
// non-blocking streams reused across bases (devmem.cu)
cudaError_t stream_get(int dev, cudaStream_t* s);
void stream_put(int dev, cudaStream_t s);
// events reused across workspaces of the current device (devmem.cu)
cudaError_t event_get(cudaEvent_t* e);
void event_put(cudaEvent_t e);
// Pinned host memory from the library's cache (capacity rounded up to a
// power of two, at least 4 KB); pinned_put returns it (no copy may still be
// in flight from or to it).
cudaError_t pinned_get(size_t bytes, void** p, size_t* cap);
void pinned_put(void* p, size_t cap);
template <typename T>
cudaError_t dev_alloc_n(T** p, size_t n, cudaStream_t s) {
  return dev_alloc(reinterpret_cast<void**>(p), n * sizeof(T), s);
}

// Two timing events destroyed with the scope, whatever path leaves it.
struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t create() {
    cudaError_t e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    return e;
  }
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  EventPair() = default;
  EventPair(const EventPair&) = delete;
  EventPair& operator=(const EventPair&) = delete;
};

// Everything a kernel needs to turn an order key into a basis index.
//
// Two-level sorted index: the top level is the segment table `segc`, one
// entry per fermion mask with the sector's particle number, addressed by the
// mask's colexicographic rank (masks with k set bits in ascending numeric
// order are in colex order, rank = sum_j C(p_j, j) over the set-bit
// positions p_1 < ... < p_k).  segc[r] is the first index of mask r's
// segment.  The hop kernels stage this level in shared memory when it fits.
// The bottom level is a binary search over the segment's low key parts.
constexpr int kMaxTabRows = 8;

struct RankView {
  const uint64_t* keys;   // sorted order keys [dim]
  const uint32_t* low;    // low (e_U) parts of the keys [dim] (when ushift <= 32)
  const uint32_t* segc;   // segment starts [nmasks + 1]
  const uint32_t* binom;  // C(p, j) at [p * 33 + j], p < 32, j <= 32
  int64_t dim;
  int nmasks;
  int ushift;
  int low32;              // 1 when `low` is valid
  // Row-count tables (tab != null): the index of a state is a sum of one
  // table entry per e_U row (see basis.cu, "rank tables").
  const uint32_t* tab;
  int64_t tab_off[kMaxTabRows];  // start of the table of e_U row r in `tab`
  int nrows;              // e_U rows with a table (ny - 1)
  int F;                  // free-digit strings per e_U row, B^(nx-1)
  int B, nx, w, nU;       // digit base, lattice width, bits per digit, up links
  int ns, nf;             // sites, fermions
  int pw[kMaxSites];      // weight of free digit ix in a row's index (0 for the last)
};

struct BasisDev {
  Geom G{};
  int64_t dim = 0;
  int nmasks = 0;
  uint64_t* keys = nullptr;
  uint32_t* low = nullptr;
  uint32_t* segc = nullptr;
  uint32_t* masks = nullptr;
  uint32_t* binom = nullptr;
  uint32_t* tab = nullptr;      // rank tables (null when they would not fit)
  int64_t tab_off[kMaxTabRows] = {};
  int tab_F = 0;
  int* err = nullptr;           // device error word (DevErr bits)
  cudaStream_t stream = nullptr;
  void* block = nullptr;        // the one allocation of a small sector's buffers
  RankView view() const {
    RankView v;
    v.keys = keys;
    v.low = low;
    v.segc = segc;
    v.binom = binom;
    v.dim = dim;
    v.nmasks = nmasks;
    v.ushift = G.ushift;
    v.low32 = (G.ushift <= 32) ? 1 : 0;
    v.tab = tab;
    for (int r = 0; r < kMaxTabRows; ++r) v.tab_off[r] = tab_off[r];
    v.nrows = G.ny - 1;
    v.F = tab_F;
    v.B = 2 * G.dg + 1;
    v.nx = G.nx;
    v.w = G.w;
    v.nU = G.nU;
    v.ns = G.ns;
    v.nf = G.nf_target;
    int p = 1;
    for (int ix = kMaxSites - 1; ix >= 0; --ix) v.pw[ix] = 0;
    for (int ix = G.nx - 2; ix >= 0; --ix) {
      v.pw[ix] = p;
      p *= v.B;
    }
    return v;
  }
};

// Kernel-launch accounting, reported by lgt_launch_count: every launch site
// adds one, a graph replay adds its kernel-node count, and launches recorded
// into a graph while the calling thread captures are not counted.
void note_launch(int n = 1);
void set_capturing(bool on);

// Host geometry set-up; returns an empty string or an error message.
std::string make_geom(int nx, int ny, int dg, const int32_t* g_charges, Geom* G);

// Enumerates the sector basis on the GPU (kernels in basis.cu).  Allocates
// the device tables of `B`.  Returns an empty string or an error message.
std::string build_basis_device(BasisDev* B);
void free_basis_device(BasisDev* B);

// Decode device keys [i0, i0+n) into Julia-layout int8 arrays on the device.
void launch_decode_states(const BasisDev& B, int64_t i0, int64_t n, int8_t* nf, int8_t* eR,
                          int8_t* eU, cudaStream_t s);
void launch_ref_keys(const BasisDev& B, int64_t i0, int64_t n, uint64_t* out, cudaStream_t s);
// Rank reference (_encode) keys; out = 1-based index or 0 when absent.
void launch_rank_ref_keys(const BasisDev& B, const uint64_t* in, int64_t n, int64_t* out,
                          cudaStream_t s);
// Rank order keys; out = 0-based index or -1 when absent.
void launch_rank_order_keys(const BasisDev& B, const uint64_t* in, int64_t n, int64_t* out,
                            cudaStream_t s);

}  // namespace lgt
