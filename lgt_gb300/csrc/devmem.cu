// devmem.cu -- the library's stream-ordered device memory.
//
// Handles (bases, Hamiltonians, their lookup tables and scratch) take their
// device memory from one memory pool per device, allocated and freed in
// stream order (cudaMallocFromPoolAsync / cudaFreeAsync on the handle's
// stream).  The pool keeps freed memory, up to kRetainBytes, for the next
// allocation instead of returning it to the driver at every
// synchronisation, so a sweep that builds and drops bases and Hamiltonians
// per batch of coupling points does not pay a driver allocation and an
// implicit device synchronisation per buffer.  The large Krylov workspaces
// of the panel drivers (allocated once per shape and kept), the stored
// neighbour tables and the allocation-free observables entry point do not
// use it.
//
// Bases take their streams, and the per-CTA solver's workspaces their timing
// events, from per-device lists of released ones.
//
// Pinned host staging buffers (the per-CTA solver's tables and outputs, the
// observables' read-back) come from a process-wide cache by size class:
// page-locking and unlocking host memory costs far more than a small solve,
// and a sweep creates and destroys handles per batch.
#include <map>
#include <mutex>
#include <vector>

#include "lgt_internal.h"

namespace lgt {

namespace {

constexpr int kMaxDevices = 64;
constexpr unsigned long long kRetainBytes = 4ull << 30;  // kept for reuse per device

std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

cudaError_t pool_of(int dev, cudaMemPool_t* out) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    cudaError_t e = cudaMemPoolCreate(&p, &props);
    if (e != cudaSuccess) return e;
    unsigned long long keep = kRetainBytes;
    e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(p);
      return e;
    }
    g_pool[dev] = p;
  }
  *out = g_pool[dev];
  return cudaSuccess;
}

constexpr size_t kPinnedMinBytes = 4096;
constexpr size_t kPinnedKeepPerClass = 16;
std::mutex g_pinned_mu;
std::map<size_t, std::vector<void*>> g_pinned;  // free buffers by capacity

}  // namespace

cudaError_t pinned_get(size_t bytes, void** p, size_t* cap) {
  size_t c = kPinnedMinBytes;
  while (c < bytes) c <<= 1;
  {
    std::lock_guard<std::mutex> lock(g_pinned_mu);
    auto it = g_pinned.find(c);
    if (it != g_pinned.end() && !it->second.empty()) {
      *p = it->second.back();
      it->second.pop_back();
      *cap = c;
      return cudaSuccess;
    }
  }
  cudaError_t e = cudaMallocHost(p, c);
  if (e != cudaSuccess) {
    *p = nullptr;
    *cap = 0;
    return e;
  }
  *cap = c;
  return cudaSuccess;
}

void pinned_put(void* p, size_t cap) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lock(g_pinned_mu);
    std::vector<void*>& v = g_pinned[cap];
    if (v.size() < kPinnedKeepPerClass) {
      v.push_back(p);
      return;
    }
  }
  cudaFreeHost(p);
}

// Basis streams: a sweep creates and drops a basis per batch, and creating
// and destroying a stream each time costs more than a small sector's build.
// A released stream goes back to its device's list (work still queued on it
// runs in order before the next user's); beyond kStreamsKept it is destroyed.
namespace {
constexpr size_t kStreamsKept = 32;
std::mutex g_stream_mu;
std::map<int, std::vector<cudaStream_t>> g_streams;
}  // namespace

cudaError_t stream_get(int dev, cudaStream_t* s) {
  {
    std::lock_guard<std::mutex> lock(g_stream_mu);
    std::vector<cudaStream_t>& v = g_streams[dev];
    if (!v.empty()) {
      *s = v.back();
      v.pop_back();
      return cudaSuccess;
    }
  }
  return cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
}

void stream_put(int dev, cudaStream_t s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(g_stream_mu);
    std::vector<cudaStream_t>& v = g_streams[dev];
    if (v.size() < kStreamsKept) {
      v.push_back(s);
      return;
    }
  }
  cudaStreamDestroy(s);
}

// Timing events of the per-CTA solver's workspaces, reused the same way.
namespace {
constexpr size_t kEventsKept = 64;
std::mutex g_event_mu;
std::map<int, std::vector<cudaEvent_t>> g_events;
}  // namespace

cudaError_t event_get(cudaEvent_t* e) {
  int dev = 0;
  cudaError_t r = cudaGetDevice(&dev);
  if (r != cudaSuccess) return r;
  {
    std::lock_guard<std::mutex> lock(g_event_mu);
    std::vector<cudaEvent_t>& v = g_events[dev];
    if (!v.empty()) {
      *e = v.back();
      v.pop_back();
      return cudaSuccess;
    }
  }
  return cudaEventCreate(e);
}

void event_put(cudaEvent_t e) {
  if (!e) return;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) {
    std::lock_guard<std::mutex> lock(g_event_mu);
    std::vector<cudaEvent_t>& v = g_events[dev];
    if (v.size() < kEventsKept) {
      v.push_back(e);
      return;
    }
  }
  cudaEventDestroy(e);
}

cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  cudaMemPool_t pool = nullptr;
  e = pool_of(dev, &pool);
  if (e != cudaSuccess) return e;
  return cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, s);
}

cudaError_t dev_free(void* p, cudaStream_t s) {
  if (!p) return cudaSuccess;
  return cudaFreeAsync(p, s);
}

}  // namespace lgt
