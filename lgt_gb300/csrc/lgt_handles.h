// lgt_handles.h -- definitions of the opaque C-ABI handles (shared by the
// translation units that implement entry points).
#pragma once

#include <atomic>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/lgt_ed.h"
#include "lgt_internal.h"
#include "lgt_krylov.h"
#include "lgt_small.h"

namespace lgt {

// Device buffer owned by a handle, grown on demand, in stream order on the
// handle's stream (library pool, devmem.cu).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t need(size_t b, cudaStream_t s) {
    if (b <= bytes) return cudaSuccess;
    dev_free(p, s);
    p = nullptr;
    bytes = 0;
    cudaError_t e = dev_alloc(&p, b, s);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  void release(cudaStream_t s) {
    dev_free(p, s);
    p = nullptr;
    bytes = 0;
  }
};


// Sets the calling thread's lgt_last_error() message.
void set_last_error(const std::string& msg);

// measure_ED's means (finite_ed.jl:387-390) plus plaquette and staggered
// density, from the per-point feature vector of the observables kernel
// (n_f per site, E^2 per site, plaquettes, norm).  One definition for the
// host summaries of lgt_observe / lgt_expm_steps and the device summaries
// of lgt_observe_noalloc, so the two cannot drift apart.
__host__ __device__ inline void summarize_obs(const Geom& G, const double* feat, double t_now,
                                              lgt_obs* o) {
  const int ns = G.ns;
  double nf = 0, e2 = 0, ne = 0, no = 0, st = 0, pl = 0;
  int cnt_e = 0, cnt_o = 0;
  for (int iy = 0; iy < G.ny; ++iy)
    for (int ix = 0; ix < G.nx; ++ix) {
      const int s = iy * G.nx + ix;
      nf += feat[s];
      e2 += feat[ns + s];
      if ((ix + iy) % 2 == 0) {
        ne += feat[s];
        st += feat[s];
        ++cnt_e;
      } else {
        no += feat[s];
        st -= feat[s];
        ++cnt_o;
      }
    }
  for (int q = 0; q < G.nP; ++q) pl += feat[2 * ns + q];
  o->t = t_now;
  o->nf_mean = nf / ns;
  o->nf_even = cnt_e ? ne / cnt_e : NAN;
  o->nf_odd = cnt_o ? no / cnt_o : NAN;
  o->E2_mean = e2 / ns;
  o->plaq_mean = G.nP ? pl / G.nP : 0.0;
  o->n_stag = st / ns;
  o->norm2 = feat[2 * ns + G.nP];
}

}  // namespace lgt

struct lgt_basis {
  using BasisDev = lgt::BasisDev;
  BasisDev B;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  // owners: the caller's handle plus one per Hamiltonian made from it; the
  // basis is freed when the last owner lets go (handles may be destroyed in
  // any order, e.g. by a garbage collector)
  std::atomic<int> refs{1};
};

struct lgt_ham {
  using DevBuf = lgt::DevBuf;
  using KrylovCache = lgt::KrylovCache;
  using Pattern = lgt::Pattern;
  using SmallWork = lgt::SmallWork;
  using OpDev = lgt::OpDev;
  const lgt_basis* b = nullptr;
  int K = 0;
  uint32_t model = 0;
  std::vector<double> g, t, m;
  double* coef_d = nullptr;  // [4][K]: g^2/2, m, -t, -1/(2g^2)
  float* coef_f = nullptr;
  int seg_smem = 0;
  KrylovCache* cache = nullptr;
  DevBuf x, y, part, out;
  double* hfeat = nullptr;  // pinned staging of the observables' features and error word
  size_t hfeat_n = 0;
  Pattern pattern;          // lookup pass of the per-CTA solver (built on demand)
  SmallWork small;
  // neighbour table of the panel H*psi (built on demand by the autotuner;
  // mutable: op() hands out a pointer through which it is built)
  mutable lgt::NbrTable table;
  mutable lgt::NbrTable table_ord;  // the same renumbered to its row order (order.cu)
  OpDev op() const {
    OpDev o;
    o.G = b->B.G;
    o.R = b->B.view();
    o.err = b->B.err;
    o.model = model;
    o.K = K;
    o.seg_smem = seg_smem;
    o.cE_d = coef_d;
    o.cm_d = coef_d + K;
    o.ch_d = coef_d + 2 * K;
    o.cp_d = coef_d + 3 * K;
    o.cE_f = coef_f;
    o.cm_f = coef_f + K;
    o.ch_f = coef_f + 2 * K;
    o.cp_f = coef_f + 3 * K;
    o.table = &table;
    o.table_ord = &table_ord;
    return o;
  }
};
