// lgt_hpsi.h -- launch interface of the H*psi and CSR-export kernels.
#pragma once

#include "lgt_internal.h"

namespace lgt {

template <typename T>
struct HpsiArgs {
  Geom G;
  RankView R;
  const T* x;
  T* y;
  int64_t N;      // rows
  int C;          // columns per row = K * ncomp
  int ncomp;      // 1 real, 2 complex (re, im)
  int K;          // coupling points
  const T* cE;    // [K] g^2 / 2
  const T* cm;    // [K] m
  const T* ch;    // [K] -t
  const T* cp;    // [K] -1 / (2 g^2)
  int* err;       // device error word
  int seg_smem;   // stage the segment table in shared memory
  // Optional device-resident panel offset: x is read at x + (*xsel) * xstride.
  // Lets one captured CUDA graph apply H to "the current Krylov vector".
  const int* xsel;
  size_t xstride;
};

// Default staging decision for the top-level rank table.
int hpsi_seg_smem_default(int nmasks);

template <typename T>
cudaError_t launch_hpsi(HpsiArgs<T> a, uint32_t model, cudaStream_t s);

cudaError_t launch_row_nnz(const Geom& G, const RankView& R, uint32_t model, int64_t* counts,
                           cudaStream_t s);
cudaError_t launch_row_fill(const Geom& G, const RankView& R, uint32_t model,
                            const int64_t* rowptr, double g, double t, double m, int32_t* cols,
                            double* vals, int* err, cudaStream_t s);

}  // namespace lgt
