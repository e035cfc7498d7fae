// lgt_observe.h -- observables kernel interface.
#pragma once

#include "lgt_internal.h"

namespace lgt {

// Number of features per point: n_f per site, E^2 per site, plaquettes, norm.
int observe_nfeat(const Geom& G);
// Block partition of the observables reduction for N rows.
void observe_plan(int64_t N, int* nblk, int64_t* rpb);

// out[k * nfeat + f] for the K points of panel x ([N][K][ncomp]); part must
// hold nblk * K * nfeat doubles (observe_plan).
template <typename T>
cudaError_t launch_observe(const Geom& G, const RankView& R, const T* x, int K, int ncomp,
                           double* part, double* out, int* err, cudaStream_t s);

// Same reduction with a caller-chosen block partition (nblk blocks of rpb
// rows; part must hold nblk * K * nfeat doubles).
template <typename T>
cudaError_t launch_observe_planned(const Geom& G, const RankView& R, const T* x, int K, int ncomp,
                                   int nblk, int64_t rpb, double* part, double* out, int* err,
                                   cudaStream_t s);

}  // namespace lgt
