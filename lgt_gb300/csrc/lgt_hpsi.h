// lgt_hpsi.h -- launch interface of the H*psi and CSR-export kernels.
#pragma once

#include <string>

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
  int force_generic = 0;  // 1: run-time-geometry kernel even for a fixed shape
  int vpl = 0;            // fixed-shape load mode: 1 one vector per lane, 2 two,
                          // 3 two as one 32-byte access; 0 the built-in rule
  // Stored neighbour table (nbr_table.cu); with use_table the table kernel
  // runs (same load modes as the fixed-shape kernel).
  const uint32_t* t_meta = nullptr;
  const uint32_t* t_off = nullptr;
  const uint32_t* t_nbr = nullptr;
  int t_mm = 0;           // most entries a row can have
  int use_table = 0;
  // the panels are in the table's own row order (a renumbered table): only
  // the table kernel may run; anything else is an error, not a fallback
  int table_order = 0;
  // rows addressable from x (all the Krylov slots behind x + xsel * xstride;
  // 0: N): the extent of the tensor map of the gathered variant (vpl 4)
  int64_t x_rows = 0;
};

// The stored-table kernel with the neighbour rows gathered by the copy
// engine (nbr_table_bulk.cu): FP32 panels of 16 columns.
bool table_bulk_applies(const HpsiArgs<float>& a, int64_t x_rows);
cudaError_t launch_table_bulk(const HpsiArgs<float>& a, uint32_t model, int64_t x_rows,
                              cudaStream_t s);

// The neighbour ranks of every row of a basis for one model, kept in HBM
// (nbr_table.cu): meta[N], tile_off[ceil(N/32) + 1], nbr[nnz].
struct NbrTable {
  int64_t N = 0, nnz = 0;
  uint32_t model = 0;
  int mm = 0;
  uint32_t* meta = nullptr;
  uint32_t* tile_off = nullptr;
  uint32_t* nbr = nullptr;
  size_t bytes = 0;
  int state = 0;  // 0 not built, 1 built, -1 declined (size or representability)
  // A renumbered copy (order.cu) also holds its row order: perm[new] = old
  // row, iperm[old] = new row.
  int* perm = nullptr;
  int* iperm = nullptr;
};

// Whether the basis fits the table format (N < 2^31, fewer than 2^32
// entries, counts and sum of e^2 below 256); *bytes: an upper bound of the
// table's size.
bool nbr_table_eligible(const Geom& G, int64_t N, uint32_t model, size_t* bytes);
std::string build_nbr_table(const Geom& G, const RankView& R, uint32_t model, int* err,
                            NbrTable* T, cudaStream_t s);
void free_nbr_table(NbrTable* T);

// T renumbered to the breadth-first row order of its hop graph (order.cu):
// T2 receives the renumbered table with its perm / iperm.  One-time cost per
// Hamiltonian (a host read per search level).
std::string build_table_order(const NbrTable& T, NbrTable* T2, cudaStream_t s);
// The same with the fermion-mask segments ordered breadth-first over the
// mask graph and the rows of a segment kept in order (order.cu).
std::string build_table_mask_order(const NbrTable& T, const Geom& G, const RankView& R,
                                   NbrTable* T2, cudaStream_t s);

// Whether the table kernel serves these arguments (table present, vector-
// aligned panels) and its widest load mode (as hpsi_fixed_applies).
template <typename T>
bool table_load_mode(const HpsiArgs<T>& a, int* max_vpl);
template <typename T>
cudaError_t launch_hpsi_table(const HpsiArgs<T>& a, uint32_t model, cudaStream_t s);

// Whether a fixed-shape kernel serves these arguments, and the widest load
// mode it may use (1, 2 when C is a multiple of two vectors, 3 when the
// panels are also 32-byte aligned).
template <typename T>
bool hpsi_fixed_applies(const HpsiArgs<T>& a, int* max_vpl);

// Default staging decision for the top-level rank table.
int hpsi_seg_smem_default(int nmasks);

// y = H x.  With use_table and a table present, the stored-table kernel;
// else lattices with a compile-time kernel (4x4, 4x3, 3x4 at dg = 1, rank
// tables present, vector-aligned panels) use it; all others the
// run-time-geometry kernel.  All give the same product.
template <typename T>
cudaError_t launch_hpsi(HpsiArgs<T> a, uint32_t model, cudaStream_t s);

// The run-time-geometry kernel alone (tests compare the two paths).
template <typename T>
cudaError_t launch_hpsi_generic(HpsiArgs<T> a, uint32_t model, cudaStream_t s);

// Fixed-shape kernels, one translation unit each (hpsi_<nx>x<ny>.cu).
#define LGT_DECLARE_FIXED_SHAPE(NX, NY)                                                   \
  cudaError_t launch_hpsi_##NX##x##NY(const HpsiArgs<float>& a, uint32_t model, cudaStream_t s); \
  cudaError_t launch_hpsi_##NX##x##NY(const HpsiArgs<double>& a, uint32_t model, cudaStream_t s);
LGT_DECLARE_FIXED_SHAPE(4, 4)
LGT_DECLARE_FIXED_SHAPE(4, 3)
LGT_DECLARE_FIXED_SHAPE(3, 4)
#undef LGT_DECLARE_FIXED_SHAPE

cudaError_t launch_row_nnz(const Geom& G, const RankView& R, uint32_t model, int64_t* counts,
                           cudaStream_t s);
cudaError_t launch_row_fill(const Geom& G, const RankView& R, uint32_t model,
                            const int64_t* rowptr, double g, double t, double m, int32_t* cols,
                            double* vals, int* err, cudaStream_t s);

}  // namespace lgt
