// krylov.cu -- batched Lanczos ground states and Krylov exp(-iHt) steps on the
// GPU (replaces KrylovKit.eigsolve in find_ground_state, finite_ed.jl:333-341,
// and KrylovKit.exponentiate in evolve_ED!, finite_ed.jl:405-431).
//
// K independent coupling points advance in lockstep on K-interleaved panels;
// each point has its own tridiagonal matrix, convergence state and restart.
// A Lanczos step is
//     W = H V_j                          (hpsi, storage precision)
//     repeat reorth times:               (classical Gram-Schmidt against the
//        h = V_{0..j}^H W                 whole basis, FP64 accumulation)
//        W -= V_{0..j} h,  alpha_j += Re h_j
//     beta_j = ||W||,  V_{j+1} = W / beta_j
// (a further pass runs only for points whose pass cancelled more than two
// digits).  Every reduction is two-stage (per-block partials, then a
// fixed-order warp-parallel sum), so results are bitwise reproducible.  All
// kernels read the step index j from device memory, so the step sequence is
// captured once as a CUDA graph and replayed.  The tridiagonal problems are
// solved on the device: lowest eigenpair by warp multisection of the Sturm
// count + inverse iteration (ground state, lgt_tridiag.cuh), full
// eigendecomposition by implicit QL (exponential, which runs the real and
// imaginary parts of each point as two real Krylov columns).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "lgt_bulk.cuh"
#include "lgt_dfloat.cuh"
#include "lgt_krylov.h"
#include "lgt_tridiag.cuh"

namespace lgt {

namespace {

constexpr int kT = 256;   // threads of the panel kernels
constexpr int kIC = 8;    // Krylov vectors per multidot pass
constexpr int kMaxDim = 64;

#define KCK(call)                                                                  \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
  } while (0)

// status codes per point
enum : int { kActive = 0, kExhausted = 1, kConverged = 2, kWritten = 3 };

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Standard normal samples from a counter-based hash (Box-Muller).  Point k
// of seed s draws the same vector whatever K is.
template <typename S>
__global__ void k_randn(S* out, int64_t N, int C, int ncomp, uint64_t seed) {
  const int64_t n = N * C;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = i / C;
    const int c = int(i - row * C);
    const int k = c / ncomp, comp = c - k * ncomp;
    uint64_t h = splitmix64(splitmix64(seed) ^ splitmix64(uint64_t(k) + 0x5851F42D4C957F2Dull));
    h = splitmix64(h ^ (uint64_t(row) * uint64_t(ncomp) + uint64_t(comp)));
    const uint64_t h2 = splitmix64(h);
    const double u1 = (double((h >> 11) + 1)) * 0x1.0p-53;  // (0, 1]
    const double u2 = double(h2 >> 11) * 0x1.0p-53;
    out[i] = S(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
  }
}

// Per-block partial dot products of W against V_0..V_{J-1}:
// part[blk][i][0][c] = sum_rows V_i[row][c] W[row][c]
// part[blk][i][1][c] = sum_rows V_i[row][c] W[row][c^1]   (complex only)
// With self = 1, index J holds W against itself (its squared norm).  Columns
// of points with need[k] == 0 contribute zero (need may be null).
// Measured on the 4x4 quench panel (K = 8 complex, FP64 and FP32 storage):
// the dot kernel issues a chunk's loads before its FMAs and keeps 4 blocks
// per SM; the update's plain two-chain loop beats hoisted loads.
#ifndef LGT_UPD_HOIST
#define LGT_UPD_HOIST 0
#endif
// rows a thread updates per loop trip on real panels: 2 gives four FMA
// chains and twice the loads in flight (4x4 FP32-mixed quench step 0.116 ->
// 0.114 s; FP64 unchanged)
#ifndef LGT_UPD_ROWS
#define LGT_UPD_ROWS 2
#endif
#ifndef LGT_MD_MINB
#define LGT_MD_MINB 4  // resident blocks per SM the dot kernel's registers must allow (FP64)
#endif
#ifndef LGT_MD_TRIP
#define LGT_MD_TRIP 3  // rows per trip of the FP32 double-float dot pass (4x4 K = 8 quench:
                       // 2 rows 17.70, 3 rows 18.21, 4 rows with 2 blocks/SM 17.96 steps/s)
#endif
#ifndef LGT_MD_MINB_F32
#define LGT_MD_MINB_F32 3  // the same for FP32 panels (measured with chunks sized to the
                           // vectors left: 4 without spills beats 5 with them)
#endif
// One chunk of a dot pass: the NQ basis vectors i0 .. i0 + NQ - 1 (those
// from J on are skipped) against W, per thread one column and every RG-th
// row of the block's range, into red[rg][q][comp][c].  Every load of a row
// is issued before the first FMA; slots past the basis read its last vector
// again (an L1 hit).  The loads stay in the storage type until their FMA
// (widened FP32 values would hold twice the registers and spill).
template <typename S, int NC, int NQ>
__device__ __forceinline__ void dots_chunk(const S* __restrict__ V, size_t vstride,
                                           const S* __restrict__ W, int64_t r0, int64_t r1,
                                           int rg, int RG, int c, int C, int i0, int J, int Jv,
                                           bool act, double* red, bool dw) {
  if (sizeof(S) == 4 && NC == 1 && dw) {
    // FP32 panels: products of FP32 entries are exact as double-floats, and
    // the running sums are double-floats (lgt_dfloat.cuh), so the dot is
    // FP64-class while the FP64 pipe only sees the final conversion
    df a[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) a[q] = df{0.f, 0.f};
    if (act) {
      const int ilast = (Jv > 0) ? Jv - 1 : 0;
      const float* vq[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q)
        vq[q] = reinterpret_cast<const float*>(V) + size_t((i0 + q < Jv) ? i0 + q : ilast) * vstride + c;
      const float* wp = reinterpret_cast<const float*>(W) + c;
      // LGT_MD_TRIP rows per trip: LGT_MD_TRIP (NQ + 1) loads in flight
      // before the arithmetic
      constexpr int kTrip = LGT_MD_TRIP;
      int64_t row = r0 + rg;
      for (; row + (kTrip - 1) * int64_t(RG) < r1; row += kTrip * int64_t(RG)) {
        size_t o[kTrip];
        float wv[kTrip], vv[kTrip][NQ];
#pragma unroll
        for (int u = 0; u < kTrip; ++u) {
          o[u] = size_t(row + u * int64_t(RG)) * C;
          wv[u] = __ldg(wp + o[u]);
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q)
#pragma unroll
          for (int u = 0; u < kTrip; ++u) vv[u][q] = __ldg(vq[q] + o[u]);
#pragma unroll
        for (int q = 0; q < NQ; ++q)
          if (i0 + q < J) {
#pragma unroll
            for (int u = 0; u < kTrip; ++u) df_fma(a[q], (i0 + q < Jv) ? vv[u][q] : wv[u], wv[u]);
          }
      }
      for (; row < r1; row += RG) {
        const size_t off = size_t(row) * C;
        const float w = __ldg(wp + off);
#pragma unroll
        for (int q = 0; q < NQ; ++q)
          if (i0 + q < J) df_fma(a[q], (i0 + q < Jv) ? __ldg(vq[q] + off) : w, w);
      }
    }
    if (rg < RG) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        red[((rg * kIC + q) * 2 + 0) * C + c] = act ? widen(a[q].hi) + widen(a[q].lo) : 0.0;
        red[((rg * kIC + q) * 2 + 1) * C + c] = 0.0;
      }
    }
    return;
  }
  constexpr int kB = (NC == 2) ? NQ : 1;  // imaginary parts (complex panels only)
  double a[NQ], b[kB];
#pragma unroll
  for (int q = 0; q < NQ; ++q) a[q] = 0.0;
#pragma unroll
  for (int q = 0; q < kB; ++q) b[q] = 0.0;
  if (act) {
    const int ilast = (Jv > 0) ? Jv - 1 : 0;
    for (int64_t row = r0 + rg; row < r1; row += RG) {
      const size_t off = size_t(row) * C;
      const double w = widen(W[off + c]);
      const double wx = (NC == 2) ? widen(W[off + (c ^ 1)]) : 0.0;
      S v[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const int i = (i0 + q < Jv) ? i0 + q : ilast;
        v[q] = V[size_t(i) * vstride + off + c];
      }
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        if (i0 + q < J) {
          const double vq = (i0 + q < Jv) ? widen(v[q]) : w;
          a[q] = fma(vq, w, a[q]);
          if (NC == 2) b[q % kB] = fma(vq, wx, b[q % kB]);
        }
      }
    }
  }
  if (rg < RG) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      red[((rg * kIC + q) * 2 + 0) * C + c] = act ? a[q] : 0.0;
      red[((rg * kIC + q) * 2 + 1) * C + c] = (act && NC == 2) ? b[q % kB] : 0.0;
    }
  }
}

// Partial dots of W against the basis vectors 0 .. J-1 (and W itself when
// self = 1) per block, in chunks of up to kIC vectors; a chunk of nq
// vectors runs the code for the next power of two >= nq, so that a short
// pass does not pay for kIC loads a row.
template <typename S, int NC>
__global__ void __launch_bounds__(kT, sizeof(S) == 4 ? LGT_MD_MINB_F32 : LGT_MD_MINB) k_multidot(const S* __restrict__ V, size_t vstride,
                                                 const int* jstate, int jfixed,
                                                 const S* __restrict__ W, int64_t N, int C,
                                                 int64_t rpb, double* part, int Jmax,
                                                 int self, const int* need, int ncomp,
                                                 int dw) {
  extern __shared__ double red[];  // [RG][kIC][2][C]
  const int Jv = jstate ? (*jstate + 1) : jfixed;
  const int J = Jv + self;
  const int RG = kT / C;
  const int c = threadIdx.x % C, rg = threadIdx.x / C;
  const bool act = rg < RG && (!need || need[c / ncomp] != 0);
  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int64_t r1 = (r0 + rpb < N) ? r0 + rpb : N;
  for (int i0 = 0; i0 < J; i0 += kIC) {
    const int nq = (J - i0 < kIC) ? J - i0 : kIC;
    const int nq2 = nq <= 1 ? 1 : nq <= 2 ? 2 : nq <= 4 ? 4 : kIC;
    if (nq2 == 1)
      dots_chunk<S, NC, 1>(V, vstride, W, r0, r1, rg, RG, c, C, i0, J, Jv, act, red, dw);
    else if (nq2 == 2)
      dots_chunk<S, NC, 2>(V, vstride, W, r0, r1, rg, RG, c, C, i0, J, Jv, act, red, dw);
    else if (nq2 == 4)
      dots_chunk<S, NC, 4>(V, vstride, W, r0, r1, rg, RG, c, C, i0, J, Jv, act, red, dw);
    else
      dots_chunk<S, NC, kIC>(V, vstride, W, r0, r1, rg, RG, c, C, i0, J, Jv, act, red, dw);
    __syncthreads();
    for (int q = threadIdx.x; q < nq2 * 2 * C; q += kT) {
      double s = 0.0;
      for (int g = 0; g < RG; ++g) s += red[g * kIC * 2 * C + q];
      const int ii = q / (2 * C);
      if (i0 + ii < J) part[(size_t(blockIdx.x) * Jmax + i0) * 2 * C + q] = s;
    }
    __syncthreads();
  }
}

// Bulk-copy streaming of a block's panel rows (k_multidot_bulk,
// k_update_bulk): tiles of kBulkTile values (kBulkTile / C rows, contiguous
// in every panel) pass through a ring of kBulkStages shared-memory stages,
// each refilled by one bulk copy once the block has consumed it.
constexpr int kBulkStages = 4;
constexpr int kBulkElems = 8;                  // values per thread and tile
constexpr int kBulkTile = kT * kBulkElems;     // values per chunk (8 KB)

// Basis vectors of dot group g (slots g kIC .. g kIC + kIC - 1 below Jv).
__device__ __forceinline__ int bulk_group_vectors(int g, int Jv) {
  const int i0 = g * kIC, i1 = (i0 + kIC < Jv) ? i0 + kIC : Jv;
  return i1 > i0 ? i1 - i0 : 0;
}

// The next chunk a multidot block issues: group g, tile t, slot s (0: W,
// s > 0: basis vector g kIC + s - 1), and the chunks issued so far.
struct BulkCursor {
  int g, t, s;
  int64_t issued;
  __device__ __forceinline__ void advance(int nt, int Jv) {
    ++issued;
    if (++s > bulk_group_vectors(g, Jv)) {
      s = 0;
      if (++t == nt) {
        t = 0;
        ++g;
      }
    }
  }
};

// k_multidot's double-float FP32 pass with the rows streamed in bulk
// copies.  Per group of up to kIC dot slots (basis vectors i0 .. i0 + nq - 1;
// a slot at Jv is W against itself), every tile of the block's range sends
// W_t, then V_{i0},t, ... through the stage ring; thread (c, g) keeps its
// kBulkElems values of W_t (column c, rows g + RG e) in registers and adds
// their products into one double-float per slot.  Rows and operations are
// those of dots_chunk in the same order, so the partials are bitwise
// k_multidot's.  Needs kT % C == 0 and 16-byte aligned chunks; a copy that
// does not arrive within the bounded wait raises kDevErrSpin in `err`.
__global__ void __launch_bounds__(kT, 3) k_multidot_bulk(const float* __restrict__ V, size_t vstride,
                                                      const int* jstate, const float* W,
                                                      int64_t N, int C, int64_t rpb,
                                                      double* part, int Jmax, int self,
                                                      const int* need, int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* s_buf = reinterpret_cast<float*>(smem_raw);  // [kBulkStages][kBulkTile]
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_buf + kBulkStages * kBulkTile);
  double* red = reinterpret_cast<double*>(s_bar + kBulkStages);  // [RG][kIC][2][C]
  const int Jv = *jstate + 1;
  const int J = Jv + self;
  const int tid = threadIdx.x;
  const int RG = kT / C;
  const int c = tid % C, rg = tid / C;
  const bool act = !need || need[c] != 0;
  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int64_t r1 = (r0 + rpb < N) ? r0 + rpb : N;
  const int TR = kBulkTile / C;
  const int nt = (r1 > r0) ? int((r1 - r0 + TR - 1) / TR) : 0;
  if (tid == 0) {
    for (int st = 0; st < kBulkStages; ++st) mbar_init(s_bar + st, 1);
    mbar_init_fence();
  }
  const int any = __syncthreads_or(act ? 1 : 0);
  const int ngroups = (J + kIC - 1) / kIC;
  int64_t total = 0;
  if (any)
    for (int g = 0; g < ngroups; ++g) total += int64_t(nt) * (1 + bulk_group_vectors(g, Jv));
  // producer cursor (thread 0): next chunk to issue as (group, tile, slot)
  BulkCursor cur{0, 0, 0, 0};
  auto issue_next = [&]() {
    const int64_t rs = r0 + int64_t(cur.t) * TR;
    const int rows = int((r1 - rs < TR) ? (r1 - rs) : TR);
    const float* src =
        (cur.s == 0 ? W : V + size_t(cur.g * kIC + cur.s - 1) * vstride) + size_t(rs) * C;
    const int st = int(cur.issued % kBulkStages);
    const uint32_t bytes = uint32_t(rows) * uint32_t(C) * 4u;
    mbar_arrive_expect_tx(s_bar + st, bytes);
    bulk_g2s(s_buf + size_t(st) * kBulkTile, src, bytes, s_bar + st);
    cur.advance(nt, Jv);
  };
  if (tid == 0)
    while (cur.issued < total && cur.issued < kBulkStages) issue_next();
  int64_t n = 0;  // chunks consumed
  bool bad = false;
  for (int g = 0; g < ngroups && !bad; ++g) {
    const int i0 = g * kIC;
    const int nq = (J - i0 < kIC) ? J - i0 : kIC;
    const int nv = bulk_group_vectors(g, Jv);
    df a[kIC];
#pragma unroll
    for (int q = 0; q < kIC; ++q) a[q] = df{0.f, 0.f};
    float w[kBulkElems];
    for (int t = 0; any && t < nt && !bad; ++t) {
      const int64_t rs = r0 + int64_t(t) * TR;
      const int vals = int((r1 - rs < TR) ? (r1 - rs) : TR) * C;
      for (int sl = 0; sl <= nv; ++sl, ++n) {
        const int st = int(n % kBulkStages);
        if (!mbar_wait_bounded(s_bar + st, uint32_t(n / kBulkStages) & 1u)) bad = true;
        const float* buf = s_buf + size_t(st) * kBulkTile;
        if (!bad && act) {
          if (sl == 0) {
#pragma unroll
            for (int e = 0; e < kBulkElems; ++e) {
              const int idx = tid + kT * e;
              w[e] = idx < vals ? buf[idx] : 0.f;
            }
          } else {
            const int q = sl - 1;
            const bool full = vals == kBulkTile;
#pragma unroll
            for (int qq = 0; qq < kIC; ++qq)
              if (qq == q) {
                if (full) {
#pragma unroll
                  for (int e = 0; e < kBulkElems; ++e) df_fma(a[qq], buf[tid + kT * e], w[e]);
                } else {
#pragma unroll
                  for (int e = 0; e < kBulkElems; ++e)
                    if (tid + kT * e < vals) df_fma(a[qq], buf[tid + kT * e], w[e]);
                }
              }
          }
          // self slots of this group (W against itself) after its last vector
          if (sl == nv) {
#pragma unroll
            for (int qq = 0; qq < kIC; ++qq)
              if (qq >= nv && qq < nq) {
#pragma unroll
                for (int e = 0; e < kBulkElems; ++e)
                  if (tid + kT * e < vals) df_fma(a[qq], w[e], w[e]);
              }
          }
        }
        if (__syncthreads_or(bad ? 1 : 0)) {
          bad = true;
          break;
        }
        if (tid == 0 && cur.issued < total) issue_next();
      }
    }
    if (bad) break;
    // red[rg][q][comp][c] as dots_chunk writes it, then the block's partials
#pragma unroll
    for (int q = 0; q < kIC; ++q) {
      if (q < nq) {
        red[((rg * kIC + q) * 2 + 0) * C + c] =
            (act && any) ? widen(a[q].hi) + widen(a[q].lo) : 0.0;
        red[((rg * kIC + q) * 2 + 1) * C + c] = 0.0;
      }
    }
    __syncthreads();
    const int nq2 = nq <= 1 ? 1 : nq <= 2 ? 2 : nq <= 4 ? 4 : kIC;
    for (int q = tid; q < nq2 * 2 * C; q += kT) {
      double s = 0.0;
      for (int gg = 0; gg < RG; ++gg) s += red[gg * kIC * 2 * C + q];
      const int ii = q / (2 * C);
      if (i0 + ii < J) part[(size_t(blockIdx.x) * Jmax + i0) * 2 * C + q] = s;
    }
    __syncthreads();
  }
  if (bad) {
    // copies issued and not consumed: chunks n .. issued - 1 (thread 0's count)
    if (tid == 0) {
      for (int64_t m = n; m < cur.issued; ++m)
        mbar_wait_bounded(s_bar + (m % kBulkStages), uint32_t(m / kBulkStages) & 1u);
      if (err) atomicOr(err, kDevErrSpin);
    }
    __syncthreads();
  }
}

// Sum over the per-block partials in a fixed order, one warp per output:
// lane l adds blocks l, l + 32, ..., then a fixed shuffle tree.  (A single
// thread walking all blocks waits on one dependent load and add per block.)
__device__ __forceinline__ double warp_total(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// h[i][k] = <V_i, W>_k (complex for NC = 2).  alpha_j of active points
// accumulates Re h_j (first pass sets it).  With self = 1 the extra dot (W
// against itself) goes to nb[k].  One warp per (i, k); launch
// finish_blocks(outputs) blocks of 128 threads.
__global__ void k_finish_dots(const double* part, int nblk, int Jmax, const int* jstate,
                              int jfixed, int K, int C, int ncomp, double* h, double* alpha,
                              int ldT, int first_pass, const int* status, int self, double* nb) {
  const int J = jstate ? (*jstate + 1) : jfixed;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (t >= (J + self) * K) return;
  const int i = t / K, k = t - i * K;
  double re = 0.0, im = 0.0;
  for (int b = lane; b < nblk; b += 32) {
    const double* p = part + (size_t(b) * Jmax + i) * 2 * C;
    if (ncomp == 1) {
      re += p[k];
    } else {
      re += p[2 * k] + p[2 * k + 1];
      im += p[C + 2 * k] - p[C + 2 * k + 1];
    }
  }
  re = warp_total(re);
  im = warp_total(im);
  if (lane != 0) return;
  if (i == J) {  // self dot
    nb[k] = re;
    return;
  }
  h[(size_t(i) * K + k) * 2 + 0] = re;
  h[(size_t(i) * K + k) * 2 + 1] = im;
  if (alpha && i == J - 1 && status[k] == kActive) {
    double* a = alpha + size_t(k) * ldT + (J - 1);
    *a = first_pass ? re : (*a + re);
  }
}

// Blocks of 128 threads (4 warps) for `outputs` warp-per-output finishers.
inline unsigned finish_blocks(int outputs) { return unsigned((outputs + 3) / 4); }

// W -= sum_{i<J} h_i V_i (complex product for NC = 2) for active points
// (only those with need[k] != 0 when need is given), and per-block partial
// sums of |W|^2 per column of every active point.
template <typename S, int NC>
__global__ void __launch_bounds__(kT) k_update(const S* __restrict__ V, size_t vstride,
                                               const int* jstate, int jfixed, S* __restrict__ W,
                                               int64_t N, int C, int ncomp,
                                               const double* __restrict__ h, int K,
                                               const int* status, int64_t rpb, double* npart,
                                               const int* need) {
  __shared__ double red[kT];
  const int J = jstate ? (*jstate + 1) : jfixed;
  const int RG = kT / C;
  const int c = threadIdx.x % C, rg = threadIdx.x / C;
  const int k = c / ncomp;
  // A point that needs no further pass keeps W and the norm partials of its
  // previous pass: its columns are neither read nor written here.
  const bool act = rg < RG && (!status || status[k] == kActive) && !(need && need[k] == 0);
  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int64_t r1 = (r0 + rpb < N) ? r0 + rpb : N;
  double nrm = 0.0;
  const int Ju = J;
  int64_t row_start = r0 + rg;
  if (act && NC == 1 && LGT_UPD_ROWS == 2) {
    // rows row and row + RG together: chains (a0, a1) and (b0, b1)
    const int64_t step2 = 2 * int64_t(RG);
    for (; row_start + RG < r1; row_start += step2) {
      const size_t oa = size_t(row_start) * C + c, ob = oa + size_t(RG) * C;
      double a0 = widen(W[oa]), b0 = widen(W[ob]), a1 = 0.0, b1 = 0.0;
      int i = 0;
      for (; i + 1 < Ju; i += 2) {
        const double h0 = __ldg(h + (size_t(i) * K + k) * 2);
        const double h1 = __ldg(h + (size_t(i + 1) * K + k) * 2);
        const S* v0 = V + size_t(i) * vstride;
        const S* v1 = v0 + vstride;
        const S va0 = v0[oa], vb0 = v0[ob], va1 = v1[oa], vb1 = v1[ob];
        a0 = fma(-h0, widen(va0), a0);
        b0 = fma(-h0, widen(vb0), b0);
        a1 = fma(-h1, widen(va1), a1);
        b1 = fma(-h1, widen(vb1), b1);
      }
      if (i < Ju) {
        const double h0 = __ldg(h + (size_t(i) * K + k) * 2);
        const S* v0 = V + size_t(i) * vstride;
        a0 = fma(-h0, widen(v0[oa]), a0);
        b0 = fma(-h0, widen(v0[ob]), b0);
      }
      const S sa = to_storage<S>(a0 + a1), sb = to_storage<S>(b0 + b1);
      W[oa] = sa;
      W[ob] = sb;
      const double wa = widen(sa), wb = widen(sb);
      nrm = fma(wa, wa, nrm);
      nrm = fma(wb, wb, nrm);
    }
  }
  if (act) {
    for (int64_t row = row_start; row < r1; row += RG) {
      const size_t off = size_t(row) * C;
      // two independent chains (even / odd basis vectors); the first starts
      // from W itself
      double w0 = widen(W[off + c]), w1 = 0.0;
      int i = 0;
      if (NC == 1 && LGT_UPD_HOIST) {
        // four basis vectors per trip, loads first (clamped to the last
        // vector, an L1 hit), FMAs only for the vectors that exist
        for (; i < Ju; i += 4) {
          double vv[4], hh[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int ii = (i + u < Ju) ? i + u : Ju - 1;
            hh[u] = __ldg(h + (size_t(ii) * K + k) * 2);
            vv[u] = widen(V[size_t(ii) * vstride + off + c]);
          }
          w0 = fma(-hh[0], vv[0], w0);
          if (i + 1 < Ju) w1 = fma(-hh[1], vv[1], w1);
          if (i + 2 < Ju) w0 = fma(-hh[2], vv[2], w0);
          if (i + 3 < Ju) w1 = fma(-hh[3], vv[3], w1);
        }
      }
      for (; i + 1 < Ju; i += 2) {
        const double hr0 = __ldg(h + (size_t(i) * K + k) * 2 + 0);
        const double hr1 = __ldg(h + (size_t(i + 1) * K + k) * 2 + 0);
        w0 = fma(-hr0, widen(V[size_t(i) * vstride + off + c]), w0);
        w1 = fma(-hr1, widen(V[size_t(i + 1) * vstride + off + c]), w1);
        if (NC == 2) {
          // (hr + i hi)(v_re + i v_im): re = hr v_re - hi v_im, im = hr v_im + hi v_re
          const double hi0 = __ldg(h + (size_t(i) * K + k) * 2 + 1);
          const double hi1 = __ldg(h + (size_t(i + 1) * K + k) * 2 + 1);
          w0 = fma((c & 1) ? -hi0 : hi0, widen(V[size_t(i) * vstride + off + (c ^ 1)]), w0);
          w1 = fma((c & 1) ? -hi1 : hi1, widen(V[size_t(i + 1) * vstride + off + (c ^ 1)]), w1);
        }
      }
      if (i < Ju) {
        const double hr = __ldg(h + (size_t(i) * K + k) * 2 + 0);
        w0 = fma(-hr, widen(V[size_t(i) * vstride + off + c]), w0);
        if (NC == 2) {
          const double hi = __ldg(h + (size_t(i) * K + k) * 2 + 1);
          w0 = fma((c & 1) ? -hi : hi, widen(V[size_t(i) * vstride + off + (c ^ 1)]), w0);
        }
      }
      const double w = w0 + w1;
      const S wst = to_storage<S>(w);
      if (Ju > 0) W[off + c] = wst;
      const double ws = widen(wst);
      nrm = fma(ws, ws, nrm);
    }
  }
  red[threadIdx.x] = (rg < RG) ? nrm : 0.0;
  __syncthreads();
  if (threadIdx.x < C && !(need && need[threadIdx.x / ncomp] == 0)) {
    double s = 0.0;
    for (int g = 0; g < RG; ++g) s += red[g * C + threadIdx.x];
    npart[size_t(blockIdx.x) * C + threadIdx.x] = s;
  }
}

// k_update for FP32 real panels with double-float arithmetic: W -= sum_i
// h_i V_i and the new |W|^2 partials, FP64-class (lgt_dfloat.cuh) with the
// FP64 pipe used only to split the coefficients.  The block first splits
// its columns' coefficients h into FP32 pairs hh + hl in shared memory
// (sh: [J][C] pairs); each thread then runs four rows at a time, four basis
// vectors per trip with their loads issued first.  Same partition,
// skipping rules and outputs as k_update.
__global__ void __launch_bounds__(kT) k_update_df(const float* __restrict__ V, size_t vstride,
                                                  const int* jstate, float* __restrict__ W,
                                                  int64_t N, int C, const double* __restrict__ h,
                                                  int K, const int* status, int64_t rpb,
                                                  double* npart, const int* need) {
  extern __shared__ float sh[];  // hh[J][C], then hl[J][C]
  __shared__ double red[kT];
  const int J = *jstate + 1;
  float* s_hh = sh;
  float* s_hl = sh + size_t(J) * C;
  for (int idx = threadIdx.x; idx < J * C; idx += kT) {
    const int i = idx / C, cc = idx - i * C;
    const double hv = h[(size_t(i) * K + cc) * 2];
    const float hh = narrow(hv);
    s_hh[idx] = hh;
    s_hl[idx] = narrow(hv - widen(hh));
  }
  __syncthreads();
  const int RG = kT / C;
  const int c = threadIdx.x % C, rg = threadIdx.x / C;
  const int k = c;
  const bool act = rg < RG && (!status || status[k] == kActive) && !(need && need[k] == 0);
  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int64_t r1 = (r0 + rpb < N) ? r0 + rpb : N;
  df nrm{0.f, 0.f};
  if (act) {
    // four rows at a time, four basis vectors per trip: sixteen loads in
    // flight before the arithmetic.  Each row's sum is Dot2-style (Ogita,
    // Rump, Oishi): the leading parts by TwoSum, the trailing parts added in
    // FP32 -- at most J + 1 terms per entry, so its error stays at the
    // FP32 rounding of the result plus J^2 2^-48 of the terms' sizes.
    constexpr int kRows = 4;
    int64_t row = r0 + rg;
    for (; row + (kRows - 1) * int64_t(RG) < r1; row += kRows * int64_t(RG)) {
      size_t o[kRows];
      float hi[kRows], lo[kRows];
#pragma unroll
      for (int q = 0; q < kRows; ++q) {
        o[q] = size_t(row + q * int64_t(RG)) * C + c;
        hi[q] = W[o[q]];
        lo[q] = 0.f;
      }
      const float* vi = V;
      int i = 0;
      for (; i + 3 < J; i += 4, vi += 4 * vstride) {
        float x[4][kRows];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int q = 0; q < kRows; ++q) x[u][q] = __ldg(vi + u * vstride + o[q]);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float hh = s_hh[(i + u) * C + c], hl = s_hl[(i + u) * C + c];
#pragma unroll
          for (int q = 0; q < kRows; ++q) {
            float p, e, t;
            two_prod(hh, x[u][q], p, e);
            e = df_fma_rn(hl, x[u][q], e);
            two_sum(hi[q], -p, hi[q], t);
            lo[q] = df_add_rn(lo[q], df_sub_rn(t, e));
          }
        }
      }
      for (; i < J; ++i, vi += vstride) {
        const float hh = s_hh[i * C + c], hl = s_hl[i * C + c];
#pragma unroll
        for (int q = 0; q < kRows; ++q) {
          const float xv = __ldg(vi + o[q]);
          float p, e, t;
          two_prod(hh, xv, p, e);
          e = df_fma_rn(hl, xv, e);
          two_sum(hi[q], -p, hi[q], t);
          lo[q] = df_add_rn(lo[q], df_sub_rn(t, e));
        }
      }
#pragma unroll
      for (int q = 0; q < kRows; ++q) {
        const float sa = df_add_rn(hi[q], lo[q]);
        W[o[q]] = sa;
        df_fma(nrm, sa, sa);
      }
    }
    for (; row < r1; row += RG) {
      const size_t oa = size_t(row) * C + c;
      float hi = W[oa], lo = 0.f;
      const float* vi = V;
      for (int i = 0; i < J; ++i, vi += vstride) {
        const float xv = __ldg(vi + oa);
        float p, e, t;
        two_prod(s_hh[i * C + c], xv, p, e);
        e = df_fma_rn(s_hl[i * C + c], xv, e);
        two_sum(hi, -p, hi, t);
        lo = df_add_rn(lo, df_sub_rn(t, e));
      }
      const float sa = df_add_rn(hi, lo);
      W[oa] = sa;
      df_fma(nrm, sa, sa);
    }
  }
  red[threadIdx.x] = (rg < RG) ? widen(nrm.hi) + widen(nrm.lo) : 0.0;
  __syncthreads();
  if (threadIdx.x < C && !(need && need[threadIdx.x] == 0)) {
    double s = 0.0;
    for (int g = 0; g < RG; ++g) s += red[g * C + threadIdx.x];
    npart[size_t(blockIdx.x) * C + threadIdx.x] = s;
  }
}

// k_update_df with the panel rows streamed through shared memory by the
// copy engine.  A block's row range is cut into tiles of kBulkTile values
// (kBulkTile / C rows, contiguous in every panel); the chunks W_t, V_0,t,
// ..., V_{J-1},t of tile t follow one another through a ring of
// kBulkStages shared-memory stages, each refilled by one bulk copy as soon
// as the block has consumed it, so kBulkStages - 1 chunks are in flight
// while the block computes.  Thread (c, g) owns the values tid + kT e of a
// tile (column c, rows g + RG e): the same rows in the same order as
// k_update_df, with the same arithmetic, so W and the norm partials are
// bitwise those of k_update_df.  Needs kT % C == 0 and 16-byte aligned
// chunks (launch_update checks).  A copy that does not arrive within the
// bounded wait raises kDevErrSpin in `err`; the block then waits (bounded)
// for the copies it issued and leaves.

__global__ void __launch_bounds__(kT) k_update_bulk(const float* __restrict__ V, size_t vstride,
                                                    const int* jstate, float* W, int64_t N,
                                                    int C, const double* __restrict__ h, int K,
                                                    const int* status, int64_t rpb,
                                                    double* npart, const int* need, int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* s_buf = reinterpret_cast<float*>(smem_raw);  // [kBulkStages][kBulkTile]
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_buf + kBulkStages * kBulkTile);
  __shared__ double red[kT];
  const int J = *jstate + 1;
  float* s_hh = reinterpret_cast<float*>(s_bar + kBulkStages);  // [J][C]
  float* s_hl = s_hh + size_t(J) * C;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < J * C; idx += kT) {
    const int i = idx / C, cc = idx - i * C;
    const double hv = h[(size_t(i) * K + cc) * 2];
    const float hh = narrow(hv);
    s_hh[idx] = hh;
    s_hl[idx] = narrow(hv - widen(hh));
  }
  if (tid == 0) {
    for (int st = 0; st < kBulkStages; ++st) mbar_init(s_bar + st, 1);
    mbar_init_fence();
  }
  const int RG = kT / C;
  const int c = tid % C;
  const bool act = (!status || status[c] == kActive) && !(need && need[c] == 0);
  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int64_t r1 = (r0 + rpb < N) ? r0 + rpb : N;
  const int TR = kBulkTile / C;
  const int nt = (r1 > r0) ? int((r1 - r0 + TR - 1) / TR) : 0;
  // no active column in this pass: nothing to read (the partials of
  // columns that need no pass keep their values)
  const int any = __syncthreads_or(act ? 1 : 0);
  const int nchunks = any ? nt * (J + 1) : 0;
  auto issue = [&](int n) {  // thread 0: chunk n into its stage
    const int t = n / (J + 1), i = n - t * (J + 1) - 1;
    const int64_t rs = r0 + int64_t(t) * TR;
    const int rows = int((r1 - rs < TR) ? (r1 - rs) : TR);
    const float* src = (i < 0 ? W : V + size_t(i) * vstride) + size_t(rs) * C;
    const int st = n % kBulkStages;
    const uint32_t bytes = uint32_t(rows) * uint32_t(C) * 4u;
    mbar_arrive_expect_tx(s_bar + st, bytes);
    bulk_g2s(s_buf + size_t(st) * kBulkTile, src, bytes, s_bar + st);
  };
  const int pre = nchunks < kBulkStages ? nchunks : kBulkStages;
  if (tid == 0)
    for (int n = 0; n < pre; ++n) issue(n);
  float hi[kBulkElems], lo[kBulkElems];
  df nrm{0.f, 0.f};
  int n = 0;
  bool bad = false;
  // chunk n = tile t, slot i (-1: W, then the basis vectors), advanced
  // incrementally (no division per chunk)
  int i = -1;
  int64_t rs = r0;
  int vals = int((r1 - rs < TR) ? (r1 - rs) : TR) * C;
  for (; n < nchunks; ++n) {
    const int st = n % kBulkStages;
    if (!mbar_wait_bounded(s_bar + st, uint32_t(n / kBulkStages) & 1u)) bad = true;
    const float* buf = s_buf + size_t(st) * kBulkTile;
    if (!bad) {
      if (i < 0) {
#pragma unroll
        for (int e = 0; e < kBulkElems; ++e) {
          const int idx = tid + kT * e;
          hi[e] = idx < vals ? buf[idx] : 0.f;
          lo[e] = 0.f;
        }
      } else if (act) {
        // values past the tile's rows (a partial last tile) are computed on
        // whatever the stage holds and never stored
        const float hh = s_hh[i * C + c], hl = s_hl[i * C + c];
#pragma unroll
        for (int e = 0; e < kBulkElems; ++e) {
          const float xv = buf[tid + kT * e];
          float p, q, t2;
          two_prod(hh, xv, p, q);
          q = df_fma_rn(hl, xv, q);
          two_sum(hi[e], -p, hi[e], t2);
          lo[e] = df_add_rn(lo[e], df_sub_rn(t2, q));
        }
      }
      if (i == J - 1 && act) {
        float* wout = W + size_t(rs) * C;
#pragma unroll
        for (int e = 0; e < kBulkElems; ++e) {
          const int idx = tid + kT * e;
          if (idx < vals) {
            const float sa = df_add_rn(hi[e], lo[e]);
            wout[idx] = sa;
            df_fma(nrm, sa, sa);
          }
        }
      }
    }
    if (++i == J) {
      i = -1;
      rs += TR;
      vals = int((r1 - rs < TR) ? (r1 - rs) : TR) * C;
    }
    // the stage is free once every thread has read it
    if (__syncthreads_or(bad ? 1 : 0)) {
      bad = true;
      break;
    }
    if (tid == 0 && n + kBulkStages < nchunks) issue(n + kBulkStages);
  }
  if (bad) {
    // copies issued and not consumed: chunks n .. min(n + kBulkStages, nchunks) - 1
    if (tid == 0) {
      const int last = (n + kBulkStages < nchunks) ? n + kBulkStages : nchunks;
      for (int m = n; m < last; ++m)
        mbar_wait_bounded(s_bar + (m % kBulkStages), uint32_t(m / kBulkStages) & 1u);
      if (err) atomicOr(err, kDevErrSpin);
    }
    __syncthreads();
  }
  red[tid] = (tid / C < RG) ? widen(nrm.hi) + widen(nrm.lo) : 0.0;
  __syncthreads();
  if (tid < C && !(need && need[tid] == 0)) {
    double s = 0.0;
    for (int g = 0; g < RG; ++g) s += red[g * C + tid];
    npart[size_t(blockIdx.x) * C + tid] = s;
  }
}

// Sum over blocks of point k's partial norms (warp per point, fixed order).
__device__ __forceinline__ double point_norm2(const double* npart, int nblk, int C, int ncomp,
                                              int k, int lane) {
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32)
    for (int q = 0; q < ncomp; ++q) s += npart[size_t(b) * C + k * ncomp + q];
  return warp_total(s);
}

// After a Gram-Schmidt pass: a further pass is needed for point k only when
// the pass cancelled more than two digits, ||W_after||^2 < 1e-4 ||W_before||^2.
// One warp per point.
__global__ void k_need_pass(const double* npart, int nblk, int K, int C, int ncomp,
                            const int* status, double* nb, int* need) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= K) return;
  const double s = point_norm2(npart, nblk, C, ncomp, k, lane);
  if (lane != 0) return;
  need[k] = (status[k] == kActive && s < 1e-4 * nb[k]) ? 1 : 0;
  nb[k] = s;
}

// beta_j = ||W|| per point.  A Krylov space that has become invariant
// (beta below the relative threshold) marks the point exhausted: its Ritz
// pair on the current basis is exact.  One warp per point.
__global__ void k_finish_norm(const double* npart, int nblk, int K, int C, int ncomp,
                              const int* jstate, double* beta, const double* alpha, int ldT,
                              int* status, int* len, double* bnorm, double tiny_rel, int write_beta) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= K) return;
  const double s = point_norm2(npart, nblk, C, ncomp, k, lane);
  if (lane != 0) return;
  const double nb = sqrt(s);
  bnorm[k] = nb;
  if (!write_beta || status[k] != kActive) return;
  const int j = *jstate;
  beta[size_t(k) * ldT + j] = nb;
  len[k] = j + 1;
  double scale = fabs(alpha[size_t(k) * ldT + j]);
  if (j > 0) scale = fmax(scale, beta[size_t(k) * ldT + j - 1]);
  scale = fmax(scale, 1.0);
  if (!(nb > tiny_rel * scale)) status[k] = kExhausted;
}

// dst = src / bnorm per column for points with status == sel.  dst is panel
// (*jstate + dst_off) of `dstbase` when jstate is given.  Each thread owns one
// column (one reciprocal, no per-element division or modulo); launched with
// kT threads per block.
template <typename SI, typename SO>
__global__ void k_scale(const SI* src, SO* dstbase, size_t vstride, const int* jstate, int dst_off,
                        int64_t N, int C, int ncomp, const double* bnorm, const int* status,
                        int sel, const int* gather) {
  SO* dst = dstbase + size_t((jstate ? *jstate : 0) + dst_off) * vstride;
  const int RG = kT / C;
  const int c = threadIdx.x % C, rg = threadIdx.x / C;
  if (rg >= RG) return;
  const int k = c / ncomp;
  if (status && status[k] != sel) return;
  const double b = bnorm[k];
  const double inv = (b > 0.0) ? 1.0 / b : 0.0;
  const float invf = float(inv);
  const int64_t step = int64_t(gridDim.x) * RG;
  int64_t row = int64_t(blockIdx.x) * RG + rg;
  if (sizeof(SI) == 4 && sizeof(SO) == 4 && !gather) {
    // FP32 to FP32 (the new Krylov vector): four rows' loads in flight
    // before their stores
    for (; row + 3 * step < N; row += 4 * step) {
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = float(src[size_t(row + u * step) * C + c]);
#pragma unroll
      for (int u = 0; u < 4; ++u) dst[size_t(row + u * step) * C + c] = SO(v[u] * invf);
    }
  }
  for (; row < N; row += step) {
    const size_t i = size_t(row) * C + c;
    // gather: row `row` of the destination is row gather[row] of the source
    const size_t si = gather ? size_t(gather[row]) * C + c : i;
    if (sizeof(SI) == 4 && sizeof(SO) == 4)
      dst[i] = SO(float(src[si]) * invf);
    else
      dst[i] = SO(double(src[si]) * inv);
  }
}

// k_scale for FP32 panels whose width is a multiple of 4 (no gather): a
// thread keeps four consecutive columns (the grid's thread count is a
// multiple of C / 4, so the columns stay put) and moves 16 bytes per access;
// columns of points not in state `sel` keep their values.
__global__ void __launch_bounds__(kT) k_scale_f4(const float* __restrict__ src, float* dstbase,
                                                 size_t vstride, const int* jstate, int dst_off,
                                                 int64_t N, int C, int ncomp,
                                                 const double* bnorm, const int* status, int sel) {
  float* dst = dstbase + size_t((jstate ? *jstate : 0) + dst_off) * vstride;
  const int C4 = C / 4;
  const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t nthr = int64_t(gridDim.x) * blockDim.x;
  const int c0 = int(tid % C4) * 4;
  float inv[4];
  bool on[4];
  bool all = true;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int k = (c0 + e) / ncomp;
    on[e] = !status || status[k] == sel;
    const double b = bnorm[k];
    inv[e] = float((b > 0.0) ? 1.0 / b : 0.0);
    all = all && on[e];
  }
  const int64_t n4 = N * C4;
  for (int64_t i = tid; i < n4; i += nthr) {
    const float4 v = reinterpret_cast<const float4*>(src)[i];
    const float4 o = make_float4(v.x * inv[0], v.y * inv[1], v.z * inv[2], v.w * inv[3]);
    if (all) {
      reinterpret_cast<float4*>(dst)[i] = o;
    } else {
      float* d = dst + 4 * i;
      if (on[0]) d[0] = o.x;
      if (on[1]) d[1] = o.y;
      if (on[2]) d[2] = o.z;
      if (on[3]) d[3] = o.w;
    }
  }
}

__global__ void k_advance(int* jstate) { jstate[0] += 1; }

__global__ void k_set_int(int* p, int n, int v, const int* status, int only_status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && (!status || status[i] == only_status)) p[i] = v;
}

// ---- tridiagonal solvers -----------------------------------------------------

// Ground-state convergence check, one warp per point:
// Ritz value theta, residual beta_{n-1} |z_{n-1}|, coefficients z.
__global__ void k_check_lowest(const double* alpha, const double* beta, int ldT, int* status,
                               const int* len, double* theta, double* resid, double* coef,
                               double tol, int fp32) {
  // one warp per point: warp multisection of the Sturm count (FP32 for the
  // mixed path, whose basis resolves no more), bracket warm-started from
  // this point's previous theta and residual (verified by Sturm counts, so
  // stale values only cost the fallback to the Gershgorin interval)
  __shared__ double s_a[kMaxDim], s_b[kMaxDim], s_z[kMaxDim], s_work[3 * kMaxDim];
  const int k = blockIdx.x, lane = threadIdx.x;
  const int st = status[k];
  if (st >= kConverged) return;
  const int n = len[k];
  if (n <= 0) return;
  for (int i = lane; i < n; i += 32) {
    s_a[i] = alpha[size_t(k) * ldT + i];
    s_b[i] = (i < n - 1) ? beta[size_t(k) * ldT + i] : 0.0;
  }
  __syncwarp();
  const double tp = theta[k], rp = resid[k];
  const bool warm = isfinite(tp) && isfinite(rp);
  const double th = fp32 ? warp_lowest_eig_f32(s_a, s_b, n, s_z, s_work, warm, false, tp, rp)
                         : warp_lowest_eig(s_a, s_b, n, s_z, s_work, warm, false, tp, rp);
  const double r = fabs(beta[size_t(k) * ldT + n - 1] * s_z[n - 1]);
  for (int i = lane; i < ldT; i += 32) {
    coef[(size_t(k) * ldT + i) * 2 + 0] = (i < n) ? s_z[i] : 0.0;
    coef[(size_t(k) * ldT + i) * 2 + 1] = 0.0;
  }
  if (lane != 0) return;
  theta[k] = th;
  resid[k] = (st == kExhausted) ? 0.0 : r;
  if (st == kExhausted || r <= tol) status[k] = kConverged;
}

// Implicit QL with eigenvectors (symmetric tridiagonal, Wilkinson-type
// shift), one block per point, thread r owning row r of Z.  Thread 0 runs
// the scalar chase and records the plane rotations; all threads then apply
// them to their own row, so no row depends on another.
__device__ bool ql_eigen(double* d, double* e, double* Z, int n, int ldz, double* rc, double* rs,
                         int* nrot_out) {
  const int r = threadIdx.x;
  for (int i = r; i < n; i += blockDim.x)
    for (int j = 0; j < n; ++j) Z[i * ldz + j] = (i == j) ? 1.0 : 0.0;
  __shared__ int s_l, s_m, s_nrot, s_done, s_fail;
  if (r == 0) {
    e[n - 1] = 0.0;
    s_l = 0;
    s_fail = 0;
  }
  __syncthreads();
  int iters = 0;
  while (true) {
    if (r == 0) {
      s_done = 0;
      s_nrot = 0;
      int l = s_l;
      // advance l past converged eigenvalues
      while (l < n) {
        int m = l;
        for (; m < n - 1; ++m) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= 2.2e-16 * dd) break;
        }
        if (m == l) {
          ++l;
          iters = 0;
          continue;
        }
        s_m = m;
        break;
      }
      s_l = l;
      if (l >= n) {
        s_done = 1;
      } else if (++iters > 100) {
        s_fail = 1;
        s_done = 1;
      } else {
        const int m = s_m;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double rr = hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + copysign(rr, g));
        double s = 1.0, c = 1.0, p = 0.0;
        int nrot = 0;
        bool early = false;
        for (int i = m - 1; i >= l; --i) {
          double f = s * e[i];
          const double b = c * e[i];
          rr = hypot(f, g);
          e[i + 1] = rr;
          if (rr == 0.0) {
            d[i + 1] -= p;
            e[m] = 0.0;
            early = true;
            break;
          }
          s = f / rr;
          c = g / rr;
          g = d[i + 1] - p;
          rr = (d[i] - g) * s + 2.0 * c * b;
          p = s * rr;
          d[i + 1] = g + p;
          g = c * rr - b;
          rc[nrot] = c;
          rs[nrot] = s;
          ++nrot;
        }
        if (!early) {
          d[l] -= p;
          e[l] = g;
          e[m] = 0.0;
        }
        s_nrot = nrot;
      }
    }
    __syncthreads();
    if (s_done) break;
    const int m = s_m, nrot = s_nrot;
    for (int row = r; row < n; row += blockDim.x) {
      double* zr = Z + row * ldz;
      for (int q = 0; q < nrot; ++q) {
        const int i = m - 1 - q;
        const double f = zr[i + 1];
        zr[i + 1] = rs[q] * zr[i] + rc[q] * f;
        zr[i] = rc[q] * zr[i] - rs[q] * f;
      }
    }
    __syncthreads();
  }
  if (nrot_out) *nrot_out = 0;
  return s_fail == 0;
}

// Krylov exponential check, one block per point: c = rho exp(-i tau T) e_0
// from the eigendecomposition of T_n, error estimate rho beta_{n-1} |c_{n-1}|.
// force: store the coefficients and mark converged regardless of the error.
__global__ void k_check_expm(const double* alpha, const double* beta, int ldT, int* status,
                             const int* len, const double* rho, double tau, double* err_out,
                             double* coef, double tol, int force, int* fail) {
  __shared__ double d[kMaxDim], e[kMaxDim], Z[kMaxDim * kMaxDim], rc[kMaxDim], rs[kMaxDim];
  __shared__ double cre[kMaxDim], cim[kMaxDim];
  const int k = blockIdx.x;
  const int st = status[k];
  if (st >= kConverged) return;
  const int n = len[k];
  if (n <= 0) return;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d[i] = alpha[size_t(k) * ldT + i];
    e[i] = (i < n - 1) ? beta[size_t(k) * ldT + i] : 0.0;
  }
  __syncthreads();
  const bool ok = ql_eigen(d, e, Z, n, kMaxDim, rc, rs, nullptr);
  if (!ok && threadIdx.x == 0) atomicOr(fail, 1);
  __syncthreads();
  // c_i = rho * sum_l Z[i][l] exp(-i tau lambda_l) Z[0][l]
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double sr = 0.0, si = 0.0;
    for (int l = 0; l < n; ++l) {
      double sn, cs;
      sincos(-tau * d[l], &sn, &cs);
      const double w = Z[i * kMaxDim + l] * Z[l];
      sr = fma(w, cs, sr);
      si = fma(w, sn, si);
    }
    cre[i] = rho[k] * sr;
    cim[i] = rho[k] * si;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double bl = beta[size_t(k) * ldT + n - 1];
    const double err = (st == kExhausted) ? 0.0 : fabs(bl) * hypot(cre[n - 1], cim[n - 1]);
    err_out[k] = err;
    if (force || st == kExhausted || err <= tol) {
      for (int i = 0; i < ldT; ++i) {
        coef[(size_t(k) * ldT + i) * 2 + 0] = (i < n) ? cre[i] : 0.0;
        coef[(size_t(k) * ldT + i) * 2 + 1] = (i < n) ? cim[i] : 0.0;
      }
      status[k] = kConverged;
    }
  }
}

// out = sum_{i < len[k]} coef[k][i] V_i for points with status == sel
// (complex coefficients for NC = 2).
template <typename S, int NC>
__global__ void k_combine(const S* __restrict__ V, size_t vstride, const double* coef, int ldT,
                          const int* len, const int* status, int sel, double* out, int64_t N,
                          int C, int ncomp, const int* scatter) {
  const int64_t n = N * C;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < n;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = idx / C;
    const int c = int(idx - row * C);
    const int k = c / ncomp;
    if (status[k] != sel) continue;
    const int nk = len[k];
    const size_t off = size_t(row) * C;
    double acc = 0.0;
    for (int i = 0; i < nk; ++i) {
      const double cr = coef[(size_t(k) * ldT + i) * 2 + 0];
      const double v = widen(V[size_t(i) * vstride + off + c]);
      if (NC == 1) {
        acc = fma(cr, v, acc);
      } else {
        const double ci = coef[(size_t(k) * ldT + i) * 2 + 1];
        const double vp = widen(V[size_t(i) * vstride + off + (c ^ 1)]);
        acc += (c & 1) ? (cr * v + ci * vp) : (cr * v - ci * vp);
      }
    }
    // scatter: row `row` of the basis is row scatter[row] of the output
    out[(scatter ? size_t(scatter[row]) * C : off) + c] = acc;
  }
}

// Split exponential (real Krylov columns 2k = Re psi_k and 2k+1 = Im psi_k,
// each with complex coefficients c = rho exp(-i tau T) e_0 from its own
// tridiagonal): psi_k = sum_i c^re_i V_i[2k] + i sum_i c^im_i V_i[2k+1].
template <typename S>
__global__ void k_combine_split(const S* __restrict__ V, size_t vstride, const double* coef,
                                int ldT, const int* len, double* out, int64_t N, int K,
                                const int* scatter) {
  const int C = 2 * K;
  const int64_t n = N * C;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < n;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = idx / C;
    const int c = int(idx - row * C);
    const int comp = c & 1, ca = c & ~1, cb = ca + 1;
    const size_t off = size_t(row) * C;
    double acc = 0.0;
    const int na = len[ca], nb = len[cb];
    // the real column contributes (Re c) v to Re psi and (Im c) v to Im psi
    for (int i = 0; i < na; ++i)
      acc = fma(coef[(size_t(ca) * ldT + i) * 2 + comp], widen(V[size_t(i) * vstride + off + ca]),
                acc);
    // i (cr + i ci) v = -ci v + i cr v
    for (int i = 0; i < nb; ++i) {
      const double cf = comp ? coef[(size_t(cb) * ldT + i) * 2 + 0]
                             : -coef[(size_t(cb) * ldT + i) * 2 + 1];
      acc = fma(cf, widen(V[size_t(i) * vstride + off + cb]), acc);
    }
    out[(scatter ? size_t(scatter[row]) * C : off) + c] = acc;
  }
}

// k_combine_split for an FP32 basis with double-float sums: one thread per
// (row, point) forms both outputs from the float pair (v_i[re col],
// v_i[im col]) of each basis vector, with the FP64 coefficients split once
// per block into FP32 pairs (shared memory, [C][ldT][2] pairs) and the sums
// carried as double-floats (TwoSum of the leading parts, trailing parts
// summed apart): FP64-class results without FP64 FMAs per element.
__global__ void __launch_bounds__(kT) k_combine_split_df(const float* __restrict__ V,
                                                         size_t vstride, const double* coef,
                                                         int ldT, const int* len, double* out,
                                                         int64_t N, int K, const int* scatter) {
  extern __shared__ float s_cf[];  // [C][ldT][2] hi, then [C][ldT][2] lo
  const int C = 2 * K;
  const int ncf = C * ldT * 2;
  float* s_hi = s_cf;
  float* s_lo = s_cf + ncf;
  for (int i = threadIdx.x; i < ncf; i += blockDim.x) {
    const double cv = coef[i];
    const float h = narrow(cv);
    s_hi[i] = h;
    s_lo[i] = narrow(cv - widen(h));
  }
  __syncthreads();
  const int64_t n = N * K;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < n;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = idx / K;
    const int k = int(idx - row * K);
    const int ca = 2 * k, cb = ca + 1;
    const size_t off = size_t(row) * C + ca;
    df re{0.f, 0.f}, im{0.f, 0.f};
    const int na = len[ca], nb = len[cb];
    const int nmax = na > nb ? na : nb;
    auto term = [](df& acc, float ch, float cl, float v) {
      float p, e, t;
      two_prod(ch, v, p, e);
      e = df_fma_rn(cl, v, e);
      two_sum(acc.hi, p, acc.hi, t);
      acc.lo = df_add_rn(acc.lo, df_add_rn(t, e));
    };
    for (int i = 0; i < nmax; ++i) {
      const float2 v = *reinterpret_cast<const float2*>(V + size_t(i) * vstride + off);
      if (i < na) {  // the real column: (Re c) v to Re psi, (Im c) v to Im psi
        const int q = (ca * ldT + i) * 2;
        term(re, s_hi[q], s_lo[q], v.x);
        term(im, s_hi[q + 1], s_lo[q + 1], v.x);
      }
      if (i < nb) {  // i (cr + i ci) v = -ci v + i cr v
        const int q = (cb * ldT + i) * 2;
        term(re, -s_hi[q + 1], -s_lo[q + 1], v.y);
        term(im, s_hi[q], s_lo[q], v.y);
      }
    }
    double* o = out + (scatter ? size_t(scatter[row]) * C : size_t(row) * C) + ca;
    o[0] = widen(re.hi) + widen(re.lo);
    o[1] = widen(im.hi) + widen(im.lo);
  }
}

__global__ void k_residual_parts(const double* X, const double* HX, const double* E, int64_t N,
                                 int C, int ncomp, int64_t rpb, double* npart) {
  __shared__ double red[kT];
  const int RG = kT / C;
  const int c = threadIdx.x % C, rg = threadIdx.x / C;
  const int k = c / ncomp;
  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int64_t r1 = (r0 + rpb < N) ? r0 + rpb : N;
  double nrm = 0.0;
  if (rg < RG) {
    for (int64_t row = r0 + rg; row < r1; row += RG) {
      const size_t off = size_t(row) * C + c;
      const double r = HX[off] - E[k] * X[off];
      nrm = fma(r, r, nrm);
    }
  }
  red[threadIdx.x] = (rg < RG) ? nrm : 0.0;
  __syncthreads();
  if (threadIdx.x < C) {
    double s = 0.0;
    for (int g = 0; g < RG; ++g) s += red[g * C + threadIdx.x];
    npart[size_t(blockIdx.x) * C + threadIdx.x] = s;
  }
}



// ---- host-side machinery -------------------------------------------------------

int grid_for(int64_t n) {
  int64_t b = (n + kT - 1) / kT;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return int(b);
}

// Row partition of the two-stage reductions: enough rows per block to keep
// its threads busy, at most LGT_RED_BLOCKS blocks.
#ifndef LGT_RED_ELEMS
#define LGT_RED_ELEMS 2048  // panel elements per reduction block (at most; 4x3 K=16: 4096 was 30% slower)
#endif
#ifndef LGT_RED_BLOCKS
#define LGT_RED_BLOCKS 608  // 4 blocks per SM: the reductions are latency-bound
#endif
constexpr int kRedMaxBlocks = 1216;  // 8 per SM: the largest candidate of the tuner
struct Reducer {
  int nblk = 1;
  int64_t rpb = 1;
  void plan(int64_t N, int C, int cap = LGT_RED_BLOCKS) {
    const int RG = kT / C;
    int64_t want = (N * C + LGT_RED_ELEMS - 1) / LGT_RED_ELEMS;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    rpb = (N + want - 1) / want;
    if (rpb < RG) rpb = RG;
    nblk = int((N + rpb - 1) / rpb);
    if (nblk < 1) nblk = 1;
  }
};

// Device workspace of one driver in one storage precision, reused across
// calls while the shape is unchanged (allocation synchronises the device).
template <typename S>
struct Work {
  int64_t N = -1;
  int C = 0, K = 0, ncomp = 1, m = 0, ldT = 0;
  // Components per coupling point seen by H*psi: equal to ncomp, except in
  // the split exponential, where the Krylov columns are real (ncomp = 1)
  // and H*psi pairs them as (re, im) of one point (hcomp = 2).
  int hcomp = 1;
  bool lite = false;  // reduction buffers only (no Krylov panels)
  size_t vstride = 0;
  S* V = nullptr;        // m+1 Krylov panels
  S* W = nullptr;        // H V_j, then the new residual vector
  double* R = nullptr;   // FP64 panel for H X and residuals
  double* part = nullptr;
  double* npart = nullptr;
  double* h = nullptr;
  double* alpha = nullptr;
  double* beta = nullptr;
  double* coef = nullptr;
  double* theta = nullptr;
  double* resid = nullptr;
  double* bnorm = nullptr;
  double* rho = nullptr;
  double* zeros = nullptr;
  double* nb = nullptr;   // ||W||^2 before the latest Gram-Schmidt pass
  int* need = nullptr;    // further pass needed, per point
  int* status = nullptr;
  int* len = nullptr;
  int* jstate = nullptr;
  int* fail = nullptr;
  Reducer red;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0, graph_reorth = 0;
  double graph_tiny = 0.0;
  uint64_t graph_op = 0;
  int graph_nodes = 0;

  std::string ensure(int64_t N_, int C_, int K_, int ncomp_, int m_, int hcomp_ = 0,
                     bool lite_ = false) {
    if (hcomp_ <= 0) hcomp_ = ncomp_;
    if (N_ == N && C_ == C && K_ == K && ncomp_ == ncomp && m_ == m && hcomp_ == hcomp &&
        lite_ == lite && part)
      return std::string();
    release();
    N = N_;
    C = C_;
    K = K_;
    ncomp = ncomp_;
    m = m_;
    hcomp = hcomp_;
    lite = lite_;
    ldT = m + 1;
    vstride = size_t(N) * C;
    red.plan(N, C, kRedMaxBlocks);  // partial-sum buffers for the largest block count
    const int nblk_max = red.nblk;
    red.plan(N, C);
    if (!lite) {
      KCK(cudaMalloc(&V, sizeof(S) * vstride * (m + 1)));
      KCK(cudaMalloc(&W, sizeof(S) * vstride));
      KCK(cudaMalloc(&R, sizeof(double) * vstride));
    }
    KCK(cudaMalloc(&part, sizeof(double) * size_t(nblk_max) * ldT * 2 * C));
    KCK(cudaMalloc(&npart, sizeof(double) * size_t(nblk_max) * C));
    KCK(cudaMalloc(&h, sizeof(double) * size_t(ldT) * K * 2));
    KCK(cudaMalloc(&alpha, sizeof(double) * size_t(K) * ldT));
    KCK(cudaMalloc(&beta, sizeof(double) * size_t(K) * ldT));
    KCK(cudaMalloc(&coef, sizeof(double) * size_t(K) * ldT * 2));
    KCK(cudaMalloc(&theta, sizeof(double) * K));
    KCK(cudaMalloc(&resid, sizeof(double) * K));
    KCK(cudaMalloc(&bnorm, sizeof(double) * K));
    KCK(cudaMalloc(&rho, sizeof(double) * K));
    KCK(cudaMalloc(&zeros, sizeof(double) * K));
    KCK(cudaMemset(zeros, 0, sizeof(double) * K));
    KCK(cudaMalloc(&nb, sizeof(double) * K));
    KCK(cudaMalloc(&need, sizeof(int) * K));
    KCK(cudaMalloc(&status, sizeof(int) * K));
    KCK(cudaMalloc(&len, sizeof(int) * K));
    KCK(cudaMalloc(&jstate, sizeof(int) * 4));
    KCK(cudaMalloc(&fail, sizeof(int)));
    return std::string();
  }
  // Re-partition the reductions (the captured graph holds the old one).
  void replan(int cap) {
    red.plan(N, C, cap);
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_steps = 0;
  }
  void release() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_steps = 0;
    cudaFree(V);
    cudaFree(W);
    cudaFree(R);
    cudaFree(part);
    cudaFree(npart);
    cudaFree(h);
    cudaFree(alpha);
    cudaFree(beta);
    cudaFree(coef);
    cudaFree(theta);
    cudaFree(resid);
    cudaFree(bnorm);
    cudaFree(rho);
    cudaFree(zeros);
    cudaFree(nb);
    cudaFree(need);
    cudaFree(status);
    cudaFree(len);
    cudaFree(jstate);
    cudaFree(fail);
    V = W = nullptr;
    R = part = npart = h = alpha = beta = coef = theta = resid = bnorm = rho = zeros = nb = nullptr;
    status = len = jstate = fail = need = nullptr;
    N = -1;
  }
};

template <typename S>
cudaError_t apply_h(const OpDev& op, const S* x, const int* xsel, size_t xstride, S* y, int ncomp,
                    cudaStream_t s, int nslots = 1);

template <typename S>
void set_table(const OpDev& op, HpsiArgs<S>* a) {
  const bool ord = op.krylov_order && op.table_ord && op.table_ord->state == 1;
  const NbrTable* T = ord ? op.table_ord : op.table;
  a->table_order = ord ? 1 : 0;
  if (!op.use_table || !T || T->state != 1) return;
  a->t_meta = T->meta;
  a->t_off = T->tile_off;
  a->t_nbr = T->nbr;
  a->t_mm = T->mm;
  a->use_table = 1;
}

template <>
cudaError_t apply_h<double>(const OpDev& op, const double* x, const int* xsel, size_t xstride,
                            double* y, int ncomp, cudaStream_t s, int) {
  HpsiArgs<double> a;
  a.G = op.G;
  a.R = op.R;
  a.x = x;
  a.y = y;
  a.N = op.R.dim;
  a.C = op.K * ncomp;
  a.ncomp = ncomp;
  a.K = op.K;
  a.cE = op.cE_d;
  a.cm = op.cm_d;
  a.ch = op.ch_d;
  a.cp = op.cp_d;
  a.err = op.err;
  a.seg_smem = op.seg_smem;
  a.xsel = xsel;
  a.xstride = xstride;
  a.force_generic = op.force_generic;
  a.vpl = op.vpl;
  set_table(op, &a);
  return launch_hpsi<double>(a, op.model, s);
}

template <>
cudaError_t apply_h<float>(const OpDev& op, const float* x, const int* xsel, size_t xstride,
                           float* y, int ncomp, cudaStream_t s, int nslots) {
  HpsiArgs<float> a;
  a.G = op.G;
  a.R = op.R;
  a.x = x;
  a.y = y;
  a.N = op.R.dim;
  a.C = op.K * ncomp;
  a.ncomp = ncomp;
  a.K = op.K;
  a.cE = op.cE_f;
  a.cm = op.cm_f;
  a.ch = op.ch_f;
  a.cp = op.cp_f;
  a.err = op.err;
  a.seg_smem = op.seg_smem;
  a.xsel = xsel;
  a.xstride = xstride;
  a.force_generic = op.force_generic;
  a.vpl = op.vpl;
  // rows behind x: every Krylov slot when x + xsel * xstride picks one
  a.x_rows = xsel ? int64_t(xstride / size_t(a.C)) * nslots : a.N;
  set_table(op, &a);
  return launch_hpsi<float>(a, op.model, s);
}

// Whether the table kernel accepts the driver's H*psi panels (the Krylov
// basis with its device-resident panel offset): the condition for keeping
// the Krylov vectors in the table's row order.
template <typename S>
bool table_serves(const OpDev& op, const Work<S>& w) {
  HpsiArgs<S> a;
  a.x = w.V;
  a.y = w.W;
  a.C = op.K * w.hcomp;
  a.xsel = w.jstate;
  a.xstride = w.vstride;
  a.t_meta = op.table_ord ? op.table_ord->meta : nullptr;
  return table_load_mode(a, nullptr);
}

// Whether the bulk-copy kernels can stream this Work's panels: the block's column
// mapping (kT % C == 0) and 16-byte aligned chunks (panel bases, the panel
// stride, every block's first row and the end of the panel).
// LGT_BULK_STREAM=0 in the environment keeps k_update_df (cross-checks).
template <typename S>
bool bulk_stream_ok(const Work<S>& w, const void* V, size_t vstride, const void* Wp,
                    const int* err) {
  const char* e = getenv("LGT_BULK_STREAM");
  if (e && e[0] == '0') return false;
  const size_t C = size_t(w.C);
  return err && C > 0 && kT % w.C == 0 && (reinterpret_cast<uintptr_t>(V) % 16) == 0 &&
         (reinterpret_cast<uintptr_t>(Wp) % 16) == 0 && (vstride % 4) == 0 &&
         ((size_t(w.red.rpb) * C) % 4) == 0 && ((size_t(w.N) * C) % 4) == 0;
}

template <typename S, typename SV>
cudaError_t launch_multidot(Work<S>& w, const SV* V, size_t vstride, const int* jstate, int jfixed,
                            const SV* Wp, cudaStream_t s, int self = 0,
                            const int* need = nullptr, int* err = nullptr) {
  const int RG = kT / w.C;
  const size_t sh = sizeof(double) * size_t(RG) * kIC * 2 * w.C;
  const int dw = df_reductions_enabled() ? 1 : 0;
  if constexpr (sizeof(SV) == 4) {
    // measured slower than k_multidot on the 4x4 quench panel (2.42 vs
    // 1.72 ms against 15 vectors): opt in with LGT_BULK_DOTS=1
    const char* bd = getenv("LGT_BULK_DOTS");
    if (bd && bd[0] == '1' && w.ncomp == 1 && dw && jstate &&
        bulk_stream_ok(w, V, vstride, Wp, err)) {
      const size_t shb = sizeof(float) * kBulkStages * kBulkTile + 8 * kBulkStages + sh;
      cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(k_multidot_bulk), int(shb));
      if (e != cudaSuccess) return e;
      k_multidot_bulk<<<w.red.nblk, kT, shb, s>>>(V, vstride, jstate, Wp, w.N, w.C, w.red.rpb,
                                                  w.part, w.ldT, self, need, err),
          lgt::note_launch();
      return cudaGetLastError();
    }
  }
  if (w.ncomp == 1)
    k_multidot<SV, 1><<<w.red.nblk, kT, sh, s>>>(V, vstride, jstate, jfixed, Wp, w.N, w.C,
                                                 w.red.rpb, w.part, w.ldT, self, need,
                                                 w.ncomp, dw), lgt::note_launch();
  else
    k_multidot<SV, 2><<<w.red.nblk, kT, sh, s>>>(V, vstride, jstate, jfixed, Wp, w.N, w.C,
                                                 w.red.rpb, w.part, w.ldT, self, need,
                                                 w.ncomp, dw), lgt::note_launch();
  return cudaGetLastError();
}

// Shared memory of k_update_df's coefficient split for the largest step of
// a Work (m + 1 vectors); above this budget the FP64 update runs.
constexpr size_t kUpdDfSmemMax = 96 * 1024;

template <typename S>
cudaError_t launch_update(Work<S>& w, S* Wp, cudaStream_t s, const int* need = nullptr,
                          int* err = nullptr) {
  if constexpr (sizeof(S) == 4) {
    const size_t sh = size_t(w.ldT) * size_t(w.C) * 2 * sizeof(float);
    if (w.ncomp == 1 && df_reductions_enabled() && sh <= kUpdDfSmemMax &&
        bulk_stream_ok(w, w.V, w.vstride, Wp, err)) {
      const size_t shb = sizeof(float) * kBulkStages * kBulkTile + 8 * kBulkStages + sh;
      cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(k_update_bulk), int(shb));
      if (e != cudaSuccess) return e;
      k_update_bulk<<<w.red.nblk, kT, shb, s>>>(w.V, w.vstride, w.jstate, Wp, w.N, w.C, w.h,
                                                w.K, w.status, w.red.rpb, w.npart, need, err),
          lgt::note_launch();
      return cudaGetLastError();
    }
    if (w.ncomp == 1 && df_reductions_enabled() && sh <= kUpdDfSmemMax) {
      cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(k_update_df), int(sh));
      if (e != cudaSuccess) return e;
      k_update_df<<<w.red.nblk, kT, sh, s>>>(w.V, w.vstride, w.jstate, Wp, w.N, w.C, w.h, w.K,
                                             w.status, w.red.rpb, w.npart, need),
          lgt::note_launch();
      return cudaGetLastError();
    }
  }
  if (w.ncomp == 1)
    k_update<S, 1><<<w.red.nblk, kT, 0, s>>>(w.V, w.vstride, w.jstate, 0, Wp, w.N, w.C, w.ncomp,
                                             w.h, w.K, w.status, w.red.rpb, w.npart,
                                             need), lgt::note_launch();
  else
    k_update<S, 2><<<w.red.nblk, kT, 0, s>>>(w.V, w.vstride, w.jstate, 0, Wp, w.N, w.C, w.ncomp,
                                             w.h, w.K, w.status, w.red.rpb, w.npart,
                                             need), lgt::note_launch();
  return cudaGetLastError();
}

// One Lanczos step on the device; every kernel reads j from w.jstate.
template <typename S>
cudaError_t lanczos_step(const OpDev& op, Work<S>& w, int reorth, double tiny_rel,
                         cudaStream_t s) {
  cudaError_t e = apply_h<S>(op, w.V, w.jstate, w.vstride, w.W, w.hcomp, s, w.m + 1);
  if (e != cudaSuccess) return e;
  const unsigned fdb = finish_blocks(w.ldT * w.K);
  // Classical Gram-Schmidt against the whole basis (this also performs the
  // three-term recurrence).  Further passes, up to `reorth`, act only on the
  // points whose previous pass cancelled more than two digits
  // (||W_after|| < 1e-2 ||W_before||); the first pass also measures
  // ||W_before||.
  for (int pass = 0; pass < reorth; ++pass) {
    const int* need = (pass == 0) ? nullptr : w.need;
    if (pass > 0)
      k_need_pass<<<finish_blocks(w.K), 128, 0, s>>>(w.npart, w.red.nblk, w.K, w.C, w.ncomp,
                                                 w.status, w.nb, w.need), lgt::note_launch();
    e = launch_multidot<S, S>(w, w.V, w.vstride, w.jstate, 0, w.W, s, pass == 0 ? 1 : 0, need,
                              op.err);
    if (e != cudaSuccess) return e;
    k_finish_dots<<<fdb, 128, 0, s>>>(w.part, w.red.nblk, w.ldT, w.jstate, 0, w.K, w.C, w.ncomp,
                                      w.h, w.alpha, w.ldT, pass == 0, w.status,
                                      pass == 0 ? 1 : 0, w.nb), lgt::note_launch();
    e = launch_update<S>(w, w.W, s, need, op.err);
    if (e != cudaSuccess) return e;
  }
  k_finish_norm<<<finish_blocks(w.K), 128, 0, s>>>(w.npart, w.red.nblk, w.K, w.C, w.ncomp, w.jstate,
                                               w.beta, w.alpha, w.ldT, w.status, w.len, w.bnorm,
                                               tiny_rel, 1), lgt::note_launch();
  bool f4 = false;
  if constexpr (sizeof(S) == 4) {
    // 16-byte accesses when the panel allows (the grid a multiple of C / 4
    // threads, so that every thread keeps its columns)
    f4 = w.C % 4 == 0 && (kT % (w.C / 4)) == 0 && (w.vstride % 4) == 0 &&
         (reinterpret_cast<uintptr_t>(w.V) & 15) == 0 && (reinterpret_cast<uintptr_t>(w.W) & 15) == 0;
    if (f4)
      k_scale_f4<<<grid_for(int64_t(w.vstride) / 4), kT, 0, s>>>(
          reinterpret_cast<const float*>(w.W), reinterpret_cast<float*>(w.V), w.vstride, w.jstate,
          1, w.N, w.C, w.ncomp, w.bnorm, w.status, kActive), lgt::note_launch();
  }
  if (!f4)
    k_scale<S, S><<<grid_for(int64_t(w.vstride)), kT, 0, s>>>(w.W, w.V, w.vstride, w.jstate, 1,
                                                              w.N, w.C, w.ncomp, w.bnorm,
                                                              w.status, kActive, nullptr),
        lgt::note_launch();
  k_advance<<<1, 1, 0, s>>>(w.jstate), lgt::note_launch();
  return cudaGetLastError();
}

// ||X_k|| of a double panel into out_norm (device, K).
template <typename S>
std::string colnorms_double(Work<S>& w, const double* X, double* out_norm, cudaStream_t s) {
  k_residual_parts<<<w.red.nblk, kT, 0, s>>>(X, X, w.zeros, w.N, w.C, w.ncomp, w.red.rpb,
                                             w.npart), lgt::note_launch();
  KCK(cudaGetLastError());
  k_finish_norm<<<finish_blocks(w.K), 128, 0, s>>>(w.npart, w.red.nblk, w.K, w.C, w.ncomp, w.jstate,
                                               w.beta, w.alpha, w.ldT, w.status, w.len, out_norm,
                                               0.0, 0), lgt::note_launch();
  KCK(cudaGetLastError());
  return std::string();
}

// Per-point Re <x|y> of two double panels through the workspace buffers.
template <typename S>
std::string dots_ws(Work<S>& w, const double* x, const double* y, double* out_host,
                    cudaStream_t s) {
  KCK((launch_multidot<S, double>(w, x, 0, nullptr, 1, y, s)));
  k_finish_dots<<<finish_blocks(w.K), 128, 0, s>>>(w.part, w.red.nblk, w.ldT, nullptr, 1, w.K, w.C,
                                                  w.ncomp, w.h, nullptr, 0, 0, nullptr, 0,
                                                  nullptr), lgt::note_launch();
  KCK(cudaGetLastError());
  std::vector<double> hh(2 * size_t(w.K));
  KCK(cudaMemcpyAsync(hh.data(), w.h, sizeof(double) * 2 * w.K, cudaMemcpyDeviceToHost, s));
  KCK(cudaStreamSynchronize(s));
  for (int k = 0; k < w.K; ++k) out_host[k] = hh[2 * k];
  return std::string();
}

// ---- autotuner ---------------------------------------------------------------
//
// Per operator shape (lattice, model, storage precision, panel width) the
// first solve times the candidates on its own workspace and keeps the
// fastest for the process:
//   * the H*psi kernel: run-time geometry, or (where one exists) the
//     fixed-shape kernel with one or two vector loads per lane;
//   * the block count of the panel reductions (Gram-Schmidt dots and
//     updates): 2, 4, 6 or 8 blocks per SM.
// LGT_AUTOTUNE=0 in the environment keeps the built-in rules.
struct TuneKey {
  int nx, ny, dg, model, bytes, C, hcomp;
  int64_t N;
  bool operator<(const TuneKey& o) const {
    return std::tie(nx, ny, dg, model, bytes, C, hcomp, N) <
           std::tie(o.nx, o.ny, o.dg, o.model, o.bytes, o.C, o.hcomp, o.N);
  }
};

std::mutex g_tune_mu;
std::map<TuneKey, TuneChoice> g_tune;

bool autotune_enabled() {
  const char* e = getenv("LGT_AUTOTUNE");
  return !(e && e[0] == '0');
}

void apply_variant(OpDev* op, int v) {
  op->force_generic = (v == kHpsiGeneric) ? 1 : 0;
  op->use_table = (v >= kHpsiTable1 && v <= kHpsiTableBulk) ? 1 : 0;
  op->vpl = (v == kHpsiFixed1 || v == kHpsiTable1)    ? 1
            : (v == kHpsiFixed2 || v == kHpsiTable2)  ? 2
            : (v == kHpsiFixed2w || v == kHpsiTable2w) ? 3
            : (v == kHpsiTableBulk)                    ? 4
                                                       : 0;
}

bool is_table_variant(int v) { return v >= kHpsiTable1 && v <= kHpsiTableBulk; }

bool stream_capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return true;
  return cap != cudaStreamCaptureStatusNone;
}

// Builds op's neighbour table on first use when the format and the memory
// budget allow; never while `s` is capturing.  Returns whether it is built.
bool ensure_table(OpDev* op, cudaStream_t s) {
  NbrTable* T = op->table;
  if (!T) return false;
  if (T->state != 0) return T->state == 1;
  if (stream_capturing(s)) return false;
  const char* en = getenv("LGT_NBR_TABLE");
  size_t bound = 0;
  if ((en && en[0] == '0') || !nbr_table_eligible(op->G, op->R.dim, op->model, &bound)) {
    T->state = -1;
    return false;
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
  size_t cap = size_t(16384) << 20;
  if (const char* mb = getenv("LGT_NBR_TABLE_MB")) cap = size_t(atoll(mb)) << 20;
  if (free_b / 4 < cap) cap = free_b / 4;
  if (bound > cap) {
    T->state = -1;
    return false;
  }
  const std::string e = build_nbr_table(op->G, op->R, op->model, op->err, T, s);
  if (!e.empty()) {
    free_nbr_table(T);
    T->state = -1;
    return false;
  }
  // the renumbered copy for the Krylov drivers, when a second table fits the
  // same budget: mask segments in breadth-first order (default),
  // LGT_TABLE_ORDER=row the row-level order, LGT_TABLE_ORDER=0 none
  NbrTable* T2 = op->table_ord;
  if (T2 && T2->state == 0) {
    const char* eo = getenv("LGT_TABLE_ORDER");
    const bool none = eo && eo[0] == '0';
    const bool rows = eo && eo[0] == 'r';
    if (none || 2 * bound > cap) {
      T2->state = -1;
    } else {
      const std::string e2 = rows ? build_table_order(*T, T2, s)
                                  : build_table_mask_order(*T, op->G, op->R, T2, s);
      if (!e2.empty()) {
        free_nbr_table(T2);
        T2->state = -1;
      }
    }
  }
  return true;
}

// Whether the Krylov drivers keep their vectors in the table's row order:
// the table kernel is chosen and its renumbered copy exists.
bool use_krylov_order(const OpDev& op) {
  return op.use_table && op.table_ord && op.table_ord->state == 1 && op.table_ord->perm;
}

// The H*psi variant forced by LGT_HPSI_VARIANT (1..8), or 0.
int hpsi_forced() {
  const char* fv = getenv("LGT_HPSI_VARIANT");
  const int v = fv ? atoi(fv) : 0;
  return (v >= kHpsiGeneric && v <= kHpsiTableBulk) ? v : 0;
}

// Applies variant v, or the built-in rule when v needs a table that cannot
// be had; returns the variant applied.
int apply_variant_checked(OpDev* op, int v, cudaStream_t s) {
  if (is_table_variant(v) && !ensure_table(op, s)) v = kHpsiDefault;
  apply_variant(op, v);
  return v;
}

struct HpsiKey {
  int nx, ny, dg, model, bytes, C;
  int64_t N;
  bool operator<(const HpsiKey& o) const {
    return std::tie(nx, ny, dg, model, bytes, C, N) <
           std::tie(o.nx, o.ny, o.dg, o.model, o.bytes, o.C, o.N);
  }
};
std::map<HpsiKey, std::pair<int, double>> g_hpsi_tune;  // variant, ms per launch

// Times the H*psi candidates on (x, y) for this shape once per process.
template <typename S>
std::string tune_hpsi(OpDev* op, const S* x, S* y, int C, int hcomp, cudaStream_t s,
                      int* variant_out, double* ms_out) {
  // LGT_HPSI_VARIANT=1..7 forces one variant (cross-checks of every kernel)
  if (const int v = hpsi_forced()) {
    const int u = apply_variant_checked(op, v, s);
    if (variant_out) *variant_out = u;
    if (ms_out) *ms_out = 0.0;
    return std::string();
  }
  const HpsiKey key{op->G.nx, op->G.ny, op->G.dg, int(op->model), int(sizeof(S)), C, op->R.dim};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_hpsi_tune.find(key);
    if (it != g_hpsi_tune.end()) {
      const int u = apply_variant_checked(op, it->second.first, s);
      if (variant_out) *variant_out = u;
      if (ms_out) *ms_out = it->second.second;
      return std::string();
    }
  }
  if (!autotune_enabled() || stream_capturing(s)) {
    apply_variant(op, kHpsiDefault);
    if (variant_out) *variant_out = kHpsiDefault;
    if (ms_out) *ms_out = 0.0;
    return std::string();  // rule (not cached: a later eager call may tune)
  }
  HpsiArgs<S> probe;
  probe.G = op->G;
  probe.R = op->R;
  probe.x = x;
  probe.y = y;
  probe.N = op->R.dim;
  probe.C = C;
  probe.xsel = nullptr;
  probe.xstride = 0;
  int mode = 0;
  std::vector<int> cand{kHpsiGeneric};
  if (hpsi_fixed_applies(probe, &mode)) {
    cand.push_back(kHpsiFixed1);
    if (mode >= 2) cand.push_back(kHpsiFixed2);
    if (mode >= 3) cand.push_back(kHpsiFixed2w);
  }
  if (ensure_table(op, s)) {
    probe.t_meta = op->table->meta;
    if (table_load_mode(probe, &mode)) {
      cand.push_back(kHpsiTable1);
      if (mode >= 2) cand.push_back(kHpsiTable2);
      if (mode >= 3) cand.push_back(kHpsiTable2w);
      // (the copy-engine gather, kHpsiTableBulk, is not a candidate: 3.3x
      // slower on the 4x4 K = 8 panel; LGT_HPSI_VARIANT=8 forces it)
    }
  }
  EventPair evp;
  KCK(evp.create());
  cudaEvent_t e0 = evp.a, e1 = evp.b;
  int best_v = kHpsiDefault;
  double best = 1e30;
  cudaError_t e = cudaSuccess;
  for (int v : cand) {
    OpDev o = *op;
    apply_variant(&o, v);
    o.krylov_order = use_krylov_order(o) ? 1 : 0;  // the table the drivers will use
    e = apply_h<S>(o, x, nullptr, 0, y, hcomp, s);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = apply_h<S>(o, x, nullptr, 0, y, hcomp, s);
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) break;
    if (ms / 3.0 < best) {
      best = ms / 3.0;
      best_v = v;
    }
  }
  if (e != cudaSuccess) return std::string("autotune: ") + cudaGetErrorString(e);
  // A built table stays with the Hamiltonian even when another kernel wins
  // here: graphs captured for its other panel widths may launch from it.
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_hpsi_tune[key] = {best_v, best};
  }
  apply_variant(op, best_v);
  if (variant_out) *variant_out = best_v;
  if (ms_out) *ms_out = best;
  return std::string();
}

template <typename S>
std::string autotune(OpDev* op, Work<S>& w, cudaStream_t s, TuneChoice* out) {
  const TuneKey key{op->G.nx, op->G.ny, op->G.dg, int(op->model), int(sizeof(S)),
                    w.C, w.hcomp, w.N};
  // a forced H*psi kernel (cross-checks) neither reads nor fills the cache
  const bool forced = hpsi_forced();
  if (!forced) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      TuneChoice c = it->second;
      c.hpsi_variant = apply_variant_checked(op, c.hpsi_variant, s);
      if (w.red.nblk != c.red_nblk) w.replan(c.red_blocks);
      if (out) *out = c;
      return std::string();
    }
  }
  TuneChoice c;
  c.hpsi_variant = kHpsiDefault;
  c.red_blocks = LGT_RED_BLOCKS;
  if (autotune_enabled() && !w.lite && w.V) {
    const int J = (w.m + 1 < 8) ? w.m + 1 : 8;
    KCK(cudaMemsetAsync(w.V, 0, sizeof(S) * w.vstride * J, s));
    KCK(cudaMemsetAsync(w.W, 0, sizeof(S) * w.vstride, s));
    // H*psi variant (shared with lgt_matvec's choice for this shape)
    std::string err = tune_hpsi<S>(op, w.V, w.W, w.C, w.hcomp, s, &c.hpsi_variant, &c.hpsi_ms);
    if (!err.empty()) return err;
    EventPair evp;
    KCK(evp.create());
    cudaEvent_t e0 = evp.a, e1 = evp.b;
    auto timed = [&](auto&& launch) -> double {  // one warm-up, mean of three
      cudaError_t e = launch();
      if (e == cudaSuccess) e = cudaEventRecord(e0, s);
      for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = launch();
      if (e == cudaSuccess) e = cudaEventRecord(e1, s);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        err = std::string("autotune: ") + cudaGetErrorString(e);
        return 1e30;
      }
      return double(ms) / 3.0;
    };
    // reduction block counts: Gram-Schmidt passes (dots and update) against
    // 2, 5 and 8 vectors (all points active, h = 0), summed
    KCK(cudaMemsetAsync(w.status, 0, sizeof(int) * w.K, s));
    KCK(cudaMemsetAsync(w.h, 0, sizeof(double) * size_t(w.ldT) * w.K * 2, s));
    double best = 1e30;
    int last_nblk = -1;
    for (int cap : {304, 608, 912, kRedMaxBlocks}) {
      if (!err.empty()) break;
      w.red.plan(w.N, w.C, cap);
      if (w.red.nblk == last_nblk) continue;
      last_nblk = w.red.nblk;
      double t = 0.0;
      for (int jv : {2, 5, 8}) {
        const int jj = (jv < J ? jv : J) - 1;  // step index: jj + 1 vectors
        KCK(cudaMemcpyAsync(w.jstate, &jj, sizeof(int), cudaMemcpyHostToDevice, s));
        t += timed([&] {
          cudaError_t e =
              launch_multidot<S, S>(w, w.V, w.vstride, w.jstate, 0, w.W, s, 0, nullptr, op->err);
          if (e == cudaSuccess) e = launch_update<S>(w, w.W, s, nullptr, op->err);
          return e;
        });
      }
      if (t < best) {
        best = t;
        c.red_blocks = cap;
      }
    }
    c.red_ms = best;
    if (!err.empty()) return err;
    c.measured = 1;
  }
  w.replan(c.red_blocks);
  c.red_nblk = w.red.nblk;
  c.hpsi_variant = apply_variant_checked(op, c.hpsi_variant, s);
  if (!forced) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = c;
  }
  if (out) *out = c;
  return std::string();
}

template <typename S>
std::string capture_steps(const OpDev& op, Work<S>& w, int steps, int reorth, double tiny_rel,
                          cudaStream_t s) {
  if (w.graph) {
    cudaGraphExecDestroy(w.graph);
    w.graph = nullptr;
    w.graph_steps = 0;
  }
  cudaGraph_t g;
  KCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  set_capturing(true);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < steps && e == cudaSuccess; ++i) e = lanczos_step<S>(op, w, reorth, tiny_rel, s);
  set_capturing(false);
  cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (e != cudaSuccess) return std::string("graph capture: ") + cudaGetErrorString(e);
  if (e2 != cudaSuccess) return std::string("graph capture end: ") + cudaGetErrorString(e2);
  size_t nodes = 0;
  cudaGraphGetNodes(g, nullptr, &nodes);
  w.graph_nodes = int(nodes);
  e = cudaGraphInstantiate(&w.graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return std::string("graph instantiate: ") + cudaGetErrorString(e);
  w.graph_steps = steps;
  w.graph_reorth = reorth;
  w.graph_tiny = tiny_rel;
  return std::string();
}

// `steps` Lanczos steps.  Full chunks replay a captured graph; the first
// chunk of a new configuration runs eagerly (which also sets the kernels'
// shared-memory attributes) and is captured for later chunks.
template <typename S>
std::string run_steps(const OpDev& op, Work<S>& w, const KrylovParams& p, int steps,
                      double tiny_rel, cudaStream_t s, int64_t* matvecs) {
  if (steps <= 0) return std::string();
  // a captured sequence is replayed only for the same step count, passes,
  // threshold and operator (kernel variant, row order)
  const uint64_t opkey = (uint64_t(op.krylov_order) << 8) ^ (uint64_t(op.use_table) << 9) ^
                         (uint64_t(op.force_generic) << 10) ^ (uint64_t(op.vpl) << 11);
  const bool cached = w.graph && w.graph_steps == steps && w.graph_reorth == p.reorth &&
                      w.graph_tiny == tiny_rel && w.graph_op == opkey;
  if (p.use_graph && steps == p.check_every && cached) {
    KCK(cudaGraphLaunch(w.graph, s));
    note_launch(w.graph_nodes);
  } else {
    for (int i = 0; i < steps; ++i) KCK(lanczos_step<S>(op, w, p.reorth, tiny_rel, s));
    if (p.use_graph && steps == p.check_every) {
      std::string err = capture_steps<S>(op, w, steps, p.reorth, tiny_rel, s);
      if (!err.empty()) return err;
      w.graph_op = opkey;
    }
  }
  *matvecs += steps;
  return std::string();
}

// V_0 = X / ||X|| for active points (X double, storage S); rho = ||X||.
// perm: the Krylov row order (V_0 row n = X row perm[n]), or null.
template <typename S>
std::string start_from(Work<S>& w, const double* X, cudaStream_t s, const int* perm) {
  std::string err = colnorms_double<S>(w, X, w.rho, s);
  if (!err.empty()) return err;
  k_scale<double, S><<<grid_for(int64_t(w.vstride)), kT, 0, s>>>(
      X, w.V, w.vstride, nullptr, 0, w.N, w.C, w.ncomp, w.rho, w.status, kActive, perm),
      lgt::note_launch();
  KCK(cudaGetLastError());
  return std::string();
}

template <typename S>
std::string reset_cycle(Work<S>& w, cudaStream_t s) {
  KCK(cudaMemsetAsync(w.jstate, 0, sizeof(int), s));
  KCK(cudaMemsetAsync(w.alpha, 0, sizeof(double) * size_t(w.K) * w.ldT, s));
  KCK(cudaMemsetAsync(w.beta, 0, sizeof(double) * size_t(w.K) * w.ldT, s));
  k_set_int<<<(w.K + 127) / 128, 128, 0, s>>>(w.len, w.K, 0, w.status, kActive), lgt::note_launch();
  KCK(cudaGetLastError());
  return std::string();
}

template <typename S>
std::string ground_state_impl(const OpDev& op_in, const KrylovParams& p, Work<S>& w, double* X,
                              double* E0, double* resid_out, cudaStream_t s, KrylovReport* rep) {
  OpDev op = op_in;  // carries the autotuner's H*psi variant
  const int64_t N = op.R.dim;
  const int K = op.K;
  const int ncomp = 1, C = K;
  int m = p.krylovdim;
  if (m > N) m = int(N);
  if (m > kMaxDim - 1) m = kMaxDim - 1;
  if (m < 1) m = 1;
  std::string err = w.ensure(N, C, K, ncomp, m);
  if (!err.empty()) {
    w.release();
    return err;
  }
  err = autotune<S>(&op, w, s, nullptr);
  if (!err.empty()) return err;
  // the Krylov vectors in the table's row order when its kernel was chosen
  // and serves these panels: X is gathered into V_0 and the combinations
  // scattered back
  op.krylov_order = (use_krylov_order(op) && table_serves(op, w)) ? 1 : 0;
  const int* perm = op.krylov_order ? op.table_ord->perm : nullptr;
  const bool fp32 = sizeof(S) == 4;
  const double tiny_rel = fp32 ? 1e-6 : 1e-12;
  // FP32 panels cannot resolve residuals much below 1e-6 |H|: the inner
  // solve stops there and the Ritz pair is finished in FP64 below.
  const double tol_inner = fp32 ? fmax(p.tol, 2e-5) : p.tol;

  EventPair ev;
  KCK(ev.create());
  cudaEventRecord(ev.a, s);
  KCK(cudaMemsetAsync(w.status, 0, sizeof(int) * K, s));
  KCK(cudaMemsetAsync(w.len, 0, sizeof(int) * K, s));
  KCK(cudaMemsetAsync(w.fail, 0, sizeof(int), s));
  KCK(cudaMemsetAsync(w.theta, 0xff, sizeof(double) * K, s));  // NaN: no warm bracket yet
  if (!p.start_given) {
    k_randn<double><<<grid_for(N * C), kT, 0, s>>>(X, N, C, ncomp, p.seed), lgt::note_launch();
    KCK(cudaGetLastError());
  }
  err = reset_cycle<S>(w, s);
  if (!err.empty()) return err;
  err = start_from<S>(w, X, s, perm);
  if (!err.empty()) return err;

  std::vector<int> st(K);
  int j = 0, restarts = 0;
  int64_t matvecs = 0;
  bool noconv = false;
  while (true) {
    const int steps = (m - j < p.check_every) ? (m - j) : p.check_every;
    err = run_steps<S>(op, w, p, steps, tiny_rel, s, &matvecs);
    if (!err.empty()) return err;
    j += steps;
    k_check_lowest<<<K, 32, 0, s>>>(w.alpha, w.beta, w.ldT, w.status, w.len, w.theta, w.resid,
                                    w.coef, tol_inner, fp32 ? 1 : 0), lgt::note_launch();
    KCK(cudaGetLastError());
    KCK(cudaMemcpyAsync(st.data(), w.status, sizeof(int) * K, cudaMemcpyDeviceToHost, s));
    KCK(cudaStreamSynchronize(s));
    bool all = true;
    for (int k = 0; k < K; ++k) all = all && (st[k] >= kConverged);
    if (all) break;
    if (j >= m) {
      if (restarts >= p.maxiter) {
        noconv = true;
        break;
      }
      // keep the points that converged in this cycle, restart the others
      // from their current Ritz vectors
      k_combine<S, 1><<<grid_for(N * C), kT, 0, s>>>(w.V, w.vstride, w.coef, w.ldT, w.len,
                                                     w.status, kConverged, X, N, C, ncomp, perm), lgt::note_launch();
      k_set_int<<<(K + 127) / 128, 128, 0, s>>>(w.status, K, kWritten, w.status, kConverged), lgt::note_launch();
      k_combine<S, 1><<<grid_for(N * C), kT, 0, s>>>(w.V, w.vstride, w.coef, w.ldT, w.len,
                                                     w.status, kActive, X, N, C, ncomp, perm), lgt::note_launch();
      KCK(cudaGetLastError());
      err = reset_cycle<S>(w, s);
      if (!err.empty()) return err;
      err = start_from<S>(w, X, s, perm);
      if (!err.empty()) return err;
      j = 0;
      ++restarts;
    }
  }
  // final vectors of the points still on the current basis
  k_set_int<<<(K + 127) / 128, 128, 0, s>>>(w.status, K, kConverged, w.status, kActive), lgt::note_launch();
  k_set_int<<<(K + 127) / 128, 128, 0, s>>>(w.status, K, kConverged, w.status, kExhausted), lgt::note_launch();
  k_combine<S, 1><<<grid_for(N * C), kT, 0, s>>>(w.V, w.vstride, w.coef, w.ldT, w.len, w.status,
                                                 kConverged, X, N, C, ncomp, perm),
      lgt::note_launch();
  KCK(cudaGetLastError());
  std::vector<double> theta(K);
  KCK(cudaMemcpyAsync(theta.data(), w.theta, sizeof(double) * K, cudaMemcpyDeviceToHost, s));

  // FP64 finish: normalise X, R = H X in FP64, E = <X|R>, ||R - E X||.
  KCK(cudaMemsetAsync(w.status, 0, sizeof(int) * K, s));
  err = colnorms_double<S>(w, X, w.rho, s);
  if (!err.empty()) return err;
  k_scale<double, double><<<grid_for(N * C), kT, 0, s>>>(X, X, 0, nullptr, 0, N, C, ncomp, w.rho,
                                                          nullptr, 0, nullptr), lgt::note_launch();
  KCK(cudaGetLastError());
  OpDev op_ref = op;  // X is in the reference order here
  op_ref.krylov_order = 0;
  KCK(apply_h<double>(op_ref, X, nullptr, 0, w.R, ncomp, s));
  ++matvecs;
  std::vector<double> erq(K), r2(K);
  err = dots_ws<S>(w, X, w.R, erq.data(), s);
  if (!err.empty()) return err;
  KCK(cudaMemcpyAsync(w.theta, erq.data(), sizeof(double) * K, cudaMemcpyHostToDevice, s));
  k_residual_parts<<<w.red.nblk, kT, 0, s>>>(X, w.R, w.theta, N, C, ncomp, w.red.rpb, w.npart), lgt::note_launch();
  k_finish_norm<<<finish_blocks(K), 128, 0, s>>>(w.npart, w.red.nblk, K, C, ncomp, w.jstate, w.beta,
                                             w.alpha, w.ldT, w.status, w.len, w.bnorm, 0.0, 0), lgt::note_launch();
  KCK(cudaGetLastError());
  KCK(cudaMemcpyAsync(r2.data(), w.bnorm, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
  cudaEventRecord(ev.b, s);
  KCK(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev.a, ev.b);
  int conv = 0;
  double maxr = 0.0;
  for (int k = 0; k < K; ++k) {
    // FP64: the Ritz value, as eigsolve returns; FP32-mixed: the FP64
    // Rayleigh quotient of the FP32-converged vector.
    E0[k] = fp32 ? erq[k] : theta[k];
    if (resid_out) resid_out[k] = r2[k];
    if (r2[k] <= tol_inner * 1.01 + 1e-300) ++conv;
    maxr = fmax(maxr, r2[k]);
  }
  if (rep) {
    rep->matvecs += matvecs;
    rep->restarts += restarts;
    rep->converged = conv;
    rep->max_residual = maxr;
    rep->seconds += ms * 1e-3;
  }
  if (noconv) return std::string("NOCONV: Lanczos did not converge within maxiter restarts");
  return std::string();
}

// Krylov exp(-i dt H) steps.  H is real, so exp(-i tau H)(a + i b) =
// exp(-i tau H) a + i exp(-i tau H) b: the real and imaginary parts of each
// point's state are propagated as two real Krylov columns (real
// Gram-Schmidt: half the FP64 work of complex columns) and recombined with
// complex coefficients.  Each column's error estimate must meet tol / sqrt 2,
// so the point's combined error meets tol.
template <typename S>
std::string expm_impl(const OpDev& op_in, const KrylovParams& p, Work<S>& w, double dt,
                      int n_steps, double* X, double* drift, StepObserver* obs, cudaStream_t s,
                      KrylovReport* rep) {
  OpDev op = op_in;  // carries the autotuner's H*psi variant
  const int64_t N = op.R.dim;
  const int K = op.K;       // coupling points (complex columns of X)
  const int C = 2 * K;      // real Krylov columns
  const int Kc = C;         // Krylov "points": one per real column
  int m = p.krylovdim;
  if (m > N) m = int(N);
  if (m > kMaxDim - 1) m = kMaxDim - 1;
  if (m < 1) m = 1;
  std::string err = w.ensure(N, C, Kc, 1, m, 2);
  if (!err.empty()) {
    w.release();
    return err;
  }
  err = autotune<S>(&op, w, s, nullptr);
  if (!err.empty()) return err;
  // the Krylov vectors in the table's row order when its kernel was chosen
  // and serves these panels: X is gathered into V_0 and the combinations
  // scattered back
  op.krylov_order = (use_krylov_order(op) && table_serves(op, w)) ? 1 : 0;
  const int* perm = op.krylov_order ? op.table_ord->perm : nullptr;
  const double tiny_rel = (sizeof(S) == 8) ? 1e-12 : 1e-6;
  const double tol = p.tol / sqrt(2.0);
  std::vector<int> st(Kc);
  std::vector<double> errs(Kc, 0.0), nrm(K);
  if (drift)
    for (int k = 0; k < K; ++k) drift[k] = 0.0;
  int64_t matvecs = 0;
  int substeps = 0;
  double maxerr = 0.0;
  EventPair ev;
  KCK(ev.create());
  cudaEventRecord(ev.a, s);
  KCK(cudaMemsetAsync(w.fail, 0, sizeof(int), s));
  if (obs) {
    err = obs->on_step(0, X);
    if (!err.empty()) return err;
  }
  auto all_converged = [&](bool* out) -> std::string {
    KCK(cudaMemcpyAsync(st.data(), w.status, sizeof(int) * Kc, cudaMemcpyDeviceToHost, s));
    KCK(cudaStreamSynchronize(s));
    bool a = true;
    for (int k = 0; k < Kc; ++k) a = a && (st[k] >= kConverged);
    *out = a;
    return std::string();
  };
  for (int step = 1; step <= n_steps; ++step) {
    double remaining = dt;
    int guard_sub = 0;
    while (remaining > 0.0) {
      KCK(cudaMemsetAsync(w.status, 0, sizeof(int) * Kc, s));
      KCK(cudaMemsetAsync(w.len, 0, sizeof(int) * Kc, s));
      err = reset_cycle<S>(w, s);
      if (!err.empty()) return err;
      // V_0 = column / ||column|| (a zero column, e.g. Im psi = 0, spans an
      // empty Krylov space: it is exhausted at once and contributes 0)
      err = start_from<S>(w, X, s, perm);
      if (!err.empty()) return err;
      int j = 0;
      bool all = false;
      while (j < m) {
        const int steps = (m - j < p.check_every) ? (m - j) : p.check_every;
        err = run_steps<S>(op, w, p, steps, tiny_rel, s, &matvecs);
        if (!err.empty()) return err;
        j += steps;
        k_check_expm<<<Kc, 64, 0, s>>>(w.alpha, w.beta, w.ldT, w.status, w.len, w.rho, remaining,
                                       w.resid, w.coef, tol, 0, w.fail), lgt::note_launch();
        KCK(cudaGetLastError());
        err = all_converged(&all);
        if (!err.empty()) return err;
        if (all) break;
      }
      double tau = remaining;
      if (!all) {
        // The Krylov space is too small for the whole interval: take the
        // largest tau = remaining / 2^q meeting the tolerance (scaled to the
        // sub-interval) for every column, then continue from there.
        double t = remaining;
        bool ok = false;
        for (int q = 0; q < 40 && !ok; ++q) {
          t *= 0.5;
          k_check_expm<<<Kc, 64, 0, s>>>(w.alpha, w.beta, w.ldT, w.status, w.len, w.rho, t,
                                         w.resid, w.coef, tol * (t / dt), 0, w.fail), lgt::note_launch();
          err = all_converged(&ok);
          if (!err.empty()) return err;
        }
        if (!ok)
          return std::string("NOCONV: no sub-step down to dt / 2^40 meets the tolerance");
        tau = t;
        KCK(cudaMemsetAsync(w.status, 0, sizeof(int) * Kc, s));
        k_check_expm<<<Kc, 64, 0, s>>>(w.alpha, w.beta, w.ldT, w.status, w.len, w.rho, tau,
                                       w.resid, w.coef, tol, 1, w.fail), lgt::note_launch();
        KCK(cudaGetLastError());
        ++substeps;
        if (++guard_sub > 4096) return std::string("NOCONV: exponential step could not be split");
      }
      KCK(cudaMemcpyAsync(errs.data(), w.resid, sizeof(double) * Kc, cudaMemcpyDeviceToHost, s));
      if constexpr (sizeof(S) == 4) {
        const size_t shc = sizeof(float) * 4 * size_t(C) * w.ldT;
        if (df_reductions_enabled() && shc <= 48 * 1024 && (w.vstride % 2) == 0) {
          k_combine_split_df<<<grid_for(N * K), kT, shc, s>>>(
              reinterpret_cast<const float*>(w.V), w.vstride, w.coef, w.ldT, w.len, X, N, K,
              perm), lgt::note_launch();
        } else {
          k_combine_split<S><<<grid_for(N * C), kT, 0, s>>>(w.V, w.vstride, w.coef, w.ldT, w.len,
                                                            X, N, K, perm), lgt::note_launch();
        }
      } else {
        k_combine_split<S><<<grid_for(N * C), kT, 0, s>>>(w.V, w.vstride, w.coef, w.ldT, w.len, X,
                                                          N, K, perm), lgt::note_launch();
      }
      KCK(cudaGetLastError());
      KCK(cudaStreamSynchronize(s));
      for (int k = 0; k < K; ++k) maxerr = fmax(maxerr, hypot(errs[2 * k], errs[2 * k + 1]));
      remaining -= tau;
      if (remaining < 1e-15 * dt) remaining = 0.0;
    }
    // psi ./= norm(psi) per point (finite_ed.jl:420): the point view of the
    // panel, K complex columns
    k_residual_parts<<<w.red.nblk, kT, 0, s>>>(X, X, w.zeros, N, C, 2, w.red.rpb,
                                               w.npart), lgt::note_launch();
    k_finish_norm<<<finish_blocks(K), 128, 0, s>>>(w.npart, w.red.nblk, K, C, 2, w.jstate, w.beta,
                                               w.alpha, w.ldT, w.status, w.len, w.rho, 0.0,
                                               0), lgt::note_launch();
    k_scale<double, double><<<grid_for(N * C), kT, 0, s>>>(X, X, 0, nullptr, 0, N, C, 2, w.rho,
                                                            nullptr, 0, nullptr), lgt::note_launch();
    KCK(cudaGetLastError());
    if (drift) {
      KCK(cudaMemcpyAsync(nrm.data(), w.rho, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
      KCK(cudaStreamSynchronize(s));
      for (int k = 0; k < K; ++k) drift[k] = fmax(drift[k], fabs(nrm[k] - 1.0));
    }
    if (obs) {
      err = obs->on_step(step, X);
      if (!err.empty()) return err;
    }
  }
  int fail = 0;
  KCK(cudaMemcpyAsync(&fail, w.fail, sizeof(int), cudaMemcpyDeviceToHost, s));
  cudaEventRecord(ev.b, s);
  KCK(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev.a, ev.b);
  if (rep) {
    rep->matvecs += matvecs;
    rep->restarts += substeps;
    rep->converged = K;
    rep->max_residual = maxerr;
    rep->seconds += ms * 1e-3;
  }
  if (fail) return std::string("NOCONV: tridiagonal eigensolver did not converge");
  return std::string();
}

}  // namespace

struct KrylovCache {
  Work<double> gs_d;
  Work<float> gs_f;
  Work<double> ex_d;
  Work<float> ex_f;
  Work<double> dots;  // reduction buffers of panel_dots only
  Work<double> tune_d;  // explicit autotuning (lgt_autotune), released after use
  Work<float> tune_f;
  ~KrylovCache() {
    gs_d.release();
    gs_f.release();
    ex_d.release();
    ex_f.release();
    dots.release();
    tune_d.release();
    tune_f.release();
  }
};

std::string krylov_autotune(const OpDev& op_in, KrylovCache* cache, int ncomp, int mixed,
                            cudaStream_t s, TuneChoice* out) {
  OpDev op = op_in;
  const int64_t N = op.R.dim;
  const int C = (ncomp == 2) ? 2 * op.K : op.K;
  if (C > kT) return "at most 256 real columns per panel";
  const int m = int(N < 8 ? N : 8);
  std::string err;
  if (mixed) {
    err = cache->tune_f.ensure(N, C, C, 1, m, ncomp == 2 ? 2 : 1);
    if (err.empty()) err = autotune<float>(&op, cache->tune_f, s, out);
    cache->tune_f.release();
  } else {
    err = cache->tune_d.ensure(N, C, C, 1, m, ncomp == 2 ? 2 : 1);
    if (err.empty()) err = autotune<double>(&op, cache->tune_d, s, out);
    cache->tune_d.release();
  }
  return err;
}

std::string ensure_row_order(OpDev* op, cudaStream_t s) {
  if (!ensure_table(op, s)) return "the stored neighbour table is not available for this basis";
  if (!op->table_ord || op->table_ord->state != 1 || !op->table_ord->perm)
    return "the table's row order is not available (LGT_TABLE_ORDER=0 or memory budget)";
  op->use_table = 1;
  op->force_generic = 0;
  op->krylov_order = 1;
  return std::string();
}

KrylovCache* krylov_cache_new() { return new KrylovCache(); }
void krylov_cache_free(KrylovCache* c) { delete c; }

cudaError_t apply_h_d(const OpDev& op, const double* x, double* y, int ncomp, cudaStream_t s) {
  return apply_h<double>(op, x, nullptr, 0, y, ncomp, s);
}

cudaError_t apply_h_f(const OpDev& op, const float* x, float* y, int ncomp, cudaStream_t s) {
  return apply_h<float>(op, x, nullptr, 0, y, ncomp, s);
}

std::string hpsi_choose_d(OpDev* op, const double* x, double* y, int ncomp, cudaStream_t s) {
  return tune_hpsi<double>(op, x, y, op->K * ncomp, ncomp, s, nullptr, nullptr);
}

std::string hpsi_choose_f(OpDev* op, const float* x, float* y, int ncomp, cudaStream_t s) {
  return tune_hpsi<float>(op, x, y, op->K * ncomp, ncomp, s, nullptr, nullptr);
}

std::string panel_dots(KrylovCache* cache, const double* x, const double* y, int64_t N, int K,
                       int ncomp, double* out, cudaStream_t s) {
  Work<double>& w = cache->dots;
  std::string err = w.ensure(N, K * ncomp, K, ncomp, 1, ncomp, true);
  if (!err.empty()) return err;
  return dots_ws<double>(w, x, y, out, s);
}

std::string lanczos_ground_state(const OpDev& op, const KrylovParams& p, KrylovCache* cache,
                                 double* X, double* E0, double* resid, cudaStream_t s,
                                 KrylovReport* rep) {
  if (op.K > kT) return "at most 256 real columns per panel";
  if (!p.mixed) return ground_state_impl<double>(op, p, cache->gs_d, X, E0, resid, s, rep);
  std::string err = ground_state_impl<float>(op, p, cache->gs_f, X, E0, resid, s, rep);
  if (!err.empty() || p.refine <= 0) return err;
  // FP64 correction: a short FP64 Lanczos started from the FP32 solution
  KrylovParams q = p;
  q.mixed = 0;
  q.start_given = 1;
  q.krylovdim = p.refine;
  if (q.check_every > q.krylovdim) q.check_every = q.krylovdim;
  return ground_state_impl<double>(op, q, cache->gs_d, X, E0, resid, s, rep);
}

std::string krylov_expm(const OpDev& op, const KrylovParams& p, KrylovCache* cache, double dt,
                        int n_steps, double* X, double* norm_drift, StepObserver* obs,
                        cudaStream_t s, KrylovReport* rep) {
  if (op.K * 2 > kT) return "at most 128 complex points per panel";
  if (p.mixed)
    return expm_impl<float>(op, p, cache->ex_f, dt, n_steps, X, norm_drift, obs, s, rep);
  return expm_impl<double>(op, p, cache->ex_d, dt, n_steps, X, norm_drift, obs, s, rep);
}

}  // namespace lgt
