// hpsi.cu -- matrix-free, row-pull, atomic-free y = H x on K-interleaved
// panels (replaces build_hamiltonian's sparse matrix, finite_ed.jl:252-322,
// and the SparseMatrixCSC * Vector product inside KrylovKit).
//
// Panel layout: x[row][col], col = k * ncomp + comp, C = K * ncomp columns
// per row, rows contiguous (C * sizeof(T) bytes).  Column k of the panel uses
// the couplings (g_k, t_k, m_k) of coupling point k; comp is 0 (real) or
// 0/1 (real/imaginary part).  H is real, so a complex vector is simply two
// columns that share coefficients.
//
// One warp owns 32 consecutive rows and works in two phases:
//  1. lane = row: decode the row's key, derive e_R, enumerate its moves and
//     rank each neighbour key ONCE (shared by all C columns) into a
//     shared-memory neighbour list (index << 2 | kind);
//  2. lane = (row, column chunk): gather V-wide vectors (double2 / float4)
//     of x from each neighbour row, accumulate in registers, write y once.
// Every output element is written by exactly one thread: no atomics, and the
// result is bitwise reproducible run to run.
#include <cstdio>

#include "lgt_hpsi.h"
#include "lgt_moves.cuh"
#include "lgt_rank.cuh"

namespace lgt {

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;

template <typename T, int V>
struct Vec;
template <>
struct Vec<double, 1> {
  using type = double;
};
template <>
struct Vec<double, 2> {
  using type = double2;
};
template <>
struct Vec<float, 1> {
  using type = float;
};
template <>
struct Vec<float, 4> {
  using type = float4;
};

template <typename T, int V>
__device__ __forceinline__ void vload(const T* p, T (&r)[V]) {
  using VT = typename Vec<T, V>::type;
  VT v = __ldg(reinterpret_cast<const VT*>(p));
  const T* s = reinterpret_cast<const T*>(&v);
#pragma unroll
  for (int e = 0; e < V; ++e) r[e] = s[e];
}

template <typename T, int V>
__device__ __forceinline__ void vstore(T* p, const T (&r)[V]) {
  using VT = typename Vec<T, V>::type;
  VT v;
  T* s = reinterpret_cast<T*>(&v);
#pragma unroll
  for (int e = 0; e < V; ++e) s[e] = r[e];
  *reinterpret_cast<VT*>(p) = v;
}

struct SmemLayout {
  int binom_off, segc_off, coef_off, nbr_off, meta_off, total;
};

template <typename T>
__host__ __device__ inline SmemLayout smem_layout(int nmasks, int seg_smem, int K, int max_moves) {
  SmemLayout L;
  int o = 0;
  L.binom_off = o;
  o += 32 * 33 * 4;
  L.segc_off = o;
  if (seg_smem) o += ((nmasks + 1) * 4 + 15) / 16 * 16;
  L.coef_off = o;
  o += (4 * K * int(sizeof(T)) + 15) / 16 * 16;
  L.meta_off = o;  // per row: cnt (int16), e2 (int16), stag (int16), pad
  o += kWarps * 32 * 8;
  L.nbr_off = o;
  o += kWarps * 32 * max_moves * 4;
  L.total = o;
  return L;
}

// Off-diagonal entries a row can have: one per bond, plus W and W^dagger
// per plaquette when the model has them.
__host__ __device__ inline int row_moves(const Geom& G, bool plaq) {
  return G.nR + G.nU + (plaq ? 2 * G.nP : 0);
}

// Shared-memory stride of a row's neighbour list: odd, so that the lists of
// the rows a warp touches at once fall in distinct banks.
__host__ __device__ inline int row_stride(const Geom& G, bool plaq) {
  return row_moves(G, plaq) | 1;
}

template <typename T, int V, bool PLAQ, bool JW>
__global__ void __launch_bounds__(kThreads) k_hpsi(HpsiArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Geom& G = a.G;
  const int MM = row_stride(G, PLAQ);
  const SmemLayout L = smem_layout<T>(a.R.nmasks, a.seg_smem, a.K, MM);
  uint32_t* s_binom = reinterpret_cast<uint32_t*>(smem + L.binom_off);
  uint32_t* s_segc = reinterpret_cast<uint32_t*>(smem + L.segc_off);
  T* s_coef = reinterpret_cast<T*>(smem + L.coef_off);  // [4][K]: cE, cm, ch, cp
  int16_t* s_meta = reinterpret_cast<int16_t*>(smem + L.meta_off);
  uint32_t* s_nbr = reinterpret_cast<uint32_t*>(smem + L.nbr_off);

  for (int i = threadIdx.x; i < 32 * 33; i += kThreads) s_binom[i] = a.R.binom[i];
  if (a.seg_smem)
    for (int i = threadIdx.x; i <= a.R.nmasks; i += kThreads) s_segc[i] = a.R.segc[i];
  for (int i = threadIdx.x; i < a.K; i += kThreads) {
    s_coef[i] = a.cE[i];
    s_coef[a.K + i] = a.cm[i];
    s_coef[2 * a.K + i] = a.ch[i];
    s_coef[3 * a.K + i] = a.cp[i];
  }
  __syncthreads();
  const uint32_t* segc = a.seg_smem ? s_segc : a.R.segc;

  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t warp_row0 = (int64_t(blockIdx.x) * kWarps + wid) * 32;
  if (warp_row0 >= a.N) return;
  int16_t* meta = s_meta + (wid * 32) * 4;
  uint32_t* nbr = s_nbr + size_t(wid * 32) * MM;

  // ---- phase 1: one lane per row: moves + ranks -------------------------
  {
    const int64_t row = warp_row0 + lane;
    int cnt = 0, e2 = 0, stag = 0;
    if (row < a.N) {
      const Config c = decode(G, __ldg(a.R.keys + row));
      diag_parts(G, c, &e2, &stag);
      uint32_t* my = nbr + lane * MM;
      if (a.R.tab) {
        // rank tables: each neighbour's index is nrows independent loads
        uint32_t fidx[kMaxTabRows];
#pragma unroll
        for (int r = 0; r < kMaxTabRows; ++r)
          fidx[r] = (r < a.R.nrows) ? row_index(a.R, c.digits, r) : 0u;
        for_each_move_rows<PLAQ, JW>(G, c, fidx, a.R.pw,
                                     [&](uint32_t nmask, int rc, uint32_t frc, uint32_t kind) {
          const int64_t j = rank_rows(a.R, nmask, fidx, rc, frc);
          if (j < 0 || j >= a.N) {
            raise_err(a.err, kDevErrBounds);
            return;
          }
          if (cnt < MM) my[cnt++] = (uint32_t(j) << 2) | kind;
        });
      } else {
        for_each_move<PLAQ, JW>(G, c, [&](uint64_t nkey, uint32_t kind) {
          const int64_t j = rank_key(a.R, segc, s_binom, nkey);
          if (j < 0) {
            raise_err(a.err, kDevErrRank);
            return;
          }
          if (cnt < MM) my[cnt++] = (uint32_t(j) << 2) | kind;
        });
      }
    }
    meta[lane * 4 + 0] = int16_t(cnt);
    meta[lane * 4 + 1] = int16_t(e2);
    meta[lane * 4 + 2] = int16_t(stag);
  }
  __syncwarp();

  // ---- phase 2: lanes over (row, column chunk) ---------------------------
  const int C = a.C;
  const int chunks = C / V;
  const int items = 32 * chunks;
  const T* __restrict__ x = a.xsel ? a.x + size_t(*a.xsel) * a.xstride : a.x;
  T* __restrict__ y = a.y;
  const int ncomp = a.ncomp;
  for (int it = lane; it < items; it += 32) {
    const int rl = it / chunks;
    const int ch = it - rl * chunks;
    const int64_t row = warp_row0 + rl;
    if (row >= a.N) continue;
    const int col0 = ch * V;
    const int cnt = meta[rl * 4 + 0];
    const T e2 = T(meta[rl * 4 + 1]);
    const T stag = T(meta[rl * 4 + 2]);
    T cd[V], chp[V], cpl[V], acc[V], xv[V];
#pragma unroll
    for (int e = 0; e < V; ++e) {
      const int k = (col0 + e) / ncomp;
      cd[e] = s_coef[k] * e2 + s_coef[a.K + k] * stag;  // (g^2/2) sum e^2 + m sum stag n_f
      chp[e] = s_coef[2 * a.K + k];                     // -t
      cpl[e] = s_coef[3 * a.K + k];                     // -1/(2 g^2)
    }
    vload<T, V>(x + size_t(row) * C + col0, xv);
#pragma unroll
    for (int e = 0; e < V; ++e) acc[e] = cd[e] * xv[e];
    const uint32_t* lst = nbr + rl * MM;
    for (int n = 0; n < cnt; ++n) {
      const uint32_t ent = lst[n];
      const size_t j = ent >> 2;
      const uint32_t kind = ent & 3u;
      vload<T, V>(x + j * C + col0, xv);
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const T cf = (kind == kPlaq) ? cpl[e] : ((kind == kHopNeg) ? -chp[e] : chp[e]);
        acc[e] = fma(cf, xv[e], acc[e]);
      }
    }
    vstore<T, V>(y + size_t(row) * C + col0, acc);
  }
}

template <typename T, int V, bool PLAQ, bool JW>
cudaError_t launch_t(const HpsiArgs<T>& a, cudaStream_t s) {
  const SmemLayout L = smem_layout<T>(a.R.nmasks, a.seg_smem, a.K, row_stride(a.G, PLAQ));
  auto kern = k_hpsi<T, V, PLAQ, JW>;
  {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), L.total);
    if (e != cudaSuccess) return e;
  }
  const int64_t blocks = (a.N + kThreads - 1) / kThreads;
  if (blocks <= 0) return cudaSuccess;
  kern<<<unsigned(blocks), kThreads, L.total, s>>>(a), lgt::note_launch();
  return cudaGetLastError();
}

template <typename T, int V>
cudaError_t launch_v(const HpsiArgs<T>& a, uint32_t model, cudaStream_t s) {
  const bool plaq = model & kModelPlaq, jw = model & kModelJW;
  if (plaq && jw) return launch_t<T, V, true, true>(a, s);
  if (plaq) return launch_t<T, V, true, false>(a, s);
  if (jw) return launch_t<T, V, false, true>(a, s);
  return launch_t<T, V, false, false>(a, s);
}

}  // namespace

int hpsi_seg_smem_default(int nmasks) { return (nmasks + 1) * 4 <= 16 * 1024 ? 1 : 0; }

template <typename T>
bool vec_ok(const HpsiArgs<T>& a) {
  constexpr int VW = 16 / int(sizeof(T));
  const size_t xs = a.xsel ? a.xstride * sizeof(T) : 0;
  return (a.C % VW == 0) && ((reinterpret_cast<uintptr_t>(a.x) & 15) == 0) &&
         ((reinterpret_cast<uintptr_t>(a.y) & 15) == 0) && (xs % 16 == 0);
}

template <typename T>
cudaError_t launch_hpsi_generic(HpsiArgs<T> a, uint32_t model, cudaStream_t s) {
  constexpr int VW = 16 / int(sizeof(T));
  if (vec_ok(a)) return launch_v<T, VW>(a, model, s);
  return launch_v<T, 1>(a, model, s);
}

template <typename T>
bool hpsi_fixed_applies(const HpsiArgs<T>& a, int* max_vpl) {
  const Geom& G = a.G;
  const bool shape = (G.nx == 4 && G.ny == 4) || (G.nx == 4 && G.ny == 3) ||
                     (G.nx == 3 && G.ny == 4);
  const bool ok = shape && G.dg == 1 && a.R.tab && a.N < (int64_t(1) << 31) && vec_ok(a);
  const bool two = a.C % (2 * (16 / int(sizeof(T)))) == 0;
  const bool wide = two && (reinterpret_cast<uintptr_t>(a.x) & 31) == 0 &&
                    (reinterpret_cast<uintptr_t>(a.y) & 31) == 0 &&
                    (a.xsel == nullptr || (a.xstride * sizeof(T)) % 32 == 0);
  if (max_vpl) *max_vpl = ok ? (wide ? 3 : (two ? 2 : 1)) : 0;
  return ok;
}

template <typename T>
cudaError_t launch_hpsi(HpsiArgs<T> a, uint32_t model, cudaStream_t s) {
  const Geom& G = a.G;
  if (a.use_table && !a.force_generic && table_load_mode(a, nullptr))
    return launch_hpsi_table(a, model, s);
  if (a.table_order) return cudaErrorInvalidValue;  // no other kernel knows that order
  if (!a.force_generic && hpsi_fixed_applies(a, nullptr)) {
    if (G.nx == 4 && G.ny == 4) return launch_hpsi_4x4(a, model, s);
    if (G.nx == 4 && G.ny == 3) return launch_hpsi_4x3(a, model, s);
    if (G.nx == 3 && G.ny == 4) return launch_hpsi_3x4(a, model, s);
  }
  return launch_hpsi_generic(a, model, s);
}

template bool hpsi_fixed_applies<double>(const HpsiArgs<double>&, int*);
template bool hpsi_fixed_applies<float>(const HpsiArgs<float>&, int*);

template cudaError_t launch_hpsi<double>(HpsiArgs<double>, uint32_t, cudaStream_t);
template cudaError_t launch_hpsi<float>(HpsiArgs<float>, uint32_t, cudaStream_t);
template cudaError_t launch_hpsi_generic<double>(HpsiArgs<double>, uint32_t, cudaStream_t);
template cudaError_t launch_hpsi_generic<float>(HpsiArgs<float>, uint32_t, cudaStream_t);

// ----------------------------------------------------------------------------
// CSR export (parity checks and the reference's nnz(H), finite_ed.jl:355)
// ----------------------------------------------------------------------------
namespace {

template <bool PLAQ, bool JW>
__global__ void k_row_nnz(Geom G, RankView R, int64_t N, int64_t* counts) {
  int64_t row = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (row >= N) return;
  const Config c = decode(G, R.keys[row]);
  int64_t n = 1;  // the diagonal is always stored (finite_ed.jl:276)
  for_each_move<PLAQ, JW>(G, c, [&](uint64_t, uint32_t) { ++n; });
  counts[row] = n;
}

// Diagonal in the reference's own summation order (finite_ed.jl:265-276), so
// exported values are bitwise those of build_hamiltonian.
__device__ double ref_diag(const Geom& G, const Config& c, double g, double m) {
  double E = 0.0;
  const double cE = __dmul_rn(g, g) / 2.0;
  for (int iy = 0; iy < G.ny; ++iy)
    for (int ix = 0; ix < G.nx; ++ix) {
      if (ix < G.nx - 1) {
        double e = double(get_eR(G, c.rpack, iy * (G.nx - 1) + ix));
        E = __dadd_rn(E, __dmul_rn(cE, __dmul_rn(e, e)));
      }
      if (iy < G.ny - 1) {
        double e = double(get_eU(G, c.digits, iy * G.nx + ix));
        E = __dadd_rn(E, __dmul_rn(cE, __dmul_rn(e, e)));
      }
      const double stag = ((ix + iy) % 2 == 0) ? 1.0 : -1.0;
      E = __dadd_rn(E, __dmul_rn(__dmul_rn(m, stag), double((c.mask >> (iy * G.nx + ix)) & 1u)));
    }
  return E;
}

template <bool PLAQ, bool JW>
__global__ void k_row_fill(Geom G, RankView R, int64_t N, const int64_t* rowptr, double g,
                           double t, double m, int32_t* cols, double* vals, int* err) {
  int64_t row = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (row >= N) return;
  const Config c = decode(G, R.keys[row]);
  int64_t p = rowptr[row];
  const int64_t end = rowptr[row + 1];
  const double invg2 = 1.0 / (2.0 * __dmul_rn(g, g));
  // insertion into a column-sorted row
  auto put = [&](int64_t col, double v) {
    int64_t q = p;
    while (q > rowptr[row] && cols[q - 1] > col) {
      cols[q] = cols[q - 1];
      vals[q] = vals[q - 1];
      --q;
    }
    cols[q] = int32_t(col);
    vals[q] = v;
    ++p;
  };
  put(row, ref_diag(G, c, g, m));
  for_each_move<PLAQ, JW>(G, c, [&](uint64_t nkey, uint32_t kind) {
    const int64_t j = rank_key(R, R.segc, R.binom, nkey);
    if (j < 0 || p >= end) {
      raise_err(err, j < 0 ? kDevErrRank : kDevErrBounds);
      return;
    }
    const double v = (kind == kPlaq) ? -invg2 : ((kind == kHopNeg) ? t : -t);
    put(j, v);
  });
}

}  // namespace

cudaError_t launch_row_nnz(const Geom& G, const RankView& R, uint32_t model, int64_t* counts,
                           cudaStream_t s) {
  const int64_t N = R.dim;
  if (N == 0) return cudaSuccess;
  const unsigned blocks = unsigned((N + 255) / 256);
  const bool plaq = model & kModelPlaq, jw = model & kModelJW;
  if (plaq && jw) k_row_nnz<true, true><<<blocks, 256, 0, s>>>(G, R, N, counts), lgt::note_launch();
  else if (plaq) k_row_nnz<true, false><<<blocks, 256, 0, s>>>(G, R, N, counts), lgt::note_launch();
  else if (jw) k_row_nnz<false, true><<<blocks, 256, 0, s>>>(G, R, N, counts), lgt::note_launch();
  else k_row_nnz<false, false><<<blocks, 256, 0, s>>>(G, R, N, counts), lgt::note_launch();
  return cudaGetLastError();
}

cudaError_t launch_row_fill(const Geom& G, const RankView& R, uint32_t model,
                            const int64_t* rowptr, double g, double t, double m, int32_t* cols,
                            double* vals, int* err, cudaStream_t s) {
  const int64_t N = R.dim;
  if (N == 0) return cudaSuccess;
  const unsigned blocks = unsigned((N + 255) / 256);
  const bool plaq = model & kModelPlaq, jw = model & kModelJW;
  if (plaq && jw)
    k_row_fill<true, true><<<blocks, 256, 0, s>>>(G, R, N, rowptr, g, t, m, cols, vals, err), lgt::note_launch();
  else if (plaq)
    k_row_fill<true, false><<<blocks, 256, 0, s>>>(G, R, N, rowptr, g, t, m, cols, vals, err), lgt::note_launch();
  else if (jw)
    k_row_fill<false, true><<<blocks, 256, 0, s>>>(G, R, N, rowptr, g, t, m, cols, vals, err), lgt::note_launch();
  else
    k_row_fill<false, false><<<blocks, 256, 0, s>>>(G, R, N, rowptr, g, t, m, cols, vals, err), lgt::note_launch();
  return cudaGetLastError();
}

}  // namespace lgt
