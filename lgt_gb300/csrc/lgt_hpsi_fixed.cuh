// lgt_hpsi_fixed.cuh -- H*psi with the lattice shape fixed at compile time
// (dg = 1, rank tables present).  Same product and same row-pull,
// atomic-free structure as k_hpsi in hpsi.cu; the difference is the cost of
// the per-row integer work.  With nx, ny constant every field offset, bond,
// Jordan-Wigner test and table stride is an immediate, the move loops are
// fully unrolled, and the three or so rank-table loads of each move are
// independent of the other moves, so they overlap.
//
// Per row the kernel computes (finite_ed.jl:265-318 for the reference model,
// matter_gauge_entanglement_pjw.jl:82-147 for the plaquette/JW model):
//   y = (cE e2 + cm stag) x_row + ch * sum_hops (+-) x_j + cp * sum_plaq x_j
// with e2 = sum of e^2 over links, stag = sum_s (+-1) n_f(s), ch = -t,
// cp = -1/(2 g^2), cE = g^2/2: the neighbour sums are plain adds (FMA by +-1
// under JW) and each coupling is applied once per row.
//
// Phase 1 (lane = row) writes the row's neighbour indices into shared
// memory, hops first, then plaquette moves; bit 31 of a hop entry is its
// Jordan-Wigner parity.  Phase 2 (lanes over (row, column slice)) gathers
// x rows (lgt_hpsi_gather.cuh).
#pragma once

#include "lgt_hpsi.h"
#include "lgt_hpsi_gather.cuh"

namespace lgt {
namespace fixed {

__host__ __device__ constexpr int pow3(int n) { return n <= 0 ? 1 : 3 * pow3(n - 1); }

template <int NX, int NY>
struct Shape {
  static constexpr int NS = NX * NY;
  static constexpr int NU = NX * (NY - 1);
  static constexpr int NR = (NX - 1) * NY;
  static constexpr int NP = (NX - 1) * (NY - 1);
  static constexpr int USHIFT = 2 * NU;  // two bits per e_U digit at dg = 1
  static constexpr int F = pow3(NX - 1); // free-digit strings per e_U row
  static constexpr int F1 = F + 1;
  static constexpr int NROWS = NY - 1;   // e_U rows, one rank table each
  static_assert(NX >= 2 && NY >= 2, "fixed shapes have at least one e_U row and bond");
  static_assert(USHIFT <= 32 && NS <= 16, "fixed shapes keep mask and digits in 32 bits");
  static_assert(NROWS <= kMaxTabRows, "too many e_U rows");
  // weight of free digit ix in its row's index (the last digit is fixed)
  __host__ __device__ static constexpr uint32_t pw(int ix) { return ix < NX - 1 ? uint32_t(pow3(NX - 2 - ix)) : 0u; }
  // sites with ix + iy even carry +m n_f, odd ones -m n_f (finite_ed.jl:272-274)
  __host__ __device__ static constexpr uint32_t parity_mask(int par) {
    uint32_t m = 0;
    for (int s = 0; s < NS; ++s)
      if (((s % NX) + (s / NX)) % 2 == par) m |= 1u << s;
    return m;
  }
};

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
// Resident blocks per SM the register budget must allow.  Measured on the
// 4x4 lattice, K = 8 complex: 6 blocks without plaquettes, 4 with them
// (their extra registers would spill).
#ifndef LGT_FIXED_MINB
#define LGT_FIXED_MINB 6
#endif
#ifndef LGT_FIXED_MINB_PLAQ
#define LGT_FIXED_MINB_PLAQ 4
#endif

template <int NX, int NY, bool PLAQ>
__host__ __device__ constexpr int max_moves() {
  return Shape<NX, NY>::NR + Shape<NX, NY>::NU + (PLAQ ? 2 * Shape<NX, NY>::NP : 0);
}

// Shared-memory stride of a row's neighbour list: odd, so the lists of the
// rows a warp touches at once fall in distinct banks.
template <int NX, int NY, bool PLAQ>
__host__ __device__ constexpr int list_stride() {
  return max_moves<NX, NY, PLAQ>() | 1;
}

using gather::coef_bytes;

template <int NX, int NY, bool PLAQ, typename T>
__host__ __device__ inline int smem_bytes(int K) {
  return coef_bytes<T>(K) + kThreads * 4 + kThreads * list_stride<NX, NY, PLAQ>() * 4;
}

// Index of the state (nm, rows f) with row rc's index replaced by frc
// (rc < 0: none): T_0[nm, f_0] + sum_r T_r[nm >> r*NX, f_{r-1}, f_r].
// g[r] = f_{r-1} * (F + 1) + f_r is the row's own (f_{r-1}, f_r) offset,
// reused by every move that leaves both digits strings alone.
template <int NX, int NY>
__device__ __forceinline__ uint32_t rank_fixed(const uint32_t* __restrict__ tab,
                                               const uint32_t (&off)[kMaxTabRows], uint32_t nm,
                                               const uint32_t (&f)[kMaxTabRows],
                                               const uint32_t (&g)[kMaxTabRows], int rc,
                                               uint32_t frc) {
  using S = Shape<NX, NY>;
  uint32_t idx = __ldg(tab + nm * uint32_t(S::F1) + ((rc == 0) ? frc : f[0]));
#pragma unroll
  for (int r = 1; r < S::NROWS; ++r) {
    uint32_t pair = g[r];
    if (rc == r) pair = f[r - 1] * uint32_t(S::F1) + frc;
    if (rc == r - 1) pair = frc * uint32_t(S::F1) + f[r];
    idx += __ldg(tab + off[r] + (nm >> (r * NX)) * uint32_t(S::F * S::F1) + pair);
  }
  return idx;
}

template <int NX, int NY, typename T, int LD, bool PLAQ, bool JW>
__global__ void __launch_bounds__(kThreads, PLAQ ? LGT_FIXED_MINB_PLAQ : LGT_FIXED_MINB)
    k_hpsi_fixed(HpsiArgs<T> a) {
  using S = Shape<NX, NY>;
  constexpr int MM = list_stride<NX, NY, PLAQ>();
  extern __shared__ __align__(16) unsigned char smem[];
  const int K = a.K;
  T* s_coef = reinterpret_cast<T*>(smem);  // [4][K]: cE, cm, ch, cp
  uint32_t* s_meta = reinterpret_cast<uint32_t*>(smem + coef_bytes<T>(K));
  uint32_t* s_nbr = s_meta + kThreads;

  for (int i = threadIdx.x; i < K; i += kThreads) {
    s_coef[i] = a.cE[i];
    s_coef[K + i] = a.cm[i];
    s_coef[2 * K + i] = a.ch[i];
    s_coef[3 * K + i] = a.cp[i];
  }
  __syncthreads();

  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t warp_row0 = (int64_t(blockIdx.x) * kWarps + wid) * 32;
  if (warp_row0 >= a.N) return;
  uint32_t* nbr = s_nbr + (wid * 32) * MM;
  const uint32_t N32 = uint32_t(a.N);

  // ---- phase 1: lane = row ------------------------------------------------
  {
    const int64_t row = warp_row0 + lane;
    uint32_t meta = 0;
    if (row < a.N) {
      const uint32_t* __restrict__ tab = a.R.tab;
      uint32_t off[kMaxTabRows];
#pragma unroll
      for (int r = 0; r < kMaxTabRows; ++r) off[r] = uint32_t(a.R.tab_off[r]);
      const uint64_t key = __ldcs(a.R.keys + row);  // read once: evict first
      const uint32_t mask = uint32_t(key >> S::USHIFT);
      const uint32_t dig =
          S::USHIFT == 32 ? uint32_t(key) : uint32_t(key) & ((1u << (S::USHIFT & 31)) - 1u);
      int eu[S::NU];
#pragma unroll
      for (int j = 0; j < S::NU; ++j) eu[j] = int((dig >> (2 * (S::NU - 1 - j))) & 3u) - 1;
      // e_R by horizontal Gauss propagation (finite_ed.jl:202-225)
      int er[S::NR];
#pragma unroll
      for (int iy = 0; iy < NY; ++iy) {
        int acc = 0;
#pragma unroll
        for (int ix = 0; ix < NX - 1; ++ix) {
          const int s = iy * NX + ix;
          acc += int((mask >> s) & 1u) + int(a.G.gq[s]);
          if (iy < NY - 1) acc -= eu[iy * NX + ix];
          if (iy > 0) acc += eu[(iy - 1) * NX + ix];
          er[iy * (NX - 1) + ix] = acc;
        }
      }
      int e2 = 0;  // e in {-1, 0, 1}: e^2 = e & 1
#pragma unroll
      for (int r = 0; r < S::NR; ++r) e2 += er[r] & 1;
#pragma unroll
      for (int j = 0; j < S::NU; ++j) e2 += eu[j] & 1;
      const int stag = __popc(mask & S::parity_mask(0)) - __popc(mask & S::parity_mask(1));
      uint32_t f[kMaxTabRows];
#pragma unroll
      for (int r = 0; r < kMaxTabRows; ++r) {
        uint32_t v = 0;
        if (r < S::NROWS) {
#pragma unroll
          for (int ix = 0; ix < NX - 1; ++ix) v += uint32_t(eu[r * NX + ix] + 1) * S::pw(ix);
        }
        f[r] = v;
      }
      uint32_t g[kMaxTabRows];
#pragma unroll
      for (int r = 0; r < kMaxTabRows; ++r)
        g[r] = (r >= 1 && r < S::NROWS) ? f[r - 1] * uint32_t(S::F1) + f[r] : 0u;
      uint32_t* my = nbr + lane * MM;
      int cnt = 0;
      bool bad = false;
      // hops on horizontal bonds (finite_ed.jl:279-297): e_U unchanged
#pragma unroll
      for (int iy = 0; iy < NY; ++iy) {
#pragma unroll
        for (int ix = 0; ix < NX - 1; ++ix) {
          const int r = iy * (NX - 1) + ix, sL = iy * NX + ix;
          const uint32_t nL = (mask >> sL) & 1u, nR = (mask >> (sL + 1)) & 1u;
          if ((nL ^ nR) && er[r] != 1 - 2 * int(nL)) {
            const uint32_t j = rank_fixed<NX, NY>(tab, off, mask ^ (3u << sL), f, g, -1, 0u);
            bad |= j >= N32;
            uint32_t ent = j;
            if (JW) ent |= uint32_t(__popc(mask & a.G.jw_between[r]) & 1) << 31;
            my[cnt++] = ent;
          }
        }
      }
      // hops on vertical bonds (finite_ed.jl:300-318): e_U(ix,iy) +-1
#pragma unroll
      for (int iy = 0; iy < NY - 1; ++iy) {
#pragma unroll
        for (int ix = 0; ix < NX; ++ix) {
          const int jl = iy * NX + ix;
          const uint32_t nD = (mask >> jl) & 1u, nU = (mask >> (jl + NX)) & 1u;
          if ((nD ^ nU) && eu[jl] != 1 - 2 * int(nD)) {
            const uint32_t fr = nD ? f[iy] - S::pw(ix) : f[iy] + S::pw(ix);
            const uint32_t j =
                rank_fixed<NX, NY>(tab, off, mask ^ ((1u << jl) | (1u << (jl + NX))), f, g, iy, fr);
            bad |= j >= N32;
            my[cnt++] = j;
          }
        }
      }
      const int cnth = cnt;
      if (PLAQ) {  // W and W^dagger (u1_lgt_hamiltonian.jl:264-289)
#pragma unroll
        for (int iy = 0; iy < NY - 1; ++iy) {
#pragma unroll
          for (int ix = 0; ix < NX - 1; ++ix) {
            const int eb = er[iy * (NX - 1) + ix], et = er[(iy + 1) * (NX - 1) + ix];
            const int el = eu[iy * NX + ix], ey = eu[iy * NX + ix + 1];
            const uint32_t d = S::pw(ix) - S::pw(ix + 1);
            if (eb > -1 && el < 1 && ey > -1 && et < 1) {
              const uint32_t j = rank_fixed<NX, NY>(tab, off, mask, f, g, iy, f[iy] + d);
              bad |= j >= N32;
              my[cnt++] = j;
            }
            if (eb < 1 && el > -1 && ey < 1 && et > -1) {
              const uint32_t j = rank_fixed<NX, NY>(tab, off, mask, f, g, iy, f[iy] - d);
              bad |= j >= N32;
              my[cnt++] = j;
            }
          }
        }
      }
      if (bad) {  // never for a consistent basis; drop the row's moves
        raise_err(a.err, kDevErrBounds);
        cnt = 0;
      }
      meta = gather::pack_meta(cnt, PLAQ ? (bad ? 0 : cnth) : cnt, e2, stag);
    }
    s_meta[wid * 32 + lane] = meta;
  }
  __syncwarp();

  gather::gather_rows<T, LD, PLAQ, JW>(a, warp_row0, lane, s_meta + wid * 32, s_coef,
                                       [&](int rl) { return nbr + rl * MM; });
}

// Launches the fixed-shape kernel for (NX, NY); the caller has checked
// dg == 1, rank tables present, N < 2^31, C % (16 / sizeof(T)) == 0 and
// 16-byte aligned panels.
template <int NX, int NY, typename T, int LD, bool PLAQ, bool JW>
cudaError_t launch_shape_v(const HpsiArgs<T>& a, cudaStream_t s) {
  auto kern = k_hpsi_fixed<NX, NY, T, LD, PLAQ, JW>;
  const int bytes = smem_bytes<NX, NY, PLAQ, T>(a.K);
  {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), bytes);
    if (e != cudaSuccess) return e;
  }
  const int64_t blocks = (a.N + kThreads - 1) / kThreads;
  if (blocks <= 0) return cudaSuccess;
  kern<<<unsigned(blocks), kThreads, bytes, s>>>(a), lgt::note_launch();
  return cudaGetLastError();
}

// Load mode: a.vpl = 1 one vector per lane, 2 two vectors, 3 two vectors as
// one 32-byte access; 0 the built-in rule (two vectors when C allows).  A mode
// the panel cannot take falls back to the next narrower one.
template <int NX, int NY, typename T, bool PLAQ, bool JW>
cudaError_t launch_shape_m(const HpsiArgs<T>& a, cudaStream_t s) {
  constexpr int V = 16 / int(sizeof(T));
  const bool two = a.C % (2 * V) == 0;
  // 32-byte accesses: panels and the Krylov panel stride keep every row
  // slice 32-byte aligned
  const bool wide = two && (reinterpret_cast<uintptr_t>(a.x) & 31) == 0 &&
                    (reinterpret_cast<uintptr_t>(a.y) & 31) == 0 &&
                    (a.xsel == nullptr || (a.xstride * sizeof(T)) % 32 == 0);
  if (a.vpl == 3 && wide) return launch_shape_v<NX, NY, T, 4, PLAQ, JW>(a, s);
  if (a.vpl != 1 && two) return launch_shape_v<NX, NY, T, 2, PLAQ, JW>(a, s);
  return launch_shape_v<NX, NY, T, 1, PLAQ, JW>(a, s);
}

template <int NX, int NY, typename T>
cudaError_t launch_shape(const HpsiArgs<T>& a, uint32_t model, cudaStream_t s) {
  const bool plaq = model & kModelPlaq, jw = model & kModelJW;
  if (plaq && jw) return launch_shape_m<NX, NY, T, true, true>(a, s);
  if (plaq) return launch_shape_m<NX, NY, T, true, false>(a, s);
  if (jw) return launch_shape_m<NX, NY, T, false, true>(a, s);
  return launch_shape_m<NX, NY, T, false, false>(a, s);
}

}  // namespace fixed
}  // namespace lgt
