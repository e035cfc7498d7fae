// lgt_hpsi_gather.cuh -- the gather phase shared by the row-pull H*psi
// kernels whose neighbour lists sit in shared memory (the fixed-shape kernel,
// which ranks the moves itself, and the stored-table kernel, which copies
// them from the neighbour table).
//
// Lanes run over (row, W-column slice) of the warp's 32 rows: each of a
// row's lanes loads one or two vectors of V elements per neighbour (LD = 1,
// 2), or two vectors as one 32-byte access (LD = 4), sums the hop
// neighbours (times the Jordan-Wigner sign) and the plaquette neighbours in
// two accumulators, and applies the couplings once per row:
//   y = (cE e2 + cm stag) x_row + ch * sum_hops (+-) x_j + cp * sum_plaq x_j
// (finite_ed.jl:265-318; matter_gauge_entanglement_pjw.jl:82-147).
#pragma once

#include "lgt_hpsi.h"

namespace lgt {
namespace gather {

// Neighbour rows gathered per loop trip: measured on the 4x4 lattice, K = 8
// complex, 8 rows in flight for FP32 (the table kernel: 0.757 -> 0.714 ms
// against 4; the fixed-shape kernel is indifferent), 2 for FP64 (bound by
// the FP64 pipe, not by latency; 8 costs 15%).
#ifndef LGT_GATHER_UNROLL
#define LGT_GATHER_UNROLL (sizeof(T) == 4 ? 8 : 2)
#endif

// Per-row meta word of a neighbour list: entry count, hop count (hops come
// first), sum of e^2 over the links and the staggered occupation + 128.
__host__ __device__ constexpr uint32_t pack_meta(int cnt, int nh, int e2, int stag) {
  return uint32_t(cnt) | (uint32_t(nh) << 8) | (uint32_t(e2) << 16) | (uint32_t(stag + 128) << 24);
}

template <typename T>
__host__ __device__ inline int coef_bytes(int K) {
  return (4 * K * int(sizeof(T)) + 15) / 16 * 16;
}

template <typename T, int V>
struct VecT;
template <>
struct VecT<double, 2> {
  using type = double2;
};
template <>
struct VecT<float, 4> {
  using type = float4;
};

template <typename T, int V>
__device__ __forceinline__ void ld(const T* p, T* r) {
  using VT = typename VecT<T, V>::type;
  const VT v = __ldg(reinterpret_cast<const VT*>(p));
  const T* s = reinterpret_cast<const T*>(&v);
#pragma unroll
  for (int e = 0; e < V; ++e) r[e] = s[e];
}

// y is written once and not read again by this kernel: streaming store, so
// its lines do not push reusable x rows out of L2
template <typename T, int V>
__device__ __forceinline__ void st(T* p, const T* r) {
  using VT = typename VecT<T, V>::type;
  VT v;
  T* s = reinterpret_cast<T*>(&v);
#pragma unroll
  for (int e = 0; e < V; ++e) s[e] = r[e];
  __stcs(reinterpret_cast<VT*>(p), v);
}

// 32-byte loads and streaming stores (sm_100+ 256-bit global accesses);
// the address must be 32-byte aligned, which the host checks.
__device__ __forceinline__ void ld32(const float* p, float* r) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]),
        "=f"(r[7])
      : "l"(p));
}
__device__ __forceinline__ void ld32(const double* p, double* r) {
  asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
      : "=d"(r[0]), "=d"(r[1]), "=d"(r[2]), "=d"(r[3])
      : "l"(p));
}
__device__ __forceinline__ void st32(float* p, const float* r) {
  asm volatile("st.global.cs.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
               :
               : "l"(p), "f"(r[0]), "f"(r[1]), "f"(r[2]), "f"(r[3]), "f"(r[4]), "f"(r[5]),
                 "f"(r[6]), "f"(r[7])
               : "memory");
}
__device__ __forceinline__ void st32(double* p, const double* r) {
  asm volatile("st.global.cs.v4.f64 [%0], {%1, %2, %3, %4};"
               :
               : "l"(p), "d"(r[0]), "d"(r[1]), "d"(r[2]), "d"(r[3])
               : "memory");
}

// A lane's columns of one row: LD = 1 one vector, 2 two vectors, 4 two
// vectors as one 32-byte access.
template <typename T, int V, int LD>
__device__ __forceinline__ void ld_slice(const T* p, T* r) {
  if (LD == 4) {
    ld32(p, r);
  } else {
#pragma unroll
    for (int q = 0; q < LD; ++q) ld<T, V>(p + q * V, r + q * V);
  }
}
template <typename T, int V, int LD>
__device__ __forceinline__ void st_slice(T* p, const T* r) {
  if (LD == 4) {
    st32(p, r);
  } else {
#pragma unroll
    for (int q = 0; q < LD; ++q) st<T, V>(p + q * V, r + q * V);
  }
}

// The gather phase for the warp's rows warp_row0 .. warp_row0 + 31:
// s_meta[rl] is row rl's meta word (pack_meta), list(rl) its entries (hop
// entries carry the Jordan-Wigner parity in bit 31), s_coef the couplings
// [4][K]: cE, cm, ch, cp.
template <typename T, int LD, bool PLAQ, bool JW, class List>
__device__ __forceinline__ void gather_rows(const HpsiArgs<T>& a, int64_t warp_row0, int lane,
                                            const uint32_t* s_meta, const T* s_coef, List list) {
  constexpr int V = 16 / int(sizeof(T));
  constexpr int W = V * (LD == 1 ? 1 : 2);  // columns per lane
  const int K = a.K;
  const int C = a.C;
  const int lpr = C / W;  // lanes per row (C % W == 0 on the host)
  const int items = 32 * lpr;
  const T* __restrict__ x = a.xsel ? a.x + size_t(*a.xsel) * a.xstride : a.x;
  T* __restrict__ y = a.y;
  const int ncomp = a.ncomp;
  for (int it = lane; it < items; it += 32) {
    const int rl = it / lpr;
    const int64_t row = warp_row0 + rl;
    if (row >= a.N) continue;
    // lane slice: W contiguous columns (interleaving the row's lanes so that
    // one load instruction covers whole sectors measured slower)
    const int col0 = (it - rl * lpr) * W;
    const uint32_t m = s_meta[rl];
    const int cnt = int(m & 255u), nh = int((m >> 8) & 255u);
    const T e2 = T(int((m >> 16) & 255u)), stag = T(int(m >> 24) - 128);
    const uint32_t* lst = list(rl);
    T ah[W], ap[W], xd[W], xs[LGT_GATHER_UNROLL][W];
    const T* px = x + size_t(row) * C + col0;
    ld_slice<T, V, LD>(px, xd);
#pragma unroll
    for (int e = 0; e < W; ++e) {
      ah[e] = T(0);
      ap[e] = T(0);
    }
    // LGT_GATHER_UNROLL neighbour rows in flight per trip; the tail trip
    // gathers only the rows that exist and adds zeros for the rest
    for (int n = 0; n < nh; n += LGT_GATHER_UNROLL) {
      uint32_t ent[LGT_GATHER_UNROLL];
#pragma unroll
      for (int u = 0; u < LGT_GATHER_UNROLL; ++u) {
        ent[u] = (n + u < nh) ? lst[n + u] : 0u;
        if (n + u < nh) {
          ld_slice<T, V, LD>(x + size_t(ent[u] & 0x7fffffffu) * C + col0, xs[u]);
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) xs[u][e] = T(0);
        }
      }
#pragma unroll
      for (int u = 0; u < LGT_GATHER_UNROLL; ++u) {
        if (JW) {
          const T sg = (ent[u] >> 31) ? T(-1) : T(1);
#pragma unroll
          for (int e = 0; e < W; ++e) ah[e] = fma(sg, xs[u][e], ah[e]);
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) ah[e] += xs[u][e];
        }
      }
    }
    if (PLAQ) {
      for (int n = nh; n < cnt; n += LGT_GATHER_UNROLL) {
#pragma unroll
        for (int u = 0; u < LGT_GATHER_UNROLL; ++u) {
          if (n + u < cnt) {
            ld_slice<T, V, LD>(x + size_t(lst[n + u]) * C + col0, xs[u]);
          } else {
#pragma unroll
            for (int e = 0; e < W; ++e) xs[u][e] = T(0);
          }
        }
#pragma unroll
        for (int u = 0; u < LGT_GATHER_UNROLL; ++u)
#pragma unroll
          for (int e = 0; e < W; ++e) ap[e] += xs[u][e];
      }
    }
    // y = (cE e2 + cm stag) x + ch * hops (+ cp * plaquettes); the diagonal
    // coefficient once per point (the re and im columns of a complex point
    // share it; W and col0 are even)
    auto finish = [&](int e, int k, T cd) {
      T v = fma(s_coef[2 * K + k], ah[e], cd * xd[e]);
      if (PLAQ) v = fma(s_coef[3 * K + k], ap[e], v);
      xd[e] = v;
    };
    if (ncomp == 2 && (W % 2) == 0) {
#pragma unroll
      for (int e = 0; e < W; e += 2) {
        const int k = (col0 + e) >> 1;
        const T cd = s_coef[k] * e2 + s_coef[K + k] * stag;  // (g^2/2) e2 + m stag
        finish(e, k, cd);
        finish(e + 1, k, cd);
      }
    } else {
#pragma unroll
      for (int e = 0; e < W; ++e) {
        const int col = col0 + e;
        const int k = (ncomp == 2) ? (col >> 1) : col;
        finish(e, k, s_coef[k] * e2 + s_coef[K + k] * stag);
      }
    }
    st_slice<T, V, LD>(y + size_t(row) * C + col0, xd);
  }
}

}  // namespace gather
}  // namespace lgt
