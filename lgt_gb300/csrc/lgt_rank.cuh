// lgt_rank.cuh -- order key -> basis index (the Dict lookup of
// finite_ed.jl:291-292 and :310-311, done without a hash table).
#pragma once

#include "lgt_internal.h"

namespace lgt {

// Colexicographic rank of a k-subset given as a bit mask:
// sum_j C(p_j, j) over the set-bit positions p_1 < p_2 < ... (j from 1).
// Masks with k bits in ascending numeric order have ranks 0, 1, 2, ...
__device__ __forceinline__ int colex_rank(uint32_t mask, const uint32_t* binom) {
  int r = 0, j = 1;
  while (mask) {
    int p = __ffs(mask) - 1;
    r += int(binom[p * 33 + j]);
    ++j;
    mask &= mask - 1;
  }
  return r;
}

// Index of the free e_U digits of row r in the row's lexicographic order
// (first digit most significant, base B).
__device__ __forceinline__ uint32_t row_index(const RankView& R, uint64_t digits, int r) {
  const uint32_t dmask = (1u << R.w) - 1u;
  uint32_t f = 0;
  for (int ix = 0; ix < R.nx - 1; ++ix) {
    const int j = r * R.nx + ix;
    f = f * uint32_t(R.B) + uint32_t((digits >> (R.w * (R.nU - 1 - j))) & dmask);
  }
  return f;
}

// Rank by the row-count tables: mask and the row indices f[r] of a basis
// state; row rc (if >= 0) uses frc instead of f[rc].
__device__ __forceinline__ int64_t rank_rows(const RankView& R, uint32_t mask, const uint32_t* f,
                                             int rc, uint32_t frc) {
  const uint32_t F1 = uint32_t(R.F) + 1u;
  uint32_t fr = (rc == 0) ? frc : f[0];
  int64_t rk = __ldg(R.tab + uint64_t(mask) * F1 + fr);
#pragma unroll
  for (int r = 1; r < kMaxTabRows; ++r) {
    if (r >= R.nrows) break;
    const uint32_t fp = fr;
    fr = (rc == r) ? frc : f[r];
    const uint64_t m = uint64_t(mask >> (r * R.nx));
    rk += __ldg(R.tab + R.tab_off[r] + (m * uint64_t(R.F) + fp) * F1 + fr);
  }
  return rk;
}

// Index of `key` in the sorted key table, or -1 when absent.  `segc` and
// `binom` may point to shared-memory copies of the top-level tables.
__device__ __forceinline__ int64_t rank_key(const RankView& R, const uint32_t* segc,
                                            const uint32_t* binom, uint64_t key) {
  if (R.tab) {
    uint32_t f[kMaxTabRows];
    const uint64_t digits = key & ((1ull << R.ushift) - 1);
#pragma unroll
    for (int r = 0; r < kMaxTabRows; ++r) f[r] = (r < R.nrows) ? row_index(R, digits, r) : 0u;
    const uint64_t m64 = key >> R.ushift;
    if ((m64 >> R.ns) != 0 || __popcll(m64) != R.nf) return -1;
    const uint32_t mask = uint32_t(m64);
    const int64_t i = rank_rows(R, mask, f, -1, 0);
    if (i < 0 || i >= R.dim || __ldg(R.keys + i) != key) return -1;
    return i;
  }
  uint32_t mask = uint32_t(key >> R.ushift);
  int cr = colex_rank(mask, binom);
  if (cr < 0 || cr >= R.nmasks) return -1;
  uint32_t lo = segc[cr], hi = segc[cr + 1];
  if (R.low32) {
    const uint32_t t = uint32_t(key & ((1ull << R.ushift) - 1));
    uint32_t n = hi - lo;
    const uint32_t* base = R.low + lo;
    // branch-reduced lower bound
    while (n > 1) {
      uint32_t half = n >> 1;
      if (__ldg(base + half - 1) < t) base += half;
      n -= half;
    }
    if (n == 1 && __ldg(base) < t) ++base;
    int64_t i = int64_t(base - R.low);
    if (i < int64_t(hi) && __ldg(R.low + i) == t) return i;
    return -1;
  } else {
    uint32_t n = hi - lo;
    const uint64_t* base = R.keys + lo;
    while (n > 1) {
      uint32_t half = n >> 1;
      if (__ldg(base + half - 1) < key) base += half;
      n -= half;
    }
    if (n == 1 && __ldg(base) < key) ++base;
    int64_t i = int64_t(base - R.keys);
    if (i < int64_t(hi) && __ldg(R.keys + i) == key) return i;
    return -1;
  }
}

}  // namespace lgt
