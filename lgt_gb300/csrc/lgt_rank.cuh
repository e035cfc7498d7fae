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

// Index of `key` in the sorted key table, or -1 when absent.  `segc` and
// `binom` may point to shared-memory copies of the top-level tables.
__device__ __forceinline__ int64_t rank_key(const RankView& R, const uint32_t* segc,
                                            const uint32_t* binom, uint64_t key) {
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
