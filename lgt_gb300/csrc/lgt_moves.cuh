// lgt_moves.cuh -- enumeration of the off-diagonal moves of one basis state.
//
// Each move is a neighbour configuration reached by one term of H:
//   * hop on a horizontal bond (finite_ed.jl:279-297) or a vertical bond
//     (finite_ed.jl:300-318).  The reference stores only the "forward" hop
//     (n_L = 0, n_R = 1, e < dg -> n_L = 1, n_R = 0, e + 1) and mirrors it
//     into both (i,j) and (j,i); a row-pull kernel therefore visits both
//     directions from the row's own state.  Coefficient -t, times the
//     Jordan-Wigner parity of the sites strictly between the bond's ends on
//     the column snake in the JW model (matter_gauge_entanglement_pjw.jl:
//     104-127; vertical bonds are snake-adjacent and carry no string).
//   * plaquette W or W^dagger (matter_gauge_entanglement_pjw.jl:129-144,
//     u1_lgt_hamiltonian.jl:264-289): W lowers e_R(ix,iy), raises e_U(ix,iy),
//     lowers e_U(ix+1,iy), raises e_R(ix,iy+1); coefficient -1/(2 g^2).
// Move kinds: 0 = hop (+), 1 = hop with negative JW parity, 2 = plaquette.
#pragma once

#include "lgt_common.cuh"
#include "lgt_internal.h"

namespace lgt {

enum MoveKind : uint32_t { kHopPos = 0, kHopNeg = 1, kPlaq = 2 };

// Calls f(neighbour_key, kind) for every move of configuration c.
template <bool PLAQ, bool JW, class F>
__host__ __device__ __forceinline__ void for_each_move(const Geom& G, const Config& c, F&& f) {
  const uint32_t mask = c.mask;
  // horizontal bonds (ix,iy)-(ix+1,iy): e_U unchanged, e_R(ix,iy) +-1
#pragma unroll 1
  for (int iy = 0; iy < G.ny; ++iy) {
#pragma unroll 1
    for (int ix = 0; ix < G.nx - 1; ++ix) {
      const int r = iy * (G.nx - 1) + ix;
      const int sL = iy * G.nx + ix;
      const uint32_t nL = (mask >> sL) & 1u, nR = (mask >> (sL + 1)) & 1u;
      if (nL == nR) continue;
      const int e = get_eR(G, c.rpack, r);
      const bool ok = (nL == 0u) ? (e < G.dg) : (e > -G.dg);
      if (!ok) continue;
      uint32_t kind = kHopPos;
      if (JW) kind = (popc32(mask & G.jw_between[r]) & 1) ? kHopNeg : kHopPos;
      f(make_key(G, mask ^ (3u << sL), c.digits), kind);
    }
  }
  // vertical bonds (ix,iy)-(ix,iy+1): e_U(ix,iy) +-1
#pragma unroll 1
  for (int iy = 0; iy < G.ny - 1; ++iy) {
#pragma unroll 1
    for (int ix = 0; ix < G.nx; ++ix) {
      const int j = iy * G.nx + ix;  // link index == lower site index
      const uint32_t nD = (mask >> j) & 1u, nU = (mask >> (j + G.nx)) & 1u;
      if (nD == nU) continue;
      const int e = get_eU(G, c.digits, j);
      const uint64_t unit = digit_unit(G, j);
      const uint32_t nm = mask ^ ((1u << j) | (1u << (j + G.nx)));
      if (nD == 0u) {
        if (e < G.dg) f(make_key(G, nm, c.digits + unit), uint32_t(kHopPos));
      } else {
        if (e > -G.dg) f(make_key(G, nm, c.digits - unit), uint32_t(kHopPos));
      }
    }
  }
  if (PLAQ) {
#pragma unroll 1
    for (int iy = 0; iy < G.ny - 1; ++iy) {
#pragma unroll 1
      for (int ix = 0; ix < G.nx - 1; ++ix) {
        const int rb = iy * (G.nx - 1) + ix, rt = rb + (G.nx - 1);
        const int jl = iy * G.nx + ix, jr = jl + 1;
        const int eb = get_eR(G, c.rpack, rb), et = get_eR(G, c.rpack, rt);
        const int el = get_eU(G, c.digits, jl), er = get_eU(G, c.digits, jr);
        const int dg = G.dg;
        const uint64_t ul = digit_unit(G, jl), ur = digit_unit(G, jr);
        if (eb > -dg && el < dg && er > -dg && et < dg)  // W
          f(make_key(G, mask, c.digits + ul - ur), uint32_t(kPlaq));
        if (eb < dg && el > -dg && er < dg && et > -dg)  // W^dagger
          f(make_key(G, mask, c.digits - ul + ur), uint32_t(kPlaq));
      }
    }
  }
}

// Moves of configuration c for the rank-table path: f(nmask, rc, frc, kind)
// with the neighbour's fermion mask and, when an e_U row's free-digit index
// changes, that row rc and its new index frc (rc = -1: none changes).
// fidx[r] are the row indices of c, pw[ix] the weight of free digit ix
// (0 for the last digit of a row, which the row sum fixes).
template <bool PLAQ, bool JW, class F>
__device__ __forceinline__ void for_each_move_rows(const Geom& G, const Config& c,
                                                   const uint32_t (&fidx)[kMaxTabRows],
                                                   const int* pw, F&& f) {
  auto pick = [&](int r) {
    uint32_t v = fidx[0];
#pragma unroll
    for (int q = 1; q < kMaxTabRows; ++q)
      if (r == q) v = fidx[q];
    return v;
  };
  const uint32_t mask = c.mask;
#pragma unroll 1
  for (int iy = 0; iy < G.ny; ++iy) {
#pragma unroll 1
    for (int ix = 0; ix < G.nx - 1; ++ix) {
      const int r = iy * (G.nx - 1) + ix;
      const int sL = iy * G.nx + ix;
      const uint32_t nL = (mask >> sL) & 1u, nR = (mask >> (sL + 1)) & 1u;
      if (nL == nR) continue;
      const int e = get_eR(G, c.rpack, r);
      const bool ok = (nL == 0u) ? (e < G.dg) : (e > -G.dg);
      if (!ok) continue;
      uint32_t kind = kHopPos;
      if (JW) kind = (popc32(mask & G.jw_between[r]) & 1) ? kHopNeg : kHopPos;
      f(mask ^ (3u << sL), -1, 0u, kind);
    }
  }
#pragma unroll 1
  for (int iy = 0; iy < G.ny - 1; ++iy) {
    const uint32_t fr = pick(iy);
#pragma unroll 1
    for (int ix = 0; ix < G.nx; ++ix) {
      const int j = iy * G.nx + ix;
      const uint32_t nD = (mask >> j) & 1u, nU = (mask >> (j + G.nx)) & 1u;
      if (nD == nU) continue;
      const int e = get_eU(G, c.digits, j);
      const uint32_t nm = mask ^ ((1u << j) | (1u << (j + G.nx)));
      if (nD == 0u) {
        if (e < G.dg) f(nm, iy, fr + uint32_t(pw[ix]), uint32_t(kHopPos));
      } else {
        if (e > -G.dg) f(nm, iy, fr - uint32_t(pw[ix]), uint32_t(kHopPos));
      }
    }
  }
  if (PLAQ) {
#pragma unroll 1
    for (int iy = 0; iy < G.ny - 1; ++iy) {
      const uint32_t fr = pick(iy);
#pragma unroll 1
      for (int ix = 0; ix < G.nx - 1; ++ix) {
        const int rb = iy * (G.nx - 1) + ix, rt = rb + (G.nx - 1);
        const int jl = iy * G.nx + ix, jr = jl + 1;
        const int eb = get_eR(G, c.rpack, rb), et = get_eR(G, c.rpack, rt);
        const int el = get_eU(G, c.digits, jl), er = get_eU(G, c.digits, jr);
        const int dg = G.dg;
        const uint32_t d = uint32_t(pw[ix]) - uint32_t(pw[ix + 1]);
        if (eb > -dg && el < dg && er > -dg && et < dg)  // W
          f(mask, iy, fr + d, uint32_t(kPlaq));
        if (eb < dg && el > -dg && er < dg && et > -dg)  // W^dagger
          f(mask, iy, fr - d, uint32_t(kPlaq));
      }
    }
  }
}

}  // namespace lgt
