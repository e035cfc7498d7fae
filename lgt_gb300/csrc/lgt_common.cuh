// lgt_common.cuh -- geometry, key layout and small device helpers shared by
// the GB300 exact-diagonalisation kernels.
//
// A basis state of the U(1) link model (finite_ed.jl:69-78) is the triple
// (n_f, e_R, e_U).  The Gauss law fixes e_R from (n_f, e_U)
// (finite_ed.jl:202-225), so a state is identified by its ORDER KEY
//
//     key = (mask << ushift) | digits
//     mask   = sum_s n_f(s) << s,   s = (iy-1)*nx + (ix-1)     (finite_ed.jl:142)
//     digits = e_U values (e+dg) in w-bit fields, iy outer, ix inner, the
//              first link most significant;  ushift = w * N_U.
//
// The reference numbers states in discovery order: masks ascending
// (finite_ed.jl:138), then e_U lexicographic with values ascending from -dg
// (finite_ed.jl:174-200).  The order key is strictly increasing in that
// order, so the index of a state is the rank of its key in the sorted key
// table, and that rank + 1 is the reference's key_dict value.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lgt {

constexpr int kMaxSites = 32;   // fermion mask fits a uint32
constexpr int kMaxLinks = 64;

enum Model : uint32_t {
  kModelRef = 0,   // finite_ed.jl:252-322: diagonal + bare hopping
  kModelJW = 1u,   // Jordan-Wigner strings on the column snake
  kModelPlaq = 2u, // magnetic plaquette -(1/2g^2)(W + W^dag)
  kModelPJW = 3u,  // matter_gauge_entanglement_pjw.jl:82-147
};

// Error bits a kernel may raise in the per-basis device error word.  Kernels
// never trap: they record and skip the access.
enum DevErr : int {
  kDevErrRank = 1,      // a neighbour key was not found in the basis
  kDevErrBounds = 2,    // an index fell outside its buffer
  kDevErrNaN = 4,       // a non-finite value was produced
  kDevErrSpin = 8,      // a bounded wait ran out
};

// Geometry passed by value to every kernel (fits the 4 KB parameter space).
struct Geom {
  int nx, ny, dg;
  int ns;          // sites
  int nR, nU, nP;  // right links, up links, plaquettes
  int w;           // bits per e_U digit
  int ushift;      // w * nU
  int nf_target;   // number of fermions, -sum(g)
  int max_moves;   // nR + nU + 2 nP: upper bound on off-diagonal entries per row
  uint32_t even_mask;        // sites with ix+iy even (1-based): staggered sign +1
  uint32_t odd_mask;         // sites with ix+iy odd: staggered sign -1
  int8_t gq[kMaxSites];      // background charge g(s)
  int8_t grow[kMaxSites];    // sum of g over row iy (0-based row index)
  uint32_t jw_between[kMaxSites];  // per horizontal bond r: sites strictly
                                   // between its ends on the column snake
};

__host__ __device__ inline uint64_t digit_unit(const Geom& G, int j) {
  // weight of e_U link j (0-based, iy outer / ix inner) in the order key
  return 1ull << (G.w * (G.nU - 1 - j));
}

__host__ __device__ inline int get_eU(const Geom& G, uint64_t digits, int j) {
  return int((digits >> (G.w * (G.nU - 1 - j))) & ((1u << G.w) - 1)) - G.dg;
}

// Decoded configuration of one state, kept in packed registers: e_U and e_R
// as w-bit (e+dg) fields, indexed eU: j = iy*nx+ix (iy < ny-1),
// eR: r = iy*(nx-1)+ix (ix < nx-1), all 0-based.
struct Config {
  uint32_t mask;
  uint64_t digits;  // e_U fields exactly as in the key
  uint64_t rpack;   // e_R fields, field r at bit w*r
};

__host__ __device__ inline int get_eR(const Geom& G, uint64_t rpack, int r) {
  return int((rpack >> (G.w * r)) & ((1u << G.w) - 1)) - G.dg;
}

// Derive e_R of a state from (mask, e_U) by horizontal Gauss propagation
// (finite_ed.jl:202-225).  Returns false when some e_R leaves [-dg, dg]
// (only possible for keys that are not basis states).
__host__ __device__ inline bool derive_eR(const Geom& G, uint32_t mask, uint64_t digits,
                                          uint64_t* rpack) {
  uint64_t rp = 0;
  for (int iy = 0; iy < G.ny; ++iy) {
    int acc = 0;
    for (int ix = 0; ix < G.nx - 1; ++ix) {
      int s = iy * G.nx + ix;
      int q = int((mask >> s) & 1u) + G.gq[s];
      int eu_now = (iy < G.ny - 1) ? get_eU(G, digits, iy * G.nx + ix) : 0;
      int eu_prev = (iy > 0) ? get_eU(G, digits, (iy - 1) * G.nx + ix) : 0;
      acc += q - eu_now + eu_prev;
      if (acc < -G.dg || acc > G.dg) return false;
      rp |= uint64_t(acc + G.dg) << (G.w * (iy * (G.nx - 1) + ix));
    }
  }
  *rpack = rp;
  return true;
}

__host__ __device__ inline Config decode(const Geom& G, uint64_t key) {
  Config c;
  c.mask = uint32_t(G.ushift >= 64 ? 0 : (key >> G.ushift));
  c.digits = G.ushift >= 64 ? key : (key & ((1ull << G.ushift) - 1));
  c.rpack = 0;
  derive_eR(G, c.mask, c.digits, &c.rpack);
  return c;
}

__host__ __device__ inline uint64_t make_key(const Geom& G, uint32_t mask, uint64_t digits) {
  return (uint64_t(mask) << G.ushift) | digits;
}

// Reference packed key _encode (finite_ed.jl:80-97), dg == 1 only: n_f bits,
// then 2-bit (e+1) fields of e_R (iy outer, ix = 1..nx-1), then of e_U.
__host__ __device__ inline uint64_t ref_encode(const Geom& G, const Config& c) {
  uint64_t key = c.mask;  // bits [0, ns): n_f at s = iy*nx+ix
  int off = G.ns;
  for (int r = 0; r < G.nR; ++r, off += 2)
    key |= uint64_t(get_eR(G, c.rpack, r) + 1) << off;
  for (int j = 0; j < G.nU; ++j, off += 2)
    key |= uint64_t(get_eU(G, c.digits, j) + 1) << off;
  return key;
}

// Integer parts of the diagonal (finite_ed.jl:265-276):
//   E_diag = (g^2/2) * e2 + m * stag,  e2 = sum e^2 over links,
//   stag = sum_s (+1 if ix+iy even else -1) n_f(s).
__host__ __device__ inline void diag_parts(const Geom& G, const Config& c, int* e2, int* stag) {
  int s2 = 0;
  for (int r = 0; r < G.nR; ++r) {
    int e = get_eR(G, c.rpack, r);
    s2 += e * e;
  }
  for (int j = 0; j < G.nU; ++j) {
    int e = get_eU(G, c.digits, j);
    s2 += e * e;
  }
  *e2 = s2;
#ifdef __CUDA_ARCH__
  *stag = __popc(c.mask & G.even_mask) - __popc(c.mask & G.odd_mask);
#else
  *stag = __builtin_popcount(c.mask & G.even_mask) - __builtin_popcount(c.mask & G.odd_mask);
#endif
}

__host__ __device__ inline int popc32(uint32_t v) {
#ifdef __CUDA_ARCH__
  return __popc(v);
#else
  return __builtin_popcount(v);
#endif
}

#ifdef __CUDACC__
__device__ inline void raise_err(int* err, int bit) {
  if (err) atomicOr(err, bit);
}

// FP32 -> FP64 widening by integer operations on the bit pattern (IEEE-754
// binary32 -> binary64: exponent rebiased by 1023 - 127, mantissa shifted
// left by 29), so mixed-precision kernels keep conversions off GB300's
// narrow FP64 pipe.  Exact for normal numbers; FP32 subnormals (below
// 1.2e-38) become zero; infinities and NaNs stay infinities and NaNs.
__device__ __forceinline__ double widen(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t m = (e == 0u) ? 0u : (u & 0x7fffffu);
  const uint32_t ed = (e == 0u) ? 0u : ((e == 0xffu) ? 0x7ffu : e + 896u);
  const uint32_t hi = (u & 0x80000000u) | (ed << 20) | (m >> 3);
  return __hiloint2double(int(hi), int(m << 29));
}
__device__ __forceinline__ double widen(double d) { return d; }

// FP64 -> FP32 rounding to nearest (ties to even) by integer operations on
// the bit pattern, the counterpart of widen: magnitudes below the FP32
// normal range (2^-126) become signed zero, those above it infinity; NaN
// stays NaN.  A mantissa that rounds up to 2^24 carries into the exponent
// through the addition.
__device__ __forceinline__ float narrow(double d) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(d));
  const uint32_t sign = uint32_t(u >> 32) & 0x80000000u;
  const int e = int((u >> 52) & 0x7ffu);
  const unsigned long long mant = u & 0xfffffffffffffull;
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (mant ? 0x400000u : 0u));
  const int e32 = e - 1023 + 127;
  if (e32 <= 0) return __uint_as_float(sign);
  uint32_t m = uint32_t(mant >> 29);
  const uint32_t rem = uint32_t(mant & 0x1fffffffull);
  if (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ++m;
  uint32_t bits = (uint32_t(e32) << 23) + m;
  if (e32 >= 255 || bits >= 0x7f800000u) bits = 0x7f800000u;
  return __uint_as_float(sign | bits);
}

// A value in the storage type S of a Krylov basis (float: narrow).
template <typename S>
__device__ __forceinline__ S to_storage(double d) {
  if constexpr (sizeof(S) == 4) return narrow(d);
  else return S(d);
}
#endif

}  // namespace lgt
