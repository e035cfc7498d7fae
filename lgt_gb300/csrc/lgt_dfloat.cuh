// lgt_dfloat.cuh -- double-float ("float-float") arithmetic for the
// FP64-class reductions of the FP32-mixed Krylov drivers.
//
// GB300 issues FP32 fused multiply-adds at 64 times the rate of FP64 ones,
// and the Gram-Schmidt dots and updates of the mixed path (FP32 Krylov
// vectors, FP64-class accumulation) are bound by the FP64 pipe when written
// in FP64.  Here a value is carried as the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi) / 2 (about 48 significant bits) and
// combined with error-free transformations:
//   * TwoSum (Knuth, The Art of Computer Programming vol. 2, 4.2.2):
//     s = fl(a + b) and the exact rounding error e, a + b = s + e;
//   * Fast2Sum (Dekker 1971), the same when |a| >= |b|, in three operations;
//   * TwoProduct with a fused multiply-add: p = fl(a b), e = fma(a, b, -p),
//     a b = p + e exactly.
// Sums and dot products built from them follow Ogita, Rump and Oishi,
// "Accurate Sum and Dot Product", SIAM J. Sci. Comput. 26(6), 2005, with
// the running sum renormalised after every term (the double-word addition
// of Joldes, Muller and Popescu, ACM TOMS 44(2), 2017, Alg. 5), so a sum of
// n terms is off by at most about 3 n 2^-48 times the sum of |terms|.
//
// Every operation goes through the _rn intrinsics on the device, which the
// compiler never contracts into fused multiply-adds or reassociates: the
// transformations are exact only for separately rounded operations.  The
// host versions (for CPU tests of the same code) need a build without
// floating-point contraction (-ffp-contract=off).
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define LGT_DF_FN __host__ __device__ __forceinline__
#else
#define LGT_DF_FN inline
#endif

namespace lgt {

struct df {
  float hi, lo;
};

LGT_DF_FN float df_add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
LGT_DF_FN float df_sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
LGT_DF_FN float df_mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
LGT_DF_FN float df_fma_rn(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

// a + b = s + e exactly (Knuth's TwoSum, no ordering needed).
LGT_DF_FN void two_sum(float a, float b, float& s, float& e) {
  s = df_add_rn(a, b);
  const float bb = df_sub_rn(s, a);
  e = df_add_rn(df_sub_rn(a, df_sub_rn(s, bb)), df_sub_rn(b, bb));
}

// a + b = s + e exactly when |a| >= |b| (or a == 0) (Dekker's Fast2Sum).
LGT_DF_FN void fast_two_sum(float a, float b, float& s, float& e) {
  s = df_add_rn(a, b);
  e = df_sub_rn(b, df_sub_rn(s, a));
}

// a * b = p + e exactly (FMA form of Dekker's product; no overflow assumed).
LGT_DF_FN void two_prod(float a, float b, float& p, float& e) {
  p = df_mul_rn(a, b);
  e = df_fma_rn(a, b, -p);
}

// x += (p + e), where p + e is a product from two_prod (or any pair with
// |e| small against |p|): TwoSum of the leading parts, the trailing parts
// added, then renormalised.
LGT_DF_FN void df_acc(df& x, float p, float e) {
  float s, t;
  two_sum(x.hi, p, s, t);
  t = df_add_rn(t, df_add_rn(x.lo, e));
  fast_two_sum(s, t, x.hi, x.lo);
}

// x += a * b for FP32 a, b: the product exactly, then accumulated.
LGT_DF_FN void df_fma(df& x, float a, float b) {
  float p, e;
  two_prod(a, b, p, e);
  df_acc(x, p, e);
}

// x += a * (bh + bl) for an FP32 a and a double-float b: the leading product
// exactly, the trailing one rounded (it is 2^-24 smaller).
LGT_DF_FN void df_fma2(df& x, float a, float bh, float bl) {
  float p, e;
  two_prod(a, bh, p, e);
  e = df_fma_rn(a, bl, e);
  df_acc(x, p, e);
}

// x -= (hh + hl) * v: the update of a double-float residual by an FP32
// basis entry v and a coefficient split into hh + hl.
LGT_DF_FN void df_sub_prod(df& x, float hh, float hl, float v) {
  float p, e;
  two_prod(hh, v, p, e);
  e = df_fma_rn(hl, v, e);
  df_acc(x, -p, -e);
}

// x + y for two double-floats (the same sequence as df_acc).
LGT_DF_FN df df_add(df x, df y) {
  df_acc(x, y.hi, y.lo);
  return x;
}

// The FP32 value nearest to hi + lo (up to a tie at the last bit).
LGT_DF_FN float df_round(df x) { return df_add_rn(x.hi, x.lo); }

}  // namespace lgt
