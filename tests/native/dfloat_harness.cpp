// Host harness of lgt_gb300/csrc/lgt_dfloat.cuh for the CPU tests: the same
// double-float routines the mixed-precision reduction kernels use, exported
// over a C ABI (built by tests/test_dfloat.py with -ffp-contract=off).
#include <cstdint>

#include "../../lgt_gb300/csrc/lgt_dfloat.cuh"

using lgt::df;

extern "C" {

// sum_i a_i b_i, accumulated as the dot kernels do (df_fma per term).
double dfh_dot(const float* a, const float* b, int64_t n) {
  df acc{0.f, 0.f};
  for (int64_t i = 0; i < n; ++i) lgt::df_fma(acc, a[i], b[i]);
  return double(acc.hi) + double(acc.lo);
}

// The Gram-Schmidt update of one entry, as k_update_df does it: w minus
// sum_i h_i v_i with each h_i split into an FP32 pair, two coefficient
// chains (even and odd i), rounded to FP32 at the end.
float dfh_update(float w, const double* h, const float* v, int64_t J) {
  df a0{w, 0.f}, a1{0.f, 0.f};
  int64_t i = 0;
  for (; i + 1 < J; i += 2) {
    const float h0 = float(h[i]), h1 = float(h[i + 1]);
    lgt::df_sub_prod(a0, h0, float(h[i] - double(h0)), v[i]);
    lgt::df_sub_prod(a1, h1, float(h[i + 1] - double(h1)), v[i + 1]);
  }
  if (i < J) {
    const float h0 = float(h[i]);
    lgt::df_sub_prod(a0, h0, float(h[i] - double(h0)), v[i]);
  }
  return lgt::df_round(lgt::df_add(a0, a1));
}

// sum_i a_i (bh_i + bl_i), the per-CTA dot against a double-float residual.
double dfh_dot2(const float* a, const float* bh, const float* bl, int64_t n) {
  df acc{0.f, 0.f};
  for (int64_t i = 0; i < n; ++i) lgt::df_fma2(acc, a[i], bh[i], bl[i]);
  return double(acc.hi) + double(acc.lo);
}

}  // extern "C"
