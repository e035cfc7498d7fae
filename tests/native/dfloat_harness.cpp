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
// sum_i h_i v_i with each h_i split into an FP32 pair hh + hl, the leading
// parts summed by TwoSum and the trailing parts in FP32 (Dot2 form),
// rounded to FP32 at the end.
float dfh_update(float w, const double* h, const float* v, int64_t J) {
  float hi = w, lo = 0.f;
  for (int64_t i = 0; i < J; ++i) {
    const float hh = float(h[i]), hl = float(h[i] - double(hh));
    float p, e, t;
    lgt::two_prod(hh, v[i], p, e);
    e = lgt::df_fma_rn(hl, v[i], e);
    lgt::two_sum(hi, -p, hi, t);
    lo = lgt::df_add_rn(lo, lgt::df_sub_rn(t, e));
  }
  return lgt::df_add_rn(hi, lo);
}

// sum_i a_i (bh_i + bl_i), the per-CTA dot against a double-float residual.
double dfh_dot2(const float* a, const float* bh, const float* bl, int64_t n) {
  df acc{0.f, 0.f};
  for (int64_t i = 0; i < n; ++i) lgt::df_fma2(acc, a[i], bh[i], bl[i]);
  return double(acc.hi) + double(acc.lo);
}

}  // extern "C"
