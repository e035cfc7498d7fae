// lgt_tridiag.cuh -- lowest eigenpair of the Lanczos tridiagonal T, on one
// warp: Sturm-count multisection (division-free recurrence) and inverse
// iteration, in FP64 or, for the FP32-mixed path, FP32.  Used by the
// per-CTA solver (small.cu) and the panel solver's checks (krylov.cu).
// The work array holds at least 3 * kTriMax doubles, z at least kTriMax.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lgt {

constexpr int kTriMax = 64;  // largest Krylov dimension + 1

// Number of eigenvalues of the tridiagonal (a, b) below x: sign changes of
// the leading principal minors p_i = det(T_i - x I), from the three-term
// recurrence p_i = (a_i - x) p_{i-1} - b_{i-1}^2 p_{i-2} (bb holds b^2).
// Division-free (FP64 division is a long dependent chain on this part); the
// minors are rescaled by 2^-600 when they grow past 2^600; an exact zero
// takes the sign opposite to its predecessor.  Signs, zeros and magnitudes
// are read from the bit patterns (integer operations), so a step costs
// three FP64 operations.
__device__ __forceinline__ int sign_bit(double v) { return int(uint32_t(__double2hiint(v)) >> 31); }
__device__ __forceinline__ bool is_zero(double v) {
  return ((uint32_t(__double2hiint(v)) & 0x7fffffffu) | uint32_t(__double2loint(v))) == 0u;
}
__device__ __forceinline__ int exp_bits(double v) {
  return int((uint32_t(__double2hiint(v)) >> 20) & 0x7ffu);
}

__device__ inline int sturm_below(const double* a, const double* bb, int n, double x) {
  double p0 = 1.0, p1 = a[0] - x;
  int sp = 0;  // sign bit of the previous minor (p_{-1} = 1 > 0)
  int s1 = is_zero(p1) ? 1 - sp : sign_bit(p1);
  int cnt = (s1 != sp) ? 1 : 0;
  sp = s1;
  for (int i = 1; i < n; ++i) {
    double p2 = fma(a[i] - x, p1, -bb[i - 1] * p0);
    const int e2 = exp_bits(p2);
    if (e2 > 1023 + 600) {
      p2 *= 0x1.0p-600;
      p1 *= 0x1.0p-600;
    } else if (e2 < 1023 - 600 && exp_bits(p1) < 1023 - 600) {
      p2 *= 0x1.0p600;
      p1 *= 0x1.0p600;
    }
    const int s2 = is_zero(p2) ? 1 - sp : sign_bit(p2);
    cnt += (s2 != sp) ? 1 : 0;
    sp = s2;
    p0 = p1;
    p1 = p2;
  }
  return cnt;
}

// Lowest eigenpair of the n x n symmetric tridiagonal (a, b) by warp-parallel
// multisection of the Sturm count (32 probes per round), then inverse
// iteration on the positive-definite T - (theta - delta) I by lane 0,
// starting from z when warm (z holds the previous eigenvector, padded with
// zeros, warm_z) or from ones.  When warm, the previous lowest Ritz value th_prev
// (an upper bound: the lowest Ritz value only decreases as the Krylov space
// grows) and its residual r_prev bracket the search, [th_prev - 2 r_prev,
// th_prev], if the Sturm count confirms the lower end; otherwise the
// Gershgorin interval is used.  Called by one full warp; bb (n entries of
// work space after the first kTriMax) and z are written by lane 0 / the warp.
__device__ inline double warp_lowest_eig(const double* a, const double* b, int n, double* z,
                                         double* work, bool warm, bool warm_z, double th_prev,
                                         double r_prev) {
  const int lane = threadIdx.x & 31;
  double* bb = work + 2 * kTriMax;
  for (int i = lane; i < n - 1; i += 32) bb[i] = b[i] * b[i];
  __syncwarp();
  double lo = a[0], hi = a[0];
  for (int i = 0; i < n; ++i) {
    const double r = ((i > 0) ? fabs(b[i - 1]) : 0.0) + ((i < n - 1) ? fabs(b[i]) : 0.0);
    lo = fmin(lo, a[i] - r);
    hi = fmax(hi, a[i] + r);
  }
  const double scale = fmax(fmax(fabs(lo), fabs(hi)), 1e-300);
  if (warm) {
    const double whi = fmin(hi, th_prev + 8.0 * 2.2e-16 * scale);
    const double wlo = fmax(lo, th_prev - fmax(2.0 * r_prev, 1e-9 * scale));
    // lane 0 probes the lower end, lane 1 the upper end
    const double xp = (lane == 0) ? wlo : whi;
    const int c = sturm_below(a, bb, n, xp);
    const int c_lo = __shfl_sync(0xffffffffu, c, 0), c_hi = __shfl_sync(0xffffffffu, c, 1);
    if (c_lo == 0 && c_hi >= 1) {
      lo = wlo;
      hi = whi;
    }
  }
  for (int it = 0; it < 40; ++it) {
    if (hi - lo <= 2.2e-16 * scale) break;
    const double step = (hi - lo) / 33.0;
    const double x = lo + step * double(lane + 1);
    const unsigned bal = __ballot_sync(0xffffffffu, sturm_below(a, bb, n, x) >= 1);
    if (bal) {
      const int L = __ffs(bal) - 1;
      const double nhi = lo + step * double(L + 1);
      const double nlo = (L > 0) ? lo + step * double(L) : lo;
      if (!(nhi < hi) && !(nlo > lo)) break;  // no progress at this precision
      hi = nhi;
      lo = nlo;
    } else {
      const double nlo = lo + step * 32.0;
      if (!(nlo > lo)) break;
      lo = nlo;
    }
  }
  const double theta = 0.5 * (lo + hi);
  // inverse iteration on the positive-definite T - (theta - delta) I: the
  // two triangular sweeps by lane 0 (factorisation merged into the forward
  // sweep, diagonal scaling into the backward one), operands read eight
  // entries ahead; the scaling by the whole warp
  const double shift = theta - 4.0 * 2.2e-16 * scale;
  double* d = work;  // reciprocal pivots
  double* l = work + kTriMax;
  if (!warm_z)
    for (int i = lane; i < n; i += 32) z[i] = 1.0;
  __syncwarp();
  const int reps = warm_z ? 1 : 2;
  for (int rep = 0; rep < reps; ++rep) {
    if (lane == 0) {
      double dprev = 0.0, bprev = 0.0, zprev = 0.0;
      for (int i0 = 0; i0 < n; i0 += 8) {
        double ac[8], bc[8], zc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i0 + u;
          ac[u] = (i < n) ? a[i] : 0.0;
          bc[u] = (i < n - 1) ? b[i] : 0.0;
          zc[u] = (i < n) ? z[i] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i0 + u;
          if (i < n) {
            double piv;
            if (i == 0) {
              piv = ac[u] - shift;
            } else {
              const double li = bprev * dprev;
              l[i - 1] = li;
              piv = (ac[u] - shift) - li * bprev;
              zc[u] = fma(-li, zprev, zc[u]);
            }
            if (piv <= 0.0) piv = 1e-300;
            const double di = 1.0 / piv;
            d[i] = di;
            z[i] = zc[u];
            dprev = di;
            bprev = bc[u];
            zprev = zc[u];
          }
        }
      }
      double znext = 0.0;
      for (int i1 = n - 1; i1 >= 0; i1 -= 8) {
        double zc[8], dc[8], lc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i1 - u;
          zc[u] = (i >= 0) ? z[i] : 0.0;
          dc[u] = (i >= 0) ? d[i] : 0.0;
          lc[u] = (i >= 0 && i < n - 1) ? l[i] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i1 - u;
          if (i >= 0) {
            double t = zc[u] * dc[u];
            if (i < n - 1) t = fma(-lc[u], znext, t);
            z[i] = t;
            znext = t;
          }
        }
      }
    }
    __syncwarp();
    double mx = 0.0;
    for (int i = lane; i < n; i += 32) mx = fmax(mx, fabs(z[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const double inv = 1.0 / mx;
    double nn = 0.0;
    for (int i = lane; i < n; i += 32) {
      const double zi = z[i] * inv;
      z[i] = zi;
      nn = fma(zi, zi, nn);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
    const double in2 = 1.0 / sqrt(nn);
    for (int i = lane; i < n; i += 32) z[i] *= in2;
    __syncwarp();
  }
  const bool neg = z[0] < 0.0;
  __syncwarp();
  if (neg)
    for (int i = lane; i < n; i += 32) z[i] = -z[i];
  __syncwarp();
  return theta;
}

// FP32 counterpart of sturm_below for the mixed path's checks (minors
// rescaled by 2^-60 / 2^60 to stay inside the FP32 range).  The count is
// that of a matrix within a few FP32 ulps of T (Sturm counts by the LDL^T
// recurrence are backward stable), so brackets are reliable to ~1e-6 |T|.
__device__ inline int sturm_below_f(const float* a, const float* bb, int n, float x) {
  float p0 = 1.0f, p1 = a[0] - x;
  int sp = 0;
  int s1 = (p1 == 0.0f) ? 1 - sp : (p1 < 0.0f ? 1 : 0);
  int cnt = (s1 != sp) ? 1 : 0;
  sp = s1;
  for (int i = 1; i < n; ++i) {
    float p2 = fmaf(a[i] - x, p1, -bb[i - 1] * p0);
    if (fabsf(p2) > 0x1.0p60f) {
      p2 *= 0x1.0p-60f;
      p1 *= 0x1.0p-60f;
    } else if (fabsf(p2) < 0x1.0p-60f && fabsf(p1) < 0x1.0p-60f) {
      p2 *= 0x1.0p60f;
      p1 *= 0x1.0p60f;
    }
    const int s2 = (p2 == 0.0f) ? 1 - sp : (p2 < 0.0f ? 1 : 0);
    cnt += (s2 != sp) ? 1 : 0;
    sp = s2;
    p0 = p1;
    p1 = p2;
  }
  return cnt;
}

// Lowest eigenpair for the FP32-mixed path: as warp_lowest_eig, in FP32
// (GB300's FP64 pipe makes a one-warp FP64 recurrence a long latency
// chain).  theta is good to ~1e-6 |T| and z to FP32 accuracy: the FP32
// Krylov basis resolves no more, and the energy returned by the solver is
// the FP64 Rayleigh quotient of the final vector.
__device__ inline double warp_lowest_eig_f32(const double* a64, const double* b64, int n,
                                             double* z, double* work, bool warm, bool warm_z,
                                             double th_prev, double r_prev) {
  const int lane = threadIdx.x & 31;
  float* a = reinterpret_cast<float*>(work);
  float* b = a + kTriMax;
  float* bb = b + kTriMax;
  float* d = bb + kTriMax;
  float* l = d + kTriMax;
  float* zf = l + kTriMax;
  for (int i = lane; i < n; i += 32) {
    a[i] = float(a64[i]);
    const float bi = (i < n - 1) ? float(b64[i]) : 0.0f;
    b[i] = bi;
    bb[i] = bi * bi;
  }
  __syncwarp();
  // Gershgorin bounds: lane i covers rows i, i + 32
  float lo = 3.0e38f, hi = -3.0e38f;
  for (int i = lane; i < n; i += 32) {
    const float r = ((i > 0) ? fabsf(b[i - 1]) : 0.0f) + fabsf(b[i]);
    lo = fminf(lo, a[i] - r);
    hi = fmaxf(hi, a[i] + r);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const float scale = fmaxf(fmaxf(fabsf(lo), fabsf(hi)), 1e-30f);
  lo -= 1e-6f * scale;  // FP32 rounding of the bounds
  hi += 1e-6f * scale;
  if (warm) {
    const float whi = fminf(hi, float(th_prev) + 4e-6f * scale);
    const float wlo = fmaxf(lo, float(th_prev) - fmaxf(2.0f * float(r_prev), 1e-5f * scale));
    const int c = sturm_below_f(a, bb, n, (lane == 0) ? wlo : whi);
    const int c_lo = __shfl_sync(0xffffffffu, c, 0), c_hi = __shfl_sync(0xffffffffu, c, 1);
    if (c_lo == 0 && c_hi >= 1) {
      lo = wlo;
      hi = whi;
    }
  }
  for (int it = 0; it < 24; ++it) {
    if (hi - lo <= 2e-7f * scale) break;
    const float step = (hi - lo) * (1.0f / 33.0f);
    const float x = lo + step * float(lane + 1);
    const unsigned bal = __ballot_sync(0xffffffffu, sturm_below_f(a, bb, n, x) >= 1);
    if (bal) {
      const int L = __ffs(bal) - 1;
      const float nhi = lo + step * float(L + 1);
      const float nlo = (L > 0) ? lo + step * float(L) : lo;
      if (!(nhi < hi) && !(nlo > lo)) break;
      hi = nhi;
      lo = nlo;
    } else {
      const float nlo = lo + step * 32.0f;
      if (!(nlo > lo)) break;
      lo = nlo;
    }
  }
  const float theta = 0.5f * (lo + hi);
  // inverse iteration on T - (theta - delta) I, positive definite: the two
  // triangular sweeps by lane 0 (the factorisation merged into the forward
  // sweep, the diagonal scaling into the backward one), each reading its
  // operands eight entries ahead so that the sweep waits on its arithmetic
  // rather than on shared-memory loads; the scaling by the whole warp
  const float shift = theta - 4e-7f * scale;
  for (int i = lane; i < n; i += 32) zf[i] = warm_z ? float(z[i]) : 1.0f;
  __syncwarp();
  const int reps = warm_z ? 1 : 2;
  for (int rep = 0; rep < reps; ++rep) {
    if (lane == 0) {
      float dprev = 0.0f, bprev = 0.0f, zprev = 0.0f;
      for (int i0 = 0; i0 < n; i0 += 8) {
        float ac[8], bc[8], zc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i0 + u;
          ac[u] = (i < n) ? a[i] : 0.0f;
          bc[u] = (i < n) ? b[i] : 0.0f;
          zc[u] = (i < n) ? zf[i] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i0 + u;
          if (i < n) {
            float piv;
            if (i == 0) {
              piv = ac[u] - shift;
            } else {
              const float li = bprev * dprev;
              l[i - 1] = li;
              piv = (ac[u] - shift) - li * bprev;
              zc[u] = fmaf(-li, zprev, zc[u]);
            }
            if (piv <= 0.0f) piv = 1e-30f;
            const float di = 1.0f / piv;
            d[i] = di;
            zf[i] = zc[u];
            dprev = di;
            bprev = bc[u];
            zprev = zc[u];
          }
        }
      }
      float znext = 0.0f;
      for (int i1 = n - 1; i1 >= 0; i1 -= 8) {
        float zc[8], dc[8], lc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i1 - u;
          zc[u] = (i >= 0) ? zf[i] : 0.0f;
          dc[u] = (i >= 0) ? d[i] : 0.0f;
          lc[u] = (i >= 0 && i < n - 1) ? l[i] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i1 - u;
          if (i >= 0) {
            float t = zc[u] * dc[u];
            if (i < n - 1) t = fmaf(-lc[u], znext, t);
            zf[i] = t;
            znext = t;
          }
        }
      }
    }
    __syncwarp();
    float mx = 0.0f;
    for (int i = lane; i < n; i += 32) mx = fmaxf(mx, fabsf(zf[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const float inv = 1.0f / mx;
    float nn = 0.0f;
    for (int i = lane; i < n; i += 32) {
      const float zi = zf[i] * inv;
      zf[i] = zi;
      nn = fmaf(zi, zi, nn);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
    const float in2 = rsqrtf(nn);
    for (int i = lane; i < n; i += 32) zf[i] *= in2;
    __syncwarp();
  }
  const float sg = (zf[0] < 0.0f) ? -1.0f : 1.0f;
  for (int i = lane; i < n; i += 32) z[i] = double(sg * zf[i]);
  __syncwarp();
  return double(theta);
}

}  // namespace lgt
