// observe.cu -- observables of K states on the GPU (replaces measure_ED,
// finite_ed.jl:369-393, and adds the plaquette expectation).
//
// Every observable is linear in the row probabilities p = |psi(row)|^2 or,
// for the plaquette, in 2 Re conj(psi(W row)) psi(row).  Features per row:
//   f = s            n_f(s)                              s = iy*nx + ix
//   f = ns + s       e_R(ix,iy)^2 [ix<nx-1] + e_U(ix,iy)^2 [iy<ny-1]
//   f = 2 ns + q     plaquette q = iy*(nx-1) + ix: W applicable -> 2 Re(...)
//   f = 2 ns + nP    1 (the norm)
// A block decodes a tile of rows (and ranks the W-neighbours once for all K
// points) into shared memory, then threads (point k, row subgroup) accumulate
// the features in registers.  Per-block partials are summed in a fixed
// order: results are bitwise reproducible.
//
// The per-row feature sums (about 40 per row and point) run in double-float
// arithmetic on the FP32 pipe (lgt_dfloat.cuh) rather than in FP64, which
// GB300 issues at 1/64 of the FP32 rate: amplitudes are split into FP32
// pairs by integer operations, |psi|^2 and the plaquette products formed
// with exact FP32 products, and each feature is a pair (hi, lo) advanced by
// TwoSum with the trailing parts summed apart and renormalised once per
// tile (Ogita, Rump and Oishi's Sum2).  The occupation features add the
// probability of a run of rows with the same fermion mask once per run.
// LGT_DF_REDUCTIONS=0 keeps the FP64 sums (cross-checks).
#include <type_traits>

#include "lgt_dfloat.cuh"
#include "lgt_observe.h"
#include "lgt_rank.cuh"

namespace lgt {

namespace {

constexpr int kT = 256;
constexpr int kFCh = 8;  // features reduced per round (two barriers a round)

// d = hi + lo with hi its leading 24 significant bits (truncated) and lo
// the next 24 (truncated), by integer operations on the bit pattern; |d|
// below the FP32 normal range gives zeros (its square is below 1e-76), lo
// below that range gives lo = 0.  Relative error at most 2^-47.
__device__ __forceinline__ df split_df(double d) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(d));
  const uint32_t uh = uint32_t(u >> 32), ul = uint32_t(u);
  const uint32_t sign = uh & 0x80000000u;
  const int e = int((uh >> 20) & 0x7ffu);
  const int e32 = e - 896;  // FP32 biased exponent of the leading bit
  if (e32 <= 0 || e32 >= 255) return df{0.f, 0.f};
  const uint32_t hm = ((uh & 0xfffffu) << 3) | (ul >> 29);
  const float hi = __uint_as_float(sign | (uint32_t(e32) << 23) | hm);
  const uint32_t rem = ul & 0x1fffffffu;  // value rem * 2^(e - 1075)
  float lo = 0.f;
  if (rem != 0u) {
    const int lz = __clz(int(rem));  // >= 3
    const int el = (31 - lz) + e - 948;  // biased exponent of rem's leading bit
    if (el > 0) lo = __uint_as_float(sign | (uint32_t(el) << 23) | ((rem << (lz + 1)) >> 9));
  }
  return df{hi, lo};
}

// acc += (xh + xl): TwoSum of the leading parts, trailing parts summed
// apart (renormalised by df_renorm once per tile).
__device__ __forceinline__ void df_add_lite(df& acc, float xh, float xl) {
  float s, t;
  two_sum(acc.hi, xh, s, t);
  acc.hi = s;
  acc.lo = df_add_rn(acc.lo, df_add_rn(t, xl));
}

__device__ __forceinline__ void df_renorm(df& acc) { fast_two_sum(acc.hi, acc.lo, acc.hi, acc.lo); }

// A small non-negative integer as FP32 (exact below 2^23), without a
// conversion instruction.
__device__ __forceinline__ float small_int_f(uint32_t w) {
  return df_sub_rn(__uint_as_float(0x4B000000u | w), 8388608.f);
}

// Features of one block's rows with the accumulators in registers: MS sites
// and MP plaquettes at most (compile time), so every accumulator index is a
// constant.  Accumulator slots: [0, MS) occupation per site, [MS, 2 MS) E^2
// per site, [2 MS, 2 MS + MP) plaquettes, 2 MS + MP the norm; slot s is
// feature obs_slot_feature(s) (negative: unused at this lattice).
__device__ __forceinline__ int obs_slot_feature(int s, int MS, int MP, int ns, int nP) {
  if (s < MS) return s < ns ? s : -1;
  if (s < 2 * MS) return (s - MS) < ns ? ns + (s - MS) : -1;
  if (s < 2 * MS + MP) return (s - 2 * MS) < nP ? 2 * ns + (s - 2 * MS) : -1;
  return 2 * ns + nP;
}

template <typename T, int NC, int MS, int MP, bool DF>
__global__ void __launch_bounds__(kT) k_observe(Geom G, RankView R, const T* __restrict__ x,
                                                int64_t N, int K, int nfeat, int64_t rpb,
                                                double* part, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* s_binom = reinterpret_cast<uint32_t*>(smem);               // 32*33
  uint32_t* s_mask = s_binom + 32 * 33;                                // kT
  uint8_t* s_e2 = reinterpret_cast<uint8_t*>(s_mask + kT);             // kT * ns
  int32_t* s_nb = reinterpret_cast<int32_t*>(s_e2 + ((kT * G.ns + 15) / 16) * 16);  // kT * nP
  for (int i = threadIdx.x; i < 32 * 33; i += kT) s_binom[i] = R.binom[i];

  constexpr int NSLOT = 2 * MS + MP + 1;
  using A = typename std::conditional<DF, df, double>::type;
  const int C = K * NC;
  const int RS = kT / K;  // row subgroups
  const int k = threadIdx.x % K, rs = threadIdx.x / K;
  const bool worker = rs < RS;
  const int ns = G.ns, nP = G.nP;
  A acc_n[MS], acc_e[MS], acc_p[MP], acc_norm;
  auto zero = [](A& a) {
    if constexpr (DF) a = df{0.f, 0.f};
    else a = 0.0;
  };
#pragma unroll
  for (int i = 0; i < MS; ++i) {
    zero(acc_n[i]);
    zero(acc_e[i]);
  }
#pragma unroll
  for (int i = 0; i < MP; ++i) zero(acc_p[i]);
  zero(acc_norm);
  // DF: probability of the current run of rows with one fermion mask, added
  // to the occupations of the mask's sites when the run ends
  df seg{0.f, 0.f};
  uint32_t seg_mask = 0u;

  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int64_t r1 = (r0 + rpb < N) ? r0 + rpb : N;
  for (int64_t t0 = r0; t0 < r1; t0 += kT) {
    __syncthreads();
    {  // phase 1: one thread per row of the tile
      const int64_t row = t0 + threadIdx.x;
      if (row < r1) {
        const Config c = decode(G, __ldg(R.keys + row));
        s_mask[threadIdx.x] = c.mask;
        for (int iy = 0; iy < G.ny; ++iy)
          for (int ix = 0; ix < G.nx; ++ix) {
            int e2 = 0;
            if (ix < G.nx - 1) {
              const int e = get_eR(G, c.rpack, iy * (G.nx - 1) + ix);
              e2 += e * e;
            }
            if (iy < G.ny - 1) {
              const int e = get_eU(G, c.digits, iy * G.nx + ix);
              e2 += e * e;
            }
            s_e2[threadIdx.x * G.ns + iy * G.nx + ix] = uint8_t(e2);
          }
        for (int iy = 0; iy < G.ny - 1; ++iy)
          for (int ix = 0; ix < G.nx - 1; ++ix) {
            const int q = iy * (G.nx - 1) + ix;
            const int rb = q, rt = q + (G.nx - 1);
            const int jl = iy * G.nx + ix, jr = jl + 1;
            const int eb = get_eR(G, c.rpack, rb), et = get_eR(G, c.rpack, rt);
            const int el = get_eU(G, c.digits, jl), er = get_eU(G, c.digits, jr);
            int32_t j = -1;
            if (eb > -G.dg && el < G.dg && er > -G.dg && et < G.dg) {
              const uint64_t nk =
                  make_key(G, c.mask, c.digits + digit_unit(G, jl) - digit_unit(G, jr));
              const int64_t jj = rank_key(R, R.segc, s_binom, nk);
              if (jj < 0) raise_err(err, kDevErrRank);
              j = int32_t(jj);
            }
            s_nb[threadIdx.x * G.nP + q] = j;
          }
      }
    }
    __syncthreads();
    if (!worker) continue;
    const int rows = int((r1 - t0 < kT) ? (r1 - t0) : kT);
    for (int rl = rs; rl < rows; rl += RS) {
      const int64_t row = t0 + rl;
      const T* xr = x + size_t(row) * C + k * NC;
      const uint32_t mask = s_mask[rl];
      if constexpr (DF) {
        df a0, a1{0.f, 0.f};
        if constexpr (sizeof(T) == 8) {
          a0 = split_df(double(xr[0]));
          if (NC == 2) a1 = split_df(double(xr[1]));
        } else {
          a0 = df{float(xr[0]), 0.f};
          if (NC == 2) a1 = df{float(xr[1]), 0.f};
        }
        // p = |a|^2: the leading squares exactly, the cross terms rounded
        float ph, pl;
        two_prod(a0.hi, a0.hi, ph, pl);
        pl = df_fma_rn(df_add_rn(a0.hi, a0.hi), a0.lo, pl);
        if (NC == 2) {
          float q, qe, t;
          two_prod(a1.hi, a1.hi, q, qe);
          qe = df_fma_rn(df_add_rn(a1.hi, a1.hi), a1.lo, qe);
          two_sum(ph, q, ph, t);
          pl = df_add_rn(pl, df_add_rn(qe, t));
        }
        fast_two_sum(ph, pl, ph, pl);
        if (mask != seg_mask) {
#pragma unroll
          for (int i = 0; i < MS; ++i)
            if (i < ns && ((seg_mask >> i) & 1u)) df_add_lite(acc_n[i], seg.hi, seg.lo);
          seg = df{0.f, 0.f};
          seg_mask = mask;
        }
        df_add_lite(seg, ph, pl);
        df_add_lite(acc_norm, ph, pl);
#pragma unroll
        for (int i = 0; i < MS; ++i)
          if (i < ns) {
            const float wv = small_int_f(s_e2[rl * ns + i]);
            float qh, qe;
            two_prod(wv, ph, qh, qe);
            qe = df_fma_rn(wv, pl, qe);
            df_add_lite(acc_e[i], qh, qe);
          }
#pragma unroll
        for (int q = 0; q < MP; ++q)
          if (q < nP) {
            const int32_t j = s_nb[rl * nP + q];
            if (j >= 0) {
              const T* xj = x + size_t(j) * C + k * NC;
              df b0, b1{0.f, 0.f};
              if constexpr (sizeof(T) == 8) {
                b0 = split_df(double(xj[0]));
                if (NC == 2) b1 = split_df(double(xj[1]));
              } else {
                b0 = df{float(xj[0]), 0.f};
                if (NC == 2) b1 = df{float(xj[1]), 0.f};
              }
              // 2 Re conj(b) a = 2 (b0 a0 + b1 a1)
              float vh, ve;
              two_prod(b0.hi, a0.hi, vh, ve);
              ve = df_fma_rn(b0.hi, a0.lo, df_fma_rn(b0.lo, a0.hi, ve));
              if (NC == 2) {
                float q2, qe, t;
                two_prod(b1.hi, a1.hi, q2, qe);
                qe = df_fma_rn(b1.hi, a1.lo, df_fma_rn(b1.lo, a1.hi, qe));
                two_sum(vh, q2, vh, t);
                ve = df_add_rn(ve, df_add_rn(qe, t));
              }
              df_add_lite(acc_p[q], df_add_rn(vh, vh), df_add_rn(ve, ve));
            }
          }
      } else {
        const double a0 = double(xr[0]);
        const double a1 = (NC == 2) ? double(xr[1]) : 0.0;
        const double p = a0 * a0 + a1 * a1;
        acc_norm += p;
#pragma unroll
        for (int i = 0; i < MS; ++i)
          if (i < ns) {
            if ((mask >> i) & 1u) acc_n[i] += p;
            acc_e[i] = fma(p, double(s_e2[rl * ns + i]), acc_e[i]);
          }
#pragma unroll
        for (int q = 0; q < MP; ++q)
          if (q < nP) {
            const int32_t j = s_nb[rl * nP + q];
            if (j >= 0) {
              const T* xj = x + size_t(j) * C + k * NC;
              double v = double(xj[0]) * a0;
              if (NC == 2) v += double(xj[1]) * a1;
              acc_p[q] += 2.0 * v;
            }
          }
      }
    }
    if constexpr (DF) {  // the trailing parts renormalised once per tile
#pragma unroll
      for (int i = 0; i < MS; ++i) {
        df_renorm(acc_n[i]);
        df_renorm(acc_e[i]);
      }
#pragma unroll
      for (int q = 0; q < MP; ++q) df_renorm(acc_p[q]);
      df_renorm(acc_norm);
      df_renorm(seg);
    }
  }
  if constexpr (DF) {
    if (worker) {
#pragma unroll
      for (int i = 0; i < MS; ++i)
        if (i < ns && ((seg_mask >> i) & 1u)) df_add_lite(acc_n[i], seg.hi, seg.lo);
    }
  }
  auto val = [](const A& a) -> double {
    if constexpr (DF) return widen(a.hi) + widen(a.lo);
    else return a;
  };
  // slot s's accumulator (s a constant after unrolling)
  auto slot = [&](int sl) -> double {
#pragma unroll
    for (int i = 0; i < MS; ++i) {
      if (sl == i) return val(acc_n[i]);
      if (sl == MS + i) return val(acc_e[i]);
    }
#pragma unroll
    for (int q = 0; q < MP; ++q)
      if (sl == 2 * MS + q) return val(acc_p[q]);
    return val(acc_norm);
  };
  // reduce the row subgroups, kFCh slots a round: red[q][thread], then
  // thread (q, k) adds subgroups g = 0 .. RS-1 in order for slot s0 + q
  __syncthreads();
  double* red = reinterpret_cast<double*>(smem);
#pragma unroll
  for (int s0 = 0; s0 < NSLOT; s0 += kFCh) {
#pragma unroll
    for (int q = 0; q < kFCh; ++q)
      red[q * kT + threadIdx.x] = (worker && s0 + q < NSLOT) ? slot(s0 + q) : 0.0;
    __syncthreads();
    for (int t = threadIdx.x; t < kFCh * K; t += kT) {
      const int q = t / K, kk = t - q * K;
      const int f = (s0 + q < NSLOT) ? obs_slot_feature(s0 + q, MS, MP, ns, nP) : -1;
      if (f >= 0) {
        double sum = 0.0;
        for (int g = 0; g < RS; ++g) sum += red[q * kT + g * K + kk];
        part[(size_t(blockIdx.x) * K + kk) * nfeat + f] = sum;
      }
    }
    __syncthreads();
  }
}

// Any lattice up to 96 features: the accumulators indexed at run time (FP64,
// or double-float pairs).
template <typename T, int NC, int MAXF, bool DF>
__global__ void __launch_bounds__(kT) k_observe_generic(Geom G, RankView R, const T* __restrict__ x,
                                                int64_t N, int K, int nfeat, int64_t rpb,
                                                double* part, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* s_binom = reinterpret_cast<uint32_t*>(smem);               // 32*33
  uint32_t* s_mask = s_binom + 32 * 33;                                // kT
  uint8_t* s_e2 = reinterpret_cast<uint8_t*>(s_mask + kT);             // kT * ns
  int32_t* s_nb = reinterpret_cast<int32_t*>(s_e2 + ((kT * G.ns + 15) / 16) * 16);  // kT * nP
  for (int i = threadIdx.x; i < 32 * 33; i += kT) s_binom[i] = R.binom[i];

  const int C = K * NC;
  const int RS = kT / K;  // row subgroups
  const int k = threadIdx.x % K, rs = threadIdx.x / K;
  const bool worker = rs < RS;
  double acc[DF ? 1 : MAXF];
  df dacc[DF ? MAXF : 1];
  df seg{0.f, 0.f};          // probability of the current run of rows with one mask (DF)
  uint32_t seg_mask = 0u;
#pragma unroll
  for (int f = 0; f < (DF ? 1 : MAXF); ++f) acc[f] = 0.0;
#pragma unroll
  for (int f = 0; f < (DF ? MAXF : 1); ++f) dacc[f] = df{0.f, 0.f};
  // the run's probability into the occupation features of its mask's sites
  auto flush_seg = [&]() {
#pragma unroll
    for (int f = 0; f < MAXF; ++f)
      if (f < G.ns && ((seg_mask >> f) & 1u)) df_add_lite(dacc[f], seg.hi, seg.lo);
    seg = df{0.f, 0.f};
  };

  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int64_t r1 = (r0 + rpb < N) ? r0 + rpb : N;
  for (int64_t t0 = r0; t0 < r1; t0 += kT) {
    __syncthreads();
    {  // phase 1: one thread per row of the tile
      const int64_t row = t0 + threadIdx.x;
      if (row < r1) {
        const Config c = decode(G, __ldg(R.keys + row));
        s_mask[threadIdx.x] = c.mask;
        for (int iy = 0; iy < G.ny; ++iy)
          for (int ix = 0; ix < G.nx; ++ix) {
            int e2 = 0;
            if (ix < G.nx - 1) {
              const int e = get_eR(G, c.rpack, iy * (G.nx - 1) + ix);
              e2 += e * e;
            }
            if (iy < G.ny - 1) {
              const int e = get_eU(G, c.digits, iy * G.nx + ix);
              e2 += e * e;
            }
            s_e2[threadIdx.x * G.ns + iy * G.nx + ix] = uint8_t(e2);
          }
        for (int iy = 0; iy < G.ny - 1; ++iy)
          for (int ix = 0; ix < G.nx - 1; ++ix) {
            const int q = iy * (G.nx - 1) + ix;
            const int rb = q, rt = q + (G.nx - 1);
            const int jl = iy * G.nx + ix, jr = jl + 1;
            const int eb = get_eR(G, c.rpack, rb), et = get_eR(G, c.rpack, rt);
            const int el = get_eU(G, c.digits, jl), er = get_eU(G, c.digits, jr);
            int32_t j = -1;
            if (eb > -G.dg && el < G.dg && er > -G.dg && et < G.dg) {
              const uint64_t nk =
                  make_key(G, c.mask, c.digits + digit_unit(G, jl) - digit_unit(G, jr));
              const int64_t jj = rank_key(R, R.segc, s_binom, nk);
              if (jj < 0) raise_err(err, kDevErrRank);
              j = int32_t(jj);
            }
            s_nb[threadIdx.x * G.nP + q] = j;
          }
      }
    }
    __syncthreads();
    if (!worker) continue;
    const int rows = int((r1 - t0 < kT) ? (r1 - t0) : kT);
    if constexpr (DF) {
      for (int rl = rs; rl < rows; rl += RS) {
        const int64_t row = t0 + rl;
        const T* xr = x + size_t(row) * C + k * NC;
        df a0, a1{0.f, 0.f};
        if constexpr (sizeof(T) == 8) {
          a0 = split_df(double(xr[0]));
          if (NC == 2) a1 = split_df(double(xr[1]));
        } else {
          a0 = df{float(xr[0]), 0.f};
          if (NC == 2) a1 = df{float(xr[1]), 0.f};
        }
        // p = |a|^2: the leading squares exactly, the cross terms rounded
        float ph, pl;
        two_prod(a0.hi, a0.hi, ph, pl);
        pl = df_fma_rn(df_add_rn(a0.hi, a0.hi), a0.lo, pl);
        if (NC == 2) {
          float q, qe, t;
          two_prod(a1.hi, a1.hi, q, qe);
          qe = df_fma_rn(df_add_rn(a1.hi, a1.hi), a1.lo, qe);
          two_sum(ph, q, ph, t);
          pl = df_add_rn(pl, df_add_rn(qe, t));
        }
        fast_two_sum(ph, pl, ph, pl);
        const uint32_t mask = s_mask[rl];
        if (mask != seg_mask) {
          flush_seg();
          seg_mask = mask;
        }
        df_add_lite(seg, ph, pl);
#pragma unroll
        for (int f = 0; f < MAXF; ++f) {
          if (f < G.ns) {
            // occupations: through the run sum
          } else if (f < 2 * G.ns) {
            const float wv = small_int_f(s_e2[rl * G.ns + (f - G.ns)]);
            float qh, qe;
            two_prod(wv, ph, qh, qe);
            qe = df_fma_rn(wv, pl, qe);
            df_add_lite(dacc[f], qh, qe);
          } else if (f < 2 * G.ns + G.nP) {
            const int32_t j = s_nb[rl * G.nP + (f - 2 * G.ns)];
            if (j >= 0) {
              const T* xj = x + size_t(j) * C + k * NC;
              df b0, b1{0.f, 0.f};
              if constexpr (sizeof(T) == 8) {
                b0 = split_df(double(xj[0]));
                if (NC == 2) b1 = split_df(double(xj[1]));
              } else {
                b0 = df{float(xj[0]), 0.f};
                if (NC == 2) b1 = df{float(xj[1]), 0.f};
              }
              // 2 Re conj(b) a = 2 (b0 a0 + b1 a1)
              float vh, ve;
              two_prod(b0.hi, a0.hi, vh, ve);
              ve = df_fma_rn(b0.hi, a0.lo, df_fma_rn(b0.lo, a0.hi, ve));
              if (NC == 2) {
                float q, qe, t;
                two_prod(b1.hi, a1.hi, q, qe);
                qe = df_fma_rn(b1.hi, a1.lo, df_fma_rn(b1.lo, a1.hi, qe));
                two_sum(vh, q, vh, t);
                ve = df_add_rn(ve, df_add_rn(qe, t));
              }
              df_add_lite(dacc[f], df_add_rn(vh, vh), df_add_rn(ve, ve));
            }
          } else if (f == nfeat - 1) {
            df_add_lite(dacc[f], ph, pl);
          }
        }
      }
#pragma unroll
      for (int f = 0; f < MAXF; ++f) df_renorm(dacc[f]);
      df_renorm(seg);
    } else {
    for (int rl = rs; rl < rows; rl += RS) {
      const int64_t row = t0 + rl;
      const T* xr = x + size_t(row) * C + k * NC;
      const double a0 = double(xr[0]);
      const double a1 = (NC == 2) ? double(xr[1]) : 0.0;
      const double p = a0 * a0 + a1 * a1;
      const uint32_t mask = s_mask[rl];
#pragma unroll
      for (int f = 0; f < MAXF; ++f) {
        if (f < G.ns) {
          if ((mask >> f) & 1u) acc[f] += p;
        } else if (f < 2 * G.ns) {
          acc[f] = fma(p, double(s_e2[rl * G.ns + (f - G.ns)]), acc[f]);
        } else if (f < 2 * G.ns + G.nP) {
          const int32_t j = s_nb[rl * G.nP + (f - 2 * G.ns)];
          if (j >= 0) {
            const T* xj = x + size_t(j) * C + k * NC;
            double v = double(xj[0]) * a0;
            if (NC == 2) v += double(xj[1]) * a1;
            acc[f] += 2.0 * v;
          }
        } else if (f == nfeat - 1) {
          acc[f] += p;
        }
      }
    }
    }
  }
  if constexpr (DF) {
    if (worker) flush_seg();
  }
  // reduce the row subgroups, kFCh features a round: red[q][thread], then
  // thread (q, k) adds subgroups g = 0 .. RS-1 in order for feature f0 + q
  __syncthreads();
  double* red = reinterpret_cast<double*>(smem);
#pragma unroll
  for (int f0 = 0; f0 < MAXF; f0 += kFCh) {
    if (f0 < nfeat) {
#pragma unroll
      for (int q = 0; q < kFCh; ++q) {
        double v = 0.0;
        if (worker && f0 + q < nfeat) {
          if constexpr (DF) v = widen(dacc[f0 + q].hi) + widen(dacc[f0 + q].lo);
          else v = acc[f0 + q];
        }
        red[q * kT + threadIdx.x] = v;
      }
      __syncthreads();
      for (int t = threadIdx.x; t < kFCh * K; t += kT) {
        const int q = t / K, kk = t - q * K;
        if (f0 + q < nfeat) {
          double s = 0.0;
          for (int g = 0; g < RS; ++g) s += red[q * kT + g * K + kk];
          part[(size_t(blockIdx.x) * K + kk) * nfeat + f0 + q] = s;
        }
      }
      __syncthreads();
    }
  }
}

// Sum of the per-block partials, one warp per output (lane l adds blocks
// l, l + 32, ..., then a fixed shuffle tree): a fixed order, and no single
// thread waiting on one dependent load per block.
__global__ void k_observe_finish(const double* part, int nblk, int K, int nfeat, double* out) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (t >= K * nfeat) return;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += part[size_t(b) * K * nfeat + t];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[t] = s;
}

inline unsigned finish_blocks(int outputs) { return unsigned((outputs + 3) / 4); }  // 4 warps

template <typename T, int NC, int MAXF, bool DF>
cudaError_t launch_obs_generic(const Geom& G, const RankView& R, const T* x, int K, int nfeat, int nblk,
                        int64_t rpb, double* part, int* err, cudaStream_t s) {
  const size_t sh0 = 32 * 33 * 4 + kT * 4 + size_t((kT * G.ns + 15) / 16) * 16 +
                     size_t(kT) * (G.nP > 0 ? G.nP : 1) * 4;
  const size_t shr = size_t(kFCh) * kT * sizeof(double);  // the reduction's rounds
  const size_t sh = sh0 > shr ? sh0 : shr;
  auto kern = k_observe_generic<T, NC, MAXF, DF>;
  {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), int(sh));
    if (e != cudaSuccess) return e;
  }
  kern<<<nblk, kT, sh, s>>>(G, R, x, R.dim, K, nfeat, rpb, part, err), lgt::note_launch();
  return cudaGetLastError();
}

inline size_t obs_smem(const Geom& G) {
  const size_t sh0 = 32 * 33 * 4 + kT * 4 + size_t((kT * G.ns + 15) / 16) * 16 +
                     size_t(kT) * (G.nP > 0 ? G.nP : 1) * 4;
  const size_t shr = size_t(kFCh) * kT * sizeof(double);  // the reduction's rounds
  return sh0 > shr ? sh0 : shr;
}

template <typename T, int NC, int MS, int MP, bool DF>
cudaError_t launch_obs_fixed(const Geom& G, const RankView& R, const T* x, int K, int nfeat,
                             int nblk, int64_t rpb, double* part, int* err, cudaStream_t s) {
  const size_t sh = obs_smem(G);
  auto kern = k_observe<T, NC, MS, MP, DF>;
  {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), int(sh));
    if (e != cudaSuccess) return e;
  }
  kern<<<nblk, kT, sh, s>>>(G, R, x, R.dim, K, nfeat, rpb, part, err), lgt::note_launch();
  return cudaGetLastError();
}

template <typename T, int NC, bool DF>
cudaError_t launch_obs_df(const Geom& G, const RankView& R, const T* x, int K, int nfeat,
                          int nblk, int64_t rpb, double* part, int* err, cudaStream_t s) {
  // register-resident accumulators for lattices up to 16 sites and 9
  // plaquettes (4x4), run-time indexed ones beyond
  if (G.ns <= 8 && G.nP <= 4)
    return launch_obs_fixed<T, NC, 8, 4, DF>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  if (G.ns <= 12 && G.nP <= 6)
    return launch_obs_fixed<T, NC, 12, 6, DF>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  if (G.ns <= 16 && G.nP <= 9)
    return launch_obs_fixed<T, NC, 16, 9, DF>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  if (nfeat <= 24) return launch_obs_generic<T, NC, 24, false>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  if (nfeat <= 48) return launch_obs_generic<T, NC, 48, false>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  return launch_obs_generic<T, NC, 96, false>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
}

template <typename T, int NC>
cudaError_t launch_obs2(const Geom& G, const RankView& R, const T* x, int K, int nfeat, int nblk,
                        int64_t rpb, double* part, int* err, cudaStream_t s) {
  // double-float feature sums, or FP64 with LGT_DF_REDUCTIONS=0
  return df_reductions_enabled()
             ? launch_obs_df<T, NC, true>(G, R, x, K, nfeat, nblk, rpb, part, err, s)
             : launch_obs_df<T, NC, false>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
}

}  // namespace

int observe_nfeat(const Geom& G) { return 2 * G.ns + G.nP + 1; }

void observe_plan(int64_t N, int* nblk, int64_t* rpb) {
  // at least 4 rows per block (a K = 64 batch of N = 645 spreads over 162
  // blocks: the per-row FP64 feature sums are the work), at most four
  // blocks per SM
  int64_t want = (N + 3) / 4;
  if (want > 152 * 4) want = 152 * 4;
  if (want < 1) want = 1;
  int64_t r = (N + want - 1) / want;
  *rpb = r < 1 ? 1 : r;
  *nblk = int((N + *rpb - 1) / *rpb);
  if (*nblk < 1) *nblk = 1;
}

template <typename T>
cudaError_t launch_observe(const Geom& G, const RankView& R, const T* x, int K, int ncomp,
                           double* part, double* out, int* err, cudaStream_t s) {
  if (K > kT) return cudaErrorInvalidValue;
  const int nfeat = observe_nfeat(G);
  if (nfeat > 96) return cudaErrorInvalidValue;
  int nblk;
  int64_t rpb;
  observe_plan(R.dim, &nblk, &rpb);
  cudaError_t e = (ncomp == 1)
                      ? launch_obs2<T, 1>(G, R, x, K, nfeat, nblk, rpb, part, err, s)
                      : launch_obs2<T, 2>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  if (e != cudaSuccess) return e;
  k_observe_finish<<<finish_blocks(K * nfeat), 128, 0, s>>>(part, nblk, K, nfeat, out), lgt::note_launch();
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_observe_planned(const Geom& G, const RankView& R, const T* x, int K, int ncomp,
                                   int nblk, int64_t rpb, double* part, double* out, int* err,
                                   cudaStream_t s) {
  if (K > kT || nblk < 1 || rpb < 1) return cudaErrorInvalidValue;
  const int nfeat = observe_nfeat(G);
  if (nfeat > 96) return cudaErrorInvalidValue;
  cudaError_t e = (ncomp == 1)
                      ? launch_obs2<T, 1>(G, R, x, K, nfeat, nblk, rpb, part, err, s)
                      : launch_obs2<T, 2>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  if (e != cudaSuccess) return e;
  k_observe_finish<<<finish_blocks(K * nfeat), 128, 0, s>>>(part, nblk, K, nfeat, out), lgt::note_launch();
  return cudaGetLastError();
}

template cudaError_t launch_observe_planned<double>(const Geom&, const RankView&, const double*,
                                                    int, int, int, int64_t, double*, double*, int*,
                                                    cudaStream_t);
template cudaError_t launch_observe_planned<float>(const Geom&, const RankView&, const float*, int,
                                                   int, int, int64_t, double*, double*, int*,
                                                   cudaStream_t);

template cudaError_t launch_observe<double>(const Geom&, const RankView&, const double*, int, int,
                                            double*, double*, int*, cudaStream_t);
template cudaError_t launch_observe<float>(const Geom&, const RankView&, const float*, int, int,
                                           double*, double*, int*, cudaStream_t);

}  // namespace lgt
