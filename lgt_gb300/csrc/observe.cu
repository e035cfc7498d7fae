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
#include "lgt_observe.h"
#include "lgt_rank.cuh"

namespace lgt {

namespace {

constexpr int kT = 256;
constexpr int kFCh = 8;  // features reduced per round (two barriers a round)

template <typename T, int NC, int MAXF>
__global__ void __launch_bounds__(kT) k_observe(Geom G, RankView R, const T* __restrict__ x,
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
  double acc[MAXF];
#pragma unroll
  for (int f = 0; f < MAXF; ++f) acc[f] = 0.0;

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
  // reduce the row subgroups, kFCh features a round: red[q][thread], then
  // thread (q, k) adds subgroups g = 0 .. RS-1 in order for feature f0 + q
  __syncthreads();
  double* red = reinterpret_cast<double*>(smem);
#pragma unroll
  for (int f0 = 0; f0 < MAXF; f0 += kFCh) {
    if (f0 < nfeat) {
#pragma unroll
      for (int q = 0; q < kFCh; ++q)
        red[q * kT + threadIdx.x] = (worker && f0 + q < nfeat) ? acc[f0 + q] : 0.0;
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

template <typename T, int NC, int MAXF>
cudaError_t launch_obs3(const Geom& G, const RankView& R, const T* x, int K, int nfeat, int nblk,
                        int64_t rpb, double* part, int* err, cudaStream_t s) {
  const size_t sh0 = 32 * 33 * 4 + kT * 4 + size_t((kT * G.ns + 15) / 16) * 16 +
                     size_t(kT) * (G.nP > 0 ? G.nP : 1) * 4;
  const size_t shr = size_t(kFCh) * kT * sizeof(double);  // the reduction's rounds
  const size_t sh = sh0 > shr ? sh0 : shr;
  auto kern = k_observe<T, NC, MAXF>;
  {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), int(sh));
    if (e != cudaSuccess) return e;
  }
  kern<<<nblk, kT, sh, s>>>(G, R, x, R.dim, K, nfeat, rpb, part, err), lgt::note_launch();
  return cudaGetLastError();
}

template <typename T, int NC>
cudaError_t launch_obs2(const Geom& G, const RankView& R, const T* x, int K, int nfeat, int nblk,
                        int64_t rpb, double* part, int* err, cudaStream_t s) {
  if (nfeat <= 24) return launch_obs3<T, NC, 24>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  if (nfeat <= 48) return launch_obs3<T, NC, 48>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
  return launch_obs3<T, NC, 96>(G, R, x, K, nfeat, nblk, rpb, part, err, s);
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
