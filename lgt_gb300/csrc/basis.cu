// basis.cu -- Gauss-law basis enumeration on the GPU (replaces build_basis and
// its recursion, finite_ed.jl:125-232) and the ranking tables.
//
// Enumeration is an ordered stream compaction over a flat candidate space.
// Candidate c = (mask rank mi, free-digit string f):
//   * mi runs over the fermion masks with N_f = -sum(g) set bits in ascending
//     order (finite_ed.jl:138-139);
//   * f runs over the e_U values of every row except the last column of each
//     row, first link most significant, each digit ascending from -dg
//     (finite_ed.jl:183-200).  The last e_U of row iy is fixed by the row sum
//     S[iy] (finite_ed.jl:146-152,186-191); e_R follows by horizontal Gauss
//     propagation and must stay in [-dg, dg] (finite_ed.jl:202-225).
// Candidate order equals the reference's discovery order, so compacting the
// valid candidates IN ORDER (warp ballot inside a warp, block prefix over the
// warps, device-wide exclusive scan over blocks) emits the order keys already
// sorted.  No sort and no hash table are needed.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "lgt_internal.h"
#include "lgt_rank.cuh"

namespace lgt {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;                       // candidates per thread per block
constexpr int kTile = kThreads * kItems;         // candidates per block

__host__ __device__ inline uint64_t ipow(uint64_t b, int e) {
  uint64_t r = 1;
  while (e-- > 0) r *= b;
  return r;
}

// Fermion masks with the sector's particle number.
struct MaskPred {
  int nf_target;
  uint64_t total;  // 2^ns
  __device__ bool operator()(uint64_t idx, uint64_t* val) const {
    *val = idx;
    return __popcll(idx) == nf_target;
  }
};

// Candidate (mask rank, free e_U string) -> order key when the state is valid.
template <int DG>
struct CandPred {
  Geom G;
  const uint32_t* masks;
  uint64_t nfree;     // (2dg+1)^F candidate strings per mask
  uint64_t total;     // nmasks * nfree
  __device__ bool operator()(uint64_t idx, uint64_t* val) const {
    constexpr int B = 2 * DG + 1;
    const uint64_t mi = idx / nfree;
    uint64_t f = idx - mi * nfree;
    const uint32_t mask = masks[mi];
    // Row sums S[iy] = sum_{j<=iy} R[j], R[j] = sum_ix (n_f + g) on row j
    // (finite_ed.jl:146-152); S[ny-1] = 0, so S[iy] = S[iy+1] - R[iy+1].
    // Free digits are peeled off f from the least significant end, i.e. from
    // the last e_U row backwards, and placed at their key positions.
    uint64_t digits = 0;
    int S = 0;
    const uint32_t rowmask = (G.nx >= 32) ? 0xffffffffu : ((1u << G.nx) - 1u);
#pragma unroll 1
    for (int iy = G.ny - 2; iy >= 0; --iy) {
      const uint32_t rowbits = (mask >> ((iy + 1) * G.nx)) & rowmask;
      S -= __popc(rowbits) + G.grow[iy + 1];
      int partial = 0;
#pragma unroll 1
      for (int ix = G.nx - 2; ix >= 0; --ix) {
        const uint64_t q = f / B;
        const int v = int(f - q * B) - DG;
        f = q;
        partial += v;
        digits |= uint64_t(v + DG) * digit_unit(G, iy * G.nx + ix);
      }
      const int last = S - partial;
      if (last < -DG || last > DG) return false;
      digits |= uint64_t(last + DG) * digit_unit(G, iy * G.nx + G.nx - 1);
    }
    uint64_t rp;
    if (!derive_eR(G, mask, digits, &rp)) return false;
    *val = make_key(G, mask, digits);
    return true;
  }
};

template <class Pred>
__global__ void __launch_bounds__(kThreads) k_compact_count(Pred p, uint32_t* block_counts) {
  __shared__ uint32_t warp_tot[kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t base = uint64_t(blockIdx.x) * kTile;
  uint32_t cnt = 0;
#pragma unroll 1
  for (int it = 0; it < kItems; ++it) {
    const uint64_t idx = base + uint64_t(it) * kThreads + threadIdx.x;
    uint64_t v;
    bool ok = idx < p.total && p(idx, &v);
    cnt += __popc(__ballot_sync(0xffffffffu, ok));
  }
  if (lane == 0) warp_tot[wid] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w = 0; w < kThreads / 32; ++w) s += warp_tot[w];
    block_counts[blockIdx.x] = s;
  }
}

template <class Pred, class Out>
__global__ void __launch_bounds__(kThreads) k_compact_write(Pred p, const uint64_t* block_off,
                                                            Out* out, uint64_t cap, int* err) {
  __shared__ uint32_t warp_cnt[kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t base = uint64_t(blockIdx.x) * kTile;
  uint64_t running = block_off[blockIdx.x];
#pragma unroll 1
  for (int it = 0; it < kItems; ++it) {
    const uint64_t idx = base + uint64_t(it) * kThreads + threadIdx.x;
    uint64_t v = 0;
    bool ok = idx < p.total && p(idx, &v);
    const uint32_t bal = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) warp_cnt[wid] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      uint32_t c = warp_cnt[w];
      before += (w < wid) ? c : 0u;
      total += c;
    }
    if (ok) {
      const uint64_t at = running + before + __popc(bal & ((1u << lane) - 1u));
      if (at < cap) out[at] = Out(v);
      else raise_err(err, kDevErrBounds);
    }
    running += total;
    __syncthreads();
  }
}

// Exclusive scan of n uint32 counts into uint64 offsets; offsets[n] = total.
// One block; the counts are few (one per 4096 candidates).
__global__ void __launch_bounds__(1024) k_scan_counts(const uint32_t* counts, int64_t n,
                                                      uint64_t* offsets) {
  __shared__ uint64_t warp_sum[32];
  __shared__ uint64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t start = 0; start < n; start += 1024) {
    const int64_t i = start + threadIdx.x;
    uint64_t v = (i < n) ? counts[i] : 0;
    uint64_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint64_t y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) warp_sum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint64_t s = warp_sum[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint64_t y = __shfl_up_sync(0xffffffffu, s, d);
        if (lane >= d) s += y;
      }
      warp_sum[lane] = s;  // inclusive over warps
    }
    __syncthreads();
    const uint64_t warp_excl = (wid > 0) ? warp_sum[wid - 1] : 0;
    if (i < n) offsets[i] = carry + warp_excl + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_sum[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) offsets[n] = carry;
}

// segc[r] = first index of the segment of mask r (lower bound of mask<<ushift);
// segc[nmasks] = dim
__device__ __forceinline__ uint32_t segment_start(const uint64_t* keys, int64_t dim,
                                                  const uint32_t* masks, int nmasks, int ushift,
                                                  int r) {
  if (r == nmasks) return uint32_t(dim);
  const uint64_t t = uint64_t(masks[r]) << ushift;
  int64_t lo = 0, hi = dim;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < t) lo = mid + 1; else hi = mid;
  }
  return uint32_t(lo);
}

__global__ void k_segments(const uint64_t* keys, int64_t dim, const uint32_t* masks, int nmasks,
                           int ushift, uint32_t* segc) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > nmasks) return;
  segc[r] = segment_start(keys, dim, masks, nmasks, ushift, r);
}

__global__ void k_low_parts(const uint64_t* keys, int64_t dim, int ushift, uint32_t* low) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < dim) low[i] = uint32_t(keys[i] & ((1ull << ushift) - 1));
}

// C(p, j) for j = 0..32 into binom[p * 33 + j] (p < 32)
__device__ __forceinline__ void binom_column(uint32_t* binom, int p) {
  uint64_t c = 1;
  for (int j = 0; j <= 32; ++j) {
    binom[p * 33 + j] = (j <= p) ? uint32_t(c) : 0u;
    if (j < p) c = c * uint64_t(p - j) / uint64_t(j + 1);
    else c = 0;
  }
}

__global__ void k_binom(uint32_t* binom) {
  if (threadIdx.x < 32) binom_column(binom, threadIdx.x);
}

__global__ void k_decode_states(Geom G, const uint64_t* keys, int64_t i0, int64_t n, int8_t* nf,
                                int8_t* eR, int8_t* eU) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Config c = decode(G, keys[i0 + i]);
  // Julia column-major blocks per state
  for (int s = 0; s < G.ns; ++s) nf[i * G.ns + s] = int8_t((c.mask >> s) & 1u);
  for (int r = 0; r < G.nR; ++r) eR[i * G.nR + r] = int8_t(get_eR(G, c.rpack, r));
  for (int j = 0; j < G.nU; ++j) eU[i * G.nU + j] = int8_t(get_eU(G, c.digits, j));
}

__global__ void k_ref_keys(Geom G, const uint64_t* keys, int64_t i0, int64_t n, uint64_t* out) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = ref_encode(G, decode(G, keys[i0 + i]));
}

// _encode key -> 1-based index (0 when the configuration is not a basis
// state): the key_dict lookup of finite_ed.jl:527-531.
__global__ void k_rank_ref_keys(Geom G, RankView R, const uint64_t* in, int64_t n, int64_t* out) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = in[i];
  uint32_t mask = uint32_t(k & ((G.ns >= 32) ? 0xffffffffu : ((1u << G.ns) - 1u)));
  int off = G.ns + 2 * G.nR;
  uint64_t digits = 0;
  bool ok = true;
  for (int j = 0; j < G.nU; ++j, off += 2) {
    int e = int((k >> off) & 3u) - 1;
    if (e < -1 || e > 1) ok = false;
    digits = (digits << G.w) | uint64_t(e + G.dg);
  }
  if (G.ns + 2 * (G.nR + G.nU) < 64 && (k >> (G.ns + 2 * (G.nR + G.nU))) != 0) ok = false;
  int64_t idx = -1;
  if (ok && __popc(mask) == G.nf_target) {
    const uint64_t key = make_key(G, mask, digits);
    idx = rank_key(R, R.segc, R.binom, key);
    // the e_R fields must agree with the Gauss-law values as well
    if (idx >= 0 && ref_encode(G, decode(G, key)) != k) idx = -1;
  }
  out[i] = idx + 1;
}

__global__ void k_rank_order_keys(Geom G, RankView R, const uint64_t* in, int64_t n,
                                  int64_t* out) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = in[i];
  const uint64_t mask = k >> R.ushift;
  int64_t idx = -1;
  if ((mask >> G.ns) == 0 && __popcll(mask) == G.nf_target && R.nmasks > 0)
    idx = rank_key(R, R.segc, R.binom, k);
  out[i] = idx;
}


// ---- rank tables ---------------------------------------------------------------
//
// Within the segment of a fermion mask, states are ordered lexicographically
// by their e_U rows u_0, u_1, ..., u_{ny-2}, each row by its free digits
// (all but the last, which the row sum fixes).  So the index of a state is
//     segc(mask) + sum_r T_r(mask rows >= r, u_{r-1}, u_r),
//     T_r = sum over v < u_r valid at row r given u_{r-1} of
//           Cnt_{r+1}(v) = number of valid completions of rows r+1.. given u_r = v.
// Validity at row r needs only q on row r, the row sum S_r (which depends on
// the mask rows below... above r: S_r = -sum_{j>r} R_j) and u_{r-1}, u_r, so
// every term is a table lookup.  Tables are built bottom-up; entry [F] of the
// last axis holds the total Cnt_r.  T_0 is indexed by the whole mask and
// carries segc folded in.  A state's rank is then ny-1 independent loads.

// digits of a row from its free-digit index f (first most significant) and
// row sum S; returns false if the determined last digit is out of range
__device__ __forceinline__ bool row_digits(int nx, int dg, int B, uint32_t f, int S, int* d) {
  int sum = 0;
  for (int ix = nx - 2; ix >= 0; --ix) {
    d[ix] = int(f % uint32_t(B)) - dg;
    f /= uint32_t(B);
    sum += d[ix];
  }
  d[nx - 1] = S - sum;
  return d[nx - 1] >= -dg && d[nx - 1] <= dg;
}

// e_R row validity: acc over ix < nx-1 of q(ix) - u(ix) + uprev(ix) within [-dg, dg]
__device__ __forceinline__ bool eR_row_ok(int nx, int dg, uint32_t rowbits, const int8_t* g,
                                          const int* u, const int* uprev) {
  int acc = 0;
  for (int ix = 0; ix < nx - 1; ++ix) {
    acc += int((rowbits >> ix) & 1u) + g[ix] - (u ? u[ix] : 0) + (uprev ? uprev[ix] : 0);
    if (acc < -dg || acc > dg) return false;
  }
  return true;
}

// Cnt_{ny-1}(u_{ny-2}): the last e_R row, for every bit pattern m of the last
// site row and every free index fp of u_{ny-2}.
__device__ __forceinline__ void tab_last_at(const Geom& G, int F, uint32_t* L, int idx) {
  const uint32_t m = uint32_t(idx / F), fp = uint32_t(idx % F);
  const int r = G.ny - 1;
  const int Rl = __popc(m) + G.grow[r];
  int up[kMaxSites];
  const bool okp = row_digits(G.nx, G.dg, 2 * G.dg + 1, fp, -Rl, up);
  L[idx] = (okp && eR_row_ok(G.nx, G.dg, m, G.gq + r * G.nx, nullptr, up)) ? 1u : 0u;
}

__global__ void k_tab_last(Geom G, int F, uint32_t* L) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < (1 << G.nx) * F) tab_last_at(G, F, L, idx);
}

// T_r for e_U row r (0 <= r <= ny-2): m = site rows >= r (nx*(ny-r) bits),
// fp = free index of u_{r-1} (Fp = 1 for r = 0).  `next` is Cnt_{r+1}:
// L when r = ny-2, else T_{r+1} (its entry [F]).
__device__ __forceinline__ void tab_row_at(const Geom& G, int F, int r, const uint32_t* next,
                                           int next_is_last, uint32_t* T, int Fp, int64_t idx) {
  const uint32_t m = uint32_t(idx / Fp), fp = uint32_t(idx % Fp);
  const int B = 2 * G.dg + 1;
  const uint32_t rowmask = (1u << G.nx) - 1u;
  int Sr = 0;  // S_r = -sum_{j>r} R_j
  for (int j = r + 1; j < G.ny; ++j) Sr -= __popc((m >> ((j - r) * G.nx)) & rowmask) + G.grow[j];
  const int Rr = __popc(m & rowmask) + G.grow[r];
  int up[kMaxSites], u[kMaxSites];
  if (r > 0) row_digits(G.nx, G.dg, B, fp, Sr - Rr, up);
  uint32_t run = 0;
  uint32_t* out = T + (uint64_t(m) * Fp + fp) * uint64_t(F + 1);
  for (int v = 0; v < F; ++v) {
    out[v] = run;
    if (!row_digits(G.nx, G.dg, B, uint32_t(v), Sr, u)) continue;
    if (!eR_row_ok(G.nx, G.dg, m & rowmask, G.gq + r * G.nx, u, r > 0 ? up : nullptr)) continue;
    const uint64_t mn = uint64_t(m >> G.nx);
    run += next_is_last ? next[mn * F + v] : next[(mn * F + v) * uint64_t(F + 1) + F];
  }
  out[F] = run;
}

__global__ void k_tab_row(Geom G, int F, int r, const uint32_t* next, int next_is_last,
                          uint32_t* T, int Fp, int64_t nm) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx < nm * Fp) tab_row_at(G, F, r, next, next_is_last, T, Fp, idx);
}

// T_0 += segc of the mask's segment (masks with the sector's particle number)
__global__ void k_tab_seg(Geom G, const uint32_t* masks, const uint32_t* segc, int nmasks, int F,
                          uint32_t* T0) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(nmasks) * (F + 1)) return;
  const int cr = int(idx / (F + 1)), v = int(idx % (F + 1));
  T0[uint64_t(masks[cr]) * (F + 1) + v] += segc[cr];
}

// every basis key must rank to its own index through the tables
__device__ __forceinline__ bool tab_ranks_own_index(const RankView& R, int64_t i) {
  const uint64_t key = R.keys[i];
  const uint64_t digits = key & ((1ull << R.ushift) - 1);
  uint32_t f[kMaxTabRows];
#pragma unroll
  for (int r = 0; r < kMaxTabRows; ++r) f[r] = (r < R.nrows) ? row_index(R, digits, r) : 0u;
  return rank_rows(R, uint32_t(key >> R.ushift), f, -1, 0) == i;
}

__global__ void k_tab_check(RankView R, int* bad) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < R.dim && !tab_ranks_own_index(R, i)) atomicOr(bad, 1);
}

// ---- small sectors in one launch -------------------------------------------
//
// For a candidate space of at most kFusedMaxCandidates and tables of at most
// kFusedMaxTable entries, one block builds the whole basis: binomials, the
// masks and the order keys by the same ordered compaction (tile by tile of
// the block, warp ballots and a prefix over the warps), the segment starts
// and low parts, the rank tables row by row and their self-check, with block
// barriers between the phases.  The host then waits once, for the sector
// dimension and the check, instead of a dozen launches and two read-backs.
constexpr int kFusedThreads = 1024;
constexpr uint64_t kFusedMaxCandidates = uint64_t(1) << 15;
constexpr int64_t kFusedMaxTable = int64_t(1) << 16;

struct FusedBasisArgs {
  Geom G;
  RankView R;        // tables and geometry (its dim is an upper bound)
  uint32_t* binom;
  uint32_t* masks;
  uint64_t* keys;
  uint32_t* low;     // null when the e_U part exceeds 32 bits
  uint32_t* segc;
  uint32_t* tab;     // null: no tables
  uint32_t* L;       // the last e_U row's counts (tables only)
  int64_t* out;      // [0] sector dimension, [1] tables failed their check
  int* err;
  int nmasks;        // C(ns, N_f)
  uint64_t nfree;    // free e_U strings per mask
  uint64_t cap;      // nmasks * nfree: room for every candidate
  int F;
  int64_t nlast;
};

// In-order compaction of p's candidates by one block; returns the count.
template <class Pred, class Out>
__device__ uint64_t block_compact(const Pred& p, Out* out, uint64_t cap, int* err,
                                  uint32_t* warp_cnt) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint64_t running = 0;
  for (uint64_t base = 0; base < p.total; base += blockDim.x) {
    const uint64_t idx = base + threadIdx.x;
    uint64_t v = 0;
    const bool ok = idx < p.total && p(idx, &v);
    const uint32_t bal = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) warp_cnt[wid] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < nw; ++w) {
      const uint32_t c = warp_cnt[w];
      before += (w < wid) ? c : 0u;
      total += c;
    }
    if (ok) {
      const uint64_t at = running + before + __popc(bal & ((1u << lane) - 1u));
      if (at < cap) out[at] = Out(v);
      else raise_err(err, kDevErrBounds);
    }
    running += total;
    __syncthreads();  // warp_cnt reused; this tile's writes visible to the block
  }
  return running;
}

template <int DG>
__global__ void __launch_bounds__(kFusedThreads) k_basis_fused(FusedBasisArgs a) {
  __shared__ uint32_t warp_cnt[kFusedThreads / 32];
  __shared__ int s_bad;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid < 32) binom_column(a.binom, tid);
  if (tid == 0) s_bad = 0;
  const int nmasks = a.nmasks;
  block_compact(MaskPred{a.G.nf_target, uint64_t(1) << a.G.ns}, a.masks, uint64_t(nmasks), a.err,
                warp_cnt);
  const CandPred<DG> cp{a.G, a.masks, a.nfree, uint64_t(nmasks) * a.nfree};
  const int64_t dim = int64_t(block_compact(cp, a.keys, a.cap, a.err, warp_cnt));
  for (int r = tid; r <= nmasks; r += nt)
    a.segc[r] = segment_start(a.keys, dim, a.masks, nmasks, a.G.ushift, r);
  if (a.low)
    for (int64_t i = tid; i < dim; i += nt)
      a.low[i] = uint32_t(a.keys[i] & ((1ull << a.G.ushift) - 1));
  if (a.tab) {
    const int F = a.F, nrows = a.G.ny - 1;
    for (int64_t idx = tid; idx < a.nlast * F; idx += nt) tab_last_at(a.G, F, a.L, int(idx));
    __syncthreads();
    for (int r = nrows - 1; r >= 0; --r) {
      const int64_t nm = int64_t(1) << (a.G.nx * (a.G.ny - r));
      const int Fp = (r == 0) ? 1 : F;
      const uint32_t* next = (r == nrows - 1) ? a.L : a.tab + a.R.tab_off[r + 1];
      for (int64_t idx = tid; idx < nm * Fp; idx += nt)
        tab_row_at(a.G, F, r, next, r == nrows - 1, a.tab + a.R.tab_off[r], Fp, idx);
      __syncthreads();
    }
    // T_0 += segc of the mask's segment (segc was written before the
    // barriers above)
    for (int64_t idx = tid; idx < int64_t(nmasks) * (F + 1); idx += nt) {
      const int cr = int(idx / (F + 1)), v = int(idx % (F + 1));
      a.tab[uint64_t(a.masks[cr]) * (F + 1) + v] += a.segc[cr];
    }
    __syncthreads();
    for (int64_t i = tid; i < dim; i += nt)
      if (!tab_ranks_own_index(a.R, i)) s_bad = 1;
    __syncthreads();
  }
  if (tid == 0) {
    a.out[0] = dim;
    a.out[1] = s_bad;
  }
}

#define CK(call)                                                                 \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
  } while (0)

// Ordered compaction driver: counts, scans, writes.  The output holds
// `expected` entries when the caller knows the count (no read-back; the
// write is bounds-checked into `err`), else an upper bound (every
// candidate) when that is small, the count then read back once; only a
// large candidate space reads the count before allocating.  Temporaries and
// the output come from the library's stream-ordered pool.
constexpr uint64_t kUpperBoundBytes = 64ull << 20;
template <class Pred, class Out>
std::string compact(const Pred& p, Out** out, int64_t* count, int* err, cudaStream_t s,
                    int64_t expected = -1) {
  *out = nullptr;
  *count = 0;
  const uint64_t nblk64 = (p.total + kTile - 1) / kTile;
  if (nblk64 == 0) return std::string();
  if (nblk64 > 0x7fffffffull) return "candidate space too large for the enumerator";
  const int nblk = int(nblk64);
  uint32_t* counts = nullptr;
  uint64_t* offs = nullptr;
  CK(dev_alloc_n(&counts, size_t(nblk), s));
  CK(dev_alloc_n(&offs, size_t(nblk) + 1, s));
  k_compact_count<<<nblk, kThreads, 0, s>>>(p, counts), lgt::note_launch();
  CK(cudaGetLastError());
  k_scan_counts<<<1, 1024, 0, s>>>(counts, nblk, offs), lgt::note_launch();
  CK(cudaGetLastError());
  uint64_t total = 0, cap = 0;
  const bool small = p.total * sizeof(Out) <= kUpperBoundBytes;
  if (expected >= 0) {
    total = cap = uint64_t(expected);
  } else if (small) {
    cap = p.total;
  } else {
    CK(cudaMemcpyAsync(&total, offs + nblk, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    cap = total;
  }
  Out* o = nullptr;
  if (cap > 0) {
    CK(dev_alloc_n(&o, size_t(cap), s));
    k_compact_write<<<nblk, kThreads, 0, s>>>(p, offs, o, cap, err), lgt::note_launch();
    CK(cudaGetLastError());
  }
  if (expected < 0 && small) {
    CK(cudaMemcpyAsync(&total, offs + nblk, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  CK(dev_free(counts, s));
  CK(dev_free(offs, s));
  *out = o;
  *count = int64_t(total);
  return std::string();
}

}  // namespace

std::string make_geom(int nx, int ny, int dg, const int32_t* g, Geom* Gp) {
  Geom G{};
  if (nx < 1 || ny < 1) return "lattice sides must be >= 1";
  if (dg < 1 || dg > 7) return "dg must be in 1..7";
  G.nx = nx;
  G.ny = ny;
  G.dg = dg;
  G.ns = nx * ny;
  G.nR = (nx - 1) * ny;
  G.nU = nx * (ny - 1);
  G.nP = (nx - 1) * (ny - 1);
  int w = 1;
  while ((1 << w) < 2 * dg + 1) ++w;
  G.w = w;
  G.ushift = w * G.nU;
  if (G.ns > 31) return "at most 31 sites are supported (fermion mask is a uint32)";
  if (G.ns + G.ushift > 64) return "order key (sites + bits * up-links) exceeds 64 bits";
  long sum = 0;
  for (int i = 0; i < G.ns; ++i) {
    if (g[i] < -127 || g[i] > 127) return "background charge out of range";
    sum += g[i];
  }
  if (-sum < 0 || -sum > G.ns)
    return "Inconsistent sector: N_f = " + std::to_string(-sum) + " (need 0 <= N_f <= nx*ny)";
  G.nf_target = int(-sum);
  G.max_moves = G.nR + G.nU + 2 * G.nP;
  for (int iy = 1; iy <= ny; ++iy)
    for (int ix = 1; ix <= nx; ++ix) {
      int s = (iy - 1) * nx + (ix - 1);
      G.gq[s] = int8_t(g[(ix - 1) + (iy - 1) * nx]);  // column-major g[ix,iy]
      if ((ix + iy) % 2 == 0) G.even_mask |= 1u << s;
      else G.odd_mask |= 1u << s;
    }
  for (int iy = 0; iy < ny; ++iy) {
    int r = 0;
    for (int ix = 0; ix < nx; ++ix) r += G.gq[iy * nx + ix];
    G.grow[iy] = int8_t(r);
  }
  // Column snake (decoupling_U_soe.jl:41-54): column ix outer, iy ascending
  // for odd ix and descending for even ix (1-based).
  auto pos = [&](int ix, int iy) { return (ix - 1) * ny + ((ix & 1) ? iy : (ny + 1 - iy)); };
  for (int iy = 1; iy <= ny; ++iy)
    for (int ix = 1; ix <= nx - 1; ++ix) {
      int a = pos(ix, iy), b = pos(ix + 1, iy);
      int lo = a < b ? a : b, hi = a < b ? b : a;
      uint32_t between = 0;
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          int p = pos(jx, jy);
          if (p > lo && p < hi) between |= 1u << ((jy - 1) * nx + (jx - 1));
        }
      G.jw_between[(iy - 1) * (nx - 1) + (ix - 1)] = between;
    }
  *Gp = G;
  return std::string();
}

// Layout of the row-count rank tables: F strings per row, the start of each
// row's table, the entries of all of them and of the last row's counts.
// False when the tables do not apply or exceed 2^25 entries.
bool tab_plan(const Geom& G, int* Fo, int64_t* off, int64_t* toto, int64_t* nlasto) {
  const int nrows = G.ny - 1;
  if (nrows < 1 || nrows > kMaxTabRows || G.nx < 2) return false;
  const int Bd = 2 * G.dg + 1;
  long double Fl = 1;
  for (int i = 0; i < G.nx - 1; ++i) Fl *= Bd;
  if (Fl > 4096) return false;
  const int F = int(Fl);
  for (int r = 0; r < kMaxTabRows; ++r) off[r] = 0;
  long double tot = (long double)(1ull << G.ns) * (F + 1);
  for (int r = 1; r < nrows; ++r) {
    off[r] = int64_t(tot);
    tot += (long double)(1ull << (G.nx * (G.ny - r))) * F * (F + 1);
  }
  const int64_t nlast = int64_t(1) << G.nx;
  if (tot + nlast * F > (long double)(int64_t(1) << 25)) return false;
  *Fo = F;
  *toto = int64_t(tot);
  *nlasto = nlast;
  return true;
}

// Builds the row-count rank tables when they fit (at most 2^25 entries) and
// keeps them only if every basis key ranks to its own index through them.
std::string build_rank_tables(BasisDev* B) {
  const Geom& G = B->G;
  cudaStream_t s = B->stream;
  const int nrows = G.ny - 1;
  int F = 0;
  int64_t off[kMaxTabRows], tot = 0, nlast = 0;
  if (B->dim == 0 || !tab_plan(G, &F, off, &tot, &nlast)) return std::string();
  uint32_t* tab = nullptr;
  uint32_t* L = nullptr;
  int* bad = nullptr;
  CK(dev_alloc_n(&tab, size_t(tot), s));
  CK(dev_alloc_n(&L, size_t(nlast * F), s));
  CK(dev_alloc_n(&bad, 1, s));
  CK(cudaMemsetAsync(bad, 0, sizeof(int), s));
  k_tab_last<<<unsigned((nlast * F + 255) / 256), 256, 0, s>>>(G, F, L), lgt::note_launch();
  for (int r = nrows - 1; r >= 0; --r) {
    const int64_t nm = int64_t(1) << (G.nx * (G.ny - r));
    const int Fp = (r == 0) ? 1 : F;
    const uint32_t* next = (r == nrows - 1) ? L : tab + off[r + 1];
    k_tab_row<<<unsigned((nm * Fp + 255) / 256), 256, 0, s>>>(G, F, r, next, r == nrows - 1,
                                                              tab + off[r], Fp, nm), lgt::note_launch();
  }
  k_tab_seg<<<unsigned((int64_t(B->nmasks) * (F + 1) + 255) / 256), 256, 0, s>>>(
      G, B->masks, B->segc, B->nmasks, F, tab), lgt::note_launch();
  CK(cudaGetLastError());
  B->tab = tab;
  B->tab_F = F;
  for (int r = 0; r < kMaxTabRows; ++r) B->tab_off[r] = off[r];
  k_tab_check<<<unsigned((B->dim + 255) / 256), 256, 0, s>>>(B->view(), bad), lgt::note_launch();
  int hbad = 0;
  CK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(dev_free(L, s));
  CK(dev_free(bad, s));
  CK(cudaStreamSynchronize(s));
  if (hbad) {  // keep the binary-search ranking
    dev_free(B->tab, s);
    B->tab = nullptr;
    B->tab_F = 0;
    return "rank tables failed their self-check";
  }
  return std::string();
}

// The whole basis of a small sector from one launch of k_basis_fused, its
// buffers carved from one pool allocation (BasisDev::block).
std::string build_basis_fused(BasisDev* B, int nmasks, uint64_t nfree) {
  const Geom& G = B->G;
  cudaStream_t s = B->stream;
  const uint64_t cap = uint64_t(nmasks) * nfree;
  int F = 0;
  int64_t off[kMaxTabRows] = {}, tot = 0, nlast = 0;
  const bool tabs = tab_plan(G, &F, off, &tot, &nlast) && tot + nlast * F <= kFusedMaxTable;
  size_t at = 0;
  auto take = [&](size_t bytes) {
    const size_t o = at;
    at += (bytes + 255) & ~size_t(255);
    return o;
  };
  const size_t o_hdr = take(64);  // error word at 0, dimension and check flag at 16
  const size_t o_binom = take(32 * 33 * sizeof(uint32_t));
  const size_t o_masks = take(size_t(nmasks) * sizeof(uint32_t));
  const size_t o_keys = take(cap * sizeof(uint64_t));
  const size_t o_low = (G.ushift <= 32) ? take(cap * sizeof(uint32_t)) : 0;
  const size_t o_segc = take((size_t(nmasks) + 1) * sizeof(uint32_t));
  const size_t o_tab = tabs ? take(size_t(tot) * sizeof(uint32_t)) : 0;
  const size_t o_L = tabs ? take(size_t(nlast) * F * sizeof(uint32_t)) : 0;
  void* blk = nullptr;
  CK(dev_alloc(&blk, at, s));
  B->block = blk;
  char* base = static_cast<char*>(blk);
  CK(cudaMemsetAsync(base + o_hdr, 0, 64, s));
  B->err = reinterpret_cast<int*>(base + o_hdr);
  int64_t* out = reinterpret_cast<int64_t*>(base + o_hdr + 16);
  B->binom = reinterpret_cast<uint32_t*>(base + o_binom);
  B->masks = reinterpret_cast<uint32_t*>(base + o_masks);
  B->keys = reinterpret_cast<uint64_t*>(base + o_keys);
  B->low = (G.ushift <= 32) ? reinterpret_cast<uint32_t*>(base + o_low) : nullptr;
  B->segc = reinterpret_cast<uint32_t*>(base + o_segc);
  B->nmasks = nmasks;
  B->dim = int64_t(cap);  // room for every candidate until the count is read
  if (tabs) {
    B->tab = reinterpret_cast<uint32_t*>(base + o_tab);
    B->tab_F = F;
    for (int r = 0; r < kMaxTabRows; ++r) B->tab_off[r] = off[r];
  }
  FusedBasisArgs a;
  a.G = G;
  a.R = B->view();
  a.binom = B->binom;
  a.masks = B->masks;
  a.keys = B->keys;
  a.low = B->low;
  a.segc = B->segc;
  a.tab = B->tab;
  a.L = tabs ? reinterpret_cast<uint32_t*>(base + o_L) : nullptr;
  a.out = out;
  a.err = B->err;
  a.nmasks = nmasks;
  a.nfree = nfree;
  a.cap = cap;
  a.F = F;
  a.nlast = nlast;
  switch (G.dg) {
#define LGT_FUSED_CASE(D)                                        \
  case D:                                                        \
    k_basis_fused<D><<<1, kFusedThreads, 0, s>>>(a);             \
    break;
    LGT_FUSED_CASE(1)
    LGT_FUSED_CASE(2)
    LGT_FUSED_CASE(3)
    LGT_FUSED_CASE(4)
    LGT_FUSED_CASE(5)
    LGT_FUSED_CASE(6)
    LGT_FUSED_CASE(7)
#undef LGT_FUSED_CASE
    default:
      return "unsupported dg";
  }
  lgt::note_launch();
  CK(cudaGetLastError());
  int64_t hout[2] = {0, 0};
  CK(cudaMemcpyAsync(hout, out, sizeof(hout), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  B->dim = hout[0];
  if (tabs && hout[1]) {  // the block keeps the memory; ranking by search
    B->tab = nullptr;
    B->tab_F = 0;
    return "rank tables failed their self-check";
  }
  return std::string();
}

std::string build_basis_device(BasisDev* B) {
  const Geom& G = B->G;
  cudaStream_t s = B->stream;
  int64_t expect = 1;  // masks with N_f set bits: C(ns, N_f)
  for (int j = 0; j < G.nf_target; ++j) expect = expect * (G.ns - j) / (j + 1);
  const int nfd = (G.ny - 1) * (G.nx - 1);
  const uint64_t base = uint64_t(2 * G.dg + 1);
  long double space = 1;
  for (int i = 0; i < nfd; ++i) space *= (long double)base;
  if (space * (long double)(expect ? expect : 1) > 1.8e19L)
    return "candidate space exceeds 64-bit indexing";
  const uint64_t nfree = ipow(base, nfd);
  const char* fz = std::getenv("LGT_BASIS_FUSED");  // "0": the multi-launch build
  if (expect > 0 && space * (long double)expect <= (long double)kFusedMaxCandidates &&
      !(fz && fz[0] == '0'))
    return build_basis_fused(B, int(expect), nfree);

  CK(dev_alloc_n(&B->err, 1, s));
  CK(cudaMemsetAsync(B->err, 0, sizeof(int), s));
  CK(dev_alloc_n(&B->binom, 32 * 33, s));
  k_binom<<<1, 32, 0, s>>>(B->binom), lgt::note_launch();
  CK(cudaGetLastError());

  // 1. masks with N_f set bits, ascending: C(ns, N_f) of them (the write is
  //    bounds-checked into the error word against that count)
  MaskPred mp{G.nf_target, 1ull << G.ns};
  int64_t nmasks = 0;
  std::string err = compact(mp, &B->masks, &nmasks, B->err, s, expect);
  if (!err.empty()) return err;
  B->nmasks = int(nmasks);

  // 2. candidates (mask, free e_U digits) -> sorted order keys
  int64_t dim = 0;
  if (nmasks > 0) {
    switch (G.dg) {
#define LGT_ENUM_CASE(D)                                                 \
  case D: {                                                              \
    CandPred<D> cp{G, B->masks, nfree, uint64_t(nmasks) * nfree};        \
    err = compact(cp, &B->keys, &dim, B->err, s);                        \
    break;                                                               \
  }
      LGT_ENUM_CASE(1)
      LGT_ENUM_CASE(2)
      LGT_ENUM_CASE(3)
      LGT_ENUM_CASE(4)
      LGT_ENUM_CASE(5)
      LGT_ENUM_CASE(6)
      LGT_ENUM_CASE(7)
#undef LGT_ENUM_CASE
      default:
        return "unsupported dg";
    }
    if (!err.empty()) return err;
  }
  if (dim >= (int64_t(1) << 32) - 1) return "sector dimension exceeds 2^32";
  B->dim = dim;

  // 3. ranking tables
  CK(dev_alloc_n(&B->segc, size_t(nmasks) + 1, s));
  k_segments<<<int((nmasks + 1 + 255) / 256), 256, 0, s>>>(B->keys, dim, B->masks, int(nmasks),
                                                          G.ushift, B->segc), lgt::note_launch();
  CK(cudaGetLastError());
  if (G.ushift <= 32 && dim > 0) {
    CK(dev_alloc_n(&B->low, size_t(dim), s));
    k_low_parts<<<int((dim + 255) / 256), 256, 0, s>>>(B->keys, dim, G.ushift, B->low), lgt::note_launch();
    CK(cudaGetLastError());
  }
  err = build_rank_tables(B);
  if (!err.empty()) return err;
  return std::string();
}

void free_basis_device(BasisDev* B) {
  cudaStream_t s = B->stream;
  if (B->block) {  // one allocation holds every buffer
    dev_free(B->block, s);
    const Geom G = B->G;
    const cudaStream_t st = B->stream;
    *B = BasisDev();
    B->G = G;
    B->stream = st;
    return;
  }
  dev_free(B->tab, s);
  B->tab = nullptr;
  dev_free(B->keys, s);
  dev_free(B->low, s);
  dev_free(B->segc, s);
  dev_free(B->masks, s);
  dev_free(B->binom, s);
  dev_free(B->err, s);
  B->keys = nullptr;
  B->low = nullptr;
  B->segc = nullptr;
  B->masks = nullptr;
  B->binom = nullptr;
  B->err = nullptr;
}

void launch_decode_states(const BasisDev& B, int64_t i0, int64_t n, int8_t* nf, int8_t* eR,
                          int8_t* eU, cudaStream_t s) {
  if (n <= 0) return;
  k_decode_states<<<int((n + 255) / 256), 256, 0, s>>>(B.G, B.keys, i0, n, nf, eR, eU), lgt::note_launch();
}

void launch_ref_keys(const BasisDev& B, int64_t i0, int64_t n, uint64_t* out, cudaStream_t s) {
  if (n <= 0) return;
  k_ref_keys<<<int((n + 255) / 256), 256, 0, s>>>(B.G, B.keys, i0, n, out), lgt::note_launch();
}

void launch_rank_ref_keys(const BasisDev& B, const uint64_t* in, int64_t n, int64_t* out,
                          cudaStream_t s) {
  if (n <= 0) return;
  k_rank_ref_keys<<<int((n + 255) / 256), 256, 0, s>>>(B.G, B.view(), in, n, out), lgt::note_launch();
}

void launch_rank_order_keys(const BasisDev& B, const uint64_t* in, int64_t n, int64_t* out,
                            cudaStream_t s) {
  if (n <= 0) return;
  k_rank_order_keys<<<int((n + 255) / 256), 256, 0, s>>>(B.G, B.view(), in, n, out), lgt::note_launch();
}

}  // namespace lgt
