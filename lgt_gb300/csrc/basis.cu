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

// segc[r] = first index of the segment of mask r (lower bound of mask<<ushift)
__global__ void k_segments(const uint64_t* keys, int64_t dim, const uint32_t* masks, int nmasks,
                           int ushift, uint32_t* segc) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > nmasks) return;
  if (r == nmasks) {
    segc[r] = uint32_t(dim);
    return;
  }
  const uint64_t t = uint64_t(masks[r]) << ushift;
  int64_t lo = 0, hi = dim;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < t) lo = mid + 1; else hi = mid;
  }
  segc[r] = uint32_t(lo);
}

__global__ void k_low_parts(const uint64_t* keys, int64_t dim, int ushift, uint32_t* low) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < dim) low[i] = uint32_t(keys[i] & ((1ull << ushift) - 1));
}

__global__ void k_binom(uint32_t* binom) {
  int p = threadIdx.x;  // 0..31
  if (p >= 32) return;
  // C(p, j) for j = 0..32
  uint64_t c = 1;
  for (int j = 0; j <= 32; ++j) {
    binom[p * 33 + j] = (j <= p) ? uint32_t(c) : 0u;
    if (j < p) c = c * uint64_t(p - j) / uint64_t(j + 1);
    else c = 0;
  }
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
__global__ void k_tab_last(Geom G, int F, uint32_t* L) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (1 << G.nx) * F) return;
  const uint32_t m = uint32_t(idx / F), fp = uint32_t(idx % F);
  const int r = G.ny - 1;
  const int Rl = __popc(m) + G.grow[r];
  int up[kMaxSites];
  const bool okp = row_digits(G.nx, G.dg, 2 * G.dg + 1, fp, -Rl, up);
  L[idx] = (okp && eR_row_ok(G.nx, G.dg, m, G.gq + r * G.nx, nullptr, up)) ? 1u : 0u;
}

// T_r for e_U row r (0 <= r <= ny-2): m = site rows >= r (nx*(ny-r) bits),
// fp = free index of u_{r-1} (Fp = 1 for r = 0).  `next` is Cnt_{r+1}:
// L when r = ny-2, else T_{r+1} (its entry [F]).
__global__ void k_tab_row(Geom G, int F, int r, const uint32_t* next, int next_is_last,
                          uint32_t* T, int Fp, int64_t nm) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= nm * Fp) return;
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

// T_0 += segc of the mask's segment (masks with the sector's particle number)
__global__ void k_tab_seg(Geom G, const uint32_t* masks, const uint32_t* segc, int nmasks, int F,
                          uint32_t* T0) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(nmasks) * (F + 1)) return;
  const int cr = int(idx / (F + 1)), v = int(idx % (F + 1));
  T0[uint64_t(masks[cr]) * (F + 1) + v] += segc[cr];
}

// every basis key must rank to its own index through the tables
__global__ void k_tab_check(RankView R, int* bad) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= R.dim) return;
  const uint64_t key = R.keys[i];
  const uint64_t digits = key & ((1ull << R.ushift) - 1);
  uint32_t f[kMaxTabRows];
#pragma unroll
  for (int r = 0; r < kMaxTabRows; ++r) f[r] = (r < R.nrows) ? row_index(R, digits, r) : 0u;
  if (rank_rows(R, uint32_t(key >> R.ushift), f, -1, 0) != i) atomicOr(bad, 1);
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

// Builds the row-count rank tables when they fit (at most 2^25 entries) and
// keeps them only if every basis key ranks to its own index through them.
std::string build_rank_tables(BasisDev* B) {
  const Geom& G = B->G;
  cudaStream_t s = B->stream;
  const int nrows = G.ny - 1;
  if (B->dim == 0 || nrows < 1 || nrows > kMaxTabRows || G.nx < 2) return std::string();
  const int Bd = 2 * G.dg + 1;
  long double Fl = 1;
  for (int i = 0; i < G.nx - 1; ++i) Fl *= Bd;
  if (Fl > 4096) return std::string();
  const int F = int(Fl);
  int64_t off[kMaxTabRows] = {};
  long double tot = (long double)(1ull << G.ns) * (F + 1);
  for (int r = 1; r < nrows; ++r) {
    off[r] = int64_t(tot);
    tot += (long double)(1ull << (G.nx * (G.ny - r))) * F * (F + 1);
  }
  const int64_t nlast = int64_t(1) << G.nx;
  if (tot + nlast * F > (long double)(int64_t(1) << 25)) return std::string();
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

std::string build_basis_device(BasisDev* B) {
  const Geom& G = B->G;
  cudaStream_t s = B->stream;
  CK(dev_alloc_n(&B->err, 1, s));
  CK(cudaMemsetAsync(B->err, 0, sizeof(int), s));
  CK(dev_alloc_n(&B->binom, 32 * 33, s));
  k_binom<<<1, 32, 0, s>>>(B->binom), lgt::note_launch();
  CK(cudaGetLastError());

  // 1. masks with N_f set bits, ascending: C(ns, N_f) of them (the write is
  //    bounds-checked into the error word against that count)
  MaskPred mp{G.nf_target, 1ull << G.ns};
  int64_t expect = 1;
  for (int j = 0; j < G.nf_target; ++j) expect = expect * (G.ns - j) / (j + 1);
  int64_t nmasks = 0;
  std::string err = compact(mp, &B->masks, &nmasks, B->err, s, expect);
  if (!err.empty()) return err;
  B->nmasks = int(nmasks);

  // 2. candidates (mask, free e_U digits) -> sorted order keys
  const int nfd = (G.ny - 1) * (G.nx - 1);
  const uint64_t base = uint64_t(2 * G.dg + 1);
  long double space = 1;
  for (int i = 0; i < nfd; ++i) space *= (long double)base;
  if (space * (long double)(nmasks ? nmasks : 1) > 1.8e19L)
    return "candidate space exceeds 64-bit indexing";
  const uint64_t nfree = ipow(base, nfd);
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
