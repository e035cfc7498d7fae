// nbr_table.cu -- the stored neighbour table: the lookup pass of H*psi
// (every row's neighbour ranks, finite_ed.jl:279-318 and
// matter_gauge_entanglement_pjw.jl:104-144) computed once per basis and
// model and kept in HBM, so that the products of a Krylov solve only gather.
//
// Nothing of H's values is stored: the coefficients stay per coupling point
// and are applied by the gather phase (lgt_hpsi_gather.cuh).  Layout:
//   meta[N]      per row: entry count, hop count, sum of e^2, staggered
//                occupation + 128 (gather::pack_meta);
//   tile_off[T+1] start of the entries of rows 32 t .. 32 t + 31 in `nbr`;
//   nbr[nnz]     row by row: hop entries (index | JW parity << 31), then
//                plaquette entries, in the move order of lgt_moves.cuh.
// 4 bytes per off-diagonal entry plus 4 per row: 0.43 GB for the 4x4
// staggered sector of the reference model (N = 8.56e6, 11.4 entries a row).
//
// Build: a count pass (meta and per-tile totals), a scan of the tile totals,
// and a fill pass that ranks every move (rank tables when the basis has
// them, else the key search) -- any lattice shape and any dg.
//
// The table kernel copies a warp's lists into shared memory with coalesced
// streaming loads (evict-first, so that the table does not push reusable x
// rows out of L2) and runs the gather phase of the fixed-shape kernel.
#include <cstdlib>

#include "lgt_hpsi.h"
#include "lgt_hpsi_gather.cuh"
#include "lgt_moves.cuh"
#include "lgt_rank.cuh"

namespace lgt {

namespace {

constexpr int kBuildThreads = 256;
constexpr int kTabWarps = 8;
constexpr int kTabThreads = kTabWarps * 32;
// Resident blocks per SM the register budget must allow.  Measured on the
// 4x4 lattice, K = 8 complex FP32: 5 blocks with 8 rows in flight beat 6
// with 4 (0.714 vs 0.757 ms); 8 blocks (32 registers) spill.
#ifndef LGT_TABLE_MINB
#define LGT_TABLE_MINB 5
#endif
#ifndef LGT_TABLE_MINB_PLAQ
#define LGT_TABLE_MINB_PLAQ 4
#endif

#define TCK(call)                                                                  \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
  } while (0)

__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += u;
  }
  return v;
}

// Count pass: meta word of every row and the entry total of every tile.
template <bool PLAQ, bool JW>
__global__ void __launch_bounds__(kBuildThreads) k_table_count(Geom G, RankView R, int64_t N,
                                                               uint32_t* meta,
                                                               uint32_t* tile_cnt) {
  const int64_t row = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int cnt = 0;
  if (row < N) {
    const Config c = decode(G, R.keys[row]);
    int e2 = 0, stag = 0, nh = 0;
    diag_parts(G, c, &e2, &stag);
    for_each_move<PLAQ, JW>(G, c, [&](uint64_t, uint32_t kind) {
      ++cnt;
      if (kind != kPlaq) ++nh;
    });
    meta[row] = gather::pack_meta(cnt, nh, e2, stag);
  }
  const int tot = warp_incl_scan(cnt, lane);
  if (lane == 31 && row - 31 < N) tile_cnt[row >> 5] = uint32_t(tot);
}

// Exclusive scan of n tile totals into off[0..n] (one block; the build runs
// once per basis and model).
__global__ void __launch_bounds__(1024) k_table_scan(const uint32_t* cnt, int64_t n, uint32_t* off) {
  __shared__ uint32_t warp_sum[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t start = 0; start < n; start += 1024) {
    const int64_t i = start + threadIdx.x;
    const uint32_t v = (i < n) ? cnt[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) warp_sum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint32_t s = warp_sum[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, s, d);
        if (lane >= d) s += y;
      }
      warp_sum[lane] = s;
    }
    __syncthreads();
    const uint32_t excl = (wid > 0) ? warp_sum[wid - 1] : 0u;
    if (i < n) off[i] = carry + excl + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_sum[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) off[n] = carry;
}

// Fill pass: rank every move of every row into its slot.
template <bool PLAQ, bool JW>
__global__ void __launch_bounds__(kBuildThreads) k_table_fill(Geom G, RankView R, int64_t N,
                                                              const uint32_t* meta,
                                                              const uint32_t* tile_off,
                                                              uint32_t* nbr, int* err) {
  const int64_t row = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int cnt = (row < N) ? int(meta[row] & 255u) : 0;
  const int incl = warp_incl_scan(cnt, lane);
  if (row >= N) return;
  uint32_t* my = nbr + tile_off[row >> 5] + uint32_t(incl - cnt);
  const Config c = decode(G, R.keys[row]);
  int n = 0;
  auto put = [&](int64_t j, uint32_t kind) {
    if (j < 0 || j >= N || n >= cnt) {
      raise_err(err, j < 0 ? kDevErrRank : kDevErrBounds);
      return;
    }
    my[n++] = uint32_t(j) | (kind == kHopNeg ? 0x80000000u : 0u);
  };
  if (R.tab) {
    uint32_t fidx[kMaxTabRows];
#pragma unroll
    for (int r = 0; r < kMaxTabRows; ++r) fidx[r] = (r < R.nrows) ? row_index(R, c.digits, r) : 0u;
    for_each_move_rows<PLAQ, JW>(G, c, fidx, R.pw,
                                 [&](uint32_t nmask, int rc, uint32_t frc, uint32_t kind) {
      put(rank_rows(R, nmask, fidx, rc, frc), kind);
    });
  } else {
    for_each_move<PLAQ, JW>(G, c, [&](uint64_t nkey, uint32_t kind) {
      put(rank_key(R, R.segc, R.binom, nkey), kind);
    });
  }
  while (n < cnt) my[n++] = 0u;  // only after a rank error (raised above)
}

template <typename T>
__host__ __device__ inline int table_smem(int K, int mm) {
  return gather::coef_bytes<T>(K) + 2 * kTabThreads * 4 + kTabThreads * mm * 4;
}

// y = H x from the stored table: per warp, the 32 meta words (an exclusive
// warp scan of their counts gives each row's list offset) and the tile's
// entries are copied into shared memory, then the gather phase runs.
template <typename T, int LD, bool PLAQ, bool JW>
__global__ void __launch_bounds__(kTabThreads, PLAQ ? LGT_TABLE_MINB_PLAQ : LGT_TABLE_MINB)
    k_hpsi_table(HpsiArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int K = a.K;
  T* s_coef = reinterpret_cast<T*>(smem);  // [4][K]: cE, cm, ch, cp
  uint32_t* s_meta = reinterpret_cast<uint32_t*>(smem + gather::coef_bytes<T>(K));
  uint32_t* s_off = s_meta + kTabThreads;
  uint32_t* s_list = s_off + kTabThreads;
  for (int i = threadIdx.x; i < K; i += kTabThreads) {
    s_coef[i] = a.cE[i];
    s_coef[K + i] = a.cm[i];
    s_coef[2 * K + i] = a.ch[i];
    s_coef[3 * K + i] = a.cp[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t warp_row0 = (int64_t(blockIdx.x) * kTabWarps + wid) * 32;
  if (warp_row0 >= a.N) return;
  const int64_t row = warp_row0 + lane;
  const uint32_t m = (row < a.N) ? __ldcs(a.t_meta + row) : 0u;
  const int cnt = int(m & 255u);
  const int incl = warp_incl_scan(cnt, lane);
  s_meta[wid * 32 + lane] = m;
  s_off[wid * 32 + lane] = uint32_t(incl - cnt);
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const uint32_t* src = a.t_nbr + __ldg(a.t_off + (warp_row0 >> 5));
  uint32_t* lst = s_list + wid * 32 * a.t_mm;
  for (int i = lane; i < total; i += 32) lst[i] = __ldcs(src + i);
  __syncwarp();
  const uint32_t* offs = s_off + wid * 32;
  gather::gather_rows<T, LD, PLAQ, JW>(a, warp_row0, lane, s_meta + wid * 32, s_coef,
                                       [&](int rl) { return lst + offs[rl]; });
}

template <typename T, int LD, bool PLAQ, bool JW>
cudaError_t launch_table_v(const HpsiArgs<T>& a, cudaStream_t s) {
  auto kern = k_hpsi_table<T, LD, PLAQ, JW>;
  const int bytes = table_smem<T>(a.K, a.t_mm);
  {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), bytes);
    if (e != cudaSuccess) return e;
  }
  const int64_t blocks = (a.N + kTabThreads - 1) / kTabThreads;
  if (blocks <= 0) return cudaSuccess;
  kern<<<unsigned(blocks), kTabThreads, bytes, s>>>(a), lgt::note_launch();
  return cudaGetLastError();
}

template <typename T, bool PLAQ, bool JW>
cudaError_t launch_table_m(const HpsiArgs<T>& a, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    // the gathered variant where it applies, else the widest load mode
    const int64_t rows = a.x_rows > 0 ? a.x_rows : a.N;
    if (a.vpl == 4 && table_bulk_applies(a, rows))
      return launch_table_bulk(a, (PLAQ ? kModelPlaq : 0u) | (JW ? kModelJW : 0u), rows, s);
  }
  int mode = 0;
  table_load_mode(a, &mode);
  const int want = a.vpl == 0 ? 2 : a.vpl;
  const int use = want < mode ? want : mode;
  if (use >= 3) return launch_table_v<T, 4, PLAQ, JW>(a, s);
  if (use == 2) return launch_table_v<T, 2, PLAQ, JW>(a, s);
  return launch_table_v<T, 1, PLAQ, JW>(a, s);
}

}  // namespace

int table_row_moves(const Geom& G, uint32_t model) {
  return G.nR + G.nU + ((model & kModelPlaq) ? 2 * G.nP : 0);
}

bool nbr_table_eligible(const Geom& G, int64_t N, uint32_t model, size_t* bytes) {
  const int mm = table_row_moves(G, model);
  const int64_t e2max = int64_t(G.nR + G.nU) * G.dg * G.dg;
  const bool ok = N > 0 && N < (int64_t(1) << 31) && N * mm < (int64_t(1) << 32) && mm <= 255 &&
                  e2max <= 255 && G.ns <= 127;
  // upper bound (every row with every move); the count pass gives the size
  if (bytes) *bytes = size_t(N) * 4 * (size_t(mm) + 1) + size_t(N / 32 + 2) * 4;
  return ok;
}

std::string build_nbr_table(const Geom& G, const RankView& R, uint32_t model, int* err,
                            NbrTable* T, cudaStream_t s) {
  free_nbr_table(T);
  const int64_t N = R.dim;
  if (!nbr_table_eligible(G, N, model, nullptr)) return "basis not representable in a table";
  const int64_t tiles = (N + 31) / 32;
  const unsigned blocks = unsigned((N + kBuildThreads - 1) / kBuildThreads);
  uint32_t* tile_cnt = nullptr;
  TCK(cudaMalloc(&T->meta, sizeof(uint32_t) * N));
  TCK(cudaMalloc(&T->tile_off, sizeof(uint32_t) * (tiles + 1)));
  TCK(cudaMalloc(&tile_cnt, sizeof(uint32_t) * tiles));
  const bool plaq = model & kModelPlaq, jw = model & kModelJW;
#define LGT_TABLE_PASS(KERN, ...)                                                           \
  do {                                                                                      \
    if (plaq && jw) KERN<true, true><<<blocks, kBuildThreads, 0, s>>>(__VA_ARGS__);         \
    else if (plaq) KERN<true, false><<<blocks, kBuildThreads, 0, s>>>(__VA_ARGS__);         \
    else if (jw) KERN<false, true><<<blocks, kBuildThreads, 0, s>>>(__VA_ARGS__);           \
    else KERN<false, false><<<blocks, kBuildThreads, 0, s>>>(__VA_ARGS__);                  \
    lgt::note_launch();                                                                     \
  } while (0)
  LGT_TABLE_PASS(k_table_count, G, R, N, T->meta, tile_cnt);
  k_table_scan<<<1, 1024, 0, s>>>(tile_cnt, tiles, T->tile_off), lgt::note_launch();
  uint32_t nnz = 0;
  TCK(cudaMemcpyAsync(&nnz, T->tile_off + tiles, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  TCK(cudaStreamSynchronize(s));
  TCK(cudaFree(tile_cnt));
  T->nnz = int64_t(nnz);
  TCK(cudaMalloc(&T->nbr, sizeof(uint32_t) * (size_t(nnz) + 1)));
  LGT_TABLE_PASS(k_table_fill, G, R, N, T->meta, T->tile_off, T->nbr, err);
#undef LGT_TABLE_PASS
  TCK(cudaGetLastError());
  TCK(cudaStreamSynchronize(s));
  T->N = N;
  T->model = model;
  T->mm = table_row_moves(G, model);
  T->bytes = sizeof(uint32_t) * (size_t(N) + size_t(tiles) + 1 + size_t(nnz) + 1);
  T->state = 1;
  return std::string();
}

void free_nbr_table(NbrTable* T) {
  cudaFree(T->meta);
  cudaFree(T->tile_off);
  cudaFree(T->nbr);
  cudaFree(T->perm);
  cudaFree(T->iperm);
  *T = NbrTable();
}

template <typename T>
bool table_load_mode(const HpsiArgs<T>& a, int* max_vpl) {
  constexpr int V = 16 / int(sizeof(T));
  const size_t xs = a.xsel ? a.xstride * sizeof(T) : 0;
  const bool ok = a.t_meta && a.C % V == 0 && ((reinterpret_cast<uintptr_t>(a.x) & 15) == 0) &&
                  ((reinterpret_cast<uintptr_t>(a.y) & 15) == 0) && (xs % 16 == 0);
  const bool two = a.C % (2 * V) == 0;
  const bool wide = two && (reinterpret_cast<uintptr_t>(a.x) & 31) == 0 &&
                    (reinterpret_cast<uintptr_t>(a.y) & 31) == 0 && (xs % 32 == 0);
  if (max_vpl) *max_vpl = ok ? (wide ? 3 : (two ? 2 : 1)) : 0;
  return ok;
}

template <typename T>
cudaError_t launch_hpsi_table(const HpsiArgs<T>& a, uint32_t model, cudaStream_t s) {
  if (!table_load_mode(a, nullptr)) return cudaErrorInvalidValue;
  const bool plaq = model & kModelPlaq, jw = model & kModelJW;
  if (plaq && jw) return launch_table_m<T, true, true>(a, s);
  if (plaq) return launch_table_m<T, true, false>(a, s);
  if (jw) return launch_table_m<T, false, true>(a, s);
  return launch_table_m<T, false, false>(a, s);
}

template bool table_load_mode<double>(const HpsiArgs<double>&, int*);
template bool table_load_mode<float>(const HpsiArgs<float>&, int*);
template cudaError_t launch_hpsi_table<double>(const HpsiArgs<double>&, uint32_t, cudaStream_t);
template cudaError_t launch_hpsi_table<float>(const HpsiArgs<float>&, uint32_t, cudaStream_t);

}  // namespace lgt
