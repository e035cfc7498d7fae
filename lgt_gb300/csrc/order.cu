// order.cu -- a locality-preserving row order for the stored-table H*psi.
//
// In the reference's basis order (fermion mask major) a row's neighbours
// sit in other mask segments all over the vector, and the x gathers of one
// product miss L2 about five times per row on the 4x4 lattice (ncu: 3.2 GB
// of DRAM reads for 0.55 GB of x).  Ordering the rows by a breadth-first
// search of the hop graph puts every row next to the rows of the levels
// around it: an exact LRU model of a 50-100 MB cache over the 4x4 basis
// gives 1.6-1.9 misses per row in that order against 4.3-5.1 in the
// reference order.  The order is the queue order of the search from row 0:
// level after level; within a level, rows in the order their first
// discoverer was placed; a discoverer's children in the order of its table
// entries.  Rows no search from placed rows reaches start a new search from
// the first of them (after a few searches, the rest are appended in index
// order).
//
// The Krylov drivers keep their basis vectors in this order and apply H with
// a copy of the neighbour table renumbered to it; a state crosses the
// boundary by a gather when a Krylov space is started and a scatter when the
// result is combined, so callers only ever see the reference order.
//
// The row-level order above scatters the gathers of neighbouring lanes
// (the rows a warp handles no longer have structured neighbours), and the
// table kernel is bound by L1/TEX transactions more than by DRAM misses; so
// the default is the same search one level up: the fermion-mask segments
// (whose rows keep their reference order inside) are ordered breadth-first
// over the mask graph, two masks being adjacent when one hop moves a
// fermion across a bond between them (LRU model: 2.1 misses per row at
// 100 MB against 4.3).  LGT_TABLE_ORDER=row selects the row-level order,
// LGT_TABLE_ORDER=0 none.
//
// Everything runs on the device, level-synchronous: per level one pass
// claims the undiscovered neighbours of the level's rows (the smallest
// (discoverer position, entry slot) key wins), one counts each row's claimed
// children, a scan turns the counts into offsets and one pass places the
// children.  The host reads one count per level.
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <vector>

#include "lgt_hpsi.h"

namespace lgt {

namespace {

constexpr int kOT = 256;
constexpr int kMaxSearches = 16;

#define OCK(call)                                                                  \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
  } while (0)

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int* total) {
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += u;
  }
  *total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

// Entry offset of every row of a table: tile offset plus the exclusive scan
// of the counts of the rows before it in its 32-row tile.
__global__ void k_row_offsets(const uint32_t* meta, const uint32_t* tile_off, int64_t N,
                              uint32_t* row_off) {
  const int64_t row = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int cnt = (row < N) ? int(meta[row] & 255u) : 0;
  int tot;
  const int ex = warp_excl_scan(cnt, lane, &tot);
  if (row < N) row_off[row] = tile_off[row >> 5] + uint32_t(ex);
}

// Claim pass of level L: rows at positions [p0, p1) offer each neighbour the
// key (position - p0) * 256 + slot; a neighbour not yet reached joins level
// L + 1 and keeps the smallest key offered to it.
__global__ void k_bfs_claim(const uint32_t* meta, const uint32_t* row_off, const uint32_t* nbr,
                            const int* perm, int64_t p0, int64_t p1, int L, int* level,
                            unsigned long long* key) {
  const int64_t p = p0 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= p1) return;
  const int o = perm[p];
  const int cnt = int(meta[o] & 255u);
  const uint32_t* e = nbr + row_off[o];
  for (int s = 0; s < cnt; ++s) {
    const int j = int(e[s] & 0x7fffffffu);
    const int old = atomicCAS(level + j, -1, L + 1);
    if (old == -1 || old == L + 1)
      atomicMin(key + j, (unsigned long long)(p - p0) * 256ull + unsigned(s));
  }
}

// The number of children each row of level L owns (the neighbours whose
// smallest key is this row's offer).
__global__ void k_bfs_count(const uint32_t* meta, const uint32_t* row_off, const uint32_t* nbr,
                            const int* perm, int64_t p0, int64_t p1, int L, const int* level,
                            const unsigned long long* key, uint32_t* count) {
  const int64_t p = p0 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= p1) return;
  const int o = perm[p];
  const int cnt = int(meta[o] & 255u);
  const uint32_t* e = nbr + row_off[o];
  uint32_t c = 0;
  for (int s = 0; s < cnt; ++s) {
    const int j = int(e[s] & 0x7fffffffu);
    if (level[j] == L + 1 && key[j] == (unsigned long long)(p - p0) * 256ull + unsigned(s)) ++c;
  }
  count[p - p0] = c;
}

// Places the children of level L after position p1, in discoverer order.
__global__ void k_bfs_place(const uint32_t* meta, const uint32_t* row_off, const uint32_t* nbr,
                            int* perm, int* iperm, int64_t p0, int64_t p1, int L, const int* level,
                            const unsigned long long* key, const uint32_t* off, int64_t N) {
  const int64_t p = p0 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= p1) return;
  const int o = perm[p];
  const int cnt = int(meta[o] & 255u);
  const uint32_t* e = nbr + row_off[o];
  int64_t at = p1 + off[p - p0];
  for (int s = 0; s < cnt; ++s) {
    const int j = int(e[s] & 0x7fffffffu);
    if (level[j] == L + 1 && key[j] == (unsigned long long)(p - p0) * 256ull + unsigned(s)) {
      if (at < N) {  // each row is claimed once, so this always holds
        perm[at] = j;
        iperm[j] = int(at);
      }
      ++at;
    }
  }
}

// Block sums of n counts (kOT per block, exclusive within the block into
// out) and the block totals into sums.
__global__ void k_scan_block(const uint32_t* in, int64_t n, uint32_t* out, uint32_t* sums) {
  __shared__ uint32_t ws[kOT / 32];
  const int64_t i = int64_t(blockIdx.x) * kOT + threadIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t v = (i < n) ? in[i] : 0u;
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += u;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < wid; ++w) before += ws[w];
  if (i < n) out[i] = before + x - v;
  if (threadIdx.x == kOT - 1) sums[blockIdx.x] = before + x;
}

// Exclusive scan of the block sums (one block, in rounds) and the grand
// total at sums_off[nb].
__global__ void __launch_bounds__(1024) k_scan_sums(const uint32_t* sums, int64_t nb,
                                                    uint32_t* sums_off) {
  __shared__ uint32_t ws[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t start = 0; start < nb; start += 1024) {
    const int64_t i = start + threadIdx.x;
    const uint32_t v = (i < nb) ? sums[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += u;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint32_t t = ws[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, t, d);
        if (lane >= d) t += u;
      }
      ws[lane] = t;
    }
    __syncthreads();
    const uint32_t ex = (wid > 0) ? ws[wid - 1] : 0u;
    if (i < nb) sums_off[i] = carry + ex + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += ws[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums_off[nb] = carry;
}

__global__ void k_scan_add(uint32_t* out, int64_t n, const uint32_t* sums_off) {
  const int64_t i = int64_t(blockIdx.x) * kOT + threadIdx.x;
  if (i < n) out[i] += sums_off[blockIdx.x];
}

// First row no search has reached (atomicMin over the unplaced rows).
__global__ void k_first_unplaced(const int* level, int64_t N, int* first) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < N && level[i] < 0) atomicMin(first, int(i));
}

__global__ void k_unplaced_flags(const int* level, int64_t N, uint32_t* flag) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < N) flag[i] = level[i] < 0 ? 1u : 0u;
}

__global__ void k_place_unplaced(const int* level, int64_t N, const uint32_t* off, int64_t at0,
                                 int* perm, int* iperm) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < N && level[i] < 0) {
    const int64_t at = at0 + off[i];
    perm[at] = int(i);
    iperm[i] = int(at);
  }
}

__global__ void k_invert(const int* perm, int64_t N, int* iperm) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n < N) iperm[perm[n]] = int(n);
}

__global__ void k_seed(int* perm, int* iperm, int* level, int64_t at, int row, int L) {
  perm[at] = row;
  iperm[row] = int(at);
  level[row] = L;
}

// The renumbered table: meta and counts of row n are those of old row
// perm[n]; its entries are the old row's, each index mapped through iperm
// (the Jordan-Wigner parity bit kept).
__global__ void k_perm_meta(const uint32_t* meta, const int* perm, int64_t N, uint32_t* meta2,
                            uint32_t* tile_cnt) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const uint32_t m = (n < N) ? meta[perm[n]] : 0u;
  if (n < N) meta2[n] = m;
  int tot;
  warp_excl_scan(int(m & 255u), lane, &tot);
  if (lane == 0 && n < N) tile_cnt[n >> 5] = uint32_t(tot);
}

__global__ void k_perm_fill(const uint32_t* meta2, const uint32_t* tile_off2,
                            const uint32_t* row_off, const uint32_t* nbr, const int* perm,
                            const int* iperm, int64_t N, uint32_t* nbr2) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int cnt = (n < N) ? int(meta2[n] & 255u) : 0;
  int tot;
  const int ex = warp_excl_scan(cnt, lane, &tot);
  if (n >= N) return;
  const uint32_t* src = nbr + row_off[perm[n]];
  uint32_t* dst = nbr2 + tile_off2[n >> 5] + uint32_t(ex);
  for (int s = 0; s < cnt; ++s) {
    const uint32_t e = src[s];
    dst[s] = uint32_t(iperm[e & 0x7fffffffu]) | (e & 0x80000000u);
  }
}

// Exclusive scan of n counts into out[0..n) with the total at *total_dev
// (stream-ordered; scratch from the pool).
std::string scan_counts(const uint32_t* in, int64_t n, uint32_t* out, uint32_t* total_dev,
                        cudaStream_t s) {
  const int64_t nb = (n + kOT - 1) / kOT;
  uint32_t* sums = nullptr;
  uint32_t* sums_off = nullptr;
  OCK(dev_alloc_n(&sums, size_t(nb) + 1, s));
  OCK(dev_alloc_n(&sums_off, size_t(nb) + 1, s));
  k_scan_block<<<unsigned(nb), kOT, 0, s>>>(in, n, out, sums), lgt::note_launch();
  k_scan_sums<<<1, 1024, 0, s>>>(sums, nb, sums_off), lgt::note_launch();
  k_scan_add<<<unsigned(nb), kOT, 0, s>>>(out, n, sums_off), lgt::note_launch();
  OCK(cudaMemcpyAsync(total_dev, sums_off + nb, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  OCK(cudaGetLastError());
  OCK(dev_free(sums, s));
  OCK(dev_free(sums_off, s));
  return std::string();
}

// The renumbered table T2 of T under perm (T2's perm and iperm are set).
std::string renumber(const NbrTable& T, const int* perm, const int* iperm,
                     const uint32_t* row_off, NbrTable* T2, cudaStream_t s) {
  const int64_t N = T.N;
  const unsigned nblk = unsigned((N + kOT - 1) / kOT);
  const int64_t tiles = (N + 31) / 32;
  uint32_t* tile_cnt = nullptr;
  OCK(cudaMalloc(&T2->meta, sizeof(uint32_t) * N));
  OCK(cudaMalloc(&T2->tile_off, sizeof(uint32_t) * (tiles + 1)));
  OCK(cudaMalloc(&T2->nbr, sizeof(uint32_t) * (size_t(T.nnz) + 1)));
  OCK(dev_alloc_n(&tile_cnt, size_t(tiles) + 1, s));
  k_perm_meta<<<nblk, kOT, 0, s>>>(T.meta, perm, N, T2->meta, tile_cnt), lgt::note_launch();
  {
    std::string e = scan_counts(tile_cnt, tiles, T2->tile_off, T2->tile_off + tiles, s);
    if (!e.empty()) return e;
  }
  k_perm_fill<<<nblk, kOT, 0, s>>>(T2->meta, T2->tile_off, row_off, T.nbr, perm, iperm, N,
                                   T2->nbr), lgt::note_launch();
  OCK(cudaGetLastError());
  OCK(dev_free(tile_cnt, s));
  return std::string();
}

void finish(const NbrTable& T, NbrTable* T2) {
  T2->N = T.N;
  T2->nnz = T.nnz;
  T2->model = T.model;
  T2->mm = T.mm;
  T2->bytes = T.bytes + sizeof(int) * 2 * size_t(T.N);
  T2->state = 1;
}

}  // namespace

std::string build_table_order(const NbrTable& T, NbrTable* T2, cudaStream_t s) {
  const int64_t N = T.N;
  if (T.state != 1 || N <= 0) return "no neighbour table to reorder";
  free_nbr_table(T2);
  const unsigned nblk = unsigned((N + kOT - 1) / kOT);
  int *perm = nullptr, *iperm = nullptr, *level = nullptr, *first = nullptr;
  uint32_t *row_off = nullptr, *count = nullptr, *off = nullptr, *total = nullptr;
  unsigned long long* key = nullptr;
  OCK(cudaMalloc(&perm, sizeof(int) * N));
  T2->perm = perm;
  OCK(cudaMalloc(&iperm, sizeof(int) * N));
  T2->iperm = iperm;
  OCK(dev_alloc_n(&level, size_t(N), s));
  OCK(dev_alloc_n(&key, size_t(N), s));
  OCK(dev_alloc_n(&row_off, size_t(N), s));
  OCK(dev_alloc_n(&count, size_t(N) + 1, s));
  OCK(dev_alloc_n(&off, size_t(N) + 1, s));
  OCK(dev_alloc_n(&total, 1, s));
  OCK(dev_alloc_n(&first, 1, s));
  OCK(cudaMemsetAsync(level, 0xff, sizeof(int) * N, s));
  OCK(cudaMemsetAsync(key, 0xff, sizeof(unsigned long long) * N, s));
  k_row_offsets<<<nblk, kOT, 0, s>>>(T.meta, T.tile_off, N, row_off), lgt::note_launch();
  OCK(cudaGetLastError());
  // searches from the first unplaced row until every row is placed
  int64_t placed = 0;
  int L = 0, seed = 0, searches = 0;
  while (placed < N) {
    k_seed<<<1, 1, 0, s>>>(perm, iperm, level, placed, seed, L), lgt::note_launch();
    int64_t p0 = placed, p1 = placed + 1;
    while (p1 > p0) {  // each level places at least one row or ends the search
      const unsigned nb = unsigned((p1 - p0 + kOT - 1) / kOT);
      k_bfs_claim<<<nb, kOT, 0, s>>>(T.meta, row_off, T.nbr, perm, p0, p1, L, level, key),
          lgt::note_launch();
      k_bfs_count<<<nb, kOT, 0, s>>>(T.meta, row_off, T.nbr, perm, p0, p1, L, level, key, count),
          lgt::note_launch();
      std::string e = scan_counts(count, p1 - p0, off, total, s);
      if (!e.empty()) return e;
      k_bfs_place<<<nb, kOT, 0, s>>>(T.meta, row_off, T.nbr, perm, iperm, p0, p1, L, level, key,
                                      off, N), lgt::note_launch();
      OCK(cudaGetLastError());
      uint32_t nt = 0;
      OCK(cudaMemcpyAsync(&nt, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      OCK(cudaStreamSynchronize(s));
      if (int64_t(nt) > N - p1) return "row ordering overran the basis";
      p0 = p1;
      p1 += int64_t(nt);
      ++L;
    }
    placed = p1;
    if (placed >= N) break;
    if (++searches >= kMaxSearches) {
      // rows no search has reached by now go last, in index order
      k_unplaced_flags<<<nblk, kOT, 0, s>>>(level, N, count), lgt::note_launch();
      std::string e = scan_counts(count, N, off, total, s);
      if (!e.empty()) return e;
      k_place_unplaced<<<nblk, kOT, 0, s>>>(level, N, off, placed, perm, iperm),
          lgt::note_launch();
      OCK(cudaGetLastError());
      placed = N;
      break;
    }
    int h = INT_MAX;
    OCK(cudaMemcpyAsync(first, &h, sizeof(int), cudaMemcpyHostToDevice, s));
    k_first_unplaced<<<nblk, kOT, 0, s>>>(level, N, first), lgt::note_launch();
    OCK(cudaMemcpyAsync(&h, first, sizeof(int), cudaMemcpyDeviceToHost, s));
    OCK(cudaStreamSynchronize(s));
    if (h == INT_MAX) return "row ordering lost rows";
    seed = h;
    ++L;
  }
  {
    std::string e = renumber(T, perm, iperm, row_off, T2, s);
    if (!e.empty()) return e;
  }
  OCK(dev_free(level, s));
  OCK(dev_free(key, s));
  OCK(dev_free(row_off, s));
  OCK(dev_free(count, s));
  OCK(dev_free(off, s));
  OCK(dev_free(total, s));
  OCK(dev_free(first, s));
  OCK(cudaStreamSynchronize(s));
  finish(T, T2);
  return std::string();
}
std::string build_table_mask_order(const NbrTable& T, const Geom& G, const RankView& R,
                                   NbrTable* T2, cudaStream_t s) {
  const int64_t N = T.N;
  if (T.state != 1 || N <= 0) return "no neighbour table to reorder";
  if (G.ns > 26) return "too many sites for the host mask search";
  free_nbr_table(T2);
  // the sector's masks, ascending (the segment order of the basis)
  std::vector<uint32_t> masks;
  for (uint32_t m = 0; m < (1u << G.ns); ++m)
    if (__builtin_popcount(m) == G.nf_target) masks.push_back(m);
  if (int64_t(masks.size()) != int64_t(R.nmasks)) return "mask count differs from the basis";
  std::vector<uint32_t> segc(masks.size() + 1);
  OCK(cudaMemcpyAsync(segc.data(), R.segc, sizeof(uint32_t) * segc.size(),
                      cudaMemcpyDeviceToHost, s));
  OCK(cudaStreamSynchronize(s));
  // bonds (site pairs) of the lattice: a hop across one moves a fermion
  std::vector<std::pair<int, int>> bonds;
  for (int iy = 0; iy < G.ny; ++iy)
    for (int ix = 0; ix + 1 < G.nx; ++ix) bonds.push_back({iy * G.nx + ix, iy * G.nx + ix + 1});
  for (int iy = 0; iy + 1 < G.ny; ++iy)
    for (int ix = 0; ix < G.nx; ++ix) bonds.push_back({iy * G.nx + ix, (iy + 1) * G.nx + ix});
  const size_t M = masks.size();
  std::vector<int> order;
  order.reserve(M);
  std::vector<char> seen(M, 0);
  for (size_t start = 0; start < M; ++start) {  // every component, first mask first
    if (seen[start]) continue;
    seen[start] = 1;
    size_t head = order.size();
    order.push_back(int(start));
    while (head < order.size()) {
      const uint32_t m = masks[order[head++]];
      for (const auto& b : bonds) {
        const uint32_t ba = 1u << b.first, bb = 1u << b.second;
        if (((m & ba) != 0) == ((m & bb) != 0)) continue;
        const uint32_t n = m ^ ba ^ bb;
        const size_t q = size_t(std::lower_bound(masks.begin(), masks.end(), n) - masks.begin());
        if (q < M && masks[q] == n && !seen[q]) {
          seen[q] = 1;
          order.push_back(int(q));
        }
      }
    }
  }
  std::vector<int> hperm;
  hperm.reserve(size_t(N));
  for (int q : order)
    for (uint32_t r = segc[q]; r < segc[q + 1]; ++r) hperm.push_back(int(r));
  if (int64_t(hperm.size()) != N) return "mask segments do not cover the basis";
  int *perm = nullptr, *iperm = nullptr;
  uint32_t* row_off = nullptr;
  OCK(cudaMalloc(&perm, sizeof(int) * N));
  T2->perm = perm;
  OCK(cudaMalloc(&iperm, sizeof(int) * N));
  T2->iperm = iperm;
  OCK(cudaMemcpyAsync(perm, hperm.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s));
  const unsigned nblk = unsigned((N + kOT - 1) / kOT);
  k_invert<<<nblk, kOT, 0, s>>>(perm, N, iperm), lgt::note_launch();
  OCK(dev_alloc_n(&row_off, size_t(N), s));
  k_row_offsets<<<nblk, kOT, 0, s>>>(T.meta, T.tile_off, N, row_off), lgt::note_launch();
  OCK(cudaGetLastError());
  std::string e = renumber(T, perm, iperm, row_off, T2, s);
  if (!e.empty()) return e;
  OCK(dev_free(row_off, s));
  OCK(cudaStreamSynchronize(s));
  finish(T, T2);
  return std::string();
}

}  // namespace lgt
