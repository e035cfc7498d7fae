// nbr_table_bulk.cu -- H*psi from the stored neighbour table with the
// neighbour rows gathered by the copy engine (TMA tile::gather4) instead of
// per-lane loads.
//
// The table kernel is bound by the L1/TEX load pipe: a gather instruction
// touches one 64-byte x row per four lanes, 64 useful bytes per wavefront.
// Here each warp stages a 32-row tile's neighbour lists in shared memory as
// the table kernel does, then, eight rows at a time, lets the copy engine
// bring every neighbour row into shared memory: one
// cp.async.bulk.tensor.2d ... tile::gather4 per four neighbour rows (a
// two-dimensional tensor map over the panel, rows of C floats, one-row
// boxes), completed on an mbarrier per buffer.  Two buffers per warp: the
// gathers of the next eight rows are in flight while these are summed.
// The sums read shared memory at 128 bytes per wavefront.  Row r's slots
// are padded to a multiple of four with r itself (gathered, never added).
//
// FP32 panels of 16 columns (8 complex or 16 real coupling points), the
// stored table in either row order, any model.  Measured on the 4x4 K = 8
// complex panel: 2.34 ms against 0.71 ms for the lane-gathering table
// kernel -- 25.7 M four-row gathers a launch, about one per 28 SM cycles,
// so the copy engine, not the load pipe, sets the pace for rows this short.
// It is therefore not an autotuner candidate (LGT_HPSI_VARIANT=8 runs it).  A gather that does not
// arrive within the bounded wait raises kDevErrSpin; the warp then waits,
// bounded, for the gathers it issued and leaves.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "lgt_bulk.cuh"
#include "lgt_hpsi.h"

namespace lgt {

namespace {

constexpr int kGWarps = 4;                  // warps per block
constexpr int kGThreads = kGWarps * 32;
constexpr int kGChunk = 8;                  // rows per gather round
constexpr int kGC = 16;                     // panel columns (floats per row)

__device__ __forceinline__ int warp_incl_scan_g(int v, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += u;
  }
  return v;
}

__device__ __forceinline__ void gather4(float* dst, const CUtensorMap* tm, int x, int y0, int y1,
                                        int y2, int y3, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(tm), "r"(x), "r"(y0), "r"(y1), "r"(y2), "r"(y3), "r"(smem_u32(bar))
      : "memory");
}

// Shared memory of a block: per warp 32 meta words, 32 list offsets, the
// tile's list (32 * mm entries), two buffers of kGChunk rows * ms4 slots *
// kGC floats, two mbarriers; the coefficients first.
__host__ __device__ inline size_t bulk_warp_bytes(int mm) {
  const int ms4 = (mm + 3) & ~3;
  const size_t b = size_t(2 * kGChunk) * ms4 * kGC * 4 + size_t(32) * mm * 4 + 32 * 4 * 2 + 16;
  return (b + 127) / 128 * 128;  // the next warp's buffers start 128-byte aligned
}

template <bool PLAQ, bool JW>
__global__ void __launch_bounds__(kGThreads) k_hpsi_table_bulk(HpsiArgs<float> a,
                                                              const __grid_constant__ CUtensorMap tmx,
                                                              int64_t xrows_per_slot) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int K = a.K;
  float* s_coef = reinterpret_cast<float*>(smem);  // [4][K]
  for (int i = threadIdx.x; i < K; i += kGThreads) {
    s_coef[i] = a.cE[i];
    s_coef[K + i] = a.cm[i];
    s_coef[2 * K + i] = a.ch[i];
    s_coef[3 * K + i] = a.cp[i];
  }
  const int mm = a.t_mm, ms4 = (mm + 3) & ~3;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const size_t coef_bytes = (size_t(4) * K * 4 + 127) / 128 * 128;
  unsigned char* wbase = smem + coef_bytes + size_t(wid) * bulk_warp_bytes(mm);
  float* buf0 = reinterpret_cast<float*>(wbase);  // [2][kGChunk][ms4][kGC]
  const size_t bufsz = size_t(kGChunk) * ms4 * kGC;
  uint32_t* s_list = reinterpret_cast<uint32_t*>(buf0 + 2 * bufsz);
  uint32_t* s_meta = s_list + 32 * mm;
  uint32_t* s_off = s_meta + 32;
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_off + 32);
  if (lane == 0) {
    mbar_init(s_bar, 1);
    mbar_init(s_bar + 1, 1);
    mbar_init_fence();
  }
  __syncthreads();  // coefficients and barriers

  const int64_t warp_row0 = (int64_t(blockIdx.x) * kGWarps + wid) * 32;
  if (warp_row0 >= a.N) return;
  const int64_t row = warp_row0 + lane;
  const uint32_t m = (row < a.N) ? __ldcs(a.t_meta + row) : 0u;
  const int cnt = int(m & 255u);
  const int incl = warp_incl_scan_g(cnt, lane);
  s_meta[lane] = m;
  s_off[lane] = uint32_t(incl - cnt);
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const uint32_t* src = a.t_nbr + __ldg(a.t_off + (warp_row0 >> 5));
  for (int i = lane; i < total; i += 32) s_list[i] = __ldcs(src + i);
  __syncwarp();

  // the panel's first row in the tensor (the Krylov slot of a.xsel)
  const int64_t slot = a.xsel ? int64_t(*a.xsel) : 0;
  const int ybase = int(slot * xrows_per_slot);
  const float* x = a.x + (a.xsel ? size_t(slot) * a.xstride : 0);

  // gathers of chunk c (rows 8c .. 8c + 7 of the tile) into buffer c & 1
  auto issue = [&](int c) {
    float* buf = buf0 + size_t(c & 1) * bufsz;
    const int rl = c * kGChunk + lane;
    int ng = 0;
    if (lane < kGChunk) ng = (int(s_meta[rl] & 255u) + 3) >> 2;
    int tot = ng;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0) mbar_arrive_expect_tx(s_bar + (c & 1), uint32_t(tot) * 4u * kGC * 4u);
    __syncwarp();
    if (lane < kGChunk) {
      const int cntr = int(s_meta[rl] & 255u);
      const uint32_t* lst = s_list + s_off[rl];
      const int own = int(warp_row0) + rl;  // padding slots gather the row itself
      for (int g = 0; g < ng; ++g) {
        int yq[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int sl = 4 * g + q;
          yq[q] = ybase + ((sl < cntr) ? int(lst[sl] & 0x7fffffffu) : own);
        }
        gather4(buf + (size_t(lane) * ms4 + 4 * g) * kGC, &tmx, 0, yq[0], yq[1], yq[2], yq[3],
                s_bar + (c & 1));
      }
    }
  };

  constexpr int nchunk = 32 / kGChunk;
  issue(0);
  issue(1);
  bool bad = false;
  int c = 0;
  for (; c < nchunk; ++c) {
    if (!mbar_wait_bounded(s_bar + (c & 1), uint32_t(c >> 1) & 1u)) bad = true;
    if (__any_sync(0xffffffffu, bad)) {
      bad = true;
      break;
    }
    const float* buf = buf0 + size_t(c & 1) * bufsz;
    // lane: row c * 8 + lane / 4, columns 4 (lane % 4) .. + 3
    const int rl = c * kGChunk + (lane >> 2);
    const int col0 = (lane & 3) * 4;
    const uint32_t mr = s_meta[rl];
    const int cntr = int(mr & 255u), nh = int((mr >> 8) & 255u);
    int cmax = cntr;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cmax = max(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
    const uint32_t* lst = s_list + s_off[rl];
    float4 ah = make_float4(0.f, 0.f, 0.f, 0.f), ap = ah;
    const float* rb = buf + size_t(lane >> 2) * ms4 * kGC + col0;
    for (int sl = 0; sl < cmax; ++sl) {
      if (sl < cntr) {
        const float4 v = *reinterpret_cast<const float4*>(rb + size_t(sl) * kGC);
        if (sl < nh) {
          if (JW && (lst[sl] >> 31)) {
            ah.x -= v.x;
            ah.y -= v.y;
            ah.z -= v.z;
            ah.w -= v.w;
          } else {
            ah.x += v.x;
            ah.y += v.y;
            ah.z += v.z;
            ah.w += v.w;
          }
        } else if (PLAQ) {
          ap.x += v.x;
          ap.y += v.y;
          ap.z += v.z;
          ap.w += v.w;
        }
      }
    }
    const int64_t r = warp_row0 + rl;
    if (r < a.N) {
      const float4 xd = *reinterpret_cast<const float4*>(x + size_t(r) * kGC + col0);
      const float e2 = float(int((mr >> 16) & 255u)), stag = float(int(mr >> 24) - 128);
      float o[4];
      const float xv[4] = {xd.x, xd.y, xd.z, xd.w}, hv[4] = {ah.x, ah.y, ah.z, ah.w},
                  pv[4] = {ap.x, ap.y, ap.z, ap.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int k = (col0 + e) / a.ncomp;
        const float cd = s_coef[k] * e2 + s_coef[K + k] * stag;
        float v = fmaf(s_coef[2 * K + k], hv[e], cd * xv[e]);
        if (PLAQ) v = fmaf(s_coef[3 * K + k], pv[e], v);
        o[e] = v;
      }
      __stcs(reinterpret_cast<float4*>(a.y + size_t(r) * kGC + col0),
             make_float4(o[0], o[1], o[2], o[3]));
    }
    __syncwarp();  // the buffer is free once every lane has read it
    if (c + 2 < nchunk) issue(c + 2);
  }
  if (bad) {
    // gathers issued and not consumed: chunks c .. min(c + 1, nchunk - 1)
    if (lane == 0) {
      for (int cc = c; cc < nchunk && cc < c + 2; ++cc)
        mbar_wait_bounded(s_bar + (cc & 1), uint32_t(cc >> 1) & 1u);
      if (a.err) atomicOr(a.err, kDevErrSpin);
    }
    __syncwarp();
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

}  // namespace

bool table_bulk_applies(const HpsiArgs<float>& a, int64_t x_rows) {
  const int64_t per_slot = a.xsel ? int64_t(a.xstride / kGC) : a.N;
  return a.t_meta && a.C == kGC && (a.xsel == nullptr || a.xstride % kGC == 0) &&
         (reinterpret_cast<uintptr_t>(a.x) & 15) == 0 && (reinterpret_cast<uintptr_t>(a.y) & 15) == 0 &&
         a.t_mm >= 1 && a.t_mm <= 32 && x_rows >= a.N && x_rows < (int64_t(1) << 31) &&
         per_slot >= a.N && encode_fn() != nullptr;
}

cudaError_t launch_table_bulk(const HpsiArgs<float>& a, uint32_t model, int64_t x_rows,
                              cudaStream_t s) {
  if (!table_bulk_applies(a, x_rows)) return cudaErrorInvalidValue;
  CUtensorMap tm;
  const cuuint64_t gdim[2] = {cuuint64_t(kGC), cuuint64_t(x_rows)};
  const cuuint64_t gstride[1] = {cuuint64_t(kGC) * 4};
  const cuuint32_t box[2] = {cuuint32_t(kGC), 1};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode_fn()(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                 const_cast<float*>(a.x), gdim, gstride, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  const int64_t per_slot = a.xsel ? int64_t(a.xstride / kGC) : a.N;
  const size_t coef_bytes = (size_t(4) * a.K * 4 + 127) / 128 * 128;
  const size_t bytes = coef_bytes + size_t(kGWarps) * bulk_warp_bytes(a.t_mm);
  const int64_t blocks = (a.N + kGThreads - 1) / kGThreads;
  if (blocks <= 0) return cudaSuccess;
  const bool plaq = model & kModelPlaq, jw = model & kModelJW;
  auto go = [&](auto kern) -> cudaError_t {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), int(bytes));
    if (e != cudaSuccess) return e;
    kern<<<unsigned(blocks), kGThreads, bytes, s>>>(a, tm, per_slot), lgt::note_launch();
    return cudaGetLastError();
  };
  if (plaq && jw) return go(k_hpsi_table_bulk<true, true>);
  if (plaq) return go(k_hpsi_table_bulk<true, false>);
  if (jw) return go(k_hpsi_table_bulk<false, true>);
  return go(k_hpsi_table_bulk<false, false>);
}

}  // namespace lgt
