// Gram products of the streamed VarPro normal equations on the tcgen05 tensor cores,
// in split-BF16x3 arithmetic with FP32 accumulation in tensor memory.
//
// Every FP32 value x is split as x = hi + lo (two bf16 values, ~16 significant bits);
// a product is hi*hi' + hi*lo' + lo*hi' (the lo*lo' term is below 2^-16 relative).
// The projected design rows are stored transposed and split, PT_hi / PT_lo
// [n_pad, k_pad] bf16 with the reduction index contiguous (K-major), so that both
// operands of G = PT PT^T are K-major tiles that TMA loads with 128-byte swizzling.
//
// One CTA owns one 128 x 128 tile of the upper triangle and a contiguous range of
// 64-element K stages: warp 0 issues TMA loads into a 3-stage shared-memory ring,
// warp 1 issues 12 tcgen05.mma (M=128, N=128, K=16) per stage into a TMEM
// accumulator, and warps 2-5 read the accumulator (tcgen05.ld), transpose each 32 x 32
// block through shared memory and store it with the lanes along the columns: with one
// K split the block is added to the FP64 output directly (one writer per element), with
// several each split writes its FP32 tile to a slab and gram_reduce_kernel adds the
// splits in ascending order, so the result is bitwise reproducible. Every mbarrier wait
// is bounded: a wait that runs out sets the status word, drains the TMA copies it
// issued, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include "dsplat_gb300.h"
#include "tc.cuh"

void dsg_count_launches(int kernels);

namespace {

constexpr int BM = 128, BN = 128, BK = 64;   // tile rows, tile columns, bf16 per stage row
constexpr int STAGES = 3;
constexpr int TILE_BYTES = BM * BK * 2;      // 16 KiB per operand tile (128 rows x 128 B)
constexpr int STAGE_BYTES = 4 * TILE_BYTES;  // A_hi, A_lo, B_hi, B_lo
constexpr int THREADS = 192;
constexpr uint32_t TMEM_COLS = 128;
constexpr uint32_t IDESC = tc::idesc_bf16(BM, BN);
using namespace tc;

__global__ void __launch_bounds__(THREADS, 1)
    gram_bf16x3_kernel(const __grid_constant__ CUtensorMap map_hi,
                       const __grid_constant__ CUtensorMap map_lo, int tiles_per_side,
                       int tile_from, int stages_total, int k_splits, double* __restrict__ out,
                       int n, int ldo, float* __restrict__ slab, int* __restrict__ status) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  // Tile (ti, tj) of this CTA: every upper-triangle tile (ti <= tj) whose column tile
  // is at least tile_from; rows above tile_from first, then the remaining triangle.
  const int band = tiles_per_side - tile_from;
  int ti, tj;
  if ((int)blockIdx.x < tile_from * band) {
    ti = blockIdx.x / band;
    tj = tile_from + blockIdx.x % band;
  } else {
    int rem = blockIdx.x - tile_from * band, per_row = band;
    ti = tile_from;
    while (rem >= per_row) {
      rem -= per_row;
      ++ti;
      --per_row;
    }
    tj = ti + rem;
  }
  const bool diag = ti == tj;
  const int s_begin = (int)((int64_t)blockIdx.y * stages_total / k_splits);
  const int s_end = (int)((int64_t)(blockIdx.y + 1) * stages_total / k_splits);
  const int nst = s_end - s_begin;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (nst > 0) {
    if (warp == 0 && lane == 0) {  // TMA producer
      int issued = 0;
      for (int it = 0; it < nst; ++it) {
        const int s = it % STAGES;
        if (it >= STAGES && !mbar_wait(&empty[s], ((it / STAGES) - 1) & 1, abort)) {
          *abort = 1;
          break;
        }
        uint8_t* base = smem + s * STAGE_BYTES;
        mbar_expect_tx(&full[s], diag ? 2 * TILE_BYTES : 4 * TILE_BYTES);
        const int kx = (s_begin + it) * BK;
        tma_load_2d(base, &map_hi, kx, ti * BM, &full[s]);
        tma_load_2d(base + TILE_BYTES, &map_lo, kx, ti * BM, &full[s]);
        if (!diag) {
          tma_load_2d(base + 2 * TILE_BYTES, &map_hi, kx, tj * BN, &full[s]);
          tma_load_2d(base + 3 * TILE_BYTES, &map_lo, kx, tj * BN, &full[s]);
        }
        ++issued;
      }
      if (*abort) {  // let the copies already in flight land before the CTA retires
        for (int it = issued > STAGES ? issued - STAGES : 0; it < issued; ++it)
          mbar_wait_plain(&full[it % STAGES], (it / STAGES) & 1);
      }
    } else if (warp == 1 && lane == 0) {  // MMA issuer
      bool ok = true;
      for (int it = 0; it < nst; ++it) {
        const int s = it % STAGES;
        if (!mbar_wait(&full[s], (it / STAGES) & 1, abort)) {
          *abort = 1;
          ok = false;
          break;
        }
        tc_fence_after();
        uint8_t* base = smem + s * STAGE_BYTES;
        const uint32_t a_hi = smem_u32(base), a_lo = smem_u32(base + TILE_BYTES);
        const uint32_t b_hi = diag ? a_hi : smem_u32(base + 2 * TILE_BYTES);
        const uint32_t b_lo = diag ? a_lo : smem_u32(base + 3 * TILE_BYTES);
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
          const uint32_t off = kk * 32;  // 16 bf16 = 32 bytes along K inside the swizzle atom
          umma_bf16(tmem, sw128_desc(a_hi + off), sw128_desc(b_hi + off), IDESC, (it | kk) != 0);
          umma_bf16(tmem, sw128_desc(a_hi + off), sw128_desc(b_lo + off), IDESC, 1u);
          umma_bf16(tmem, sw128_desc(a_lo + off), sw128_desc(b_hi + off), IDESC, 1u);
        }
        umma_commit(&empty[s]);
      }
      if (ok) umma_commit(done);
    } else if (warp >= 2) {  // epilogue: TMEM -> transpose in shared memory -> FP64 output / slab
      const bool ok = mbar_wait(done, 0, abort);
      tc_fence_after();
      if (ok) {
        const int q = warp & 3;  // TMEM lanes 32 q .. 32 q + 31 (the warp's accessible quarter)
        // the stage ring is idle once every MMA finished: reuse it, 32 x 33 floats per warp
        float* block = reinterpret_cast<float*>(smem) + q * 32 * 33;
        const int row0 = 32 * q;
        for (int c0 = 0; c0 < BN; c0 += 32) {
          uint32_t v[32];
          tmem_ld32(tmem + ((uint32_t)row0 << 16) + (uint32_t)c0, v);
#pragma unroll
          for (int j = 0; j < 32; ++j) block[lane * 33 + j] = __uint_as_float(v[j]);  // row lane, column j
          __syncwarp();
          const int gj = tj * BN + c0 + lane;
          if (k_splits == 1) {
            for (int r = 0; r < 32; ++r) {
              const int gi = ti * BM + row0 + r;
              if (gi < n && gj < n) out[(size_t)gi * ldo + gj] += (double)block[r * 33 + lane];
            }
          } else {
            float* tile = slab + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * (BM * BN);
            for (int r = 0; r < 32; ++r) tile[(row0 + r) * BN + c0 + lane] = block[r * 33 + lane];
          }
          __syncwarp();
        }
      } else {
        *abort = 1;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
  }
  if (threadIdx.x == 0 && *abort) atomicExch(status, 1);
}

// out[tile] += sum over splits s = 0, 1, ... of slab[s][tile], in that order, in FP64.
// Grid (tiles, BM / 8): a CTA adds 8 rows of one tile, a thread per column.
__global__ void __launch_bounds__(BN) gram_reduce_kernel(const float* __restrict__ slab, int tiles, int k_splits,
                                                         int tiles_per_side, int tile_from, double* __restrict__ out,
                                                         int n, int ldo) {
  const int pair = blockIdx.x;
  const int band = tiles_per_side - tile_from;
  int ti, tj;
  if (pair < tile_from * band) {
    ti = pair / band;
    tj = tile_from + pair % band;
  } else {
    int rem = pair - tile_from * band, per_row = band;
    ti = tile_from;
    while (rem >= per_row) {
      rem -= per_row;
      ++ti;
      --per_row;
    }
    tj = ti + rem;
  }
  const int c = threadIdx.x;
  const int gj = tj * BN + c;
  for (int r = blockIdx.y * 8; r < blockIdx.y * 8 + 8; ++r) {
    const int gi = ti * BM + r;
    double sum = 0.0;
    for (int split = 0; split < k_splits; ++split)
      sum += (double)slab[((size_t)split * tiles + pair) * (BM * BN) + r * BN + c];
    if (gi < n && gj < n) out[(size_t)gi * ldo + gj] += sum;
  }
}

// rows [m, n] FP32 -> hi/lo [.., ld] bf16 transposed, at column offset col0.
__global__ void split_transpose_kernel(const float* __restrict__ rows, int64_t m, int n,
                                       int64_t col0, __nv_bfloat16* __restrict__ hi,
                                       __nv_bfloat16* __restrict__ lo, int64_t ld) {
  __shared__ float tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  const int s0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t r = r0 + i;
    const int s = s0 + threadIdx.x;
    tile[i][threadIdx.x] = (r < m && s < n) ? rows[r * n + s] : 0.0f;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int s = s0 + i;
    const int64_t r = r0 + threadIdx.x;
    if (s < n && r < m) {
      const float x = tile[threadIdx.x][i];
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
      hi[(int64_t)s * ld + col0 + r] = h;
      lo[(int64_t)s * ld + col0 + r] = l;
    }
  }
}

std::mutex g_map_mutex;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool encode_fn() {
  std::lock_guard<std::mutex> lock(g_map_mutex);
  if (g_encode) return true;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                       &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || fn == nullptr)
    return false;
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return true;
}

bool make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols) {
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {BK, BM};
  const cuuint32_t estr[2] = {1, 1};
  return g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

extern "C" {

int dsg_split_transpose_bf16(const float* rows, int64_t m, int32_t n, int64_t column_offset,
                             void* hi, void* lo, int64_t ld, void* stream) {
  if (m < 0 || n < 0 || column_offset < 0 || ld < column_offset + m) return DSG_ERR_ARGUMENT;
  if (m == 0 || n == 0) return DSG_OK;
  if (!rows || !hi || !lo) return DSG_ERR_ARGUMENT;
  dim3 grid((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
  split_transpose_kernel<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(
      rows, m, n, column_offset, reinterpret_cast<__nv_bfloat16*>(hi),
      reinterpret_cast<__nv_bfloat16*>(lo), ld);
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

// Tiles of the upper triangle whose column tile is at least column_from's.
static int gram_pairs(int n_pad, int column_from) {
  const int tiles = n_pad / BM, tile_from = column_from / BN, band = tiles - tile_from;
  return tile_from * band + band * (band + 1) / 2;
}

size_t dsg_gram_bf16x3_workspace_bytes(int32_t n_pad, int64_t k_pad, int32_t column_from, int32_t k_splits) {
  if (n_pad <= 0 || n_pad % BM != 0 || k_pad <= 0 || column_from < 0 || column_from > n_pad || k_splits < 1)
    return 0;
  const int64_t stages = k_pad / BK;
  const int splits = (int)(k_splits > stages ? stages : k_splits);
  if (splits <= 1) return 0;
  return (size_t)splits * gram_pairs(n_pad, column_from) * BM * BN * sizeof(float);
}

int dsg_gram_bf16x3(const void* hi, const void* lo, int32_t n, int32_t n_pad, int64_t k_pad,
                    int32_t column_from, int32_t k_splits, double* out, int32_t ldo, void* workspace,
                    size_t workspace_bytes, int32_t* status, void* stream) {
  if (n < 0 || n_pad < n || n_pad % BM != 0 || k_pad < 0 || k_pad % BK != 0 || ldo < n ||
      column_from < 0 || column_from > n)
    return DSG_ERR_ARGUMENT;
  if (n == 0 || k_pad == 0) return DSG_OK;
  if (!hi || !lo || !out || !status || k_splits < 1) return DSG_ERR_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(hi) | reinterpret_cast<uintptr_t>(lo)) & 15u) return DSG_ERR_ARGUMENT;
  if (k_pad > (int64_t)0x7fffffff) return DSG_ERR_ARGUMENT;  // TMA coordinates are int32
  if (!encode_fn()) return DSG_ERR_LIBRARY;
  CUtensorMap map_hi, map_lo;
  if (!make_map(&map_hi, hi, n_pad, k_pad) || !make_map(&map_lo, lo, n_pad, k_pad))
    return DSG_ERR_ARGUMENT;
  const int tiles = n_pad / BM;
  const int tile_from = column_from / BN;
  const int pairs = gram_pairs(n_pad, column_from);
  const int stages = (int)(k_pad / BK);
  if (k_splits > stages) k_splits = stages;
  const size_t need = dsg_gram_bf16x3_workspace_bytes(n_pad, k_pad, column_from, k_splits);
  if (need > 0 && (workspace == nullptr || workspace_bytes < need)) return DSG_ERR_WORKSPACE;
  const size_t smem = (size_t)STAGES * STAGE_BYTES + 1024 + 256;
  if (cudaFuncSetAttribute(gram_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return DSG_ERR_LAUNCH;
  dim3 grid(pairs, k_splits);
  cudaStream_t st = (cudaStream_t)stream;
  float* slab = reinterpret_cast<float*>(workspace);
  gram_bf16x3_kernel<<<grid, THREADS, smem, st>>>(map_hi, map_lo, tiles, tile_from, stages, k_splits, out, n, ldo,
                                                  slab, status);
  dsg_count_launches(1);
  if (cudaGetLastError() != cudaSuccess) return DSG_ERR_LAUNCH;
  if (k_splits > 1) {
    gram_reduce_kernel<<<dim3(pairs, BM / 8), BN, 0, st>>>(slab, pairs, k_splits, tiles, tile_from, out, n, ldo);
    dsg_count_launches(1);
  }
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // extern "C"
