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
// accumulator, and warps 2-5 read the accumulator (tcgen05.ld) and add it to the
// FP64 output with atomics. Every mbarrier wait is bounded: a wait that runs out sets
// the status word, drains the TMA copies it issued, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

constexpr int BM = 128, BN = 128, BK = 64;   // tile rows, tile columns, bf16 per stage row
constexpr int STAGES = 3;
constexpr int TILE_BYTES = BM * BK * 2;      // 16 KiB per operand tile (128 rows x 128 B)
constexpr int STAGE_BYTES = 4 * TILE_BYTES;  // A_hi, A_lo, B_hi, B_lo
constexpr int THREADS = 192;
constexpr uint32_t SPIN_LIMIT = 1u << 24;
constexpr uint32_t TMEM_COLS = 128;
// kind::f16 instruction descriptor: FP32 accumulate, BF16 A and B, both K-major, N, M.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait that ignores the abort flag (used to drain copies already in flight).
__device__ __forceinline__ bool mbar_wait_plain(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < SPIN_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Bounded wait; false when the limit ran out or another role gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
  for (uint32_t i = 0; i < SPIN_LIMIT; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && *abort) return false;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor of a K-major tile with 128-byte swizzling: rows of
// 128 B, 8-row atoms 1024 B apart (SBO); LBO is unused for this layout.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__global__ void __launch_bounds__(THREADS, 1)
    gram_bf16x3_kernel(const __grid_constant__ CUtensorMap map_hi,
                       const __grid_constant__ CUtensorMap map_lo, int tiles_per_side,
                       int tile_from, int stages_total, int k_splits, double* __restrict__ out,
                       int n, int ldo, int* __restrict__ status) {
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
          umma_bf16(tmem, sw128_desc(a_hi + off), sw128_desc(b_hi + off), (it | kk) != 0);
          umma_bf16(tmem, sw128_desc(a_hi + off), sw128_desc(b_lo + off), 1u);
          umma_bf16(tmem, sw128_desc(a_lo + off), sw128_desc(b_hi + off), 1u);
        }
        umma_commit(&empty[s]);
      }
      if (ok) umma_commit(done);
    } else if (warp >= 2) {  // epilogue: TMEM -> FP64 output
      const bool ok = mbar_wait(done, 0, abort);
      tc_fence_after();
      if (ok) {
        const int q = warp & 3;
        const int gi = ti * BM + 32 * q + lane;
        for (int c0 = 0; c0 < BN; c0 += 32) {
          uint32_t v[32];
          tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
          if (gi < n) {
            double* row = out + (size_t)gi * ldo;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int gj = tj * BN + c0 + j;
              if (gj < n) atomicAdd(row + gj, (double)__uint_as_float(v[j]));
            }
          }
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

int dsg_gram_bf16x3(const void* hi, const void* lo, int32_t n, int32_t n_pad, int64_t k_pad,
                    int32_t column_from, int32_t k_splits, double* out, int32_t ldo,
                    int32_t* status, void* stream) {
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
  const int band = tiles - tile_from;
  const int pairs = tile_from * band + band * (band + 1) / 2;
  const int stages = (int)(k_pad / BK);
  if (k_splits > stages) k_splits = stages;
  const size_t smem = (size_t)STAGES * STAGE_BYTES + 1024 + 256;
  if (cudaFuncSetAttribute(gram_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return DSG_ERR_LAUNCH;
  dim3 grid(pairs, k_splits);
  gram_bf16x3_kernel<<<grid, THREADS, smem, (cudaStream_t)stream>>>(
      map_hi, map_lo, tiles, tile_from, stages, k_splits, out, n, ldo, status);
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // extern "C"
