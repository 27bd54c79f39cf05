// Dictionary rows generated on chip and projected onto the row basis on the tcgen05
// tensor cores: the mixed-precision replacement of design_bins + RowBasis.reduce_major
// (reference: dsplat/kernels/surfel.slang:313-378 and dsplat/fmcw.py:128-131, 276-294).
//
// For one aperture a and a tile of 128 surfels, the real dictionary column of each surfel,
// v[2k + part] = (re, im) of sqrt(area) c D(k - k0), is evaluated in the cotangent form of
// common.cuh straight into shared memory, split into bf16 hi + lo, and multiplied by the
// interleaved basis U [rank2, 2K] (also split, zero padded to N = rank2 rounded up to 32
// rows) with three tcgen05.mma products per K step (hi.hi, lo.hi, hi.lo): the tile is the
// M = 128 operand, U the N operand, so the tensor work scales with the basis rank. The
// projected values P[s, a rank2 + rho] = (U v_s)[rho] leave the tensor memory split and
// already in the layout of the Gram operand PT_hi / PT_lo [S, ld]: the design matrix never
// touches HBM.
//
// CTA of 21 warps, persistent over work units of (aperture, 256 surfels):
//   warps 0-15  geometry of the unit's 256 pairs (one per thread of warps 0-7), then the
//               dictionary tiles, one K-subtile (32 bins of 128 surfels, 8 surfels per
//               warp, four bins per lane) per pipeline stage;
//   warps 16-19 epilogue: tcgen05.ld of a finished accumulator, bf16 split, a transpose
//               through shared memory, and row-contiguous stores of PT;
//   warp 20     TMEM allocation, the TMA copy of U, and the MMA issue (one thread).
// Stages and accumulators are rings guarded by mbarriers; every wait is bounded and a
// wait that runs out raises the status word instead of hanging.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include "common.cuh"
#include "tc.cuh"

using namespace dsg;
using namespace tc;

namespace {

constexpr int TM = 128;                    // MMA M: surfels per tile
constexpr int UNIT = 256;                  // surfels per work unit (two tiles)
constexpr int NPROD = 512;                 // producer threads (warps 0-15)
constexpr int ROWS_PER_WARP = TM / (NPROD / 32);
constexpr int EPI_WARP = NPROD / 32;       // first of the four epilogue warps
constexpr int MMA_WARP = EPI_WARP + 4;
constexpr int PTHREADS = (MMA_WARP + 1) * 32;
constexpr int A_SUB = TM * 128;            // one [128 x 64] bf16 K-subtile: 16 KiB
constexpr int STAGE_BYTES = 2 * A_SUB;     // hi + lo
constexpr int MAX_STAGES = 4;
constexpr int XPOSE_WORDS = 2 * 32 * 17 + 16;  // per epilogue warp: hi [32][17], lo [32][17]
constexpr int SMEM_LIMIT = 227 * 1024;

__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t (&v)[32]) {
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

// Named barrier over `count` threads that also returns the OR of every thread's predicate.
__device__ __forceinline__ bool bar_or(int id, int count, bool pred) {
  uint32_t out;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(out)
      : "r"((uint32_t)pred), "r"(id), "r"(count)
      : "memory");
  return out != 0;
}

__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) {
  return *reinterpret_cast<uint32_t*>(&v);
}

// Shared-memory plan of one CTA; identical on host and device.
struct Plan {
  int nsub;        // K-subtiles of 64 elements: 2K / 64
  int ncols;       // N: rank2 rounded up to 32
  int stages;      // pipeline depth
  int u_bytes;     // one of U hi / U lo
  int table_off, recs_off, xpose_off, bars_off, total;
};

__host__ __device__ inline Plan make_plan(int K, int N_fft, int P, int rank2, int stages) {
  Plan p;
  p.nsub = 2 * K / 64;
  p.ncols = (rank2 + 31) / 32 * 32;
  p.stages = stages;
  p.u_bytes = p.nsub * p.ncols * 128;
  int off = 2 * p.u_bytes + stages * STAGE_BYTES;  // 1024-aligned blocks first
  p.table_off = off;
  off += (N_fft + K) * 8;  // tan pairs (t_i, t_{i+1})
  p.recs_off = off;
  off += UNIT * ((2 * P + 2 + 3) & ~3) * 4;
  p.xpose_off = off;
  off += 4 * XPOSE_WORDS * 4;
  p.bars_off = (off + 7) & ~7;
  off = p.bars_off + (1 + 2 * MAX_STAGES + 4 + 1) * 8 + 8;
  p.total = off + 1024;  // slack for the 1024-byte alignment of the base
  return p;
}

template <int P>
__global__ void __launch_bounds__(PTHREADS, 1)
    design_project_kernel(Consts c, const __grid_constant__ CUtensorMap u_hi_map,
                          const __grid_constant__ CUtensorMap u_lo_map, const float* __restrict__ pos,
                          int A, const float* __restrict__ cen, const float* __restrict__ nrm,
                          const float* __restrict__ areas, int S, int rank2, int stages,
                          __nv_bfloat16* __restrict__ pt_hi, __nv_bfloat16* __restrict__ pt_lo,
                          int64_t ld, int64_t col0, int* __restrict__ status) {
  // record of a pair: numerators gg[0..P) at 0, tl at 2P, lobe at 2P + 1; 16-byte multiple
  constexpr int REC = (2 * P + 2 + 3) & ~3;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const Plan plan = make_plan(c.K, c.N, P, rank2, stages);
  const int nsub = plan.nsub, N = plan.ncols;
  uint8_t* u_hi = smem;
  uint8_t* u_lo = smem + plan.u_bytes;
  uint8_t* stage_base = smem + 2 * plan.u_bytes;
  float2* table = reinterpret_cast<float2*>(smem + plan.table_off);
  float* recs = reinterpret_cast<float*>(smem + plan.recs_off);
  uint32_t* xpose = reinterpret_cast<uint32_t*>(smem + plan.xpose_off);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + plan.bars_off);
  uint64_t* u_full = bars;                    // U landed
  uint64_t* full = bars + 1;                  // [stages] a stage holds a finished K-subtile
  uint64_t* empty = full + MAX_STAGES;        // [stages] the MMAs reading a stage finished
  uint64_t* done = empty + MAX_STAGES;        // [2] an accumulator holds a finished tile
  uint64_t* tfree = done + 2;                 // [2] the epilogue has read an accumulator
  uint64_t* drain = tfree + 2;                // every issued MMA finished
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int groups = (S + UNIT - 1) / UNIT;
  const int units = A * groups;
  uint32_t tmem_cols = 32;
  while ((int)tmem_cols < 2 * N) tmem_cols <<= 1;

  for (int i = threadIdx.x; i < c.N + c.K; i += PTHREADS)
    table[i] = make_float2(tan_entry(i, c.N, false), i + 1 < c.N + c.K ? tan_entry(i + 1, c.N, false) : 0.0f);
  if (threadIdx.x == 0) {
    mbar_init(u_full, 1);
    for (int b = 0; b < stages; ++b) {
      mbar_init(&full[b], NPROD / 32);
      mbar_init(&empty[b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&done[b], 1);
      mbar_init(&tfree[b], 4);
    }
    mbar_init(drain, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = idesc_bf16(TM, N);

  if (warp < EPI_WARP) {
    // ---------------- producers: pair geometry and dictionary K-subtiles ----------------
    int stage = 0;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
      const int a = unit / groups, g = unit % groups;
      // Everyone is done with the last records; the OR over the barrier makes the abort
      // decision the same in every producer thread.
      if (bar_or(1, NPROD, *abort != 0)) break;
      if (threadIdx.x < UNIT) {
        const int s = g * UNIT + threadIdx.x;
        float* r = recs + threadIdx.x * REC;
        Pair q;
        const int sc = s < S ? s : 0;
        pair_setup(c, __ldg(pos + 3 * a), __ldg(pos + 3 * a + 1), __ldg(pos + 3 * a + 2),
                   __ldg(cen + 3 * sc), __ldg(cen + 3 * sc + 1), __ldg(cen + 3 * sc + 2),
                   __ldg(nrm + 3 * sc), __ldg(nrm + 3 * sc + 1), __ldg(nrm + 3 * sc + 2), q);
        if (s < S && q.amp > 0.0f) {
          const float2 cw = cscale(q.rot, q.amp * sqrtf(__ldg(areas + s)) * c.inv_S);
          float2 nu[P];
          numerators<P>(q.off, nu);
          r[2 * P] = q.tl;
          r[2 * P + 1] = __int_as_float(q.lobe);
#pragma unroll
          for (int k = 0; k < P; ++k) *reinterpret_cast<float2*>(r + 2 * k) = cmul(cw, nu[k]);
        } else {
          r[2 * P] = 1.0f;
          r[2 * P + 1] = __int_as_float(c.N - 1);
#pragma unroll
          for (int k = 0; k < P; ++k) *reinterpret_cast<float2*>(r + 2 * k) = make_float2(0.f, 0.f);
        }
      }
      asm volatile("bar.sync 1, %0;" ::"r"(NPROD) : "memory");
      const int tiles = min(2, (S - g * UNIT + TM - 1) / TM);
      for (int u = 0; u < tiles; ++u) {
        for (int j = 0; j < nsub; ++j, ++stage) {
          const int slot = stage % stages;
          const int round = stage / stages;
          bool ok = true;
          if (lane == 0 && round > 0 && !mbar_wait_sleep(&empty[slot], (round - 1) & 1, abort)) {
            *abort = 1;
            ok = false;
          }
          ok = __shfl_sync(0xffffffffu, ok, 0);
          if (ok) {
            uint8_t* hi = stage_base + slot * STAGE_BYTES;
            uint8_t* lo = hi + A_SUB;
            // A lane evaluates four neighbouring bins of one row (one 16-byte chunk of the
            // swizzled row); eight lanes fill a row, so a store instruction fills four rows.
            const int quad = lane >> 3, pos = lane & 7;
            const int k = j * 32 + 4 * pos;
#pragma unroll
            for (int i = 0; i < ROWS_PER_WARP / 4; ++i) {
              const int row = warp * ROWS_PER_WARP + 4 * i + quad;  // surfel within the tile
              const float* r = recs + (u * TM + row) * REC;
              const float2 tl_lobe = *reinterpret_cast<const float2*>(r + 2 * P);
              const float tl = tl_lobe.x;
              const int m = k - __float_as_int(tl_lobe.y);  // bin offset from the lobe
              float2 g[4];  // numerators of bins k .. k + 3
              if (P == 1) {
                g[0] = g[1] = g[2] = g[3] = *reinterpret_cast<const float2*>(r);
              } else if (P == 2) {
                const float4 both = *reinterpret_cast<const float4*>(r);
                const bool odd = (m & 1) != 0;
                g[0] = g[2] = odd ? make_float2(both.z, both.w) : make_float2(both.x, both.y);
                g[1] = g[3] = odd ? make_float2(both.x, both.y) : make_float2(both.z, both.w);
              } else {
#pragma unroll
                for (int t = 0; t < 4; ++t) g[t] = *reinterpret_cast<const float2*>(r + 2 * ((m + t) & (P - 1)));
              }
              const float2 t01 = table[m + c.N - 1], t23 = table[m + c.N + 1];
              const float tan4[4] = {t01.x, t01.y, t23.x, t23.y};
              uint32_t hw[4], lw[4];
#pragma unroll
              for (int t = 0; t < 4; ++t) {
                const float cot = cot_from(tan4[t], tl);
                const float re = g[t].x * cot - g[t].y, im = g[t].y * cot + g[t].x;
                const __nv_bfloat162 h = __floats2bfloat162_rn(re, im);
                const __nv_bfloat162 l = __floats2bfloat162_rn(re - __low2float(h), im - __high2float(h));
                hw[t] = bf16x2_bits(h);
                lw[t] = bf16x2_bits(l);
              }
              // K-major, 128-byte swizzle: row, then the 16-byte chunk XOR (row mod 8)
              const uint32_t off = (uint32_t)((row >> 3) * 1024 + (row & 7) * 128) +
                                   ((uint32_t)(pos ^ (row & 7)) << 4);
              *reinterpret_cast<uint4*>(hi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
              *reinterpret_cast<uint4*>(lo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          }
          __syncwarp();
          if (lane == 0) mbar_arrive(&full[slot]);
        }
      }
    }
  } else if (warp < MMA_WARP) {
    // ---------------- epilogue: TMEM -> split PT rows ----------------
    const int quarter = warp & 3;  // TMEM lanes 32 quarter .. 32 quarter + 31
    uint32_t* xh = xpose + quarter * XPOSE_WORDS;
    uint32_t* xl = xh + 32 * 17 + 16;
    int tile = 0;
    bool ok = true;
    for (int unit = blockIdx.x; unit < units && ok; unit += gridDim.x) {
      const int a = unit / groups, g = unit % groups;
      const int tiles = min(2, (S - g * UNIT + TM - 1) / TM);
      const int64_t base_col = col0 + (int64_t)a * rank2;
      for (int u = 0; u < tiles; ++u, ++tile) {
        const int acc = tile & 1, use = tile >> 1;
        if (!mbar_wait_sleep(&done[acc], use & 1, abort)) {
          *abort = 1;
          ok = false;
          break;
        }
        tc_fence_after();
        const int row0 = g * UNIT + u * TM + quarter * 32;  // surfel of lane 0
        for (int c0 = 0; c0 < N; c0 += 32) {
          uint32_t v[32];
          tmem_ld32_nowait(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * N + c0), v);
#pragma unroll
          for (int w = 0; w < 16; ++w) {
            const float x0 = __uint_as_float(v[2 * w]), x1 = __uint_as_float(v[2 * w + 1]);
            const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
            const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - __low2float(h), x1 - __high2float(h));
            xh[lane * 17 + w] = bf16x2_bits(h);
            xl[lane * 17 + w] = bf16x2_bits(l);
          }
          __syncwarp();
          // one row per step: lanes 0-15 store its hi words, lanes 16-31 its lo words
          const int word = lane & 15;
          const bool col_ok = c0 + 2 * word < rank2;
          __nv_bfloat16* dst_base = lane < 16 ? pt_hi : pt_lo;
          const uint32_t* src = lane < 16 ? xh : xl;
          for (int r = 0; r < 32; ++r) {
            const int s = row0 + r;
            if (s < S && col_ok)
              *reinterpret_cast<uint32_t*>(dst_base + (int64_t)s * ld + base_col + c0 + 2 * word) =
                  src[r * 17 + word];
          }
          __syncwarp();
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tfree[acc]);
      }
    }
  } else {
    // ---------------- MMA issue (one thread) ----------------
    if (lane == 0) {
    mbar_expect_tx(u_full, 2 * plan.u_bytes);
    for (int t = 0; t < nsub; ++t) {
      tma_load_2d(u_hi + t * (N * 128), &u_hi_map, 64 * t, 0, u_full);
      tma_load_2d(u_lo + t * (N * 128), &u_lo_map, 64 * t, 0, u_full);
    }
    bool ok = mbar_wait_sleep(u_full, 0, abort);
    int stage = 0, tile = 0;
    for (int unit = blockIdx.x; unit < units && ok; unit += gridDim.x) {
      const int g = unit % groups;
      const int tiles = min(2, (S - g * UNIT + TM - 1) / TM);
      for (int u = 0; u < tiles && ok; ++u, ++tile) {
        const int acc = tile & 1, use = tile >> 1;
        if (use > 0 && !mbar_wait_sleep(&tfree[acc], (use - 1) & 1, abort)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(acc * N);
        for (int j = 0; j < nsub; ++j, ++stage) {
          const int slot = stage % stages;
          if (!mbar_wait_sleep(&full[slot], (stage / stages) & 1, abort)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_hi = smem_u32(stage_base + slot * STAGE_BYTES);
          const uint32_t a_lo = a_hi + A_SUB;
          const uint32_t b_hi = smem_u32(u_hi + j * (N * 128));
          const uint32_t b_lo = smem_u32(u_lo + j * (N * 128));
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint32_t step = (uint32_t)kk * 32;
            umma_bf16(d, sw128_desc(a_hi + step), sw128_desc(b_hi + step), idesc, (j | kk) != 0);
            umma_bf16(d, sw128_desc(a_lo + step), sw128_desc(b_hi + step), idesc, 1u);
            umma_bf16(d, sw128_desc(a_hi + step), sw128_desc(b_lo + step), idesc, 1u);
          }
          umma_commit(&empty[slot]);
        }
        if (ok) umma_commit(&done[acc]);
      }
    }
    if (!ok) *abort = 1;
    // Every MMA issued so far completes before the accumulators are released.
    umma_commit(drain);
    mbar_wait_plain(drain, 0);
    }
    __syncwarp();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == MMA_WARP) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
  }
  if (threadIdx.x == 0 && *abort) atomicExch(status, 1);
}

std::mutex g_mutex;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool encode_ready() {
  std::lock_guard<std::mutex> lock(g_mutex);
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

// Rows [0, box_rows) of the [128, cols] bf16 basis, 64 columns per copy, 128-byte swizzle.
bool basis_map(CUtensorMap* map, const void* base, int cols, int box_rows) {
  const cuuint64_t dims[2] = {(cuuint64_t)cols, 128};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Deepest stage ring (at most MAX_STAGES) that fits the shared-memory limit; 0 if fewer than 2.
int plan_stages(int K, int N_fft, int P, int rank2) {
  for (int stages = MAX_STAGES; stages >= 2; --stages)
    if (make_plan(K, N_fft, P, rank2, stages).total <= SMEM_LIMIT) return stages;
  return 0;
}

template <int P>
int launch_project(const Consts& c, const CUtensorMap& mh, const CUtensorMap& ml, const float* pos,
                   int A, const float* cen, const float* nrm, const float* areas, int S, int rank2,
                   void* hi, void* lo, int64_t ld, int64_t col0, int* status, cudaStream_t st) {
  const int deepest = plan_stages(c.K, c.N, P, rank2);
  if (deepest == 0) return DSG_ERR_UNSUPPORTED;
  const int tuned = dsg_tuning_value(DSG_TUNE_PROJECT_STAGES);
  const int stages = tuned >= 2 && tuned < deepest ? tuned : deepest;
  const size_t smem = (size_t)make_plan(c.K, c.N, P, rank2, stages).total;
  auto kern = design_project_kernel<P>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DSG_ERR_LAUNCH;
  const long long units = (long long)A * ((S + UNIT - 1) / UNIT);
  int sms = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = (int)(units < sms ? units : sms);
  kern<<<grid, PTHREADS, smem, st>>>(c, mh, ml, pos, A, cen, nrm, areas, S, rank2, stages,
                                     reinterpret_cast<__nv_bfloat16*>(hi),
                                     reinterpret_cast<__nv_bfloat16*>(lo), ld, col0, status);
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // namespace

extern "C" {

int dsg_design_project_bf16x3(const DsgChirp* chirp, const float* positions, int32_t apertures,
                              const float* centers, const float* normals, const float* areas,
                              int32_t surfels, const void* basis_hi, const void* basis_lo,
                              int32_t rank2, void* pt_hi, void* pt_lo, int64_t ld,
                              int64_t column_offset, int32_t* status, void* stream) {
  if (!chirp || chirp->samples <= 0 || chirp->n_fft != chirp->samples * chirp->pad ||
      chirp->num_bins != chirp->n_fft / 2)
    return DSG_ERR_UNSUPPORTED;
  const int K = chirp->num_bins;
  if (!(K == 32 || K == 64 || K == 128) || !(chirp->pad == 1 || chirp->pad == 2 || chirp->pad == 4))
    return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || surfels < 0 || rank2 < 2 || rank2 > 128 || (rank2 & 1) || column_offset < 0 ||
      (column_offset & 1) || (ld & 1))
    return DSG_ERR_ARGUMENT;
  if (apertures == 0 || surfels == 0) return DSG_OK;
  if (!positions || !centers || !normals || !areas || !basis_hi || !basis_lo || !pt_hi || !pt_lo || !status)
    return DSG_ERR_ARGUMENT;
  if (ld < column_offset + (int64_t)apertures * rank2) return DSG_ERR_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(basis_hi) | reinterpret_cast<uintptr_t>(basis_lo)) & 15u)
    return DSG_ERR_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(pt_hi) | reinterpret_cast<uintptr_t>(pt_lo)) & 3u) return DSG_ERR_ARGUMENT;
  if (!encode_ready()) return DSG_ERR_LIBRARY;
  const int ncols = (rank2 + 31) / 32 * 32;
  CUtensorMap mh, ml;
  if (!basis_map(&mh, basis_hi, 2 * K, ncols) || !basis_map(&ml, basis_lo, 2 * K, ncols))
    return DSG_ERR_ARGUMENT;
  const Consts c = make_consts(*chirp);
  cudaStream_t st = (cudaStream_t)stream;
  switch (chirp->pad) {
    case 1:
      return launch_project<1>(c, mh, ml, positions, apertures, centers, normals, areas, surfels, rank2,
                               pt_hi, pt_lo, ld, column_offset, status, st);
    case 2:
      return launch_project<2>(c, mh, ml, positions, apertures, centers, normals, areas, surfels, rank2,
                               pt_hi, pt_lo, ld, column_offset, status, st);
    default:
      return launch_project<4>(c, mh, ml, positions, apertures, centers, normals, areas, surfels, rank2,
                               pt_hi, pt_lo, ld, column_offset, status, st);
  }
}

}  // extern "C"
