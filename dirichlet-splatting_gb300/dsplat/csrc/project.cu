// Dictionary rows generated on chip and projected onto the row basis on the tcgen05
// tensor cores: the mixed-precision replacement of design_bins + RowBasis.reduce_major
// (reference: dsplat/kernels/surfel.slang:313-378 and dsplat/fmcw.py:128-131, 276-294).
//
// For every aperture a of a block and every tile of 32 surfels, the real dictionary
// column of each surfel, v[2k + part] = (re, im) of sqrt(area) c D(k - k0), is evaluated
// in the cotangent form of common.cuh straight into shared memory, split into bf16
// hi + lo, and multiplied by the block's interleaved basis U [2 rank, 2K] (also split,
// zero padded to 128 rows) with three tcgen05.mma products per K step (hi.hi, hi.lo,
// lo.hi). The projected values P[a 2rank + rho, s] = (U v_s)[rho] leave the tensor
// memory already split and transposed into the Gram operand PT_hi / PT_lo [S_pad, ld],
// so the design matrix never touches HBM.
//
// CTA: 8 warps. Warps 0-3 evaluate the dictionary tile (lane = range bin, loop over the
// tile's 32 surfels, whose geometry warp 0 computed first) into one of two shared
// buffers; thread 0 then issues the MMAs into one of two TMEM accumulators. Warps 4-7
// load the accumulator (tcgen05.ld) and store the split rows. All waits are bounded.
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

constexpr int PM = 128;                 // MMA M: basis rows, zero padded
constexpr int PN = 32;                  // MMA N: surfels per tile
constexpr int PTHREADS = 256;
constexpr int UB_SUB = PM * 64 * 2;     // one [128 x 64] bf16 K-subtile of U: 16 KiB
constexpr int BB_SUB = PN * 64 * 2;     // one [32 x 64] bf16 K-subtile of a tile: 4 KiB
constexpr uint32_t PIDESC = idesc_bf16(PM, PN);

template <int P>
struct ProjectSmem {
  static constexpr int REC = 2 + 2 * P;
};

// Byte offset of element (row n, k) inside a K-major, 128-byte-swizzled operand made of
// K-subtiles of 64 elements (rows of 128 B, 8-row atoms of 1024 B).
__device__ __forceinline__ uint32_t sw128_offset(int n, int k, int sub_bytes) {
  const int sub = k >> 6, within = k & 63;
  const int chunk = (within >> 3) ^ (n & 7);
  return (uint32_t)(sub * sub_bytes + (n >> 3) * 1024 + (n & 7) * 128 + chunk * 16 + (within & 7) * 2);
}

__device__ __forceinline__ uint32_t pack_bf16x2(__nv_bfloat16 lo_half, __nv_bfloat16 hi_half) {
  return (uint32_t)__bfloat16_as_ushort(lo_half) | ((uint32_t)__bfloat16_as_ushort(hi_half) << 16);
}

template <int P>
__global__ void __launch_bounds__(PTHREADS, 1)
    design_project_kernel(Consts c, const __grid_constant__ CUtensorMap u_hi_map,
                          const __grid_constant__ CUtensorMap u_lo_map, const float* __restrict__ pos,
                          int A, const float* __restrict__ cen, const float* __restrict__ nrm,
                          const float* __restrict__ areas, int S, int rank2,
                          __nv_bfloat16* __restrict__ pt_hi, __nv_bfloat16* __restrict__ pt_lo,
                          int64_t ld, int64_t col0, int* __restrict__ status) {
  constexpr int REC = ProjectSmem<P>::REC;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int K2 = 2 * c.K;           // reduction length: (re, im) of every bin
  const int nsub = K2 / 64;         // K-subtiles of 64 elements
  uint8_t* u_hi = smem;
  uint8_t* u_lo = u_hi + nsub * UB_SUB;
  uint8_t* tiles = u_lo + nsub * UB_SUB;  // [2 buffers][hi, lo][nsub][PN x 64]
  const int tile_bytes = 2 * nsub * BB_SUB;
  float* table = reinterpret_cast<float*>(tiles + 2 * tile_bytes);
  const int tbl_n = c.N + c.K;
  float* recs = table + ((tbl_n + 3) & ~3);
  uint64_t* bars = reinterpret_cast<uint64_t*>(recs + ((PN * REC + 1) & ~1));
  uint64_t* u_full = bars;          // U landed
  uint64_t* mma_done = bars + 1;    // [2] MMA of a buffer finished (tile smem and TMEM ready)
  uint64_t* tmem_free = bars + 3;   // [2] epilogue finished reading a TMEM buffer
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 5);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int groups = (S + PN - 1) / PN;
  const int tiles_total = A * groups;

  for (int i = threadIdx.x; i < tbl_n; i += PTHREADS) table[i] = tan_entry(i, c.N, false);
  if (threadIdx.x == 0) {
    mbar_init(u_full, 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&mma_done[b], 1);
      mbar_init(&tmem_free[b], 4);
    }
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(64));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0) {  // the basis, once per CTA
    mbar_expect_tx(u_full, 2 * nsub * UB_SUB);
    for (int t = 0; t < nsub; ++t) {
      tma_load_2d(u_hi + t * UB_SUB, &u_hi_map, 64 * t, 0, u_full);
      tma_load_2d(u_lo + t * UB_SUB, &u_lo_map, 64 * t, 0, u_full);
    }
  }

  if (warp < 4) {
    // ---------------- producers: dictionary tiles and MMA issue ----------------
    bool u_ready = false;
    int local = 0;
    for (int t = blockIdx.x; t < tiles_total; t += gridDim.x, ++local) {
      const int a = t / groups, g = t % groups;
      const int buf = local & 1, use = local >> 1;
      // geometry of the tile's 32 pairs (warp 0, one pair per lane)
      if (warp == 0) {
        const int s = g * PN + lane;
        float* r = recs + lane * REC;
        Pair q;
        const int sc = s < S ? s : 0;
        pair_setup(c, __ldg(pos + 3 * a), __ldg(pos + 3 * a + 1), __ldg(pos + 3 * a + 2),
                   __ldg(cen + 3 * sc), __ldg(cen + 3 * sc + 1), __ldg(cen + 3 * sc + 2),
                   __ldg(nrm + 3 * sc), __ldg(nrm + 3 * sc + 1), __ldg(nrm + 3 * sc + 2), q);
        if (s < S && q.amp > 0.0f) {
          float2 cw = cscale(q.rot, q.amp * sqrtf(__ldg(areas + s)) * c.inv_S);
          float2 nu[P];
          numerators<P>(q.off, nu);
          r[0] = q.tl;
          r[1] = __int_as_float(q.lobe);
#pragma unroll
          for (int k = 0; k < P; ++k) *reinterpret_cast<float2*>(r + 2 + 2 * k) = cmul(cw, nu[k]);
        } else {
          r[0] = 1.0f;
          r[1] = __int_as_float(c.N - 1);
#pragma unroll
          for (int k = 0; k < P; ++k) *reinterpret_cast<float2*>(r + 2 + 2 * k) = make_float2(0.f, 0.f);
        }
        // the buffer is free once the MMA that read it two tiles ago has finished
        if (lane == 0 && use > 0 && !mbar_wait(&mma_done[buf], (use - 1) & 1, abort)) *abort = 1;
      }
      asm volatile("bar.sync 1, 128;" ::: "memory");
      if (*abort) break;  // uniform: read after the barrier
      uint8_t* hi = tiles + buf * tile_bytes;
      uint8_t* lo = hi + nsub * BB_SUB;
      const int k = warp * 32 + lane;  // range bin of this thread
      if (k < c.K) {
#pragma unroll 4
        for (int n = 0; n < PN; ++n) {
          const float* r = recs + n * REC;
          const float tl = r[0];
          const int lobe = __float_as_int(r[1]);
          const float2 gg = *reinterpret_cast<const float2*>(r + 2 + 2 * ((k - lobe) & (P - 1)));
          const float cot = cot_from(table[k - lobe + c.N - 1], tl);
          const float re = gg.x * cot - gg.y, im = gg.y * cot + gg.x;
          const __nv_bfloat16 re_h = __float2bfloat16_rn(re), im_h = __float2bfloat16_rn(im);
          const __nv_bfloat16 re_l = __float2bfloat16_rn(re - __bfloat162float(re_h));
          const __nv_bfloat16 im_l = __float2bfloat16_rn(im - __bfloat162float(im_h));
          const uint32_t off = sw128_offset(n, 2 * k, BB_SUB);
          *reinterpret_cast<uint32_t*>(hi + off) = pack_bf16x2(re_h, im_h);
          *reinterpret_cast<uint32_t*>(lo + off) = pack_bf16x2(re_l, im_l);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("bar.sync 1, 128;" ::: "memory");
      if (threadIdx.x == 0) {
        bool ok = true;
        if (!u_ready) ok = u_ready = mbar_wait(u_full, 0, abort);
        if (ok && use > 0) ok = mbar_wait(&tmem_free[buf], (use - 1) & 1, abort);
        if (!ok) {
          *abort = 1;
        } else {
          tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(buf * PN);
          for (int kk = 0; kk < K2 / 16; ++kk) {
            const uint32_t uoff = (uint32_t)((kk >> 2) * UB_SUB + (kk & 3) * 32);
            const uint32_t boff = (uint32_t)((kk >> 2) * BB_SUB + (kk & 3) * 32);
            const uint64_t ah = sw128_desc(smem_u32(u_hi) + uoff), al = sw128_desc(smem_u32(u_lo) + uoff);
            const uint64_t bh = sw128_desc(smem_u32(hi) + boff), bl = sw128_desc(smem_u32(lo) + boff);
            umma_bf16(d, ah, bh, PIDESC, kk != 0);
            umma_bf16(d, ah, bl, PIDESC, 1u);
            umma_bf16(d, al, bh, PIDESC, 1u);
          }
          umma_commit(&mma_done[buf]);
        }
      }
    }
  } else {
    // ---------------- consumers: TMEM -> split, transposed rows ----------------
    const int quarter = warp & 3;
    const int rho = 32 * quarter + lane;
    int local = 0;
    for (int t = blockIdx.x; t < tiles_total; t += gridDim.x, ++local) {
      const int a = t / groups, g = t % groups;
      const int buf = local & 1, use = local >> 1;
      if (!mbar_wait(&mma_done[buf], use & 1, abort)) {
        *abort = 1;
        break;
      }
      tc_fence_after();
      uint32_t v[32];
      const bool rows_here = 32 * quarter < rank2;
      if (rows_here) tmem_ld32(tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(buf * PN), v);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tmem_free[buf]);
      if (rows_here && rho < rank2) {
        const int64_t col = col0 + (int64_t)a * rank2 + rho;
#pragma unroll
        for (int n = 0; n < PN; ++n) {
          const int s = g * PN + n;
          const float x = __uint_as_float(v[n]);
          const __nv_bfloat16 h = __float2bfloat16_rn(x);
          const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
          pt_hi[(int64_t)s * ld + col] = h;
          pt_lo[(int64_t)s * ld + col] = l;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(64));
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

bool basis_map(CUtensorMap* map, const void* base, int cols) {
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)PM};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {64, PM};
  const cuuint32_t estr[2] = {1, 1};
  return g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t project_smem(int K, int N, int P) {
  const int nsub = 2 * K / 64;
  const size_t tbl = (size_t)((N + K + 3) & ~3) * 4;
  const size_t recs = (size_t)((PN * (2 + 2 * P) + 1) & ~1) * 4;
  return 1024 + 2 * (size_t)nsub * UB_SUB + 2 * 2 * (size_t)nsub * BB_SUB + tbl + recs + 64;
}

template <int P>
int launch_project(const Consts& c, const CUtensorMap& mh, const CUtensorMap& ml, const float* pos,
                   int A, const float* cen, const float* nrm, const float* areas, int S, int rank2,
                   void* hi, void* lo, int64_t ld, int64_t col0, int* status, cudaStream_t st) {
  const size_t smem = project_smem(c.K, c.N, P);
  auto kern = design_project_kernel<P>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DSG_ERR_LAUNCH;
  const int groups = (S + PN - 1) / PN;
  const long long tiles = (long long)A * groups;
  int sms = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = (int)(tiles < sms ? tiles : sms);
  kern<<<grid, PTHREADS, smem, st>>>(c, mh, ml, pos, A, cen, nrm, areas, S, rank2,
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
  if (apertures < 0 || surfels < 0 || rank2 < 1 || rank2 > PM || column_offset < 0) return DSG_ERR_ARGUMENT;
  if (apertures == 0 || surfels == 0) return DSG_OK;
  if (!positions || !centers || !normals || !areas || !basis_hi || !basis_lo || !pt_hi || !pt_lo || !status)
    return DSG_ERR_ARGUMENT;
  if (ld < column_offset + (int64_t)apertures * rank2) return DSG_ERR_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(basis_hi) | reinterpret_cast<uintptr_t>(basis_lo)) & 15u)
    return DSG_ERR_ARGUMENT;
  if (!encode_ready()) return DSG_ERR_LIBRARY;
  CUtensorMap mh, ml;
  if (!basis_map(&mh, basis_hi, 2 * K) || !basis_map(&ml, basis_lo, 2 * K)) return DSG_ERR_ARGUMENT;
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
