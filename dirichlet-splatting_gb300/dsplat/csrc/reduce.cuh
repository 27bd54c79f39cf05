// Shared parts of the aperture-reduced kernels (correlations, their gradients and the
// VJP): the per-mode output layout, the chain rule from a pair's sufficient statistics
//   Z0 = sum_k conj(D(k - k0)) r_k,   Z1 = sum_k conj(D'(k - k0)) r_k,
//   N0 = sum_k |D(k - k0)|^2,         N1 = sum_k Re(conj(D) D')
// to the per-surfel outputs, and the float64 fixed-order sum of per-chunk partials.
// Reference: dsplat/kernels/correlate.slang:75-108 (surfel_correlate), :171-235
// (surfel_correlate_gradient), dsplat/kernels/surfel.slang:223-311 (vjp_bins).
#pragma once
#include "common.cuh"

namespace dsg {

// Values per surfel (NV) and gradient width (W) of each mode. MODE 0: correlate (corr,
// norm). 1 / 2: correlate_gradient, width 3 / 6. 3: vjp.
template <int MODE>
struct ModeInfo;
template <> struct ModeInfo<0> { static constexpr int NV = 3; static constexpr int W = 0; };
template <> struct ModeInfo<1> { static constexpr int NV = 12; static constexpr int W = 3; };
template <> struct ModeInfo<2> { static constexpr int NV = 21; static constexpr int W = 6; };
template <> struct ModeInfo<3> { static constexpr int NV = 8; static constexpr int W = 0; };

// Adds one pair's contribution to the surfel's outputs. amp, amp_cos, cosv, inv_r, rate,
// uu (unit vector to the aperture) and rot (carrier) describe the pair; nv is the
// surfel's normal and ws its weight (VJP only).
template <int MODE>
__device__ __forceinline__ void chain_outputs(const Consts& c, float amp, float amp_cos, float cosv,
                                              float inv_r, float rate, const float uu[3], float2 rot,
                                              const float nv[3], float2 ws, float2 z0, float2 z1,
                                              float n0, float n1, float* accv) {
  constexpr bool kGrad = MODE == 1 || MODE == 2;
  const float2 e0 = cmulc(rot, z0);
  if (MODE == 0) {
    accv[0] += amp * e0.x;
    accv[1] += amp * e0.y;
    accv[2] += amp * amp * n0;
    return;
  }
  const float2 e1 = cmulc(rot, z1);
  // kpm E1 + i rate E0
  const float2 inner = make_float2(c.kpm * e1.x - rate * e0.y, c.kpm * e1.y + rate * e0.x);
  if (kGrad) {
    constexpr int W = ModeInfo<MODE>::W;
    accv[0] += amp * e0.x;
    accv[1] += amp * e0.y;
    accv[2] += amp * amp * n0;
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
      const float da = (amp * uu[jj] + amp_cos * (cosv * uu[jj] - nv[jj])) * inv_r;
      const float au = amp * uu[jj];
      accv[3 + jj] += da * e0.x + au * inner.x;
      accv[3 + W + jj] += da * e0.y + au * inner.y;
      accv[3 + 2 * W + jj] += 2.0f * amp * (da * n0 + au * c.kpm * n1);
      if (W == 6) {
        const float acu = amp_cos * uu[jj];
        accv[6 + jj] += acu * e0.x;
        accv[3 + W + 3 + jj] += acu * e0.y;
        accv[3 + 2 * W + 3 + jj] += 2.0f * amp * acu * n0;
      }
    }
  } else {  // VJP: Re(conj(w) dcorr) per coordinate, and corr for the weight
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
      const float da = (amp * uu[jj] + amp_cos * (cosv * uu[jj] - nv[jj])) * inv_r;
      const float au = amp * uu[jj];
      const float2 dcj = make_float2(da * e0.x + au * inner.x, da * e0.y + au * inner.y);
      accv[jj] += ws.x * dcj.x + ws.y * dcj.y;
      const float acu = amp_cos * uu[jj];
      accv[3 + jj] += acu * (ws.x * e0.x + ws.y * e0.y);
    }
    accv[6] += amp * e0.x;
    accv[7] += amp * e0.y;
  }
}

namespace {

// Double-precision, fixed-order sum of chunk partials; scatters to the outputs. A thread
// owns one value of one candidate (adjacent threads take adjacent values, so a warp reads
// whole partial records) and adds its chunks in order.
template <int MODE>
__global__ void chunk_sum_kernel(const float* __restrict__ partial, int S, int chunks,
                                 float* __restrict__ o0, float* __restrict__ o1,
                                 float* __restrict__ o2, float* __restrict__ o3) {
  constexpr int NV = ModeInfo<MODE>::NV;
  const long long index = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (index >= (long long)S * NV) return;
  const int s = (int)(index / NV), v = (int)(index % NV);
  const float* p = partial + (size_t)s * chunks * NV + v;
  double t = 0.0;
  for (int g = 0; g < chunks; ++g) t += (double)p[(size_t)g * NV];
  const float out = (float)t;
  if (MODE == 0) {  // corr [S,2], norm [S]
    if (v < 2) o0[2 * s + v] = out;
    else o1[s] = out;
  } else if (MODE == 3) {  // grad centers [S,3], normals [S,3], weights [S,2]
    if (v < 3) o0[3 * s + v] = out;
    else if (v < 6) o1[3 * s + v - 3] = out;
    else o2[2 * s + v - 6] = out;
  } else {  // corr, norm, dcorr [S,W,2], dnorm [S,W]
    constexpr int W = ModeInfo<MODE>::W;
    if (v < 2) o0[2 * s + v] = out;
    else if (v == 2) o1[s] = out;
    else if (v < 3 + W) o2[((size_t)s * W + v - 3) * 2] = out;
    else if (v < 3 + 2 * W) o2[((size_t)s * W + v - 3 - W) * 2 + 1] = out;
    else o3[(size_t)s * W + v - 3 - 2 * W] = out;
  }
}

}  // namespace

// Sum of chunk partials [S][chunks][NV] into the mode's outputs (one launch).
template <int MODE>
inline void launch_chunk_sum(const float* partial, int S, int chunks, float* o0, float* o1, float* o2,
                             float* o3, cudaStream_t st) {
  const long long n = (long long)S * ModeInfo<MODE>::NV;
  chunk_sum_kernel<MODE><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(partial, S, chunks, o0, o1, o2, o3);
  dsg_count_launches(1);
}

// CTAs the segment / chunk splits aim for: 152 SMs x (DSG_TUNE_SPLAT_CTAS_PER_SM, default 6).
inline int target_ctas() {
  const int per_sm = dsg_tuning_value(DSG_TUNE_SPLAT_CTAS_PER_SM);
  return 152 * (per_sm > 0 ? per_sm : 6);
}

// Interpolated form of the reduced family (interp.cu): MODE's outputs from the residual
// through a type-2 nonuniform FFT; workspace as sized by interp_workspace_bytes.
size_t interp_workspace_bytes(const Consts& c, int A, int S, int nv);
int interp_reduce(int mode, const Consts& c, const float* pos, int A, const float* cen, const float* nrm,
                  const float2* w, int S, const float2* res, void* workspace, size_t workspace_bytes,
                  float* o0, float* o1, float* o2, float* o3, const int* active, int period,
                  cudaStream_t st);
// The two halves of interp_reduce, for callers that correlate one residual many times:
// the residual's aperture tables [u0 | u1] (interp_tables_bytes; u1 only with derivative),
// then any mode's outputs from them (workspace: interp_partial_bytes).
size_t interp_partial_bytes(int A, int S, int nv);
size_t interp_tables_bytes(const Consts& c, int A, bool derivative);
int interp_residual_tables(const Consts& c, const float2* res, int A, bool derivative, float2* tables,
                           cudaStream_t st);
int interp_reduce_tabled(int mode, const Consts& c, const float* pos, int A, const float* cen, const float* nrm,
                         const float2* w, int S, const float2* tables, void* workspace, size_t workspace_bytes,
                         float* o0, float* o1, float* o2, float* o3, const int* active, int period,
                         cudaStream_t st);

}  // namespace dsg
