// Angular-spectrum focusing sum of the range-migration initializer (reference:
// dsplat/fmcw.py:361-454, migration): for every depth d and every transverse wavenumber
// (kx, ky) of the replicated aperture spectrum,
//
//   focused[d, x, y] = sum_f S[f, iu(x), iv(y)] kz_f exp(-i kz_f d),
//   kz_f = sqrt(max(k_f^2 - kx^2 - ky^2, 0)),  iu(x) = (x - qu/2 + pu/2) mod pu,
//
// where S is the 2-D FFT of the zero-padded aperture data per ADC sample f and the
// replicas (qu = pu * copies) keep every propagating spatial frequency of an undersampled
// aperture. A thread owns one (depth, x, y) and walks the frequencies in order; the FFTs,
// the crop and the trilinear interpolation stay with the caller's library.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

__global__ void focus_kernel(const float2* __restrict__ spectrum, int F, int pu, int pv,
                             const float* __restrict__ k, const float* __restrict__ kx,
                             const float* __restrict__ ky, int qu, int qv, const float* __restrict__ depths,
                             float2* __restrict__ focused) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= (long long)qu * qv) return;
  const int depth = blockIdx.y;
  const int x = (int)(cell / qv), y = (int)(cell % qv);
  int iu = (x - qu / 2 + pu / 2) % pu;
  int iv = (y - qv / 2 + pv / 2) % pv;
  if (iu < 0) iu += pu;
  if (iv < 0) iv += pv;
  const float transverse = kx[x] * kx[x] + ky[y] * ky[y];
  const float d = depths[depth];
  float2 acc = make_float2(0.f, 0.f);
  const float2* column = spectrum + (size_t)iu * pv + iv;
  for (int f = 0; f < F; ++f) {
    const float kz = sqrtf(fmaxf(k[f] * k[f] - transverse, 0.0f));
    const float2 s = column[(size_t)f * pu * pv];
    float sn, cs;
    sincosf(-kz * d, &sn, &cs);
    const float2 w = make_float2(s.x * kz, s.y * kz);
    acc.x += w.x * cs - w.y * sn;
    acc.y += w.x * sn + w.y * cs;
  }
  focused[(size_t)depth * qu * qv + cell] = acc;
}

}  // namespace

extern "C" int dsg_migration_focus(const float* spectrum, int32_t frequencies, int32_t pu, int32_t pv,
                                   const float* k, const float* kx, const float* ky, int32_t qu, int32_t qv,
                                   const float* depths, int32_t depth_count, float* focused, void* stream) {
  if (frequencies < 0 || pu <= 0 || pv <= 0 || qu <= 0 || qv <= 0 || depth_count < 0 || depth_count > 65535)
    return DSG_ERR_ARGUMENT;
  if (depth_count == 0) return DSG_OK;
  if (!focused || !depths || !kx || !ky || (frequencies > 0 && (!spectrum || !k))) return DSG_ERR_ARGUMENT;
  const long long cells = (long long)qu * qv;
  const dim3 grid((unsigned)((cells + 255) / 256), (unsigned)depth_count);
  focus_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2*>(spectrum), frequencies, pu,
                                                       pv, k, kx, ky, qu, qv, depths,
                                                       reinterpret_cast<float2*>(focused));
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}
