// ADC-domain synthesis of FMCW scans in float64 (reference: dsplat/groundtruth.py:58-90,
// synthesize, and :40-55, _echoes). Every aperture-surfel echo is a beat tone sampled by
// the ADC,
//
//   adc[a, n] = sum_s b_s amp(a, s) exp(2 pi i cycles(a, s)) exp(2 pi i beat(a, s) n / fs),
//
// with amp = cos^2 F(cos) lambda / (8 pi r) (0 when cos <= 0), cycles the carrier phase
// fc tau + K tau (t0 - tau / 2), tau = 2 r / c0, beat = 2 K r / c0. The range FFT that
// follows is a library call on the host side.
//
// One CTA per aperture, 256 threads. For each chunk of 256 surfels a thread evaluates one
// echo in float64 and the per-sample rotation w = exp(2 pi i beat / fs), and leaves the
// echo rotated to the start of each block of 16 samples (w^16 by four squarings, then a
// product per block) in shared memory. The threads then split into sample blocks x surfel
// lanes: each walks its surfels in order, adding 16 consecutive samples by the recurrence
// z <- z w, and the lanes are then summed in lane order through shared memory. The sum
// order is fixed, so the result is deterministic; each recurrence runs 16 steps from an
// anchor, so its rounding stays near float64 precision.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

constexpr int kThreads = 256;
constexpr int kBlock = 16;     // samples per recurrence block
constexpr int kMaxBlocks = 16; // up to 256 ADC samples

struct Z {
  double x, y;
};

__device__ __forceinline__ Z zmul(Z a, Z b) { return Z{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }

// exp(2 pi i cycles), the integer part of the cycles dropped exactly first.
__device__ __forceinline__ Z turn(double cycles) {
  const double frac = cycles - rint(cycles);
  double s, c;
  sincospi(2.0 * frac, &s, &c);
  return Z{c, s};
}

struct Params {
  double fc, slope, t0, lambda, c0, fresnel_n, fs;
  int samples;
};

__global__ void __launch_bounds__(kThreads) synth_kernel(Params p, const double* __restrict__ pos, int A,
                                                         const double* __restrict__ cen,
                                                         const double* __restrict__ nrm,
                                                         const double* __restrict__ amps, int S,
                                                         double* __restrict__ adc) {
  extern __shared__ double smem[];
  const int blocks = (p.samples + kBlock - 1) / kBlock;  // sample blocks
  const int lanes = kThreads / blocks;                    // surfel lanes per sample block
  Z* anchors = reinterpret_cast<Z*>(smem);                // [256 surfels][blocks]
  Z* rot = anchors + kThreads * blocks;                   // [256 surfels]
  const int a = blockIdx.x;
  const double px = pos[3 * a], py = pos[3 * a + 1], pz = pos[3 * a + 2];
  const int t = threadIdx.x;
  const int nb = t / lanes, lane = t % lanes;  // phase 2 roles (t < blocks * lanes)
  const bool active = nb < blocks;
  Z acc[kBlock];
#pragma unroll
  for (int k = 0; k < kBlock; ++k) acc[k] = Z{0.0, 0.0};

  for (int s0 = 0; s0 < S; s0 += kThreads) {
    const int count = min(kThreads, S - s0);
    __syncthreads();  // the last chunk's anchors are consumed
    if (t < count) {
      const int s = s0 + t;
      const double dx = px - cen[3 * s], dy = py - cen[3 * s + 1], dz = pz - cen[3 * s + 2];
      const double r = fmax(sqrt(dx * dx + dy * dy + dz * dz), 1e-9);
      double cosv = (dx * nrm[3 * s] + dy * nrm[3 * s + 1] + dz * nrm[3 * s + 2]) / r;
      cosv = fmax(cosv, 0.0);
      double amp = cosv * cosv * p.lambda / (8.0 * 3.14159265358979323846 * r);
      if (p.fresnel_n > 1.0) {
        const double root = sqrt(p.fresnel_n * p.fresnel_n - 1.0 + cosv * cosv);
        amp = amp * (root - cosv) / (root + cosv);
      }
      const double tau = 2.0 * r / p.c0;
      const double cycles = p.fc * tau + p.slope * tau * (p.t0 - 0.5 * tau);
      const Z carrier = turn(cycles);
      const Z b = Z{amps[2 * s], amps[2 * s + 1]};
      Z z = zmul(b, Z{amp * carrier.x, amp * carrier.y});
      const double step = 2.0 * p.slope * r / p.c0 / p.fs;  // beat cycles per sample
      const Z w = turn(step);
      Z w16 = zmul(w, w);
      w16 = zmul(w16, w16);
      w16 = zmul(w16, w16);
      w16 = zmul(w16, w16);
      rot[t] = w;
      for (int k = 0; k < blocks; ++k) {
        anchors[t * blocks + k] = z;
        z = zmul(z, w16);
      }
    }
    __syncthreads();
    if (active) {
      for (int j = lane; j < count; j += lanes) {
        const Z w = rot[j];
        Z z = anchors[j * blocks + nb];
#pragma unroll
        for (int k = 0; k < kBlock; ++k) {
          acc[k].x += z.x;
          acc[k].y += z.y;
          z = zmul(z, w);
        }
      }
    }
  }
  // Sum the surfel lanes of each sample block in lane order.
  __syncthreads();
  Z* partial = reinterpret_cast<Z*>(smem);  // [256 threads][kBlock]
  if (active) {
#pragma unroll
    for (int k = 0; k < kBlock; ++k) partial[t * kBlock + k] = acc[k];
  }
  __syncthreads();
  for (int n = t; n < blocks * kBlock; n += blockDim.x) {
    const int b = n / kBlock, k = n % kBlock;
    if (b * kBlock + k >= p.samples) continue;
    Z sum{0.0, 0.0};
    for (int l = 0; l < lanes; ++l) {
      const Z v = partial[(b * lanes + l) * kBlock + k];
      sum.x += v.x;
      sum.y += v.y;
    }
    adc[((size_t)a * p.samples + b * kBlock + k) * 2] = sum.x;
    adc[((size_t)a * p.samples + b * kBlock + k) * 2 + 1] = sum.y;
  }
}

}  // namespace

extern "C" int dsg_synthesize_adc(const DsgChirp* chirp, double sample_rate, const double* positions,
                                  int32_t apertures, const double* centers, const double* normals,
                                  const double* amplitudes, int32_t surfels, double* adc, void* stream) {
  if (!chirp || chirp->samples <= 0 || chirp->samples > kBlock * kMaxBlocks || !(sample_rate > 0.0))
    return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || surfels < 0) return DSG_ERR_ARGUMENT;
  if (apertures == 0) return DSG_OK;
  if (!positions || !adc || (surfels > 0 && (!centers || !normals || !amplitudes))) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (surfels == 0) {
    cudaMemsetAsync(adc, 0, (size_t)apertures * chirp->samples * 2 * sizeof(double), st);
    return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
  }
  Params p{chirp->fc, chirp->slope, chirp->t_start, chirp->lambda_m, chirp->c0, chirp->fresnel_n,
           sample_rate, chirp->samples};
  const int blocks = (chirp->samples + kBlock - 1) / kBlock;
  const size_t anchors = (size_t)kThreads * blocks * 16 + (size_t)kThreads * 16;
  const size_t partial = (size_t)kThreads * kBlock * 16;
  const size_t smem = anchors > partial ? anchors : partial;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(synth_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DSG_ERR_LAUNCH;
  synth_kernel<<<apertures, kThreads, smem, st>>>(p, positions, apertures, centers, normals, amplitudes, surfels,
                                                 adc);
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}
