// Per-candidate algebra of the batched certificate ascent of the spatial search, fused
// into three kernels (reference: dsplat/certificate.py:11-37 certificate, :136-142 the
// ascent map, :159-194 one iteration of search_certificate).
//
// One batched iteration runs: the quasi-Newton direction (dsg_direction), every
// backtracking trial (dsg_trials), the correlation of the full steps,
// dsg_ascent_partition, the correlation of the smaller fractions for the candidates the
// full step did not improve (dsg_surfel_correlate_active), dsg_ascent_select, the
// correlation gradient at the accepted points and dsg_ascent_update. The kernels here
// take the unscaled correlations of the surfel kernels and apply the area scaling of the
// model (sqrt(area) on correlations, area on norms, in float32), then the certificate
// algebra in float64, as the reference does between its correlation calls.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

constexpr int kPartitionThreads = 1024;
constexpr int kThreads = 128;
constexpr int kMaxFractions = 16;

// The norm clamped below at 1e-60 in float64; NaN compares false and is kept.
__device__ __forceinline__ double clamp_norm(float norm) {
  const double n = (double)norm;
  return n < 1e-60 ? 1e-60 : n;
}

// Squared normalized certificate |s|^2 / (n |r|^2), s the real part (real mode) or the
// whole scaled correlation.
__device__ __forceinline__ float certificate_value(float2 corr, float norm, float area, double power,
                                                   bool real_mode) {
  const float root = sqrtf(area);
  const double cr = (double)(corr.x * root), ci = (double)(corr.y * root);
  const double n = clamp_norm(norm * area);
  const double s2 = real_mode ? cr * cr : cr * cr + ci * ci;
  return (float)(s2 / n / power);
}

// Improvement flags of the full steps, and a stable partition of the candidates with the
// ones still pending first: position[i] is candidate i's slot, pending the number of
// pending candidates, and rows r - 1 of the batch hold trial fraction r at those slots.
// One CTA; chunks of 1024 candidates are ranked by warp ballots in index order.
__global__ void __launch_bounds__(kPartitionThreads)
    partition_kernel(const float2* __restrict__ corr, const float* __restrict__ norm,
                     const float* __restrict__ areas, const double* __restrict__ power, int real_mode,
                     const float* __restrict__ value, int count, const float* __restrict__ trial_centers,
                     const float* __restrict__ trial_normals, int fraction_count, const uint8_t* __restrict__ stuck,
                     uint8_t* __restrict__ improved, int32_t* __restrict__ position, int32_t* __restrict__ pending,
                     float* __restrict__ batch_centers, float* __restrict__ batch_normals) {
  constexpr int kWarps = kPartitionThreads / 32;
  __shared__ int warp_count[kWarps];
  __shared__ int pending_total;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const double p = *power;
  int waiting_here = 0;
  for (int i = t; i < count; i += kPartitionThreads) {
    const float v = certificate_value(corr[i], norm[i], areas[i], p, real_mode != 0);
    const bool up = isfinite(v) && v > value[i];
    improved[i] = up ? 1 : 0;
    waiting_here += up || (stuck != nullptr && stuck[i]) ? 0 : 1;
  }
  for (int offset = 16; offset > 0; offset >>= 1) waiting_here += __shfl_xor_sync(0xffffffffu, waiting_here, offset);
  if (lane == 0) warp_count[warp] = waiting_here;
  __syncthreads();
  if (t == 0) {
    int sum = 0;
    for (int w = 0; w < kWarps; ++w) sum += warp_count[w];
    pending_total = sum;
    *pending = sum;
  }
  __syncthreads();
  const int first_improved = pending_total;
  int base_pending = 0, base_improved = 0;
  for (int start = 0; start < count; start += kPartitionThreads) {
    const int i = start + t;
    const bool live = i < count;
    // written by this thread above; a stuck candidate waits for nothing (no fraction is scored)
    const bool waiting = live && improved[i] == 0 && !(stuck != nullptr && stuck[i]);
    const unsigned ballot = __ballot_sync(0xffffffffu, waiting);
    __syncthreads();  // every thread has read the previous chunk's counts
    if (lane == 0) warp_count[warp] = __popc(ballot);
    __syncthreads();
    int before = __popc(ballot & ((1u << lane) - 1u)), chunk_pending = 0;
    for (int w = 0; w < kWarps; ++w) {
      const int c = warp_count[w];
      before += w < warp ? c : 0;
      chunk_pending += c;
    }
    if (live) {
      const int slot = waiting ? base_pending + before : first_improved + base_improved + (t - before);
      position[i] = slot;
      for (int r = 1; r < fraction_count; ++r) {
        const size_t from = ((size_t)r * count + i) * 3, to = ((size_t)(r - 1) * count + slot) * 3;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          batch_centers[to + j] = trial_centers[from + j];
          batch_normals[to + j] = trial_normals[from + j];
        }
      }
    }
    const int chunk_live = min(kPartitionThreads, count - start);
    base_pending += chunk_pending;
    base_improved += chunk_live - chunk_pending;
  }
}

// Each candidate takes the first (largest) fraction whose finite certificate exceeds its
// current value: fraction 0 when the full step improved, else the first of the batch
// rows at its slot; without one it keeps its parameters.
__global__ void select_kernel(const float2* __restrict__ corr, const float* __restrict__ norm,
                              const float* __restrict__ areas, const double* __restrict__ power, int real_mode,
                              const float* __restrict__ value, int count, const uint8_t* __restrict__ improved,
                              const int32_t* __restrict__ position, const float* __restrict__ trial_centers,
                              const float* __restrict__ trial_normals, int fraction_count,
                              const uint8_t* __restrict__ stuck, const float* __restrict__ centers,
                              const float* __restrict__ normals, int move_normals, float* __restrict__ new_centers,
                              float* __restrict__ new_normals, uint8_t* __restrict__ accepted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int chosen = -1;
  if (stuck != nullptr && stuck[i]) {
    chosen = -1;  // rejected every fraction from this same state before: it rejects them again
  } else if (improved[i]) {
    chosen = 0;
  } else if (fraction_count > 1) {
    const int slot = position[i];
    const double p = *power;
    const float area = areas[i], current = value[i];
    for (int r = 1; r < fraction_count; ++r) {
      const size_t k = (size_t)(r - 1) * count + slot;
      const float v = certificate_value(corr[k], norm[k], area, p, real_mode != 0);
      if (isfinite(v) && v > current) {
        chosen = r;
        break;
      }
    }
  }
  accepted[i] = chosen >= 0 ? 1 : 0;
  const size_t from = ((size_t)(chosen < 0 ? 0 : chosen) * count + i) * 3;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    new_centers[3 * i + j] = chosen >= 0 ? trial_centers[from + j] : centers[3 * i + j];
    new_normals[3 * i + j] = chosen >= 0 && move_normals ? trial_normals[from + j] : normals[3 * i + j];
  }
}

struct Spec {
  int normalize[2];
  float scale[2];
  float mask[6];
};

// Certificate value and gradient at the accepted points, the gradient mapped to scaled
// tangent coordinates and negated (the ascent map), and the damped BFGS update of the
// candidate's inverse Hessian; the state (parameters, value, gradient, inverse) is
// overwritten in place, one thread per candidate.
template <int W>
__global__ void update_kernel(Spec spec, const float2* __restrict__ corr, const float* __restrict__ norm,
                              const float2* __restrict__ dcorr, const float* __restrict__ dnorm,
                              const float* __restrict__ areas, const double* __restrict__ power, int real_mode,
                              int count, const float* __restrict__ new_centers, const float* __restrict__ new_normals,
                              const uint8_t* __restrict__ accepted, float* __restrict__ centers,
                              float* __restrict__ normals, float* __restrict__ value, float* __restrict__ gradient,
                              float* __restrict__ inverse) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const bool real = real_mode != 0;
  const double p = *power;
  const float area = areas[i];
  const float root = sqrtf(area);
  const float2 c = corr[i];
  const double cr = (double)(c.x * root), ci = (double)(c.y * root);
  const double n = clamp_norm(norm[i] * area);
  const double v = (real ? cr * cr : cr * cr + ci * ci) / n / p;
  const bool has_norm = n > 1e-60;
  float g[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const float2 d = dcorr[(size_t)i * W + w];
    const double dcr = (double)(d.x * root), dci = (double)(d.y * root);
    const double dn = has_norm ? (double)(dnorm[(size_t)i * W + w] * area) : 0.0;
    const double ds = real ? 2.0 * cr * dcr : 2.0 * (cr * dcr + ci * dci);
    g[w] = (float)((ds - v * p * dn) / n / p);
  }
  float moved[6];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    moved[j] = new_centers[3 * i + j];
    moved[3 + j] = new_normals[3 * i + j];
  }
  // Ascent map: the part of the gradient a projection keeps (tangent to unit vectors,
  // frozen components dropped), times the mask and the group's scale, negated.
  float a[W];
#pragma unroll
  for (int k = 0; k < W / 3; ++k) {
    float vec[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) vec[j] = g[3 * k + j];
    if (spec.normalize[k]) {
      float moving[3], fixed2 = 0.0f, dot = 0.0f;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const bool free_axis = spec.mask[3 * k + j] > 0.0f;
        const float x = moved[3 * k + j];
        moving[j] = free_axis ? x : 0.0f;
        fixed2 += free_axis ? 0.0f : x * x;
        vec[j] = free_axis ? vec[j] : 0.0f;
        dot += vec[j] * moving[j];
      }
      const float room = fmaxf(1.0f - fixed2, 0.0f);
#pragma unroll
      for (int j = 0; j < 3; ++j) vec[j] = room > 0.0f ? vec[j] - dot * moving[j] / fmaxf(room, 1e-30f) : 0.0f;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) a[3 * k + j] = -(vec[j] * spec.mask[3 * k + j] * spec.scale[k]);
  }
  // Damped BFGS update, skipped unless the step was accepted and has enough curvature.
  float step[W], change[W], sy = 0.0f, ss = 0.0f, cc = 0.0f;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const float before = w < 3 ? centers[3 * i + w] : normals[3 * i + w - 3];
    step[w] = (moved[w] - before) / spec.scale[w / 3];
    change[w] = a[w] - gradient[(size_t)i * W + w];
    sy += step[w] * change[w];
    ss += step[w] * step[w];
    cc += change[w] * change[w];
  }
  const bool valid = accepted[i] && sy > 1e-8f * sqrtf(ss) * sqrtf(cc) && sy > 1e-20f;
  if (valid) {
    const float rho = 1.0f / fmaxf(sy, 1e-30f);
    float* h = inverse + (size_t)i * W * W;
    float left[W][W], product[W][W];
#pragma unroll
    for (int r = 0; r < W; ++r)
#pragma unroll
      for (int q = 0; q < W; ++q) left[r][q] = (r == q ? 1.0f : 0.0f) - rho * step[r] * change[q];
#pragma unroll
    for (int r = 0; r < W; ++r)
#pragma unroll
      for (int q = 0; q < W; ++q) {
        float sum = 0.0f;
#pragma unroll
        for (int k = 0; k < W; ++k) sum += left[r][k] * h[k * W + q];
        product[r][q] = sum;
      }
#pragma unroll
    for (int r = 0; r < W; ++r)
#pragma unroll
      for (int q = 0; q < W; ++q) {
        float sum = 0.0f;
#pragma unroll
        for (int k = 0; k < W; ++k) sum += product[r][k] * left[q][k];
        h[r * W + q] = sum + rho * step[r] * step[q];
      }
  }
  value[i] = (float)v;
#pragma unroll
  for (int w = 0; w < W; ++w) gradient[(size_t)i * W + w] = a[w];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    centers[3 * i + j] = moved[j];
    normals[3 * i + j] = moved[3 + j];
  }
}

int status() { return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH; }

}  // namespace

extern "C" {

int dsg_ascent_partition(const float* corr, const float* norm, const float* areas, const double* power,
                         int32_t real_mode, const float* value, int32_t count, const float* trial_centers,
                         const float* trial_normals, int32_t fraction_count, const uint8_t* stuck, uint8_t* improved,
                         int32_t* position, int32_t* pending, float* batch_centers, float* batch_normals,
                         void* stream) {
  if (count < 0 || fraction_count < 1 || fraction_count > kMaxFractions) return DSG_ERR_ARGUMENT;
  if (!pending || !power) return DSG_ERR_ARGUMENT;
  if (count > 0 && (!corr || !norm || !areas || !value || !trial_centers || !trial_normals || !improved ||
                    !position || (fraction_count > 1 && (!batch_centers || !batch_normals))))
    return DSG_ERR_ARGUMENT;
  partition_kernel<<<1, kPartitionThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(corr), norm, areas, power, real_mode, value, count, trial_centers,
      trial_normals, fraction_count, stuck, improved, position, pending, batch_centers, batch_normals);
  dsg_count_launches(1);
  return status();
}

int dsg_ascent_select(const float* corr, const float* norm, const float* areas, const double* power,
                      int32_t real_mode, const float* value, int32_t count, const uint8_t* improved,
                      const int32_t* position, const float* trial_centers, const float* trial_normals,
                      int32_t fraction_count, const uint8_t* stuck, const float* centers, const float* normals,
                      int32_t move_normals, float* new_centers, float* new_normals, uint8_t* accepted,
                      void* stream) {
  if (count < 0 || fraction_count < 1 || fraction_count > kMaxFractions) return DSG_ERR_ARGUMENT;
  if (count == 0) return DSG_OK;
  if (!areas || !power || !value || !improved || !position || !trial_centers || !trial_normals || !centers ||
      !normals || !new_centers || !new_normals || !accepted || (fraction_count > 1 && (!corr || !norm)))
    return DSG_ERR_ARGUMENT;
  select_kernel<<<(count + kThreads - 1) / kThreads, kThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(corr), norm, areas, power, real_mode, value, count, improved, position,
      trial_centers, trial_normals, fraction_count, stuck, centers, normals, move_normals, new_centers, new_normals,
      accepted);
  dsg_count_launches(1);
  return status();
}

int dsg_ascent_update(const DsgAscentSpec* spec, const float* corr, const float* norm, const float* dcorr,
                      const float* dnorm, const float* areas, const double* power, int32_t real_mode,
                      int32_t count, const float* new_centers, const float* new_normals, const uint8_t* accepted,
                      float* centers, float* normals, float* value, float* gradient, float* inverse,
                      void* stream) {
  if (!spec || count < 0 || (spec->width != 3 && spec->width != 6)) return DSG_ERR_ARGUMENT;
  if (count == 0) return DSG_OK;
  if (!corr || !norm || !dcorr || !dnorm || !areas || !power || !new_centers || !new_normals || !accepted ||
      !centers || !normals || !value || !gradient || !inverse)
    return DSG_ERR_ARGUMENT;
  for (int k = 0; k < spec->width / 3; ++k)
    if (!(spec->scale[k] != 0.0f)) return DSG_ERR_ARGUMENT;
  Spec s{};
  for (int k = 0; k < 2; ++k) {
    s.normalize[k] = spec->normalize[k];
    s.scale[k] = spec->scale[k];
  }
  for (int j = 0; j < 6; ++j) s.mask[j] = spec->mask[j];
  const dim3 grid((unsigned)((count + kThreads - 1) / kThreads));
  cudaStream_t st = (cudaStream_t)stream;
  const float2* c = reinterpret_cast<const float2*>(corr);
  const float2* dc = reinterpret_cast<const float2*>(dcorr);
  if (spec->width == 3)
    update_kernel<3><<<grid, kThreads, 0, st>>>(s, c, norm, dc, dnorm, areas, power, real_mode, count, new_centers,
                                                new_normals, accepted, centers, normals, value, gradient, inverse);
  else
    update_kernel<6><<<grid, kThreads, 0, st>>>(s, c, norm, dc, dnorm, areas, power, real_mode, count, new_centers,
                                                new_normals, accepted, centers, normals, value, gradient, inverse);
  dsg_count_launches(1);
  return status();
}

}  // extern "C"
