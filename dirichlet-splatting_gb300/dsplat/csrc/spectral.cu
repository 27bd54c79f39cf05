// Separable windowed Dirichlet atoms on a 1-3D periodic grid: forward, JVP, VJP and
// dictionary (reference: dsplat/kernels/spectral.slang:1-114). Every sine and cosine of
// a fraction of a turn goes through sincospif, whose argument reduction is exact, so a
// centre at 255.3 bins keeps the float32 precision of its offset from each bin.
#include <cuda_runtime.h>
#include <math.h>
#include "common.cuh"

namespace dsg {

// Unit-peak kernel of `samples` taps on an `nfft` grid and its derivative by delta.
__device__ __forceinline__ void grid_dirichlet(float delta, int samples, int nfft, float2& k,
                                               float2& dk) {
  const float fn = (float)nfft;
  const float x = delta - fn * rintf(delta / fn);
  const float a = kPi * (float)samples / fn, b = kPi / fn;
  const float h = kPi * (float)(samples - 1) / fn;
  float ratio, dr;
  if (fabsf(x) < 0.1f) {
    const float a2 = a * a, b2 = b * b;
    const float c2 = (b2 - a2) / 6.0f;
    const float c4 = (3.0f * a2 * a2 + 7.0f * b2 * b2 - 10.0f * a2 * b2) / 360.0f;
    const float c6 = (31.0f * b2 * b2 * b2 - 49.0f * a2 * b2 * b2 + 21.0f * a2 * a2 * b2 -
                      3.0f * a2 * a2 * a2) / 15120.0f;
    const float x2 = x * x;
    ratio = 1.0f + x2 * (c2 + x2 * (c4 + x2 * c6));
    dr = x * (2.0f * c2 + x2 * (4.0f * c4 + x2 * 6.0f * c6));
  } else {
    float sa, ca, sb, cb;
    sincospif(x * (float)samples / fn, &sa, &ca);
    sincospif(x / fn, &sb, &cb);
    const float inv = 1.0f / ((float)samples * sb);
    ratio = sa * inv;
    dr = (a * ca * sb - b * sa * cb) * inv / sb;
  }
  float sp, cp;
  sincospif(-(float)(samples - 1) * x / fn, &sp, &cp);
  k = make_float2(ratio * cp, ratio * sp);
  const float2 t = make_float2(dr, -h * ratio);
  dk = make_float2(cp * t.x - sp * t.y, cp * t.y + sp * t.x);
}

struct GridC {
  int dim, window, max_taps;
  int nfft[3], samples[3];
  float radius;
};

// Per-axis kernel value and derivative at delta = bin - centre (before wrapping).
__device__ __forceinline__ void axis_kernel(const GridC& g, const float* __restrict__ taps, int d,
                                            float delta, float2& k, float2& dk) {
  const float fn = (float)g.nfft[d];
  const float x = delta - fn * rintf(delta / fn);
  if (g.radius > 0.0f && fabsf(x) > g.radius) {
    k = make_float2(0.f, 0.f);
    dk = make_float2(0.f, 0.f);
    return;
  }
  if (g.window == 3) {  // Kaiser: explicit tap sum
    k = make_float2(0.f, 0.f);
    dk = make_float2(0.f, 0.f);
    const int n_s = g.samples[d];
    for (int n = 0; n < n_s; ++n) {
      const float tap = __ldg(taps + d * g.max_taps + n);
      float sn, cn;
      // exp(-2 pi i n x / nfft); reduce n x / nfft to a fraction of a turn first
      const float turns = (float)n * x / fn;
      sincospif(-2.0f * (turns - rintf(turns)), &sn, &cn);
      const float omega = -2.0f * kPi * (float)n / fn;
      k.x += tap * cn;
      k.y += tap * sn;
      dk.x += -omega * tap * sn;
      dk.y += omega * tap * cn;
    }
    return;
  }
  grid_dirichlet(x, g.samples[d], g.nfft[d], k, dk);
  if (g.window == 0) return;
  const float shift = fn / (float)g.samples[d];
  float2 km, dm, kp, dp;
  grid_dirichlet(x - shift, g.samples[d], g.nfft[d], km, dm);
  grid_dirichlet(x + shift, g.samples[d], g.nfft[d], kp, dp);
  const float wgt = g.window == 1 ? 0.5f : 0.46f / 1.08f;
  k.x -= wgt * (km.x + kp.x);
  k.y -= wgt * (km.y + kp.y);
  dk.x -= wgt * (dm.x + dp.x);
  dk.y -= wgt * (dm.y + dp.y);
}

// Atom value a and its derivatives by the centre coordinates, d[j] = -dK_j prod_{i!=j} K_i.
__device__ __forceinline__ void footprint(const GridC& g, const float* __restrict__ taps,
                                          const float* __restrict__ bin,
                                          const float* __restrict__ centre, float2& a,
                                          float2 (&d)[3]) {
  float2 k[3], dk[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    k[j] = make_float2(1.f, 0.f);
    dk[j] = make_float2(0.f, 0.f);
  }
  for (int j = 0; j < g.dim; ++j) axis_kernel(g, taps, j, bin[j] - centre[j], k[j], dk[j]);
  a = cmul(cmul(k[0], k[1]), k[2]);
  d[0] = cscale(cmul(cmul(dk[0], k[1]), k[2]), -1.0f);
  d[1] = cscale(cmul(cmul(k[0], dk[1]), k[2]), -1.0f);
  d[2] = cscale(cmul(cmul(k[0], k[1]), dk[2]), -1.0f);
}

// Per-axis tables of the separable atoms: for axis d, grid bin u < nfft[d] and atom s,
// values[d][u][s] = K_d(u - c_s[d]) and derivatives[d][u][s] = dK_d / d(delta) (complex,
// interleaved; atoms contiguous, so a table is the row-major [nfft[d], count] operand of
// the products that assemble the grid). A thread per (axis, bin, atom).
__global__ void axis_tables_kernel(GridC g, const float* __restrict__ taps, const float* __restrict__ centers,
                                   int count, int width, float2* __restrict__ values, float2* __restrict__ derivs) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per_axis = (long long)width * count;
  if (e >= per_axis * g.dim) return;
  const int d = (int)(e / per_axis);
  const int u = (int)((e % per_axis) / count), s = (int)(e % count);
  if (u >= g.nfft[d]) return;
  float2 k, dk;
  axis_kernel(g, taps, d, (float)u - __ldg(centers + (size_t)s * g.dim + d), k, dk);
  values[e] = k;
  derivs[e] = dk;
}

__global__ void spectral_forward_kernel(GridC g, const float* __restrict__ taps,
                                        const float* __restrict__ centers, int count,
                                        const float2* __restrict__ coeff,
                                        const float* __restrict__ dcenters,
                                        const float2* __restrict__ dcoeff,
                                        const float* __restrict__ bins, int size,
                                        float2* __restrict__ out) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= size) return;
  float bin[3] = {0.f, 0.f, 0.f};
  for (int j = 0; j < g.dim; ++j) bin[j] = __ldg(bins + m * g.dim + j);
  float2 sum = make_float2(0.f, 0.f);
  for (int s = 0; s < count; ++s) {
    float cen[3] = {0.f, 0.f, 0.f};
    for (int j = 0; j < g.dim; ++j) cen[j] = __ldg(centers + s * g.dim + j);
    float2 a, d[3];
    footprint(g, taps, bin, cen, a, d);
    if (dcenters == nullptr) {
      sum = cadd(sum, cmul(a, __ldg(coeff + s)));
    } else {  // JVP: (sum_j d_j dc_j) b + a db
      float2 da = make_float2(0.f, 0.f);
      for (int j = 0; j < g.dim; ++j) da = cadd(da, cscale(d[j], __ldg(dcenters + s * g.dim + j)));
      sum = cadd(sum, cadd(cmul(da, __ldg(coeff + s)), cmul(a, __ldg(dcoeff + s))));
    }
  }
  out[m] = sum;
}

// Partial gradients per (atom, span of bins): [count][spans][dim + 2].
__global__ void spectral_vjp_kernel(GridC g, const float* __restrict__ taps,
                                    const float* __restrict__ centers, int count,
                                    const float2* __restrict__ coeff,
                                    const float2* __restrict__ upstream,
                                    const float* __restrict__ bins, int size, int span,
                                    int spans, float* __restrict__ partial) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= count) return;
  float cen[3] = {0.f, 0.f, 0.f};
  for (int j = 0; j < g.dim; ++j) cen[j] = __ldg(centers + s * g.dim + j);
  const float2 b = __ldg(coeff + s);
  float gc[3] = {0.f, 0.f, 0.f};
  float2 gb = make_float2(0.f, 0.f);
  const int start = blockIdx.y * span, stop = min(size, start + span);
  for (int m = start; m < stop; ++m) {
    float bin[3] = {0.f, 0.f, 0.f};
    for (int j = 0; j < g.dim; ++j) bin[j] = __ldg(bins + m * g.dim + j);
    float2 a, d[3];
    footprint(g, taps, bin, cen, a, d);
    const float2 u = __ldg(upstream + m);
    for (int j = 0; j < g.dim; ++j) {
      const float2 bd = cmul(b, d[j]);
      gc[j] += u.x * bd.x + u.y * bd.y;
    }
    gb = cadd(gb, cmulc(a, u));
  }
  float* p = partial + ((size_t)s * spans + blockIdx.y) * (g.dim + 2);
  for (int j = 0; j < g.dim; ++j) p[j] = gc[j];
  p[g.dim] = gb.x;
  p[g.dim + 1] = gb.y;
}

__global__ void spectral_vjp_sum_kernel(const float* __restrict__ partial, int count, int spans,
                                        int dim, float* __restrict__ gcent,
                                        float* __restrict__ gcoef) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= count) return;
  double t[5] = {0, 0, 0, 0, 0};
  for (int g = 0; g < spans; ++g) {
    const float* p = partial + ((size_t)s * spans + g) * (dim + 2);
    for (int v = 0; v < dim + 2; ++v) t[v] += (double)p[v];
  }
  for (int j = 0; j < dim; ++j) gcent[s * dim + j] = (float)t[j];
  gcoef[2 * s] = (float)t[dim];
  gcoef[2 * s + 1] = (float)t[dim + 1];
}

__global__ void spectral_design_kernel(GridC g, const float* __restrict__ taps,
                                       const float* __restrict__ centers, int count,
                                       const float* __restrict__ bins, int size,
                                       float2* __restrict__ out, float2* __restrict__ jac) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)size * count) return;
  const int m = (int)(i / count), s = (int)(i % count);
  float bin[3] = {0.f, 0.f, 0.f}, cen[3] = {0.f, 0.f, 0.f};
  for (int j = 0; j < g.dim; ++j) {
    bin[j] = __ldg(bins + m * g.dim + j);
    cen[j] = __ldg(centers + s * g.dim + j);
  }
  float2 a, d[3];
  footprint(g, taps, bin, cen, a, d);
  out[i] = a;
  if (jac != nullptr)
    for (int j = 0; j < g.dim; ++j) jac[i * g.dim + j] = d[j];
}

}  // namespace dsg

using namespace dsg;

namespace {

bool grid_ok(const DsgGrid* g, GridC& c) {
  if (!g || g->dim < 1 || g->dim > 3 || g->window < 0 || g->window > 3) return false;
  c.dim = g->dim;
  c.window = g->window;
  c.max_taps = g->max_taps;
  c.radius = g->radius;
  for (int j = 0; j < 3; ++j) {
    c.nfft[j] = j < g->dim ? g->nfft[j] : 1;
    c.samples[j] = j < g->dim ? g->samples[j] : 1;
    if (j < g->dim && (c.nfft[j] <= 0 || c.samples[j] <= 0)) return false;
  }
  if (g->window == 3 && g->max_taps <= 0) return false;
  return true;
}

int status() { return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH; }

int spectral_spans(int count, int size, int& span) {
  // about 256 bins per span, more spans while atoms alone do not fill the GPU
  span = 256;
  int spans = (size + span - 1) / span;
  if (spans > 65535) {
    span = (size + 65534) / 65535;
    spans = (size + span - 1) / span;
  }
  (void)count;
  return spans;
}

}  // namespace

extern "C" {

int dsg_spectral_axis_tables(const DsgGrid* grid, const float* taps, const float* centers, int32_t count,
                             float* values, float* derivatives, void* stream) {
  GridC g;
  if (!grid_ok(grid, g)) return DSG_ERR_ARGUMENT;
  if (count < 0) return DSG_ERR_ARGUMENT;
  if (count == 0) return DSG_OK;
  if (!centers || !values || !derivatives || (g.window == 3 && !taps)) return DSG_ERR_ARGUMENT;
  int width = 1;
  for (int d = 0; d < g.dim; ++d) width = g.nfft[d] > width ? g.nfft[d] : width;
  const long long total = (long long)g.dim * width * count;
  if (total > 0x7fffffffLL * 128) return DSG_ERR_ARGUMENT;
  axis_tables_kernel<<<(unsigned)((total + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      g, taps, centers, count, width, reinterpret_cast<float2*>(values), reinterpret_cast<float2*>(derivatives));
  dsg_count_launches(1);
  return status();
}

int dsg_spectral_render(const DsgGrid* grid, const float* taps, const float* centers,
                        int32_t count, const float* coeff, const float* bins, int32_t size,
                        float* out, void* stream) {
  GridC g;
  if (!grid_ok(grid, g)) return DSG_ERR_ARGUMENT;
  if (count < 0 || size < 0) return DSG_ERR_ARGUMENT;
  if (size == 0) return DSG_OK;
  if (!bins || !out || (count > 0 && (!centers || !coeff))) return DSG_ERR_ARGUMENT;
  spectral_forward_kernel<<<(size + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      g, taps, centers, count, reinterpret_cast<const float2*>(coeff), nullptr, nullptr, bins, size,
      reinterpret_cast<float2*>(out));
  dsg_count_launches(1);
  return status();
}

int dsg_spectral_jvp(const DsgGrid* grid, const float* taps, const float* centers,
                     int32_t count, const float* coeff, const float* delta_centers,
                     const float* delta_coeff, const float* bins, int32_t size, float* out,
                     void* stream) {
  GridC g;
  if (!grid_ok(grid, g)) return DSG_ERR_ARGUMENT;
  if (count < 0 || size < 0) return DSG_ERR_ARGUMENT;
  if (size == 0) return DSG_OK;
  if (!bins || !out || (count > 0 && (!centers || !coeff || !delta_centers || !delta_coeff)))
    return DSG_ERR_ARGUMENT;
  if (count == 0) {
    cudaMemsetAsync(out, 0, (size_t)size * 2 * sizeof(float), (cudaStream_t)stream);
    return status();
  }
  spectral_forward_kernel<<<(size + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      g, taps, centers, count, reinterpret_cast<const float2*>(coeff), delta_centers,
      reinterpret_cast<const float2*>(delta_coeff), bins, size, reinterpret_cast<float2*>(out));
  dsg_count_launches(1);
  return status();
}

size_t dsg_spectral_vjp_workspace_bytes(const DsgGrid* grid, int32_t count, int32_t size) {
  GridC g;
  if (!grid_ok(grid, g) || count <= 0 || size <= 0) return 0;
  int span;
  const int spans = spectral_spans(count, size, span);
  return (size_t)count * spans * (g.dim + 2) * sizeof(float);
}

int dsg_spectral_vjp(const DsgGrid* grid, const float* taps, const float* centers,
                     int32_t count, const float* coeff, const float* upstream,
                     const float* bins, int32_t size, float* grad_centers, float* grad_coeff,
                     void* workspace, size_t workspace_bytes, void* stream) {
  GridC g;
  if (!grid_ok(grid, g)) return DSG_ERR_ARGUMENT;
  if (count < 0 || size < 0) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (count == 0) return DSG_OK;
  if (!centers || !coeff || !grad_centers || !grad_coeff) return DSG_ERR_ARGUMENT;
  if (size == 0) {
    cudaMemsetAsync(grad_centers, 0, (size_t)count * g.dim * sizeof(float), st);
    cudaMemsetAsync(grad_coeff, 0, (size_t)count * 2 * sizeof(float), st);
    return status();
  }
  if (!upstream || !bins) return DSG_ERR_ARGUMENT;
  const size_t need = dsg_spectral_vjp_workspace_bytes(grid, count, size);
  if (!workspace || workspace_bytes < need) return DSG_ERR_WORKSPACE;
  int span;
  const int spans = spectral_spans(count, size, span);
  dim3 gridd((count + 63) / 64, spans);
  float* part = reinterpret_cast<float*>(workspace);
  spectral_vjp_kernel<<<gridd, 64, 0, st>>>(g, taps, centers, count,
                                            reinterpret_cast<const float2*>(coeff),
                                            reinterpret_cast<const float2*>(upstream), bins, size,
                                            span, spans, part);
  spectral_vjp_sum_kernel<<<(count + 127) / 128, 128, 0, st>>>(part, count, spans, g.dim,
                                                                grad_centers, grad_coeff);
  dsg_count_launches(2);
  return status();
}

int dsg_spectral_design(const DsgGrid* grid, const float* taps, const float* centers,
                        int32_t count, const float* bins, int32_t size, float* out,
                        float* jacobian, void* stream) {
  GridC g;
  if (!grid_ok(grid, g)) return DSG_ERR_ARGUMENT;
  if (count < 0 || size < 0) return DSG_ERR_ARGUMENT;
  const int64_t n = (int64_t)count * size;
  if (n == 0) return DSG_OK;
  if (!centers || !bins || !out) return DSG_ERR_ARGUMENT;
  spectral_design_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      g, taps, centers, count, bins, size, reinterpret_cast<float2*>(out),
      reinterpret_cast<float2*>(jacobian));
  dsg_count_launches(1);
  return status();
}

}  // extern "C"
