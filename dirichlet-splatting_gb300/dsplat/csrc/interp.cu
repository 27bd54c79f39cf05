// Correlations, correlation gradients and the VJP of the FMCW surfels by interpolation:
// a type-2 nonuniform FFT instead of the closed-form kernel summed over every bin.
//
// For one aperture with residual r over the K kept bins, every sufficient statistic of a
// pair is a function of the pair's fractional bin k0 alone:
//
//   Z0(k0) = sum_k conj(D(k - k0)) r_k = sum_{n<S} R_n e^{-2 pi i n k0 / N},
//   R_n = (1/S) sum_k r_k e^{2 pi i n k / N}        (D(d) = (1/S) sum_n e^{-2 pi i n d / N})
//
// a trigonometric polynomial of S terms in t = k0 / N; Z1 = -dZ0/dk0 has the coefficients
// R_n (2 pi i n / N). N0 = sum_k |D(k - k0)|^2 = sum_{|q|<S} c_q e^{2 pi i q k0 / N}, with
// c_q = (S - |q|) / S^2 sum_k e^{-2 pi i q k / N}, does not depend on the aperture, and
// N1 = -dN0/dk0 / 2. Each polynomial is evaluated the way a type-2 nonuniform FFT does
// (Dutt and Rokhlin 1993; the "exponential of semicircle" kernel and its shape
// beta = 2.30 w of Barnett, Magland and af Klinteberg, SIAM J. Sci. Comput. 41 (2019)):
// its coefficients divided by the kernel's Fourier transform are sampled on a grid twice
// as fine as the polynomial's degree, and a pair adds w = 8 grid values weighted by the
// kernel psi(x - j) at its position x. The aperture tables u0 = r H0 (and u1 = r H1 for
// the derivative modes) come from a fixed-order complex GEMM kernel per call (H0, H1:
// [K, grid], built once per chirp); the N tables are fixed per chirp.
//
// Per pair this costs two sets of 8 kernel weights (sqrt and exp each) and 8 to 24
// multiply-adds instead of K bins of cotangent evaluations: the bin-sum form's K MUFU
// reciprocals per pair become 32 MUFU operations. The interpolation error is about 1e-7
// of the statistics' scale, below the float32 rounding of the sums. The outputs are
// chained and summed exactly as in the bin-sum form (surfel.cu reduce_kernel): over the
// apertures of a chunk in a fixed order, over chunks in float64.
#include <cuda_runtime.h>
#include <math.h>
#include <mutex>
#include <vector>
#include "reduce.cuh"

namespace dsg {
namespace {

constexpr int kTaps = 8;                   // kernel support w, in grid cells
constexpr double kBeta = 2.30 * kTaps;     // kernel shape
constexpr int kInterpWarps = 4;            // warps per CTA: aperture streams of the same 32 surfels
constexpr int kCorrGrid = 1;               // correlation grid: 2 cells per bin / pad (2^1)
constexpr int kNormGrid = 2;               // norm grid: 4 cells per bin / pad (2^2)
constexpr double kTwoPi = 6.28318530717958647692;
constexpr double kPiD = 3.14159265358979323846;

int log2_int(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

// psi(y) = exp(beta (sqrt(1 - (2y / w)^2) - 1)) for |y| < w / 2, else 0.
double es_host(double y) {
  const double z = 2.0 * y / kTaps;
  const double a = 1.0 - z * z;
  return a > 0.0 ? exp(kBeta * (sqrt(a) - 1.0)) : 0.0;
}

// Fourier transform of psi at xi cycles per cell, integral of psi(y) cos(2 pi xi y) by the
// midpoint rule (psi is smooth inside its support and about e^-beta = 1e-8 at its ends).
double es_transform(double xi) {
  const int n = 4096;
  const double h = (double)kTaps / n;
  double sum = 0.0;
  for (int i = 0; i < n; ++i) {
    const double y = -0.5 * kTaps + (i + 0.5) * h;
    sum += es_host(y) * cos(kTwoPi * xi * y);
  }
  return sum * h;
}

struct HostTables {
  int S, P, K, N, M, M0;
  std::vector<float2> h0;    // [K][M]
  std::vector<float2> h1;    // [K][M]
  std::vector<float2> norm;  // [M0]: (v0, v1) per grid cell
};

// The fixed tables of a chirp (samples S, pad P, kept bins K = S P / 2), in double.
//   H0[k][j] = (1/S) sum_{m=-S/2}^{S/2-1} e^{2 pi i (m + S/2) k / N} e^{-2 pi i m j / M} / Psi(m / M)
//   H1[k][j] = the same with each term times 2 pi i (m + S/2) / N
//   v0[j] + i 0 = sum_q (c_q / Psi(q / M0)) e^{2 pi i q j / M0}, v1 likewise with -pi i q c_q / N
// with M = 2 S cells for the correlations and M0 = 4 S for the norms.
HostTables build_tables(int S, int P) {
  HostTables t;
  t.S = S;
  t.P = P;
  t.N = S * P;
  t.K = t.N / 2;
  t.M = 2 * S;
  t.M0 = 4 * S;
  const int K = t.K, N = t.N, M = t.M, M0 = t.M0;
  std::vector<double> tw_re(M), tw_im(M);  // e^{-2 pi i p / M}
  for (int p = 0; p < M; ++p) {
    tw_re[p] = cos(kTwoPi * p / M);
    tw_im[p] = -sin(kTwoPi * p / M);
  }
  std::vector<double> inv_psi(S);
  for (int i = 0; i < S; ++i) inv_psi[i] = 1.0 / es_transform((double)(i - S / 2) / M);
  t.h0.resize((size_t)K * M);
  t.h1.resize((size_t)K * M);
  std::vector<double> a_re(S), a_im(S), b_re(S), b_im(S);
  for (int k = 0; k < K; ++k) {
    for (int i = 0; i < S; ++i) {  // n = i = m + S/2
      const double ang = kTwoPi * (double)((long long)i * k % N) / N;
      const double scale = inv_psi[i] / S;
      a_re[i] = cos(ang) * scale;
      a_im[i] = sin(ang) * scale;
      const double f = kTwoPi * i / N;  // times i f
      b_re[i] = -a_im[i] * f;
      b_im[i] = a_re[i] * f;
    }
    for (int j = 0; j < M; ++j) {
      double h0r = 0, h0i = 0, h1r = 0, h1i = 0;
      for (int i = 0; i < S; ++i) {
        const int m = i - S / 2;
        const int p = (int)((((long long)m * j) % M + M) % M);
        const double cr = tw_re[p], ci = tw_im[p];
        h0r += a_re[i] * cr - a_im[i] * ci;
        h0i += a_re[i] * ci + a_im[i] * cr;
        h1r += b_re[i] * cr - b_im[i] * ci;
        h1i += b_re[i] * ci + b_im[i] * cr;
      }
      t.h0[(size_t)k * M + j] = make_float2((float)h0r, (float)h0i);
      t.h1[(size_t)k * M + j] = make_float2((float)h1r, (float)h1i);
    }
  }
  // norm coefficients c_q, q = -(S-1) .. S-1
  const int Q = 2 * S - 1;
  std::vector<double> c_re(Q), c_im(Q), inv_psi0(Q);
  for (int i = 0; i < Q; ++i) {
    const int q = i - (S - 1);
    double wr = 0, wi = 0;
    for (int k = 0; k < K; ++k) {
      const double ang = -kTwoPi * (double)(((long long)q * k % N + N) % N) / N;
      wr += cos(ang);
      wi += sin(ang);
    }
    const double scale = (double)(S - (q < 0 ? -q : q)) / ((double)S * S);
    c_re[i] = wr * scale;
    c_im[i] = wi * scale;
    inv_psi0[i] = 1.0 / es_transform((double)q / M0);
  }
  t.norm.resize(M0);
  for (int j = 0; j < M0; ++j) {
    double v0 = 0, v1 = 0;
    for (int i = 0; i < Q; ++i) {
      const int q = i - (S - 1);
      const double ang = kTwoPi * (double)(((long long)q * j % M0 + M0) % M0) / M0;
      const double er = cos(ang), ei = sin(ang);
      // Re((c / Psi) e), and Re((-pi i q c / N / Psi) e)
      v0 += (c_re[i] * er - c_im[i] * ei) * inv_psi0[i];
      const double d_re = kPiD * q * c_im[i] / N, d_im = -kPiD * q * c_re[i] / N;
      v1 += (d_re * er - d_im * ei) * inv_psi0[i];
    }
    t.norm[j] = make_float2((float)v0, (float)v1);
  }
  return t;
}

struct DeviceTables {
  unsigned long long context = 0;
  int device = -1, S = 0, P = 0;
  float2* h0 = nullptr;
  float2* h1 = nullptr;
  float2* norm = nullptr;
};

std::mutex g_tables_mutex;
std::vector<DeviceTables> g_tables;

// The tables of (S, P) on the current device and context: built and uploaded at the first
// request (cudaMalloc and a synchronous copy), then reused.
int device_tables(int S, int P, DeviceTables* out) {
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return DSG_ERR_LAUNCH;
  const unsigned long long context = dsg_current_context_id();
  std::lock_guard<std::mutex> lock(g_tables_mutex);
  for (const DeviceTables& e : g_tables)
    if (e.device == device && e.context == context && context != 0 && e.S == S && e.P == P) {
      *out = e;
      return DSG_OK;
    }
  const HostTables h = build_tables(S, P);
  const size_t n_h = h.h0.size(), n_norm = h.norm.size();
  float2* base = nullptr;
  if (cudaMalloc(&base, (2 * n_h + n_norm) * sizeof(float2)) != cudaSuccess) {
    cudaGetLastError();
    return DSG_ERR_LAUNCH;
  }
  DeviceTables e;
  e.context = dsg_current_context_id();
  e.device = device;
  e.S = S;
  e.P = P;
  e.h0 = base;
  e.h1 = base + n_h;
  e.norm = base + 2 * n_h;
  bool ok = cudaMemcpy(e.h0, h.h0.data(), n_h * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaMemcpy(e.h1, h.h1.data(), n_h * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaMemcpy(e.norm, h.norm.data(), n_norm * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    cudaFree(base);
    return DSG_ERR_LAUNCH;
  }
  if (e.context != 0) g_tables.push_back(e);  // without context ids the tables are rebuilt per call
  *out = e;
  return DSG_OK;
}

// Position of a pair on a grid of 2^g cells per bin / pad: x = (lobe - off) 2^g / P as an
// integer cell base plus a fraction f in [0, 1), both exact (lobe, the shifts and the
// power-of-two scalings are exact in float).
__device__ __forceinline__ void grid_position(int lobe, float off, int g, int log2P, int& base, float& f) {
  const int num = lobe << g;
  const int whole = num >> log2P;
  const int rem = num - (whole << log2P);
  const float x = ldexpf((float)rem, -log2P) - ldexpf(off, g - log2P);
  const float fl = floorf(x);
  f = x - fl;
  base = whole + (int)fl;
}

// Kernel weights psi(f + 3 - t) of the cells base - 3 + t, t = 0..7.
__device__ __forceinline__ void kernel_weights(float f, float* wt) {
  constexpr float kB2 = (float)(kBeta * 1.4426950408889634);  // beta log2(e)
#pragma unroll
  for (int t = 0; t < kTaps; ++t) {
    const float z = (f + (float)(3 - t)) * (2.0f / kTaps);
    const float a = 1.0f - z * z;
    wt[t] = a > 0.0f ? exp2f(kB2 * (a * rsqrtf(a) - 1.0f)) : 0.0f;
  }
}

// Thread = surfel (32 per CTA, one per lane); warp w of the CTA takes the chunk's
// apertures a0 + w, a0 + w + 4, ... in ascending order; the four warps' sums are added in
// warp order at the end. u0, u1: per-aperture grid values [A][M] of Z0 and Z1 (u1 unused
// by MODE 0). Z0 and N0 take the same arithmetic in every mode, so a correlation and a
// correlation gradient of the same pair agree bitwise on the value.
template <int MODE>
__global__ void __launch_bounds__(kInterpWarps * 32) interp_kernel(
    Consts c, int log2P, const float* __restrict__ pos, int A, const float* __restrict__ cen,
    const float* __restrict__ nrm, const float2* __restrict__ w, int S, const float2* __restrict__ u0,
    const float2* __restrict__ u1, int M,
    const float2* __restrict__ norm_table, int M0, int chunk_len, int chunks, float* __restrict__ partial,
    const int* __restrict__ active, int period) {
  constexpr int NV = ModeInfo<MODE>::NV;
  constexpr bool kNorm = MODE != 3;
  constexpr bool kDeriv = MODE != 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s0 = blockIdx.x * 32;
  if (active != nullptr) {  // a CTA without an active surfel writes zero partials and leaves
    const int limit = __ldg(active);
    bool any = false;
    for (int j = 0; j < 32 && !any; ++j) any = s0 + j < S && (s0 + j) % period < limit;
    if (!any) {
      for (int i = threadIdx.x; i < 32 * NV; i += blockDim.x) {
        const int t = s0 + i / NV;
        if (t < S) partial[((size_t)t * chunks + blockIdx.y) * NV + i % NV] = 0.0f;
      }
      return;
    }
  }
  extern __shared__ float2 shared[];
  float2* ntab = shared;                                            // [M0] when kNorm
  float* combine = reinterpret_cast<float*>(shared + (kNorm ? M0 : 0));  // [warps][32][NV]
  if (kNorm)
    for (int i = threadIdx.x; i < M0; i += blockDim.x) ntab[i] = __ldg(norm_table + i);
  __syncthreads();

  const int s = s0 + lane;
  const bool live = s < S && (active == nullptr || s % period < __ldg(active));
  float accv[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) accv[v] = 0.0f;
  if (live) {
    const float cx = __ldg(cen + 3 * s), cy = __ldg(cen + 3 * s + 1), cz = __ldg(cen + 3 * s + 2);
    const float nv[3] = {__ldg(nrm + 3 * s), __ldg(nrm + 3 * s + 1), __ldg(nrm + 3 * s + 2)};
    const float2 ws = MODE == 3 ? __ldg(w + s) : make_float2(0.f, 0.f);
    const int P = 1 << log2P;
    const int a_end = min(A, (blockIdx.y + 1) * chunk_len);
    for (int a = blockIdx.y * chunk_len + warp; a < a_end; a += kInterpWarps) {
      Pair q;
      pair_setup(c, __ldg(pos + 3 * a), __ldg(pos + 3 * a + 1), __ldg(pos + 3 * a + 2), cx, cy, cz, nv[0],
                 nv[1], nv[2], q);
      if (!(q.amp > 0.0f)) continue;
      int base;
      float f, wt[kTaps];
      grid_position(q.lobe, q.off, kCorrGrid, log2P, base, f);
      kernel_weights(f, wt);
      float2 z0 = make_float2(0.f, 0.f), z1 = make_float2(0.f, 0.f);
      const float2* row0 = u0 + (size_t)a * M;
      const float2* row1 = u1 + (size_t)a * M;
#pragma unroll
      for (int t = 0; t < kTaps; ++t) {
        const int j = (base + t - 3) & (M - 1);
        const float2 v = __ldg(row0 + j);
        z0.x = fmaf(wt[t], v.x, z0.x);
        z0.y = fmaf(wt[t], v.y, z0.y);
        if (kDeriv) {
          const float2 d = __ldg(row1 + j);
          z1.x = fmaf(wt[t], d.x, z1.x);
          z1.y = fmaf(wt[t], d.y, z1.y);
        }
      }
      // e^{-i pi S k0 / N} = e^{-i pi k0 / P}, k0 = lobe - off, with lobe reduced mod 2P
      float sp, cp;
      sincospif((q.off - (float)(q.lobe & (2 * P - 1))) / (float)P, &sp, &cp);
      const float2 phase = make_float2(cp, sp);
      z0 = cmul(phase, z0);
      if (kDeriv) z1 = cmul(phase, z1);
      float n0 = 0.0f, n1 = 0.0f;
      if (kNorm) {
        grid_position(q.lobe, q.off, kNormGrid, log2P, base, f);
        kernel_weights(f, wt);
#pragma unroll
        for (int t = 0; t < kTaps; ++t) {
          const float2 v = ntab[(base + t - 3) & (M0 - 1)];
          n0 = fmaf(wt[t], v.x, n0);
          n1 = fmaf(wt[t], v.y, n1);
        }
      }
      const float uu[3] = {q.ux, q.uy, q.uz};
      chain_outputs<MODE>(c, q.amp, q.amp_cos, q.cosv, q.inv_r, q.rate, uu, q.rot, nv, ws, z0, z1, n0, n1,
                          accv);
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) combine[(warp * 32 + lane) * NV + v] = accv[v];
  __syncthreads();
  if (warp == 0 && s < S) {
    float* p = partial + ((size_t)s * chunks + blockIdx.y) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      float total = 0.0f;
#pragma unroll
      for (int g = 0; g < kInterpWarps; ++g) total += combine[(g * 32 + lane) * NV + v];
      p[v] = live ? total : 0.0f;
    }
  }
}

// u [m][n] = r [m][k] . h [k][n], complex64, row-major: the aperture tables. A CTA of 256
// threads owns a 64 x 64 block of u (a thread 4 x 4 values, rows ty + 16 i, columns tx + 16 j)
// and walks k in steps of 16 through shared memory, always in ascending order, so a
// table's values do not depend on the launch, the stream or graph capture (the same
// residual gives bitwise the same table to every correlation and gradient).
constexpr int kTile = 64, kStepK = 16;

__global__ void __launch_bounds__(256) table_gemm_kernel(const float2* __restrict__ r, int m, int k,
                                                         const float2* __restrict__ h, int n,
                                                         float2* __restrict__ u) {
  __shared__ float2 ra[kStepK][kTile + 1];  // [kk][row]
  __shared__ float2 hb[kStepK][kTile];      // [kk][column]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int row0 = blockIdx.y * kTile, col0 = blockIdx.x * kTile;
  float2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < k; k0 += kStepK) {
    for (int e = threadIdx.x; e < kTile * kStepK; e += 256) {
      const int rr = e / kStepK, kk = e % kStepK;  // r tile: 16 consecutive k of one row
      const int row = row0 + rr;
      ra[kk][rr] = row < m && k0 + kk < k ? __ldg(r + (size_t)row * k + k0 + kk) : make_float2(0.f, 0.f);
      const int kb = e / kTile, cc = e % kTile;  // h tile: 64 consecutive columns of one k
      const int col = col0 + cc;
      hb[kb][cc] = col < n && k0 + kb < k ? __ldg(h + (size_t)(k0 + kb) * n + col) : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kStepK; ++kk) {
      float2 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = ra[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = hb[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[i][j].x = fmaf(a[i].x, b[j].x, fmaf(-a[i].y, b[j].y, acc[i][j].x));
          acc[i][j].y = fmaf(a[i].x, b[j].y, fmaf(a[i].y, b[j].x, acc[i][j].y));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = row0 + ty + 16 * i;
    if (row >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = col0 + tx + 16 * j;
      if (col < n) u[(size_t)row * n + col] = acc[i][j];
    }
  }
}

int table_gemm(const float2* r, int m, int k, const float2* h, int n, float2* u, cudaStream_t st) {
  if (m <= 0) return DSG_OK;
  const dim3 grid((n + kTile - 1) / kTile, (m + kTile - 1) / kTile);
  if (grid.y > 65535u) return DSG_ERR_ARGUMENT;
  table_gemm_kernel<<<grid, 256, 0, st>>>(r, m, k, h, n, u);
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

int interp_chunks(int A, int S) {
  const int tiles = (S + 31) / 32;
  int ch = (target_ctas() + tiles - 1) / tiles;
  const int max_ch = (A + kInterpWarps - 1) / kInterpWarps;
  if (ch > max_ch) ch = max_ch;
  if (ch < 1) ch = 1;
  return ch;
}

size_t align_up(size_t n) { return (n + 255) / 256 * 256; }

int nv_of(int mode) { return mode == 0 ? 3 : mode == 1 ? 12 : mode == 2 ? 21 : 8; }

template <int MODE>
int launch_interp(const Consts& c, const float* pos, int A, const float* cen, const float* nrm, const float2* w,
                  int S, const float2* u0, const float2* u1, int M, const float2* norm_table, int M0,
                  float* partial, float* o0,
                  float* o1, float* o2, float* o3, const int* active, int period, cudaStream_t st) {
  constexpr int NV = ModeInfo<MODE>::NV;
  const int chunks = interp_chunks(A, S);
  const int chunk_len = (A + chunks - 1) / chunks;
  const int nch = (A + chunk_len - 1) / chunk_len;
  const size_t smem = (MODE != 3 ? (size_t)M0 * sizeof(float2) : 0) + (size_t)kInterpWarps * 32 * NV * sizeof(float);
  auto kern = interp_kernel<MODE>;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DSG_ERR_LAUNCH;
  const dim3 grid((S + 31) / 32, nch);
  kern<<<grid, kInterpWarps * 32, smem, st>>>(c, log2_int(c.P), pos, A, cen, nrm, w, S, u0, u1, M, norm_table,
                                                M0, chunk_len, nch, partial, active, period);
  dsg_count_launches(1);
  launch_chunk_sum<MODE>(partial, S, nch, o0, o1, o2, o3, st);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // namespace

size_t interp_partial_bytes(int A, int S, int nv) {
  return align_up((size_t)S * interp_chunks(A, S) * nv * sizeof(float));
}

size_t interp_tables_bytes(const Consts& c, int A, bool derivative) {
  return (size_t)A * (2 * c.S) * (derivative ? 2 : 1) * sizeof(float2);
}

size_t interp_workspace_bytes(const Consts& c, int A, int S, int nv) {
  return interp_partial_bytes(A, S, nv) + interp_tables_bytes(c, A, nv != 3);
}

int interp_residual_tables(const Consts& c, const float2* res, int A, bool derivative, float2* tables,
                           cudaStream_t st) {
  DeviceTables fixed;
  const int status = device_tables(c.S, c.P, &fixed);
  if (status != DSG_OK) return status;
  const int M = 2 * c.S;
  // u0 [A][M] = residual [A][K] . H0 [K][M], then u1 with H1: one GEMM gives u0 to every mode
  int out = table_gemm(res, A, c.K, fixed.h0, M, tables, st);
  if (out == DSG_OK && derivative) out = table_gemm(res, A, c.K, fixed.h1, M, tables + (size_t)A * M, st);
  return out;
}

int interp_reduce_tabled(int mode, const Consts& c, const float* pos, int A, const float* cen, const float* nrm,
                         const float2* w, int S, const float2* tables, void* workspace, size_t workspace_bytes,
                         float* o0, float* o1, float* o2, float* o3, const int* active, int period,
                         cudaStream_t st) {
  const int nv = nv_of(mode);
  if (workspace == nullptr || workspace_bytes < interp_partial_bytes(A, S, nv)) return DSG_ERR_WORKSPACE;
  DeviceTables fixed;
  const int status = device_tables(c.S, c.P, &fixed);
  if (status != DSG_OK) return status;
  const int M = 2 * c.S, M0 = 4 * c.S;
  float* partial = reinterpret_cast<float*>(workspace);
  const float2* u0 = tables;
  const float2* u1 = tables + (size_t)A * M;  // read by the derivative modes only
  switch (mode) {
    case 0: return launch_interp<0>(c, pos, A, cen, nrm, w, S, u0, u1, M, fixed.norm, M0, partial, o0, o1, o2, o3, active, period, st);
    case 1: return launch_interp<1>(c, pos, A, cen, nrm, w, S, u0, u1, M, fixed.norm, M0, partial, o0, o1, o2, o3, active, period, st);
    case 2: return launch_interp<2>(c, pos, A, cen, nrm, w, S, u0, u1, M, fixed.norm, M0, partial, o0, o1, o2, o3, active, period, st);
    default: return launch_interp<3>(c, pos, A, cen, nrm, w, S, u0, u1, M, fixed.norm, M0, partial, o0, o1, o2, o3, active, period, st);
  }
}

int interp_reduce(int mode, const Consts& c, const float* pos, int A, const float* cen, const float* nrm,
                  const float2* w, int S, const float2* res, void* workspace, size_t workspace_bytes,
                  float* o0, float* o1, float* o2, float* o3, const int* active, int period,
                  cudaStream_t st) {
  const int nv = nv_of(mode);
  if (workspace == nullptr || workspace_bytes < interp_workspace_bytes(c, A, S, nv)) return DSG_ERR_WORKSPACE;
  const size_t partial_bytes = interp_partial_bytes(A, S, nv);
  float2* tables = reinterpret_cast<float2*>(reinterpret_cast<char*>(workspace) + partial_bytes);
  const int status = interp_residual_tables(c, res, A, mode != 0, tables, st);
  if (status != DSG_OK) return status;
  return interp_reduce_tabled(mode, c, pos, A, cen, nrm, w, S, tables, workspace, partial_bytes, o0, o1, o2, o3,
                              active, period, st);
}

}  // namespace dsg

extern "C" int dsg_surfel_interp_tables(int32_t samples, int32_t pad, float* correlation, size_t correlation_floats,
                                        float* norm, size_t norm_floats) {
  if (samples < 8 || (samples & (samples - 1)) != 0 || !(pad == 1 || pad == 2 || pad == 4)) return DSG_ERR_ARGUMENT;
  const int K = samples * pad / 2, M = 2 * samples, M0 = 4 * samples;
  if (!correlation || !norm || correlation_floats < (size_t)K * M * 4 || norm_floats < (size_t)M0 * 2)
    return DSG_ERR_ARGUMENT;
  const dsg::HostTables t = dsg::build_tables(samples, pad);
  for (size_t i = 0; i < t.h0.size(); ++i) {  // [K][M][2] complex: H0, H1 per grid cell
    correlation[4 * i] = t.h0[i].x;
    correlation[4 * i + 1] = t.h0[i].y;
    correlation[4 * i + 2] = t.h1[i].x;
    correlation[4 * i + 3] = t.h1[i].y;
  }
  for (size_t i = 0; i < t.norm.size(); ++i) {
    norm[2 * i] = t.norm[i].x;
    norm[2 * i + 1] = t.norm[i].y;
  }
  return DSG_OK;
}
