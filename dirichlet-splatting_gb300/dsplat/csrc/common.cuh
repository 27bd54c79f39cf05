// Shared device code of the FMCW surfel kernels: chirp constants, the per-pair
// geometry in double-float arithmetic, the tangent tables of the cotangent form of the
// Dirichlet kernel, and the directly evaluated kernel used at the bin nearest a peak.
//
// Kernel of the range FFT (unit peak, negative exponent), with N = n_fft, S ADC
// samples, P = N / S and d = bin - k0 (reference: dsplat/kernels/common.slang:1-33,
// dsplat/kernels/surfel.slang:4-16):
//
//   D(d)  = sin(pi d / P) / (S sin(pi d / N)) * exp(-i pi (S - 1) d / N)
//         = nu(d) / S * (cot(pi d / N) + i),      nu(d) = sin(pi d / P) exp(-i pi d / P)
//   D'(d) = ((pi / P) q(d) (cot + i) - (pi / N) nu(d) (1 + cot^2)) / S,  q = exp(-2 i pi d / P)
//
// nu and q depend on d only modulo P, so a pair (aperture, surfel) has P numerator
// classes. For bin k with m = k - lobe (lobe = nearest bin to k0, o = lobe - k0):
//
//   cot(pi (m + o) / N) = (1 - tan(pi m / N) tan(pi o / N)) / (tan(pi m / N) + tan(pi o / N))
//
// with tan(pi m / N) read from a table. |pi o / N| <= pi / (2N) is small, so every
// bin's cotangent is a few roundings from exact; m = 0 gives 1 / tan(pi o / N) exactly,
// which keeps the forward accurate at the peak without a special case.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "dsplat_gb300.h"

// Host-side count of kernel launches made by the library (defined in misc.cu).
void dsg_count_launches(int kernels);
// Launch-shape knob (DSG_TUNE_*) set through dsg_tuning_set; 0 means automatic.
int dsg_tuning_value(int knob);
// Unique id of the calling thread's current CUDA context; 0 when unavailable (surfel.cu).
unsigned long long dsg_current_context_id();

namespace dsg {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kBig = 1.0e30f;  // tan entry standing in for +-infinity

struct Consts {
  int K, N, S, P;
  float kpm_hi, kpm_lo;  // bins per metre, double-float
  float cyc_hi, cyc_lo;  // C1 = 2 (fc + slope t0) / c0, carrier cycles per metre, double-float
  float cyc2;            // C2 = -2 slope / c0^2, cycles per metre^2
  float amp_scale;       // lambda / (8 pi)
  float fresnel_n;
  float inv_S;
  float pi_N, pi_P;      // pi / N, pi / P
  float kpm;             // bins per metre (float)
};

inline Consts make_consts(const DsgChirp& c) {
  Consts k;
  k.K = c.num_bins;
  k.N = c.n_fft;
  k.S = c.samples;
  k.P = c.pad;
  k.kpm_hi = (float)c.k0_per_meter;
  k.kpm_lo = (float)(c.k0_per_meter - (double)k.kpm_hi);
  double c1 = 2.0 * (c.fc + c.slope * c.t_start) / c.c0;
  k.cyc_hi = (float)c1;
  k.cyc_lo = (float)(c1 - (double)k.cyc_hi);
  k.cyc2 = (float)(-2.0 * c.slope / (c.c0 * c.c0));
  k.amp_scale = (float)(c.lambda_m / (8.0 * 3.14159265358979323846));
  k.fresnel_n = (float)c.fresnel_n;
  k.inv_S = (float)(1.0 / c.samples);
  k.pi_N = (float)(3.14159265358979323846 / c.n_fft);
  k.pi_P = (float)(3.14159265358979323846 / c.pad);
  k.kpm = (float)c.k0_per_meter;
  return k;
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}

__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // conj(a) * b
  return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// tan(pi m / N) for m = index - (N - 1); entries at +-N/2 are +-kBig. With big_center the
// m = 0 entry is kBig too: its cotangent then comes out near -tan(pi o / N), a finite
// stand-in that derivative kernels replace by the directly evaluated kernel.
__device__ __forceinline__ float tan_entry(int index, int N, bool big_center) {
  int m = index - (N - 1);
  if (m == 0) return big_center ? kBig : 0.0f;
  float s, c;
  sincospif((float)m / (float)N, &s, &c);
  if (fabsf(c) < 1e-30f) return s > 0.0f ? kBig : -kBig;
  return s / c;
}

// Cotangent of pi (m + o) / N from the table entry tan(pi m / N) and tl = tan(pi o / N).
__device__ __forceinline__ float cot_from(float tA, float tl) {
  return fmaf(-tA, tl, 1.0f) * rcp_approx(tA + tl);
}

// Geometry of one aperture-surfel pair (reference: dsplat/kernels/scattering.slang:16-50,
// dsplat/kernels/surfel.slang:29-85). The range r and the peak position k0 = r / spacing
// are carried as double-float so that the carrier phase (about 280 cycles at 0.35 m) and
// the offset of k0 from its nearest bin keep float32 relative precision.
struct Pair {
  float r, inv_r;
  float ux, uy, uz;
  float cosv;
  float amp, amp_cos;  // cos^2 F(cos) lambda / (8 pi r) and d/dcos; zero when cos <= 0
  float2 rot;          // carrier exp(2 pi i (fc tau + K tau (t0 - tau / 2)))
  float rate;          // d(carrier phase)/dr, rad / m
  int lobe;            // nearest bin to k0, wrapped into [0, N)
  float off;           // lobe - k0 in [-1/2, 1/2], never exactly 0
  float tl;            // tan(pi off / N)
};

__device__ __forceinline__ void fresnel_factor(float cosv, float n, float& f, float& df) {
  f = 1.0f;
  df = 0.0f;
  if (n <= 1.0f) return;
  float root = sqrtf(n * n - 1.0f + cosv * cosv);
  float inv = 1.0f / (root + cosv);
  f = (root - cosv) * inv;
  df = -2.0f * (root - cosv) * inv / root;
}

__device__ __forceinline__ void scattering(const Consts& c, float cosv, float inv_r, float& amp,
                                           float& amp_cos) {
  amp = 0.0f;
  amp_cos = 0.0f;
  if (!(cosv > 0.0f)) return;
  float f, df;
  fresnel_factor(cosv, c.fresnel_n, f, df);
  float path = c.amp_scale * inv_r;
  amp = path * cosv * cosv * f;
  amp_cos = path * (2.0f * cosv * f + cosv * cosv * df);
}

__device__ __forceinline__ void pair_range(const Consts& c, float px, float py, float pz, float cx,
                                           float cy, float cz, Pair& q, float& rl) {
  float dxh, dxl, dyh, dyl, dzh, dzl;
  two_sum(px, -cx, dxh, dxl);
  two_sum(py, -cy, dyh, dyl);
  two_sum(pz, -cz, dzh, dzl);
  float ph, pe, s, e;
  two_prod(dxh, dxh, ph, pe);
  float r2h = ph, r2l = fmaf(2.0f * dxh, dxl, pe);
  two_prod(dyh, dyh, ph, pe);
  two_sum(r2h, ph, s, e);
  r2h = s;
  r2l += e + fmaf(2.0f * dyh, dyl, pe);
  two_prod(dzh, dzh, ph, pe);
  two_sum(r2h, ph, s, e);
  r2h = s;
  r2l += e + fmaf(2.0f * dzh, dzl, pe);
  float rh;
  if (r2h > 0.0f) {
    rh = sqrtf(r2h);
    rl = (fmaf(-rh, rh, r2h) + r2l) / (2.0f * rh);
  } else {
    rh = 1e-12f;
    rl = 0.0f;
  }
  q.r = rh;
  q.inv_r = 1.0f / rh;
  q.ux = dxh * q.inv_r;
  q.uy = dyh * q.inv_r;
  q.uz = dzh * q.inv_r;
}

__device__ __forceinline__ void pair_setup(const Consts& c, float px, float py, float pz, float cx,
                                           float cy, float cz, float nx, float ny, float nz,
                                           Pair& q) {
  float rl;
  pair_range(c, px, py, pz, cx, cy, cz, q, rl);
  float rh = q.r;
  q.cosv = q.ux * nx + q.uy * ny + q.uz * nz;
  scattering(c, q.cosv, q.inv_r, q.amp, q.amp_cos);
  // k0 = r * bins-per-metre, its nearest bin and the offset lobe - k0.
  float kh, ke;
  two_prod(rh, c.kpm_hi, kh, ke);
  float kl = ke + fmaf(rh, c.kpm_lo, rl * c.kpm_hi);
  float lobe_f = rintf(kh);
  float off = (lobe_f - kh) - kl;
  if (off > 0.5f) {
    lobe_f -= 1.0f;
    off -= 1.0f;
  } else if (off < -0.5f) {
    lobe_f += 1.0f;
    off += 1.0f;
  }
  // N = 2 K is a power of two for every supported chirp (K in {32, 64, 128, 256}): the
  // residue in [0, N) is a mask, not an integer division
  const int lobe = (int)lobe_f & (c.N - 1);
  q.lobe = lobe;
  // A zero offset would make nu = 0 meet cot = inf; 1e-20 bins is far below float
  // resolution of the result and keeps every intermediate normal.
  if (fabsf(off) < 1e-20f) off = off < 0.0f ? -1e-20f : 1e-20f;
  q.off = off;
  float x = c.pi_N * off, x2 = x * x;
  q.tl = x * fmaf(x2, fmaf(x2, fmaf(x2, 17.0f / 315.0f, 2.0f / 15.0f), 1.0f / 3.0f), 1.0f);
  // Carrier phase in cycles: r C1 + r^2 C2; the integer part of r C1 is dropped exactly.
  float ch, ce;
  two_prod(rh, c.cyc_hi, ch, ce);
  float cl = ce + fmaf(rh, c.cyc_lo, rl * c.cyc_hi);
  float frac = (ch - rintf(ch)) + cl;
  frac = fmaf(c.cyc2 * rh, rh, frac);
  float sp, cp;
  sincospif(2.0f * frac, &sp, &cp);
  q.rot = make_float2(cp, sp);
  q.rate = 2.0f * kPi * fmaf(2.0f * c.cyc2, rh, c.cyc_hi);
}

// Numerator classes nu_r = sin(pi (r + o) / P) exp(-i pi (r + o) / P), r = (k - lobe) mod P.
template <int P>
__device__ __forceinline__ void numerators(float off, float2 (&nu)[P]) {
  float s0, c0;
  sincospif(off / (float)P, &s0, &c0);
#pragma unroll
  for (int r = 0; r < P; ++r) {
    float s = s0, cc = c0;
    if (r > 0) {
      float sr, cr;
      sincospif((float)r / (float)P, &sr, &cr);  // folded to constants
      s = s0 * cr + c0 * sr;
      cc = c0 * cr - s0 * sr;
    }
    nu[r] = make_float2(s * cc, -s * s);
  }
}

// q = exp(-2 i pi (r + o) / P) from nu = (1 - q) / (2 i).
__device__ __forceinline__ float2 q_from_nu(float2 nu) {
  return make_float2(1.0f + 2.0f * nu.y, -2.0f * nu.x);
}

// Directly evaluated kernel and derivative at d in [-1/2, 1/2] (the bin nearest a peak),
// with a Taylor branch at small |d| (reference: dsplat/kernels/common.slang:10-33,
// tests/reference/kernel.py:8-28). The series of sin(a d)/(S sin(b d)) is carried to d^6.
__device__ __forceinline__ void dirichlet_near(float d, int S, int N, float2& value, float2& deriv) {
  float a = kPi * (float)S / (float)N, b = kPi / (float)N;
  float h = kPi * (float)(S - 1) / (float)N;
  float ratio, dr;
  if (fabsf(d) < 0.1f) {
    float a2 = a * a, b2 = b * b;
    float c2 = (b2 - a2) / 6.0f;
    float c4 = (3.0f * a2 * a2 + 7.0f * b2 * b2 - 10.0f * a2 * b2) / 360.0f;
    float c6 = (31.0f * b2 * b2 * b2 - 49.0f * a2 * b2 * b2 + 21.0f * a2 * a2 * b2 -
                3.0f * a2 * a2 * a2) / 15120.0f;
    float d2 = d * d;
    ratio = 1.0f + d2 * (c2 + d2 * (c4 + d2 * c6));
    dr = d * (2.0f * c2 + d2 * (4.0f * c4 + d2 * 6.0f * c6));
  } else {
    float sa, ca, sb, cb;
    sincospif(d * (float)S / (float)N, &sa, &ca);
    sincospif(d / (float)N, &sb, &cb);
    float inv = 1.0f / ((float)S * sb);
    ratio = sa * inv;
    dr = (a * ca * sb - b * sa * cb) * inv / sb;
  }
  float sp, cp;
  sincospif(-(float)(S - 1) * d / (float)N, &sp, &cp);
  value = make_float2(ratio * cp, ratio * sp);
  // deriv = phase * (dr - i h ratio)
  float2 t = make_float2(dr, -h * ratio);
  deriv = make_float2(cp * t.x - sp * t.y, cp * t.y + sp * t.x);
}

}  // namespace dsg
