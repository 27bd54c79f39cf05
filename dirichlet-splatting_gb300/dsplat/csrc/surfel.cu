// FMCW surfel kernels: range profiles, JVP, the aperture-reduced family (VJP,
// correlations and their gradients), dictionary rows, the explicit Jacobian and the
// normal-bank scores. See common.cuh for the kernel algebra.
//
// Warp layout of the bin-parallel kernels: a warp is four quarters of eight lanes.
// Lane l of a quarter owns the bins k = l + 8 i, i < K / 8, so for one pair the bin
// offset m = k - lobe has the same residue modulo P (P divides 8) on all of a lane's
// bins, and its numerator class is fixed per pair. The 32 lanes first compute the
// geometry of 32 (or 128) pairs in parallel into shared memory, then every quarter
// sweeps its pairs' bins reading the geometry by broadcast.
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <atomic>
#include <mutex>
#include <algorithm>
#include <vector>
#include "common.cuh"
#include "reduce.cuh"
#include "tc.cuh"

namespace dsg {

constexpr int kWarps = 4;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float2 ldg2(const float2* p) { return __ldg(p); }

// ------------------------------------------------------------------------------------
// Range profiles: out[seg][a][k] = sum over the segment's surfels of w c D(k - k0).
// Reference: dsplat/kernels/surfel.slang:87-142 (render_bins), :61-85 (pair_geometry).
// ------------------------------------------------------------------------------------
// One CTA's share of the profiles: apertures [16 tile, 16 tile + 16) over the surfels
// [s_begin, s_end), written to out[seg][a][k]. smem: the tan table, then the warps' records.
template <int BPL, int P>
__device__ __forceinline__ void render_tile(const Consts& c, const float* __restrict__ pos, int A,
                                            const float* __restrict__ cen, const float* __restrict__ nrm,
                                            const float2* __restrict__ w, int s_begin, int s_end, int tile,
                                            int seg, float2* __restrict__ out, float* smem) {
  constexpr int REC = 2 + 2 * P;
  const int tbl_n = c.N + 8 * BPL;
  const int tbl_pad = (tbl_n + 3) & ~3;
  float* tbl = smem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qd = lane >> 3, lp = lane & 7;
  float* recs = smem + tbl_pad + warp * (32 * 4 * REC);
  for (int i = threadIdx.x; i < tbl_n; i += blockDim.x) tbl[i] = tan_entry(i, c.N, false);
  __syncthreads();

  const int a_base = (tile * kWarps + warp) * 4;
  float apx[4], apy[4], apz[4];
  bool aok[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    int a = a_base + t;
    aok[t] = a < A;
    int ac = aok[t] ? a : 0;
    apx[t] = __ldg(pos + 3 * ac);
    apy[t] = __ldg(pos + 3 * ac + 1);
    apz[t] = __ldg(pos + 3 * ac + 2);
  }
  float2 acc[BPL];
#pragma unroll
  for (int i = 0; i < BPL; ++i) acc[i] = make_float2(0.f, 0.f);
  float2 gsum = make_float2(0.f, 0.f);

  for (int s0 = s_begin; s0 < s_end; s0 += 32) {
    const int s = s0 + lane;
    const bool sv = s < s_end;
    float cx = 0.f, cy = 0.f, cz = 0.f, nx = 0.f, ny = 0.f, nz = 1.f;
    float2 ws = make_float2(0.f, 0.f);
    if (sv) {
      cx = __ldg(cen + 3 * s);
      cy = __ldg(cen + 3 * s + 1);
      cz = __ldg(cen + 3 * s + 2);
      nx = __ldg(nrm + 3 * s);
      ny = __ldg(nrm + 3 * s + 1);
      nz = __ldg(nrm + 3 * s + 2);
      ws = ldg2(w + s);
    }
    bool any = false;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      Pair q;
      pair_setup(c, apx[t], apy[t], apz[t], cx, cy, cz, nx, ny, nz, q);
      const bool ok = sv && aok[t] && q.amp > 0.0f && (ws.x != 0.0f || ws.y != 0.0f);
      float* r = recs + (lane * 4 + t) * REC;
      if (ok) {
        float2 cw = cscale(cmul(q.rot, ws), q.amp * c.inv_S);
        float2 nu[P];
        numerators<P>(q.off, nu);
        r[0] = q.tl;
        r[1] = __int_as_float(q.lobe);
#pragma unroll
        for (int k = 0; k < P; ++k) *reinterpret_cast<float2*>(r + 2 + 2 * k) = cmul(cw, nu[k]);
      } else {
        r[0] = 1.0f;
        r[1] = __int_as_float(0);
#pragma unroll
        for (int k = 0; k < P; ++k) *reinterpret_cast<float2*>(r + 2 + 2 * k) = make_float2(0.f, 0.f);
      }
      any |= ok;
    }
    const unsigned mask = __ballot_sync(kFull, any);
    __syncwarp();
    const int nb = min(32, s_end - s0);
    for (int j = 0; j < nb; ++j) {
      if (!((mask >> j) & 1u)) continue;
      const float* r = recs + (j * 4 + qd) * REC;
      const float tl = r[0];
      const int lobe = __float_as_int(r[1]);
      const int cls = (lp - lobe) & (P - 1);
      const float2 g = *reinterpret_cast<const float2*>(r + 2 + 2 * cls);
      gsum.x += g.x;
      gsum.y += g.y;
      const float* tb = tbl + (lp - lobe + c.N - 1);
#pragma unroll
      for (int i = 0; i < BPL; ++i) {
        const float cot = cot_from(tb[8 * i], tl);
        acc[i].x = fmaf(g.x, cot, acc[i].x);
        acc[i].y = fmaf(g.y, cot, acc[i].y);
      }
    }
    __syncwarp();
  }
  const int a = a_base + qd;
  if (a < A) {
    float2* o = out + ((size_t)seg * A + a) * c.K;
#pragma unroll
    for (int i = 0; i < BPL; ++i) o[lp + 8 * i] = make_float2(acc[i].x - gsum.y, acc[i].y + gsum.x);
  }
}

template <int BPL, int P>
__global__ void __launch_bounds__(128) render_kernel(Consts c, const float* __restrict__ pos,
                                                     int A, const float* __restrict__ cen,
                                                     const float* __restrict__ nrm,
                                                     const float2* __restrict__ w, int S,
                                                     int seg_len, float2* __restrict__ out) {
  extern __shared__ float smem[];
  const int s_begin = blockIdx.y * seg_len;
  render_tile<BPL, P>(c, pos, A, cen, nrm, w, s_begin, min(S, s_begin + seg_len), blockIdx.x, blockIdx.y, out,
                      smem);
}

// ------------------------------------------------------------------------------------
// Range profiles through the ADC samples (the reference sums the closed-form kernel over
// bins; this variant sums over samples): profile[a][k] = sum_{n<S} y[a][n] e^{-2 pi i n k/N}
// with y[a][n] = sum_s w_s c_s / S e^{2 pi i n k0_s / N}, so the profiles are the N-point DFT
// of the zero-padded samples (cuFFT, by the caller). A pair's samples form a geometric
// sequence: a lane owns SPL consecutive samples n0 .. n0 + SPL - 1, anchors the first one
// exactly (sincospif of the turn (n0 lobe mod N) / N - n0 off / N, lobe and off as in
// pair_setup) and advances by the pair's step e^{2 pi i (lobe - off) / N}, one complex
// multiply per sample: the sweep issues no MUFU operation, and every lane re-anchors each
// pair, so a rounding never travels more than SPL samples. Chunks of 32 surfels (centers,
// normals, weights) reach shared memory by bulk copies (cp.async.bulk with mbarrier
// completion, double buffered) when the inputs are 16-byte aligned; every wait is bounded
// and a wait that runs out sets the status word.
// ------------------------------------------------------------------------------------
constexpr int kAdcChunk = 32;
constexpr int kAdcRec = 6;  // per (surfel, aperture): g.re, g.im, step.re, step.im, lobe bits, off

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          tc::smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
      : "memory");
}

template <int SPL>
__global__ void __launch_bounds__(128) render_adc_kernel(Consts c, const float* __restrict__ pos, int A,
                                                         const float* __restrict__ cen,
                                                         const float* __restrict__ nrm,
                                                         const float2* __restrict__ w, int S, int seg_len,
                                                         int bulk, float2* __restrict__ out,
                                                         int* __restrict__ status) {
  __shared__ __align__(16) float s_cen[2][3 * kAdcChunk];
  __shared__ __align__(16) float s_nrm[2][3 * kAdcChunk];
  __shared__ __align__(16) float2 s_w[2][kAdcChunk];
  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ __align__(16) float s_rec[kWarps][kAdcChunk * 4 * kAdcRec];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qd = lane >> 3, lp = lane & 7;
  const int s_begin = blockIdx.y * seg_len;
  const int s_end = min(S, s_begin + seg_len);
  const int count = max(0, s_end - s_begin);
  const int whole = bulk ? count / kAdcChunk : 0;  // chunks that arrive by bulk copies
  const int nchunk = (count + kAdcChunk - 1) / kAdcChunk;
  if (threadIdx.x == 0) {
    tc::mbar_init(&s_bar[0], 1);
    tc::mbar_init(&s_bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (whole > 0) {
      tc::mbar_expect_tx(&s_bar[0], 32 * kAdcChunk);
      bulk_load(s_cen[0], cen + 3 * (size_t)s_begin, 12 * kAdcChunk, &s_bar[0]);
      bulk_load(s_nrm[0], nrm + 3 * (size_t)s_begin, 12 * kAdcChunk, &s_bar[0]);
      bulk_load(s_w[0], w + s_begin, 8 * kAdcChunk, &s_bar[0]);
    }
  }
  __syncthreads();

  const int a_base = (blockIdx.x * kWarps + warp) * 4;
  float apx[4], apy[4], apz[4];
  bool aok[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int a = a_base + t;
    aok[t] = a < A;
    const int ac = aok[t] ? a : 0;
    apx[t] = __ldg(pos + 3 * ac);
    apy[t] = __ldg(pos + 3 * ac + 1);
    apz[t] = __ldg(pos + 3 * ac + 2);
  }
  float2 acc[SPL];
#pragma unroll
  for (int i = 0; i < SPL; ++i) acc[i] = make_float2(0.f, 0.f);
  float* rec = s_rec[warp];
  const int n0 = lp * SPL;
  uint32_t parity0 = 0, parity1 = 0;
  bool failed = false;
  const float two_over_N = 2.0f / (float)c.N;

  for (int ch = 0; ch < nchunk; ++ch) {
    const int buf = ch & 1;
    const int s = s_begin + ch * kAdcChunk + lane;
    const bool sv = s < s_end;
    float cx = 0.f, cy = 0.f, cz = 0.f, nx = 0.f, ny = 0.f, nz = 1.f;
    float2 ws = make_float2(0.f, 0.f);
    if (ch < whole) {
      const bool ok = tc::mbar_wait_plain(&s_bar[buf], buf ? parity1 : parity0);
      if (buf) parity1 ^= 1u; else parity0 ^= 1u;
      failed |= !ok;
      cx = s_cen[buf][3 * lane];
      cy = s_cen[buf][3 * lane + 1];
      cz = s_cen[buf][3 * lane + 2];
      nx = s_nrm[buf][3 * lane];
      ny = s_nrm[buf][3 * lane + 1];
      nz = s_nrm[buf][3 * lane + 2];
      ws = s_w[buf][lane];
    } else if (sv) {
      cx = __ldg(cen + 3 * s);
      cy = __ldg(cen + 3 * s + 1);
      cz = __ldg(cen + 3 * s + 2);
      nx = __ldg(nrm + 3 * s);
      ny = __ldg(nrm + 3 * s + 1);
      nz = __ldg(nrm + 3 * s + 2);
      ws = ldg2(w + s);
    }
    // every thread has read this chunk's buffer; the other one was read before the last
    // barrier, so the next chunk may overwrite it
    __syncthreads();
    if (threadIdx.x == 0 && ch + 1 < whole) {
      const int nb = buf ^ 1, s1 = s_begin + (ch + 1) * kAdcChunk;
      tc::mbar_expect_tx(&s_bar[nb], 32 * kAdcChunk);
      bulk_load(s_cen[nb], cen + 3 * (size_t)s1, 12 * kAdcChunk, &s_bar[nb]);
      bulk_load(s_nrm[nb], nrm + 3 * (size_t)s1, 12 * kAdcChunk, &s_bar[nb]);
      bulk_load(s_w[nb], w + s1, 8 * kAdcChunk, &s_bar[nb]);
    }
    bool any = false;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      Pair q;
      pair_setup(c, apx[t], apy[t], apz[t], cx, cy, cz, nx, ny, nz, q);
      const bool ok = sv && aok[t] && q.amp > 0.0f && (ws.x != 0.0f || ws.y != 0.0f);
      float* r = rec + (lane * 4 + t) * kAdcRec;
      if (ok) {
        const float2 g = cscale(cmul(q.rot, ws), q.amp * c.inv_S);
        float s1, c1, s2, c2;
        sincospif((float)q.lobe * two_over_N, &s1, &c1);  // exact turn: lobe < N, N a power of two
        sincospif(-q.off * two_over_N, &s2, &c2);
        const float2 step = cmul(make_float2(c1, s1), make_float2(c2, s2));
        r[0] = g.x;
        r[1] = g.y;
        r[2] = step.x;
        r[3] = step.y;
        r[4] = __int_as_float(q.lobe);
        r[5] = q.off;
      } else {
        r[0] = 0.0f;
        r[1] = 0.0f;
      }
      any |= ok;
    }
    const unsigned mask = __ballot_sync(kFull, any);
    __syncwarp();
    const int nb = min(kAdcChunk, s_end - (s_begin + ch * kAdcChunk));
    for (int j = 0; j < nb; ++j) {
      if (!((mask >> j) & 1u)) continue;
      const float* r = rec + (j * 4 + qd) * kAdcRec;
      const float2 g = make_float2(r[0], r[1]);
      if (g.x == 0.0f && g.y == 0.0f) continue;  // the quarter's own pair is empty
      const float2 step = make_float2(r[2], r[3]);
      const int lobe = __float_as_int(r[4]);
      // turn of sample n0: (n0 lobe mod N) / N - n0 off / N, the integer part exactly
      const int whole_turn = (n0 * lobe) & (c.N - 1);
      const float turn = (float)whole_turn / (float)c.N - (float)n0 * r[5] / (float)c.N;
      float sa, ca;
      sincospif(2.0f * turn, &sa, &ca);
      float2 z = cmul(g, make_float2(ca, sa));
#pragma unroll
      for (int i = 0; i < SPL; ++i) {
        acc[i].x += z.x;
        acc[i].y += z.y;
        z = cmul(z, step);
      }
    }
    __syncwarp();
  }
  if (failed) {  // a copy never arrived: the status word says so and the tile's samples are NaN
    atomicExch(status, 1);
#pragma unroll
    for (int i = 0; i < SPL; ++i) acc[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
  }
  const int a = a_base + qd;
  if (a < A) {
    float2* o = out + ((size_t)blockIdx.y * A + a) * c.S + n0;
#pragma unroll
    for (int i = 0; i < SPL; ++i) o[i] = acc[i];
  }
}

// ------------------------------------------------------------------------------------
// Profiles of many scenes in one persistent launch (no counterpart in the reference,
// which renders one scene per call): the work items are (scene, 16-aperture tile), the
// largest scenes' tiles first, and every CTA takes the next item from a device counter
// until none is left; a tile covers all of its scene's surfels, so nothing needs a second
// pass. Scenes may differ in apertures, surfels and chirp (range bins 128 or 256, pad 2).
// ------------------------------------------------------------------------------------
struct SceneWork {
  Consts c;
  const float* pos;
  const float* cen;
  const float* nrm;
  const float2* w;
  float2* out;
  int A, S;
};

__global__ void __launch_bounds__(128) render_scenes_kernel(const SceneWork* __restrict__ scenes,
                                                            const int2* __restrict__ items, int count,
                                                            int* __restrict__ next, int* __restrict__ status) {
  extern __shared__ float smem[];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= count) return;  // the same value in every thread of the CTA
    const int2 work = items[item];
    const SceneWork& d = scenes[work.x];
    if (d.c.P == 2 && d.c.K == 128)
      render_tile<16, 2>(d.c, d.pos, d.A, d.cen, d.nrm, d.w, 0, d.S, work.y, 0, d.out, smem);
    else if (d.c.P == 2 && d.c.K == 256)
      render_tile<32, 2>(d.c, d.pos, d.A, d.cen, d.nrm, d.w, 0, d.S, work.y, 0, d.out, smem);
    else if (threadIdx.x == 0)
      atomicExch(status, 1);  // the host validates the chirps; this is a second line of defence
    __syncthreads();  // the table and s_item are rewritten for the next item
  }
}

// ------------------------------------------------------------------------------------
// JVP: out[a][k] = sum_s e1 D(k - k0) + e2 D'(k - k0) (reference:
// dsplat/kernels/surfel.slang:144-221, jvp_bins). With the big-centre table the bin
// nearest each peak first receives a finite stand-in; the quarter's owner lane replaces
// it by the directly evaluated term through a per-warp correction row, in pair order.
// ------------------------------------------------------------------------------------
template <int BPL, int P>
__global__ void __launch_bounds__(128) jvp_kernel(Consts c, const float* __restrict__ pos, int A,
                                                  const float* __restrict__ cen,
                                                  const float* __restrict__ nrm,
                                                  const float2* __restrict__ w,
                                                  const float* __restrict__ dcen,
                                                  const float* __restrict__ dnrm,
                                                  const float2* __restrict__ dw, int S,
                                                  int seg_len, float2* __restrict__ out) {
  constexpr int REC = 4 + 4 * P;  // tl, lobe, h1[P], h2[P], delta
  extern __shared__ float smem[];
  const int tbl_n = c.N + 8 * BPL;
  const int tbl_pad = (tbl_n + 3) & ~3;
  float* tbl = smem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qd = lane >> 3, lp = lane & 7;
  float* recs = smem + tbl_pad + warp * (32 * 4 * REC + 4 * 2 * c.K);
  float2* corr = reinterpret_cast<float2*>(recs + 32 * 4 * REC);  // [4][K]
  for (int i = threadIdx.x; i < tbl_n; i += blockDim.x) tbl[i] = tan_entry(i, c.N, true);
  for (int i = lane; i < 4 * c.K; i += 32) corr[i] = make_float2(0.f, 0.f);
  __syncthreads();

  const int a_base = (blockIdx.x * kWarps + warp) * 4;
  float apx[4], apy[4], apz[4];
  bool aok[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    int a = a_base + t;
    aok[t] = a < A;
    int ac = aok[t] ? a : 0;
    apx[t] = __ldg(pos + 3 * ac);
    apy[t] = __ldg(pos + 3 * ac + 1);
    apz[t] = __ldg(pos + 3 * ac + 2);
  }
  float2 acc[BPL];
#pragma unroll
  for (int i = 0; i < BPL; ++i) acc[i] = make_float2(0.f, 0.f);
  float2 csum = make_float2(0.f, 0.f);

  const int s_begin = blockIdx.y * seg_len;
  const int s_end = min(S, s_begin + seg_len);
  for (int s0 = s_begin; s0 < s_end; s0 += 32) {
    const int s = s0 + lane;
    const bool sv = s < s_end;
    float cx = 0.f, cy = 0.f, cz = 0.f, nx = 0.f, ny = 0.f, nz = 1.f;
    float dcx = 0.f, dcy = 0.f, dcz = 0.f, dnx = 0.f, dny = 0.f, dnz = 0.f;
    float2 ws = make_float2(0.f, 0.f), dws = make_float2(0.f, 0.f);
    if (sv) {
      cx = __ldg(cen + 3 * s); cy = __ldg(cen + 3 * s + 1); cz = __ldg(cen + 3 * s + 2);
      nx = __ldg(nrm + 3 * s); ny = __ldg(nrm + 3 * s + 1); nz = __ldg(nrm + 3 * s + 2);
      dcx = __ldg(dcen + 3 * s); dcy = __ldg(dcen + 3 * s + 1); dcz = __ldg(dcen + 3 * s + 2);
      dnx = __ldg(dnrm + 3 * s); dny = __ldg(dnrm + 3 * s + 1); dnz = __ldg(dnrm + 3 * s + 2);
      ws = ldg2(w + s);
      dws = ldg2(dw + s);
    }
    bool any = false;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      Pair q;
      pair_setup(c, apx[t], apy[t], apz[t], cx, cy, cz, nx, ny, nz, q);
      const bool ok = sv && aok[t] && q.amp > 0.0f;
      float* r = recs + (lane * 4 + t) * REC;
      if (ok) {
        const float dr = -(q.ux * dcx + q.uy * dcy + q.uz * dcz);
        const float dcos = ((q.cosv * q.ux - nx) * dcx + (q.cosv * q.uy - ny) * dcy +
                            (q.cosv * q.uz - nz) * dcz) * q.inv_r +
                           q.ux * dnx + q.uy * dny + q.uz * dnz;
        const float damp = -q.amp * dr * q.inv_r + q.amp_cos * dcos;
        const float dphi = q.rate * dr;
        // e1 = rot (w (damp + i amp dphi) + amp dw), e2 = -rot w amp kpm dr
        float2 inner = cadd(cmul(ws, make_float2(damp, q.amp * dphi)), cscale(dws, q.amp));
        const float2 e1 = cmul(q.rot, inner);
        const float2 e2 = cscale(cmul(q.rot, ws), -q.amp * c.kpm * dr);
        float2 nu[P];
        numerators<P>(q.off, nu);
        r[0] = q.tl;
        r[1] = __int_as_float(q.lobe);
        float2 h1_0 = make_float2(0.f, 0.f), h2_0 = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < P; ++k) {
          const float2 qv = q_from_nu(nu[k]);
          float2 h1 = cscale(cadd(cmul(e1, nu[k]), cscale(cmul(e2, qv), c.pi_P)), c.inv_S);
          float2 h2 = cscale(cmul(e2, nu[k]), -c.pi_N * c.inv_S);
          *reinterpret_cast<float2*>(r + 2 + 2 * k) = h1;
          *reinterpret_cast<float2*>(r + 2 + 2 * P + 2 * k) = h2;
          if (k == 0) { h1_0 = h1; h2_0 = h2; }
        }
        float2 delta = make_float2(0.f, 0.f);
        if (q.lobe < c.K) {
          float2 d0, d1;
          dirichlet_near(q.off, c.S, c.N, d0, d1);
          const float cg = cot_from(kBig, q.tl);
          // stand-in the sweep adds at the nearest bin: h1 (cg + i) + h2 (1 + cg^2)
          float2 stand = cadd(cmul(h1_0, make_float2(cg, 1.0f)), cscale(h2_0, 1.0f + cg * cg));
          delta = csub(cadd(cmul(e1, d0), cmul(e2, d1)), stand);
        }
        *reinterpret_cast<float2*>(r + 2 + 4 * P) = delta;
      } else {
        r[0] = 1.0f;
        r[1] = __int_as_float(c.N - 1);  // m = k - lobe never 0 on observed bins
#pragma unroll
        for (int k = 0; k < 2 * P + 1; ++k) *reinterpret_cast<float2*>(r + 2 + 2 * k) = make_float2(0.f, 0.f);
      }
      any |= ok;
    }
    const unsigned mask = __ballot_sync(kFull, any);
    __syncwarp();
    const int nb = min(32, s_end - s0);
    for (int j = 0; j < nb; ++j) {
      if (!((mask >> j) & 1u)) continue;
      const float* r = recs + (j * 4 + qd) * REC;
      const float tl = r[0];
      const int lobe = __float_as_int(r[1]);
      const int cls = (lp - lobe) & (P - 1);
      const float2 h1 = *reinterpret_cast<const float2*>(r + 2 + 2 * cls);
      const float2 h2 = *reinterpret_cast<const float2*>(r + 2 + 2 * P + 2 * cls);
      csum.x += h2.x - h1.y;
      csum.y += h2.y + h1.x;
      const float* tb = tbl + (lp - lobe + c.N - 1);
#pragma unroll
      for (int i = 0; i < BPL; ++i) {
        const float cot = cot_from(tb[8 * i], tl);
        const float cot2 = cot * cot;
        acc[i].x = fmaf(h1.x, cot, fmaf(h2.x, cot2, acc[i].x));
        acc[i].y = fmaf(h1.y, cot, fmaf(h2.y, cot2, acc[i].y));
      }
      if (lobe < c.K && (lobe & 7) == lp) {
        const float2 d = *reinterpret_cast<const float2*>(r + 2 + 4 * P);
        float2 cur = corr[qd * c.K + lobe];
        corr[qd * c.K + lobe] = cadd(cur, d);
      }
    }
    __syncwarp();
  }
  const int a = a_base + qd;
  if (a < A) {
    float2* o = out + ((size_t)blockIdx.y * A + a) * c.K;
#pragma unroll
    for (int i = 0; i < BPL; ++i) {
      const int k = lp + 8 * i;
      const float2 cr = corr[qd * c.K + k];
      o[k] = make_float2(acc[i].x + csum.x + cr.x, acc[i].y + csum.y + cr.y);
    }
  }
}

// Sum of segment partials [segments][n] into out[n], in segment order.
__global__ void segment_sum_kernel(const float2* __restrict__ partial, int segments, int64_t n,
                                   float2* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 s = partial[i];
  for (int g = 1; g < segments; ++g) {
    float2 v = partial[(int64_t)g * n + i];
    s.x += v.x;
    s.y += v.y;
  }
  out[i] = s;
}

// ------------------------------------------------------------------------------------
// Aperture-reduced family. Per pair the sufficient statistics over all bins
//   Z0 = sum conj(D) r, Z1 = sum conj(D') r, N0 = sum |D|^2, N1 = sum Re(conj(D) D')
// are chained to the outputs and summed over the CTA's aperture chunk in order.
// MODE 0: correlate (corr, norm). 1/2: correlate_gradient, width 3/6. 3: vjp.
// Reference: dsplat/kernels/correlate.slang:75-108 (surfel_correlate), :171-235
// (surfel_correlate_gradient), dsplat/kernels/surfel.slang:223-311 (vjp_bins).
// ------------------------------------------------------------------------------------
template <int P>
__host__ __device__ constexpr int reduce_record() { return 16 + 2 * P; }

template <int BPL, int P, int MODE>
__global__ void __launch_bounds__(128) reduce_kernel(Consts c, const float* __restrict__ pos, int A,
                                                     const float* __restrict__ cen,
                                                     const float* __restrict__ nrm,
                                                     const float2* __restrict__ w, int S,
                                                     const float2* __restrict__ res,
                                                     int chunk_len, int chunks,
                                                     float* __restrict__ partial,
                                                     const int* __restrict__ active, int period) {
  constexpr int NV = ModeInfo<MODE>::NV;
  // Optional active set: surfel s counts only when s mod period < *active. A CTA without
  // any active surfel writes zero partials and leaves (the same decision in every thread).
  if (active != nullptr) {
    const int limit = __ldg(active);
    const int s0 = blockIdx.x * kWarps * 4;
    bool any = false;
    for (int j = 0; j < kWarps * 4 && !any; ++j) any = s0 + j < S && (s0 + j) % period < limit;
    if (!any) {
      for (int i = threadIdx.x; i < kWarps * 4 * NV; i += blockDim.x) {
        const int t = s0 + i / NV;
        if (t < S) partial[((size_t)t * chunks + blockIdx.y) * NV + i % NV] = 0.0f;
      }
      return;
    }
  }
  constexpr bool kGrad = MODE == 1 || MODE == 2;
  constexpr bool kNorm = MODE != 3;
  constexpr bool kDeriv = MODE != 0;
  // record: tl, lobe, nu[P], d0, d1, amp, amp_cos, ux, uy, uz, cos, inv_r, rate, rot
  constexpr int R_NU = 2, R_D0 = 2 + 2 * P, R_D1 = R_D0 + 2, R_AMP = R_D1 + 2;
  constexpr int R_AMPC = R_AMP + 1, R_U = R_AMPC + 1, R_COS = R_U + 3, R_INVR = R_COS + 1;
  constexpr int R_RATE = R_INVR + 1, R_ROT = R_RATE + 1;
  constexpr int REC = reduce_record<P>();
  static_assert(REC >= R_ROT + 2, "record layout");
  extern __shared__ float smem[];
  const int tbl_n = c.N + 8 * BPL;
  const int tbl_pad = (tbl_n + 3) & ~3;
  float* tbl = smem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qd = lane >> 3, lp = lane & 7;
  float* recs = smem + tbl_pad + warp * (32 * REC);
  for (int i = threadIdx.x; i < tbl_n; i += blockDim.x) tbl[i] = tan_entry(i, c.N, true);
  __syncthreads();

  const int s = (blockIdx.x * kWarps + warp) * 4 + qd;
  const bool s_ok = s < S;
  const int sc = s_ok ? s : 0;
  const float cx = __ldg(cen + 3 * sc), cy = __ldg(cen + 3 * sc + 1), cz = __ldg(cen + 3 * sc + 2);
  const float nx = __ldg(nrm + 3 * sc), ny = __ldg(nrm + 3 * sc + 1), nz = __ldg(nrm + 3 * sc + 2);
  float2 ws = make_float2(0.f, 0.f);
  if (MODE == 3) ws = ldg2(w + sc);

  float accv[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) accv[v] = 0.0f;

  const int a_begin = blockIdx.y * chunk_len;
  const int a_end = min(A, a_begin + chunk_len);
  const float pi_P = c.pi_P, pi_N = c.pi_N, inv_S = c.inv_S;
  for (int a0 = a_begin; a0 < a_end; a0 += 8) {
    {  // pair geometry: lane (lp, qd) takes aperture a0 + lp with its quarter's surfel
      const int aa = a0 + lp;
      const bool ok = s_ok && aa < a_end;
      float* r = recs + (lp * 4 + qd) * REC;
      Pair q;
      const int ac = ok ? aa : 0;
      pair_setup(c, __ldg(pos + 3 * ac), __ldg(pos + 3 * ac + 1), __ldg(pos + 3 * ac + 2), cx, cy,
                 cz, nx, ny, nz, q);
      if (ok && q.amp > 0.0f) {
        float2 nu[P];
        numerators<P>(q.off, nu);
        r[0] = q.tl;
        r[1] = __int_as_float(q.lobe);
#pragma unroll
        for (int k = 0; k < P; ++k) *reinterpret_cast<float2*>(r + R_NU + 2 * k) = nu[k];
        float2 d0 = make_float2(0.f, 0.f), d1 = make_float2(0.f, 0.f);
        if (q.lobe < c.K) dirichlet_near(q.off, c.S, c.N, d0, d1);
        *reinterpret_cast<float2*>(r + R_D0) = d0;
        *reinterpret_cast<float2*>(r + R_D1) = d1;
        r[R_AMP] = q.amp;
        r[R_AMPC] = q.amp_cos;
        r[R_U] = q.ux;
        r[R_U + 1] = q.uy;
        r[R_U + 2] = q.uz;
        r[R_COS] = q.cosv;
        r[R_INVR] = q.inv_r;
        r[R_RATE] = q.rate;
        r[R_ROT] = q.rot.x;
        r[R_ROT + 1] = q.rot.y;
      } else {
        for (int k = 0; k < REC; ++k) r[k] = 0.0f;
        r[0] = 1.0f;
        r[1] = __int_as_float(c.N - 1);
      }
    }
    __syncwarp();
    const int nb = min(8, a_end - a0);
    for (int j = 0; j < nb; ++j) {
      const float* r = recs + (j * 4 + qd) * REC;
      const float amp = r[R_AMP];
      if (__ballot_sync(kFull, amp > 0.0f) == 0u) continue;
      const float2* row = res + (size_t)(a0 + j) * c.K;
      float2 u[BPL];
      float2 ru = make_float2(0.f, 0.f);
#pragma unroll
      for (int i = 0; i < BPL; ++i) {
        u[i] = ldg2(row + lp + 8 * i);
        ru.x += u[i].x;
        ru.y += u[i].y;
      }
      const float tl = r[0];
      const int lobe = __float_as_int(r[1]);
      const int cls = (lp - lobe) & (P - 1);
      const float* tb = tbl + (lp - lobe + c.N - 1);
      float2 sa = make_float2(0.f, 0.f), sb = make_float2(0.f, 0.f);
      float c1 = 0.f, c2 = 0.f, c3 = 0.f;
#pragma unroll
      for (int i = 0; i < BPL; ++i) {
        const float cot = cot_from(tb[8 * i], tl);
        sa.x = fmaf(cot, u[i].x, sa.x);
        sa.y = fmaf(cot, u[i].y, sa.y);
        if (kDeriv) {
          const float cot2 = cot * cot;
          sb.x = fmaf(cot2, u[i].x, sb.x);
          sb.y = fmaf(cot2, u[i].y, sb.y);
          if (kGrad) {
            c1 += cot;
            c3 = fmaf(cot2, cot, c3);
          }
        }
        if (kNorm) c2 = fmaf(cot, cot, c2);
      }
      float nc = (float)BPL;
      const bool near = lobe < c.K;
      const float2 ul = near ? ldg2(row + lobe) : make_float2(0.f, 0.f);
      if (near && (lobe & 7) == lp) {  // remove the stand-in of the nearest bin
        const float cg = cot_from(kBig, tl);
        const float cg2 = cg * cg;
        sa.x -= cg * ul.x; sa.y -= cg * ul.y;
        sb.x -= cg2 * ul.x; sb.y -= cg2 * ul.y;
        c1 -= cg; c2 -= cg2; c3 -= cg2 * cg;
        ru.x -= ul.x; ru.y -= ul.y;
        nc -= 1.0f;
      }
#pragma unroll
      for (int o = P; o < 8; o <<= 1) {
        sa.x += __shfl_xor_sync(kFull, sa.x, o);
        sa.y += __shfl_xor_sync(kFull, sa.y, o);
        ru.x += __shfl_xor_sync(kFull, ru.x, o);
        ru.y += __shfl_xor_sync(kFull, ru.y, o);
        if (kDeriv) {
          sb.x += __shfl_xor_sync(kFull, sb.x, o);
          sb.y += __shfl_xor_sync(kFull, sb.y, o);
        }
        if (kNorm) {
          c2 += __shfl_xor_sync(kFull, c2, o);
          nc += __shfl_xor_sync(kFull, nc, o);
        }
        if (kGrad) {
          c1 += __shfl_xor_sync(kFull, c1, o);
          c3 += __shfl_xor_sync(kFull, c3, o);
        }
      }
      const float2 nu = *reinterpret_cast<const float2*>(r + R_NU + 2 * cls);
      const float2 qv = q_from_nu(nu);
      const float2 amir = make_float2(sa.x + ru.y, sa.y - ru.x);  // A - i R
      float2 z0 = cscale(cmulc(nu, amir), inv_S);
      float2 z1 = make_float2(0.f, 0.f);
      float n0 = 0.f, n1 = 0.f;
      if (kDeriv) {
        const float2 rb = make_float2(ru.x + sb.x, ru.y + sb.y);
        z1 = cscale(csub(cscale(cmulc(qv, amir), pi_P), cscale(cmulc(nu, rb), pi_N)), inv_S);
      }
      const float nn = nu.x * nu.x + nu.y * nu.y;
      if (kNorm) n0 = nn * (c2 + nc) * inv_S * inv_S;
      if (kGrad) {
        const float re_nq = nu.x * qv.x + nu.y * qv.y;
        n1 = (pi_P * re_nq * (c2 + nc) - pi_N * nn * (c1 + c3)) * inv_S * inv_S;
      }
#pragma unroll
      for (int o = 1; o < P; o <<= 1) {
        z0.x += __shfl_xor_sync(kFull, z0.x, o);
        z0.y += __shfl_xor_sync(kFull, z0.y, o);
        if (kDeriv) {
          z1.x += __shfl_xor_sync(kFull, z1.x, o);
          z1.y += __shfl_xor_sync(kFull, z1.y, o);
        }
        if (kNorm) n0 += __shfl_xor_sync(kFull, n0, o);
        if (kGrad) n1 += __shfl_xor_sync(kFull, n1, o);
      }
      if (near) {
        const float2 d0 = *reinterpret_cast<const float2*>(r + R_D0);
        const float2 d1 = *reinterpret_cast<const float2*>(r + R_D1);
        z0 = cadd(z0, cmulc(d0, ul));
        if (kDeriv) z1 = cadd(z1, cmulc(d1, ul));
        if (kNorm) n0 += d0.x * d0.x + d0.y * d0.y;
        if (kGrad) n1 += d0.x * d1.x + d0.y * d1.y;
      }
      // chain to the outputs
      const float uu[3] = {r[R_U], r[R_U + 1], r[R_U + 2]};
      const float nv[3] = {nx, ny, nz};
      chain_outputs<MODE>(c, amp, r[R_AMPC], r[R_COS], r[R_INVR], r[R_RATE], uu,
                          make_float2(r[R_ROT], r[R_ROT + 1]), nv, ws, z0, z1, n0, n1, accv);
    }
    __syncwarp();
  }
  if (lp == 0 && s_ok) {
    // an inactive candidate of a CTA that had active ones still reports zeros
    const bool live = active == nullptr || s % period < __ldg(active);
    float* p = partial + ((size_t)s * chunks + blockIdx.y) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) p[v] = live ? accv[v] : 0.0f;
  }
}

// ------------------------------------------------------------------------------------
// Dictionary rows c sqrt(area) D(k - k0) (reference: dsplat/kernels/surfel.slang:313-378).
// Thread = (surfel, aperture); adjacent threads take adjacent surfels, so every bin's
// store is coalesced. real: row (2k + part) A + a; else [a K + k, s] complex.
// ------------------------------------------------------------------------------------
template <int P>
__global__ void __launch_bounds__(128) design_kernel(Consts c, const float* __restrict__ pos, int A,
                                                     const float* __restrict__ cen,
                                                     const float* __restrict__ nrm,
                                                     const float* __restrict__ areas, int S,
                                                     int real, float* __restrict__ out) {
  extern __shared__ float smem[];
  const int tbl_n = c.N + c.K;
  for (int i = threadIdx.x; i < tbl_n; i += blockDim.x) smem[i] = tan_entry(i, c.N, false);
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y;
  if (s >= S) return;
  Pair q;
  pair_setup(c, __ldg(pos + 3 * a), __ldg(pos + 3 * a + 1), __ldg(pos + 3 * a + 2),
             __ldg(cen + 3 * s), __ldg(cen + 3 * s + 1), __ldg(cen + 3 * s + 2),
             __ldg(nrm + 3 * s), __ldg(nrm + 3 * s + 1), __ldg(nrm + 3 * s + 2), q);
  float2 g[P];
  const bool vis = q.amp > 0.0f;
  if (vis) {
    float2 cw = cscale(q.rot, q.amp * sqrtf(__ldg(areas + s)) * c.inv_S);
    float2 nu[P];
    numerators<P>(q.off, nu);
#pragma unroll
    for (int k = 0; k < P; ++k) g[k] = cmul(cw, nu[k]);
  } else {
#pragma unroll
    for (int k = 0; k < P; ++k) g[k] = make_float2(0.f, 0.f);
  }
  const float* tb = smem + (c.N - 1 - q.lobe);
  for (int k0 = 0; k0 < c.K; k0 += P) {
#pragma unroll
    for (int j = 0; j < P; ++j) {
      const int k = k0 + j;
      float2 term = make_float2(0.f, 0.f);
      if (vis) {
        const float cot = cot_from(tb[k], q.tl);
        const float2 gg = g[(k - q.lobe) & (P - 1)];
        term = make_float2(gg.x * cot - gg.y, gg.y * cot + gg.x);
      }
      if (real) {
        out[((size_t)(2 * k) * A + a) * S + s] = term.x;
        out[((size_t)(2 * k + 1) * A + a) * S + s] = term.y;
      } else {
        reinterpret_cast<float2*>(out)[((size_t)a * c.K + k) * S + s] = term;
      }
    }
  }
}

// ------------------------------------------------------------------------------------
// Explicit columns and their center/normal derivatives, without area (reference:
// dsplat/kernels/correlate.slang:237-281). Thread = (surfel, aperture), loop over bins.
// ------------------------------------------------------------------------------------
template <int P>
__global__ void __launch_bounds__(128) jacobian_kernel(Consts c, const float* __restrict__ pos,
                                                       int A, const float* __restrict__ cen,
                                                       const float* __restrict__ nrm, int S,
                                                       float2* __restrict__ cols,
                                                       float2* __restrict__ jac) {
  extern __shared__ float smem[];
  const int tbl_n = c.N + c.K;
  for (int i = threadIdx.x; i < tbl_n; i += blockDim.x) smem[i] = tan_entry(i, c.N, true);
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y;
  if (s >= S) return;
  const float nv[3] = {__ldg(nrm + 3 * s), __ldg(nrm + 3 * s + 1), __ldg(nrm + 3 * s + 2)};
  Pair q;
  pair_setup(c, __ldg(pos + 3 * a), __ldg(pos + 3 * a + 1), __ldg(pos + 3 * a + 2),
             __ldg(cen + 3 * s), __ldg(cen + 3 * s + 1), __ldg(cen + 3 * s + 2), nv[0], nv[1],
             nv[2], q);
  const bool vis = q.amp > 0.0f;
  float2 nu[P];
  numerators<P>(q.off, nu);
  float2 d0 = make_float2(0.f, 0.f), d1 = make_float2(0.f, 0.f);
  dirichlet_near(q.off, c.S, c.N, d0, d1);
  const float uu[3] = {q.ux, q.uy, q.uz};
  float da[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) da[j] = (q.amp * uu[j] + q.amp_cos * (q.cosv * uu[j] - nv[j])) * q.inv_r;
  const float* tb = smem + (c.N - 1 - q.lobe);
  for (int k = 0; k < c.K; ++k) {
    const size_t e = ((size_t)a * c.K + k) * S + s;
    if (!vis) {
      cols[e] = make_float2(0.f, 0.f);
      for (int j = 0; j < 6; ++j) jac[e * 6 + j] = make_float2(0.f, 0.f);
      continue;
    }
    float2 D, Dp;
    if (k == q.lobe) {
      D = d0;
      Dp = d1;
    } else {
      const float cot = cot_from(tb[k], q.tl);
      const int cls = (k - q.lobe) & (P - 1);
      const float2 n = nu[cls], qv = q_from_nu(n);
      const float2 ci = make_float2(cot, 1.0f);
      D = cscale(cmul(n, ci), c.inv_S);
      Dp = cscale(csub(cscale(cmul(qv, ci), c.pi_P), cscale(n, c.pi_N * (1.0f + cot * cot))), c.inv_S);
    }
    const float2 z = cmul(D, q.rot);
    const float2 dz = cmul(Dp, q.rot);
    cols[e] = cscale(z, q.amp);
    // d col / d c_j = da_j z + amp u_j (kpm dz - i rate z)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float au = q.amp * uu[j];
      float2 v = make_float2(da[j] * z.x + au * (c.kpm * dz.x + q.rate * z.y),
                             da[j] * z.y + au * (c.kpm * dz.y - q.rate * z.x));
      jac[e * 6 + j] = v;
      jac[e * 6 + 3 + j] = cscale(z, q.amp_cos * uu[j]);
    }
  }
}

// ------------------------------------------------------------------------------------
// Normal-bank scores (reference: dsplat/kernels/correlate.slang:110-169). A warp owns
// one candidate. Its lanes first evaluate 32 apertures' pair geometry and per-aperture
// correlation in parallel (from the exact bin sum, or by Catmull-Rom interpolation of an
// oversampled FFT range table) into a per-warp record; then each lane takes one normal
// of the bank (lane 0 of the first chunk: the candidate's own normal) and adds the 32
// apertures two at a time with packed FP32x2 arithmetic (fma.rn.f32x2: one instruction
// for an even and an odd aperture), so the bank phase issues about half the
// instructions of a scalar loop. The even and the odd apertures are summed in ascending
// order in the two halves and the halves added at the end, so the result is fixed; a
// lane holds three packed accumulators, not three per normal, which keeps the kernel at
// full occupancy.
// ------------------------------------------------------------------------------------
constexpr int kOrientWarps = 8;
// per aperture 6 floats: ux, uy, uz, path corr.re, path corr.im, path^2 norm, with
// path = lambda / (8 pi r); the amplitude of a normal is then path cos^2 F(cos). An
// aperture pair (2i, 2i + 1) is stored as 12 floats, each quantity's even value beside
// its odd one: [ux ux uy uy | uz uz cr cr | ci ci nn nn], three 16-byte loads.
constexpr int kOrientRec = 6;

// cos^2 F(cos) for cos > 0, else 0 (the angular part of the scattering amplitude).
template <bool FRESNEL>
__device__ __forceinline__ float bank_angular(const Consts& c, float cosv) {
  if (!(cosv > 0.0f)) return 0.0f;
  float a = cosv * cosv;
  if (FRESNEL) {
    float f, df;
    fresnel_factor(cosv, c.fresnel_n, f, df);
    a *= f;
  }
  return a;
}

// Selection of the best normal per candidate (BEST): the certificate of each normal,
// |Re corr|^2 (real mode) or |corr|^2, over max(norm, 1e-60) times the residual energy, in
// float64, with corr and norm scaled by the candidate's sqrt(area) and area in float32 first
// (the arithmetic of dsplat.certificate.orient_candidates); the largest wins, NaN first and
// the lowest normal index on ties, as torch.max. which = 0 is the candidate's own normal.
struct OrientBest {
  const float* areas;    // [C]
  const double* energy;  // one value on the device
  int real_mode;
  int* which;            // [C]
  float* top;            // [C]
};

__device__ __forceinline__ bool orient_better(double v, int i, double bv, int bi) {
  const bool vn = v != v, bn = bv != bv;
  if (vn != bn) return vn;
  if (vn) return i < bi;
  return v > bv || (v == bv && i < bi);
}

template <int P, bool FRESNEL, bool BEST>
__global__ void __launch_bounds__(kOrientWarps * 32, 4) orientations_kernel(
    Consts c, const float* __restrict__ pos, int A, const float* __restrict__ cen,
    const float* __restrict__ nrm, int C, const float* __restrict__ bank, int bank_size,
    const float2* __restrict__ res, const float2* __restrict__ table,
    const float* __restrict__ norm_table, int oversample, float* __restrict__ out, OrientBest best) {
  extern __shared__ float smem[];
  const int tbl_n = c.N + c.K;
  float* tbl = smem;
  if (table == nullptr)
    for (int i = threadIdx.x; i < tbl_n; i += blockDim.x) tbl[i] = tan_entry(i, c.N, true);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* rec = smem + ((tbl_n + 3) & ~3) + warp * 32 * kOrientRec;
  const int s = blockIdx.x * (int)(blockDim.x >> 5) + warp;  // blockDim: 1..kOrientWarps warps
  if (s >= C) return;  // warp-uniform; no block barrier follows
  const float cx = __ldg(cen + 3 * s), cy = __ldg(cen + 3 * s + 1), cz = __ldg(cen + 3 * s + 2);
  const float own[3] = {__ldg(nrm + 3 * s), __ldg(nrm + 3 * s + 1), __ldg(nrm + 3 * s + 2)};
  const int size = c.N * oversample;
  const int normals = bank_size + 1;
  float* o = BEST ? nullptr : out + (size_t)s * normals * 3;
  double best_value = 0.0;
  int best_index = 0x7fffffff;
  for (int j0 = 0; j0 < normals; j0 += 32) {
    const int j = j0 + lane;
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    if (j == 0) {
      ex = own[0];
      ey = own[1];
      ez = own[2];
    } else if (j < normals) {
      ex = __ldg(bank + 3 * (j - 1));
      ey = __ldg(bank + 3 * (j - 1) + 1);
      ez = __ldg(bank + 3 * (j - 1) + 2);
    }
    const float2 ex2 = make_float2(ex, ex), ey2 = make_float2(ey, ey), ez2 = make_float2(ez, ez);
    float2 acc0 = make_float2(0.f, 0.f), acc1 = acc0, acc2 = acc0;
    for (int a0 = 0; a0 < A; a0 += 32) {
      const int a = a0 + lane;
      if (a < A) {
        Pair q;
        pair_setup(c, __ldg(pos + 3 * a), __ldg(pos + 3 * a + 1), __ldg(pos + 3 * a + 2), cx, cy, cz,
                   own[0], own[1], own[2], q);
        float2 corr;
        float norm;
        if (table != nullptr) {
          // x = k0 * oversample with k0 = lobe - off
          const float x = ((float)q.lobe - q.off) * (float)oversample;
          const float fb = floorf(x);
          const float t = x - fb;
          const int base = (int)fb;
          const float t2 = t * t, t3 = t2 * t;
          const float wts[4] = {-0.5f * t + t2 - 0.5f * t3, 1.0f - 2.5f * t2 + 1.5f * t3,
                                0.5f * t + 2.0f * t2 - 1.5f * t3, -0.5f * t2 + 0.5f * t3};
          float2 v = make_float2(0.f, 0.f);
          float nn = 0.0f;
          int first;  // the taps base - 1 .. base + 2, wrapped
          if ((size & (size - 1)) == 0) {
            first = (base - 1) & (size - 1);  // a power-of-two table (the usual oversample)
          } else {
            first = (base - 1) % size;
            if (first < 0) first += size;
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int k = first + i < size ? first + i : first + i - size;
            const float2 tv = ldg2(table + (size_t)a * size + k);
            v.x += wts[i] * tv.x;
            v.y += wts[i] * tv.y;
            nn += wts[i] * __ldg(norm_table + k);
          }
          corr = cmulc(q.rot, v);  // conj(rot) * v
          norm = fmaxf(nn, 0.0f);
        } else {
          float2 nu[P];
          numerators<P>(q.off, nu);
          float2 z = make_float2(0.f, 0.f);
          float n0 = 0.0f;
          const float* tb = tbl + (c.N - 1 - q.lobe);
          const float2* row = res + (size_t)a * c.K;
          for (int k = 0; k < c.K; ++k) {
            float2 D;
            if (k == q.lobe) {
              float2 d1;
              dirichlet_near(q.off, c.S, c.N, D, d1);
            } else {
              const float cot = cot_from(tb[k], q.tl);
              D = cscale(cmul(nu[(k - q.lobe) & (P - 1)], make_float2(cot, 1.0f)), c.inv_S);
            }
            z = cadd(z, cmulc(D, ldg2(row + k)));
            n0 += D.x * D.x + D.y * D.y;
          }
          corr = cmulc(q.rot, z);
          norm = n0;
        }
        const float path = c.amp_scale * q.inv_r;
        float* slot = rec + (lane >> 1) * 12 + (lane & 1);
        slot[0] = q.ux;
        slot[2] = q.uy;
        slot[4] = q.uz;
        slot[6] = path * corr.x;
        slot[8] = path * corr.y;
        slot[10] = path * path * norm;
      } else {  // past the last aperture: a zero record adds nothing to the odd half
        float* slot = rec + (lane >> 1) * 12 + (lane & 1);
#pragma unroll
        for (int k = 0; k < 12; k += 2) slot[k] = 0.0f;
      }
      __syncwarp();
      const int pairs = (min(32, A - a0) + 1) >> 1;
#pragma unroll 2
      for (int i = 0; i < pairs; ++i) {
        const float4 g0 = *reinterpret_cast<const float4*>(rec + i * 12);
        const float4 g1 = *reinterpret_cast<const float4*>(rec + i * 12 + 4);
        const float4 g2 = *reinterpret_cast<const float4*>(rec + i * 12 + 8);
        float2 cosv = __fmul2_rn(make_float2(g0.x, g0.y), ex2);
        cosv = __ffma2_rn(make_float2(g0.z, g0.w), ey2, cosv);
        cosv = __ffma2_rn(make_float2(g1.x, g1.y), ez2, cosv);
        float2 a;
        if (FRESNEL) {
          a = make_float2(bank_angular<true>(c, cosv.x), bank_angular<true>(c, cosv.y));
        } else {  // cos^2 where cos > 0, else 0 (fmaxf also maps NaN to 0)
          a = make_float2(fmaxf(cosv.x, 0.0f), fmaxf(cosv.y, 0.0f));
          a = __fmul2_rn(a, a);
        }
        acc0 = __ffma2_rn(a, make_float2(g1.z, g1.w), acc0);
        acc1 = __ffma2_rn(a, make_float2(g2.x, g2.y), acc1);
        acc2 = __ffma2_rn(__fmul2_rn(a, a), make_float2(g2.z, g2.w), acc2);
      }
      __syncwarp();
    }
    if (j < normals) {
      if (BEST) {
        const float root = sqrtf(__ldg(best.areas + s));
        const float re = (acc0.x + acc0.y) * root, im = (acc1.x + acc1.y) * root;
        const float nm = (acc2.x + acc2.y) * (root * root);
        double num;
        if (best.real_mode) {
          num = (double)re * (double)re;
        } else {
          const double mag = hypot((double)re, (double)im);
          num = mag * mag;
        }
        const double value = num / (fmax((double)nm, 1e-60) * __ldg(best.energy));
        if (best_index == 0x7fffffff || orient_better(value, j, best_value, best_index)) {
          best_value = value;
          best_index = j;
        }
      } else {
        o[3 * j] = acc0.x + acc0.y;
        o[3 * j + 1] = acc1.x + acc1.y;
        o[3 * j + 2] = acc2.x + acc2.y;
      }
    }
  }
  if (BEST) {
    for (int off = 16; off > 0; off >>= 1) {
      const double ov = __shfl_xor_sync(kFull, best_value, off);
      const int oi = __shfl_xor_sync(kFull, best_index, off);
      if (oi != 0x7fffffff && (best_index == 0x7fffffff || orient_better(ov, oi, best_value, best_index))) {
        best_value = ov;
        best_index = oi;
      }
    }
    if (lane == 0) {
      best.which[s] = best_index;
      best.top[s] = (float)best_value;
    }
  }
}

}  // namespace dsg

// ======================================================================================
// Host side
// ======================================================================================
using namespace dsg;

namespace {

bool chirp_ok(const DsgChirp* c) {
  if (!c) return false;
  if (c->samples <= 0 || c->pad <= 0 || c->n_fft != c->samples * c->pad) return false;
  if (c->num_bins != c->n_fft / 2) return false;
  if (!(c->pad == 1 || c->pad == 2 || c->pad == 4)) return false;
  const int K = c->num_bins;
  return K == 32 || K == 64 || K == 128 || K == 256;
}

int render_segments(const DsgChirp* c, int A, int S) {
  const int tiles = (A + 15) / 16;
  int seg = (target_ctas() + tiles - 1) / tiles;
  const int max_seg = (S + 31) / 32;
  if (seg > max_seg) seg = max_seg;
  if (seg < 1) seg = 1;
  (void)c;
  return seg;
}

int reduce_chunks(int A, int S) {
  const int tiles = (S + 15) / 16;
  int ch = (target_ctas() + tiles - 1) / tiles;
  const int max_ch = (A + 7) / 8;
  if (ch > max_ch) ch = max_ch;
  if (ch < 1) ch = 1;
  return ch;
}

int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

template <typename F>
int dispatch_kp(int K, int P, F&& f) {
  // f.template operator()<BPL, P>()
  switch (K) {
    case 32:
      if (P == 1) return f.template run<4, 1>();
      if (P == 2) return f.template run<4, 2>();
      return f.template run<4, 4>();
    case 64:
      if (P == 1) return f.template run<8, 1>();
      if (P == 2) return f.template run<8, 2>();
      return f.template run<8, 4>();
    case 128:
      if (P == 1) return f.template run<16, 1>();
      if (P == 2) return f.template run<16, 2>();
      return f.template run<16, 4>();
    case 256:
      if (P == 1) return f.template run<32, 1>();
      if (P == 2) return f.template run<32, 2>();
      return f.template run<32, 4>();
  }
  return DSG_ERR_UNSUPPORTED;
}

template <typename F>
int dispatch_p(int P, F&& f) {
  if (P == 1) return f.template run<1>();
  if (P == 2) return f.template run<2>();
  if (P == 4) return f.template run<4>();
  return DSG_ERR_UNSUPPORTED;
}

size_t table_floats(int N, int K) { return (size_t)((N + K + 8 + 3) & ~3); }

struct RenderLaunch {
  Consts c; const float* pos; int A; const float* cen; const float* nrm; const float2* w; int S;
  float2* out; float2* partial; int seg; cudaStream_t st;
  template <int BPL, int P>
  int run() {
    constexpr int REC = 2 + 2 * P;
    const size_t smem = (table_floats(c.N, 8 * BPL) + kWarps * 32 * 4 * REC) * sizeof(float);
    auto kern = render_kernel<BPL, P>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int seg_len = ((S + seg - 1) / seg + 31) / 32 * 32;
    const int nseg = (S + seg_len - 1) / seg_len;
    dim3 grid((A + 15) / 16, nseg > 0 ? nseg : 1);
    float2* dst = grid.y == 1 ? out : partial;
    kern<<<grid, 128, smem, st>>>(c, pos, A, cen, nrm, w, S, seg_len, dst);
    dsg_count_launches(1);
    if (grid.y > 1) {
      const int64_t n = (int64_t)A * c.K;
      segment_sum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(partial, grid.y, n, out);
      dsg_count_launches(1);
    }
    return launch_status();
  }
};

struct JvpLaunch {
  Consts c; const float* pos; int A; const float* cen; const float* nrm; const float2* w;
  const float* dcen; const float* dnrm; const float2* dw; int S; float2* out; float2* partial;
  int seg; cudaStream_t st;
  template <int BPL, int P>
  int run() {
    constexpr int REC = 4 + 4 * P;
    const size_t smem = (table_floats(c.N, 8 * BPL) + kWarps * (32 * 4 * REC + 8 * c.K)) * sizeof(float);
    auto kern = jvp_kernel<BPL, P>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int seg_len = ((S + seg - 1) / seg + 31) / 32 * 32;
    const int nseg = (S + seg_len - 1) / seg_len;
    dim3 grid((A + 15) / 16, nseg > 0 ? nseg : 1);
    float2* dst = grid.y == 1 ? out : partial;
    kern<<<grid, 128, smem, st>>>(c, pos, A, cen, nrm, w, dcen, dnrm, dw, S, seg_len, dst);
    dsg_count_launches(1);
    if (grid.y > 1) {
      const int64_t n = (int64_t)A * c.K;
      segment_sum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(partial, grid.y, n, out);
      dsg_count_launches(1);
    }
    return launch_status();
  }
};

template <int MODE>
struct ReduceLaunch {
  Consts c; const float* pos; int A; const float* cen; const float* nrm; const float2* w; int S;
  const float2* res; float* partial; float* o0; float* o1; float* o2; float* o3; cudaStream_t st;
  const int* active = nullptr; int period = 1;
  template <int BPL, int P>
  int run() {
    constexpr int REC = reduce_record<P>();
    const size_t smem = (table_floats(c.N, 8 * BPL) + kWarps * 32 * REC) * sizeof(float);
    auto kern = reduce_kernel<BPL, P, MODE>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int chunks = reduce_chunks(A, S);
    const int chunk_len = ((A + chunks - 1) / chunks + 7) / 8 * 8;
    const int nch = (A + chunk_len - 1) / chunk_len;
    dim3 grid((S + 15) / 16, nch);
    kern<<<grid, 128, smem, st>>>(c, pos, A, cen, nrm, w, S, res, chunk_len, nch, partial, active, period);
    const long long values = (long long)S * ModeInfo<MODE>::NV;
    chunk_sum_kernel<MODE><<<(unsigned)((values + 255) / 256), 256, 0, st>>>(partial, S, nch, o0, o1, o2, o3);
    dsg_count_launches(2);
    return launch_status();
  }
};

struct DesignLaunch {
  Consts c; const float* pos; int A; const float* cen; const float* nrm; const float* areas; int S;
  int real; float* out; cudaStream_t st;
  template <int P>
  int run() {
    const size_t smem = table_floats(c.N, c.K) * sizeof(float);
    dim3 grid((S + 127) / 128, A);
    design_kernel<P><<<grid, 128, smem, st>>>(c, pos, A, cen, nrm, areas, S, real, out);
    dsg_count_launches(1);
    return launch_status();
  }
};

struct JacobianLaunch {
  Consts c; const float* pos; int A; const float* cen; const float* nrm; int S;
  float2* cols; float2* jac; cudaStream_t st;
  template <int P>
  int run() {
    const size_t smem = table_floats(c.N, c.K) * sizeof(float);
    dim3 grid((S + 127) / 128, A);
    jacobian_kernel<P><<<grid, 128, smem, st>>>(c, pos, A, cen, nrm, S, cols, jac);
    dsg_count_launches(1);
    return launch_status();
  }
};

struct OrientLaunch {
  Consts c; const float* pos; int A; const float* cen; const float* nrm; int C; const float* bank;
  int nb; const float2* res; const float2* table; const float* ntab; int ov; float* out;
  cudaStream_t st;
  OrientBest best{};  // selection mode when best.which is set
  template <int P>
  int run() {
    const int tuned = dsg_tuning_value(DSG_TUNE_ORIENT_WARPS);
    const int warps = tuned > 0 && tuned <= kOrientWarps ? tuned : kOrientWarps;
    const size_t smem = (((c.N + c.K + 3) & ~3) + warps * 32 * kOrientRec) * sizeof(float);
    const dim3 grid((C + warps - 1) / warps);
    const bool fresnel = c.fresnel_n > 1.0f, select = best.which != nullptr;
    if (fresnel && select)
      orientations_kernel<P, true, true><<<grid, warps * 32, smem, st>>>(c, pos, A, cen, nrm, C, bank, nb, res,
                                                                         table, ntab, ov, out, best);
    else if (fresnel)
      orientations_kernel<P, true, false><<<grid, warps * 32, smem, st>>>(c, pos, A, cen, nrm, C, bank, nb, res,
                                                                          table, ntab, ov, out, best);
    else if (select)
      orientations_kernel<P, false, true><<<grid, warps * 32, smem, st>>>(c, pos, A, cen, nrm, C, bank, nb, res,
                                                                          table, ntab, ov, out, best);
    else
      orientations_kernel<P, false, false><<<grid, warps * 32, smem, st>>>(c, pos, A, cen, nrm, C, bank, nb, res,
                                                                           table, ntab, ov, out, best);
    dsg_count_launches(1);
    return launch_status();
  }
};

}  // namespace

extern "C" {

size_t dsg_surfel_render_workspace_bytes(const DsgChirp* chirp, int32_t apertures, int32_t surfels) {
  if (!chirp_ok(chirp) || apertures <= 0 || surfels <= 0) return 0;
  const int seg = render_segments(chirp, apertures, surfels);
  if (seg <= 1) return 0;
  return (size_t)seg * apertures * chirp->num_bins * 2 * sizeof(float);
}

int dsg_surfel_render(const DsgChirp* chirp, const float* positions, int32_t apertures,
                      const float* centers, const float* normals, const float* weights,
                      int32_t surfels, float* out, void* workspace, size_t workspace_bytes,
                      void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || surfels < 0 || (apertures > 0 && (!positions || !out))) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (apertures == 0) return DSG_OK;
  if (surfels == 0) {
    cudaMemsetAsync(out, 0, (size_t)apertures * chirp->num_bins * 2 * sizeof(float), st);
    return launch_status();
  }
  if (!centers || !normals || !weights) return DSG_ERR_ARGUMENT;
  const size_t need = dsg_surfel_render_workspace_bytes(chirp, apertures, surfels);
  if (need > 0 && (workspace == nullptr || workspace_bytes < need)) return DSG_ERR_WORKSPACE;
  RenderLaunch L{make_consts(*chirp), positions, apertures, centers, normals,
                 reinterpret_cast<const float2*>(weights), surfels, reinterpret_cast<float2*>(out),
                 reinterpret_cast<float2*>(workspace), render_segments(chirp, apertures, surfels), st};
  return dispatch_kp(chirp->num_bins, chirp->pad, L);
}

size_t dsg_surfel_render_samples_workspace_bytes(const DsgChirp* chirp, int32_t apertures, int32_t surfels) {
  if (!chirp_ok(chirp) || apertures <= 0 || surfels <= 0) return 0;
  const int seg = render_segments(chirp, apertures, surfels);
  if (seg <= 1) return 0;
  return (size_t)seg * apertures * chirp->samples * 2 * sizeof(float);
}

int dsg_surfel_render_samples(const DsgChirp* chirp, const float* positions, int32_t apertures,
                              const float* centers, const float* normals, const float* weights,
                              int32_t surfels, float* samples, void* workspace, size_t workspace_bytes,
                              int32_t* status, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  const int spl = chirp->samples / 8;
  if (chirp->samples % 8 != 0 || !(spl == 2 || spl == 4 || spl == 8 || spl == 16 || spl == 32))
    return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || surfels < 0 || (apertures > 0 && (!positions || !samples))) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (apertures == 0) return DSG_OK;
  if (surfels == 0) {
    cudaMemsetAsync(samples, 0, (size_t)apertures * chirp->samples * 2 * sizeof(float), st);
    return launch_status();
  }
  if (!centers || !normals || !weights || !status) return DSG_ERR_ARGUMENT;
  const size_t need = dsg_surfel_render_samples_workspace_bytes(chirp, apertures, surfels);
  if (need > 0 && (workspace == nullptr || workspace_bytes < need)) return DSG_ERR_WORKSPACE;
  const Consts c = make_consts(*chirp);
  const int seg = render_segments(chirp, apertures, surfels);
  const int seg_len = ((surfels + seg - 1) / seg + 31) / 32 * 32;  // whole chunks: 16-byte-aligned copies
  const int nseg = (surfels + seg_len - 1) / seg_len;
  const bool aligned = ((reinterpret_cast<uintptr_t>(centers) | reinterpret_cast<uintptr_t>(normals) |
                         reinterpret_cast<uintptr_t>(weights)) & 15u) == 0;
  dim3 grid((apertures + 15) / 16, nseg > 0 ? nseg : 1);
  float2* dst = grid.y == 1 ? reinterpret_cast<float2*>(samples) : reinterpret_cast<float2*>(workspace);
  const float2* w = reinterpret_cast<const float2*>(weights);
  switch (spl) {
    case 2: render_adc_kernel<2><<<grid, 128, 0, st>>>(c, positions, apertures, centers, normals, w, surfels, seg_len, aligned, dst, status); break;
    case 4: render_adc_kernel<4><<<grid, 128, 0, st>>>(c, positions, apertures, centers, normals, w, surfels, seg_len, aligned, dst, status); break;
    case 8: render_adc_kernel<8><<<grid, 128, 0, st>>>(c, positions, apertures, centers, normals, w, surfels, seg_len, aligned, dst, status); break;
    case 16: render_adc_kernel<16><<<grid, 128, 0, st>>>(c, positions, apertures, centers, normals, w, surfels, seg_len, aligned, dst, status); break;
    default: render_adc_kernel<32><<<grid, 128, 0, st>>>(c, positions, apertures, centers, normals, w, surfels, seg_len, aligned, dst, status); break;
  }
  dsg_count_launches(1);
  if (grid.y > 1) {
    const int64_t n = (int64_t)apertures * chirp->samples;
    segment_sum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(reinterpret_cast<const float2*>(workspace),
                                                                     grid.y, n, reinterpret_cast<float2*>(samples));
    dsg_count_launches(1);
  }
  return launch_status();
}

int dsg_surfel_jvp(const DsgChirp* chirp, const float* positions, int32_t apertures,
                   const float* centers, const float* normals, const float* weights,
                   const float* delta_centers, const float* delta_normals,
                   const float* delta_weights, int32_t surfels, float* out, void* workspace,
                   size_t workspace_bytes, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || surfels < 0 || (apertures > 0 && (!positions || !out))) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (apertures == 0) return DSG_OK;
  if (surfels == 0) {
    cudaMemsetAsync(out, 0, (size_t)apertures * chirp->num_bins * 2 * sizeof(float), st);
    return launch_status();
  }
  if (!centers || !normals || !weights || !delta_centers || !delta_normals || !delta_weights)
    return DSG_ERR_ARGUMENT;
  const size_t need = dsg_surfel_render_workspace_bytes(chirp, apertures, surfels);
  if (need > 0 && (workspace == nullptr || workspace_bytes < need)) return DSG_ERR_WORKSPACE;
  JvpLaunch L{make_consts(*chirp), positions, apertures, centers, normals,
              reinterpret_cast<const float2*>(weights), delta_centers, delta_normals,
              reinterpret_cast<const float2*>(delta_weights), surfels,
              reinterpret_cast<float2*>(out), reinterpret_cast<float2*>(workspace),
              render_segments(chirp, apertures, surfels), st};
  return dispatch_kp(chirp->num_bins, chirp->pad, L);
}

// Workspace of dsg_surfel_render_scenes: the device scene table, the work items and the
// queue counter, each 256-byte aligned.
static size_t scenes_layout(const DsgRenderScene* scenes, int32_t count, size_t* items_at, size_t* counter_at,
                            int* items) {
  int total = 0;
  for (int i = 0; i < count; ++i) total += (scenes[i].apertures + 15) / 16;
  const size_t table = ((size_t)count * sizeof(SceneWork) + 255) & ~(size_t)255;
  const size_t list = ((size_t)total * sizeof(int2) + 255) & ~(size_t)255;
  *items_at = table;
  *counter_at = table + list;
  *items = total;
  return table + list + 256;
}

size_t dsg_surfel_render_scenes_workspace_bytes(const DsgRenderScene* scenes, int32_t count) {
  if (!scenes || count <= 0) return 0;
  size_t items_at, counter_at;
  int items;
  return scenes_layout(scenes, count, &items_at, &counter_at, &items);
}

int dsg_surfel_render_scenes(const DsgRenderScene* scenes, int32_t count, void* workspace, size_t workspace_bytes,
                             int32_t* status, void* stream) {
  if (count < 0 || (count > 0 && !scenes)) return DSG_ERR_ARGUMENT;
  if (count == 0) return DSG_OK;
  if (!status) return DSG_ERR_ARGUMENT;
  for (int i = 0; i < count; ++i) {
    const DsgRenderScene& d = scenes[i];
    if (!chirp_ok(&d.chirp) || d.chirp.pad != 2 || (d.chirp.num_bins != 128 && d.chirp.num_bins != 256))
      return DSG_ERR_UNSUPPORTED;
    if (d.apertures < 0 || d.surfels < 0) return DSG_ERR_ARGUMENT;
    if (d.apertures > 0 && (!d.positions || !d.out)) return DSG_ERR_ARGUMENT;
    if (d.apertures > 0 && d.surfels > 0 && (!d.centers || !d.normals || !d.weights)) return DSG_ERR_ARGUMENT;
  }
  size_t items_at, counter_at;
  int total;
  const size_t need = scenes_layout(scenes, count, &items_at, &counter_at, &total);
  if (!workspace || workspace_bytes < need) return DSG_ERR_WORKSPACE;
  if (total == 0) return DSG_OK;
  // host staging: scene table, items (largest scenes first), counter = 0
  std::vector<uint8_t> staging(need, 0);
  SceneWork* table = reinterpret_cast<SceneWork*>(staging.data());
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) {
    const DsgRenderScene& d = scenes[i];
    table[i] = SceneWork{make_consts(d.chirp), d.positions, d.centers, d.normals,
                         reinterpret_cast<const float2*>(d.weights), reinterpret_cast<float2*>(d.out), d.apertures,
                         d.surfels};
    order[i] = i;
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (double)scenes[x].surfels * scenes[x].chirp.num_bins > (double)scenes[y].surfels * scenes[y].chirp.num_bins;
  });
  int2* list = reinterpret_cast<int2*>(staging.data() + items_at);
  int k = 0;
  for (int i : order)
    for (int t = 0; t < (scenes[i].apertures + 15) / 16; ++t) list[k++] = make_int2(i, t);
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(workspace, staging.data(), need, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return launch_status();
  // shared memory of the widest chirp (256 bins): the table and four warps' records
  const size_t smem = (table_floats(512, 256) + kWarps * 32 * 4 * (2 + 2 * 2)) * sizeof(float);
  if (cudaFuncSetAttribute(render_scenes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return launch_status();
  int per_sm = 0, sms = 152, device = 0;
  if (cudaGetDevice(&device) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, render_scenes_kernel, 128, smem);
  const int grid = std::min(total, std::max(1, per_sm) * sms);
  uint8_t* base = reinterpret_cast<uint8_t*>(workspace);
  render_scenes_kernel<<<grid, 128, smem, st>>>(reinterpret_cast<const SceneWork*>(base),
                                                reinterpret_cast<const int2*>(base + items_at), total,
                                                reinterpret_cast<int*>(base + counter_at), status);
  dsg_count_launches(1);
  return launch_status();
}

// Chunk partials of the exact (bin-sum) form.
static size_t exact_workspace_bytes(int32_t apertures, int32_t surfels, int32_t values_per_surfel) {
  return (size_t)surfels * reduce_chunks(apertures, surfels) * values_per_surfel * sizeof(float);
}

// Both forms fit: the interpolated form (the default) also holds the aperture tables.
size_t dsg_surfel_reduce_workspace_bytes(const DsgChirp* chirp, int32_t apertures, int32_t surfels,
                                         int32_t values_per_surfel) {
  if (!chirp_ok(chirp) || apertures <= 0 || surfels <= 0 || values_per_surfel <= 0) return 0;
  const size_t exact = exact_workspace_bytes(apertures, surfels, values_per_surfel);
  const size_t interp = interp_workspace_bytes(make_consts(*chirp), apertures, surfels, values_per_surfel);
  return exact > interp ? exact : interp;
}

// The interpolated form unless the caller needs the exact one (fixed scratch) or the
// DSG_TUNE_CORRELATION_FORM knob selects it.
static bool use_interp(bool allowed) {
  return allowed && dsg_tuning_value(DSG_TUNE_CORRELATION_FORM) != DSG_CORRELATION_EXACT;
}

static int reduce_common(int mode, const DsgChirp* chirp, const float* positions, int32_t A,
                         const float* centers, const float* normals, const float* weights,
                         int32_t S, const float* residual, float* o0, float* o1, float* o2,
                         float* o3, void* workspace, size_t workspace_bytes, void* stream,
                         bool interp_allowed = true) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (A < 0 || S < 0) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  const int nv = mode == 0 ? 3 : mode == 1 ? 12 : mode == 2 ? 21 : 8;
  if (S == 0) return DSG_OK;
  if (!centers || !normals || !o0 || !o1) return DSG_ERR_ARGUMENT;
  if (A == 0) {  // empty sums
    size_t n0 = (size_t)S * (mode == 3 ? 3 : 2), n1 = (size_t)S * (mode == 3 ? 3 : 1);
    cudaMemsetAsync(o0, 0, n0 * sizeof(float), st);
    cudaMemsetAsync(o1, 0, n1 * sizeof(float), st);
    const int W = mode == 1 ? 3 : 6;
    if (mode == 3) cudaMemsetAsync(o2, 0, (size_t)S * 2 * sizeof(float), st);
    if (mode == 1 || mode == 2) {
      cudaMemsetAsync(o2, 0, (size_t)S * W * 2 * sizeof(float), st);
      cudaMemsetAsync(o3, 0, (size_t)S * W * sizeof(float), st);
    }
    return launch_status();
  }
  if (!positions || !residual) return DSG_ERR_ARGUMENT;
  const Consts c = make_consts(*chirp);
  const float2* w = reinterpret_cast<const float2*>(weights);
  const float2* res = reinterpret_cast<const float2*>(residual);
  if (use_interp(interp_allowed))
    return interp_reduce(mode, c, positions, A, centers, normals, w, S, res, workspace, workspace_bytes,
                         o0, o1, o2, o3, nullptr, 1, st);
  const size_t need = exact_workspace_bytes(A, S, nv);
  if (workspace == nullptr || workspace_bytes < need) return DSG_ERR_WORKSPACE;
  float* part = reinterpret_cast<float*>(workspace);
  switch (mode) {
    case 0: { ReduceLaunch<0> L{c, positions, A, centers, normals, w, S, res, part, o0, o1, o2, o3, st};
              return dispatch_kp(c.K, c.P, L); }
    case 1: { ReduceLaunch<1> L{c, positions, A, centers, normals, w, S, res, part, o0, o1, o2, o3, st};
              return dispatch_kp(c.K, c.P, L); }
    case 2: { ReduceLaunch<2> L{c, positions, A, centers, normals, w, S, res, part, o0, o1, o2, o3, st};
              return dispatch_kp(c.K, c.P, L); }
    default: { ReduceLaunch<3> L{c, positions, A, centers, normals, w, S, res, part, o0, o1, o2, o3, st};
               return dispatch_kp(c.K, c.P, L); }
  }
}

int dsg_surfel_vjp(const DsgChirp* chirp, const float* positions, int32_t apertures,
                   const float* centers, const float* normals, const float* weights,
                   int32_t surfels, const float* upstream, float* grad_centers,
                   float* grad_normals, float* grad_weights, void* workspace,
                   size_t workspace_bytes, void* stream) {
  if (surfels > 0 && (!weights || !grad_weights)) return DSG_ERR_ARGUMENT;
  return reduce_common(3, chirp, positions, apertures, centers, normals, weights, surfels, upstream,
                       grad_centers, grad_normals, grad_weights, nullptr, workspace,
                       workspace_bytes, stream);
}

int dsg_surfel_correlate(const DsgChirp* chirp, const float* positions, int32_t apertures,
                         const float* centers, const float* normals, int32_t candidates,
                         const float* residual, float* corr, float* norm, void* workspace,
                         size_t workspace_bytes, void* stream) {
  return reduce_common(0, chirp, positions, apertures, centers, normals, nullptr, candidates,
                       residual, corr, norm, nullptr, nullptr, workspace, workspace_bytes, stream);
}

int dsg_surfel_correlate_active(const DsgChirp* chirp, const float* positions, int32_t apertures,
                                const float* centers, const float* normals, int32_t candidates,
                                const float* residual, const int32_t* active, int32_t period,
                                float* corr, float* norm, void* workspace, size_t workspace_bytes,
                                void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || candidates < 0 || period < 1 || !active) return DSG_ERR_ARGUMENT;
  if (candidates == 0) return DSG_OK;
  if (apertures == 0)
    return reduce_common(0, chirp, positions, apertures, centers, normals, nullptr, candidates,
                         residual, corr, norm, nullptr, nullptr, workspace, workspace_bytes, stream);
  if (!positions || !residual || !centers || !normals || !corr || !norm) return DSG_ERR_ARGUMENT;
  const Consts c = make_consts(*chirp);
  if (use_interp(true))
    return interp_reduce(0, c, positions, apertures, centers, normals, nullptr, candidates,
                         reinterpret_cast<const float2*>(residual), workspace, workspace_bytes, corr, norm,
                         nullptr, nullptr, active, period, (cudaStream_t)stream);
  const size_t need = exact_workspace_bytes(apertures, candidates, 3);
  if (workspace == nullptr || workspace_bytes < need) return DSG_ERR_WORKSPACE;
  ReduceLaunch<0> L{c, positions, apertures, centers, normals, nullptr, candidates,
                    reinterpret_cast<const float2*>(residual), reinterpret_cast<float*>(workspace),
                    corr, norm, nullptr, nullptr, (cudaStream_t)stream};
  L.active = active;
  L.period = period;
  return dispatch_kp(c.K, c.P, L);
}

int dsg_surfel_correlate_gradient(const DsgChirp* chirp, const float* positions,
                                  int32_t apertures, const float* centers, const float* normals,
                                  int32_t candidates, const float* residual, int32_t width,
                                  float* corr, float* norm, float* dcorr, float* dnorm,
                                  void* workspace, size_t workspace_bytes, void* stream) {
  if (width != 3 && width != 6) return DSG_ERR_ARGUMENT;
  if (candidates > 0 && (!dcorr || !dnorm)) return DSG_ERR_ARGUMENT;
  return reduce_common(width == 3 ? 1 : 2, chirp, positions, apertures, centers, normals, nullptr,
                       candidates, residual, corr, norm, dcorr, dnorm, workspace,
                       workspace_bytes, stream);
}

size_t dsg_surfel_residual_tables_bytes(const DsgChirp* chirp, int32_t apertures, int32_t derivative) {
  if (!chirp_ok(chirp) || apertures <= 0) return 0;
  return interp_tables_bytes(make_consts(*chirp), apertures, derivative != 0);
}

int dsg_surfel_residual_tables(const DsgChirp* chirp, const float* residual, int32_t apertures,
                               int32_t derivative, float* tables, size_t tables_bytes, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0) return DSG_ERR_ARGUMENT;
  if (apertures == 0) return DSG_OK;
  if (!residual || !tables) return DSG_ERR_ARGUMENT;
  const Consts c = make_consts(*chirp);
  if (tables_bytes < interp_tables_bytes(c, apertures, derivative != 0)) return DSG_ERR_WORKSPACE;
  return interp_residual_tables(c, reinterpret_cast<const float2*>(residual), apertures, derivative != 0,
                                reinterpret_cast<float2*>(tables), (cudaStream_t)stream);
}

size_t dsg_surfel_tabled_workspace_bytes(int32_t apertures, int32_t candidates, int32_t values_per_surfel) {
  if (apertures <= 0 || candidates <= 0 || values_per_surfel <= 0) return 0;
  return interp_partial_bytes(apertures, candidates, values_per_surfel);
}

int dsg_surfel_correlate_tabled(const DsgChirp* chirp, const float* positions, int32_t apertures,
                                const float* centers, const float* normals, int32_t candidates,
                                const float* tables, const int32_t* active, int32_t period, float* corr,
                                float* norm, void* workspace, size_t workspace_bytes, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || candidates < 0 || (active && period < 1)) return DSG_ERR_ARGUMENT;
  if (candidates == 0) return DSG_OK;
  if (!centers || !normals || !corr || !norm) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (apertures == 0) {
    cudaMemsetAsync(corr, 0, (size_t)candidates * 2 * sizeof(float), st);
    cudaMemsetAsync(norm, 0, (size_t)candidates * sizeof(float), st);
    return launch_status();
  }
  if (!positions || !tables) return DSG_ERR_ARGUMENT;
  return interp_reduce_tabled(0, make_consts(*chirp), positions, apertures, centers, normals, nullptr, candidates,
                              reinterpret_cast<const float2*>(tables), workspace, workspace_bytes, corr, norm,
                              nullptr, nullptr, active, active ? period : 1, st);
}

int dsg_surfel_correlate_gradient_tabled(const DsgChirp* chirp, const float* positions, int32_t apertures,
                                         const float* centers, const float* normals, int32_t candidates,
                                         const float* tables, int32_t width, float* corr, float* norm,
                                         float* dcorr, float* dnorm, void* workspace, size_t workspace_bytes,
                                         void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || candidates < 0 || (width != 3 && width != 6)) return DSG_ERR_ARGUMENT;
  if (candidates == 0) return DSG_OK;
  if (!centers || !normals || !corr || !norm || !dcorr || !dnorm) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (apertures == 0) {
    cudaMemsetAsync(corr, 0, (size_t)candidates * 2 * sizeof(float), st);
    cudaMemsetAsync(norm, 0, (size_t)candidates * sizeof(float), st);
    cudaMemsetAsync(dcorr, 0, (size_t)candidates * width * 2 * sizeof(float), st);
    cudaMemsetAsync(dnorm, 0, (size_t)candidates * width * sizeof(float), st);
    return launch_status();
  }
  if (!positions || !tables) return DSG_ERR_ARGUMENT;
  return interp_reduce_tabled(width == 3 ? 1 : 2, make_consts(*chirp), positions, apertures, centers, normals,
                              nullptr, candidates, reinterpret_cast<const float2*>(tables), workspace,
                              workspace_bytes, corr, norm, dcorr, dnorm, nullptr, 1, st);
}

int dsg_surfel_correlate_orientations(const DsgChirp* chirp, const float* positions,
                                      int32_t apertures, const float* centers,
                                      const float* normals, int32_t candidates, const float* bank,
                                      int32_t bank_size, const float* residual,
                                      const float* range_table, const float* norm_table,
                                      int32_t oversample, float* out, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || candidates < 0 || bank_size < 0) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (candidates == 0) return DSG_OK;
  if (!centers || !normals || !out || (bank_size > 0 && !bank)) return DSG_ERR_ARGUMENT;
  if (apertures == 0) {
    cudaMemsetAsync(out, 0, (size_t)candidates * (bank_size + 1) * 3 * sizeof(float), st);
    return launch_status();
  }
  if (!positions) return DSG_ERR_ARGUMENT;
  const bool use_table = range_table != nullptr;
  if (use_table && (!norm_table || oversample < 1)) return DSG_ERR_ARGUMENT;
  if (!use_table && !residual) return DSG_ERR_ARGUMENT;
  OrientLaunch L{make_consts(*chirp), positions, apertures, centers, normals, candidates, bank,
                 bank_size, reinterpret_cast<const float2*>(residual),
                 reinterpret_cast<const float2*>(range_table), norm_table,
                 use_table ? oversample : 1, out, st};
  return dispatch_p(chirp->pad, L);
}

int dsg_surfel_orient_best(const DsgChirp* chirp, const float* positions, int32_t apertures,
                           const float* centers, const float* normals, const float* areas, int32_t candidates,
                           const float* bank, int32_t bank_size, const float* residual, const float* range_table,
                           const float* norm_table, int32_t oversample, const double* energy, int32_t real_mode,
                           int32_t* which, float* top, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures <= 0 || candidates < 0 || bank_size < 0) return DSG_ERR_ARGUMENT;
  if (candidates == 0) return DSG_OK;
  if (!positions || !centers || !normals || !areas || !energy || !which || !top || (bank_size > 0 && !bank))
    return DSG_ERR_ARGUMENT;
  const bool use_table = range_table != nullptr;
  if (use_table && (!norm_table || oversample < 1)) return DSG_ERR_ARGUMENT;
  if (!use_table && !residual) return DSG_ERR_ARGUMENT;
  OrientLaunch L{make_consts(*chirp), positions, apertures, centers, normals, candidates, bank,
                 bank_size, reinterpret_cast<const float2*>(residual),
                 reinterpret_cast<const float2*>(range_table), norm_table,
                 use_table ? oversample : 1, nullptr, (cudaStream_t)stream};
  L.best = OrientBest{areas, energy, real_mode != 0, which, top};
  return dispatch_p(chirp->pad, L);
}

int dsg_surfel_design(const DsgChirp* chirp, const float* positions, int32_t apertures,
                      const float* centers, const float* normals, const float* areas,
                      int32_t surfels, int32_t real, float* out, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || surfels < 0) return DSG_ERR_ARGUMENT;
  if (apertures == 0 || surfels == 0) return DSG_OK;
  if (!positions || !centers || !normals || !areas || !out) return DSG_ERR_ARGUMENT;
  if (apertures > 65535) return DSG_ERR_ARGUMENT;
  DesignLaunch L{make_consts(*chirp), positions, apertures, centers, normals, areas, surfels, real,
                 out, (cudaStream_t)stream};
  return dispatch_p(chirp->pad, L);
}

int dsg_surfel_jacobian(const DsgChirp* chirp, const float* positions, int32_t apertures,
                        const float* centers, const float* normals, int32_t surfels,
                        float* columns, float* derivatives, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || surfels < 0) return DSG_ERR_ARGUMENT;
  if (apertures == 0 || surfels == 0) return DSG_OK;
  if (!positions || !centers || !normals || !columns || !derivatives) return DSG_ERR_ARGUMENT;
  if (apertures > 65535) return DSG_ERR_ARGUMENT;
  JacobianLaunch L{make_consts(*chirp), positions, apertures, centers, normals, surfels,
                   reinterpret_cast<float2*>(columns), reinterpret_cast<float2*>(derivatives),
                   (cudaStream_t)stream};
  return dispatch_p(chirp->pad, L);
}

}  // extern "C"

// ------------------------------------------------------------------------------------
// VJP without a caller workspace, for callers that cannot allocate device memory: a host
// whose device memory is owned entirely by another allocator (a framework's caching pool
// that has reserved the GPU), or a latency-bound pipeline that must not call cudaMalloc
// because it synchronizes the whole device. The aperture-chunk partials live in one
// fixed array below, DSG_VJP_SCRATCH_MAX_BYTES long, which every GPU that loads this
// library holds until the process exits.
//
// In host code the array's name is only a stand-in for the symbol; its device address
// is looked up with cudaGetSymbolAddress, with that device current, on the first call
// made on that device (and again after the device's context changed, e.g. after a
// cudaDeviceReset). That first call may also load this module onto the device, so it
// should come before any stream capture on that device.
//
// Every call on a device shares the one array and leaves its partials there. Nothing in
// it needs to start at zero: the partial kernel writes every (surfel, chunk) slot that
// the chunk sum then reads. Calls whose kernels overlap on the GPU (different streams
// without ordering between them) race on the array and give wrong gradients.
// ------------------------------------------------------------------------------------
namespace {

static __device__ __align__(256) float g_vjp_scratch[DSG_VJP_SCRATCH_MAX_BYTES / sizeof(float)];

constexpr int kScratchDevices = 64;

// The scratch address is valid for one CUDA context: a cudaDeviceReset, or a caller that
// makes another (non-primary) context current, loads the module anew. Each device slot
// therefore remembers the unique id (cuCtxGetId) of the context it was looked up in, and
// a call from any other context looks the address up again.
struct ScratchSlot {
  unsigned long long context_id = 0;
  void* address = nullptr;
};
ScratchSlot g_vjp_scratch_slots[kScratchDevices];
std::mutex g_vjp_scratch_mutex;

using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrent g_ctx_get_current = nullptr;
CtxGetId g_ctx_get_id = nullptr;
std::once_flag g_ctx_entry_once;

void resolve_context_entry_points() {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess && fn != nullptr)
    g_ctx_get_current = reinterpret_cast<CtxGetCurrent>(fn);
  fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess && fn != nullptr)
    g_ctx_get_id = reinterpret_cast<CtxGetId>(fn);
  cudaGetLastError();
}

// Unique id of the calling thread's current context; 0 when none is current.
unsigned long long current_context_id() {
  std::call_once(g_ctx_entry_once, resolve_context_entry_points);
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  CUcontext context = nullptr;
  if (g_ctx_get_current(&context) != CUDA_SUCCESS || context == nullptr) return 0;
  unsigned long long id = 0;
  if (g_ctx_get_id(context, &id) != CUDA_SUCCESS) return 0;
  return id;
}

int vjp_scratch_address(void** out) {
  int device = -1;
  if (cudaGetDevice(&device) != cudaSuccess) return DSG_ERR_LAUNCH;
  if (device < 0 || device >= kScratchDevices) return DSG_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_vjp_scratch_mutex);
  ScratchSlot& slot = g_vjp_scratch_slots[device];
  const unsigned long long id = current_context_id();
  if (id != 0 && id == slot.context_id && slot.address != nullptr) {
    *out = slot.address;
    return DSG_OK;
  }
  void* address = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&address, g_vjp_scratch);  // makes the primary context current
  if (e != cudaSuccess || address == nullptr) {
    cudaGetLastError();
    return DSG_ERR_LAUNCH;
  }
  slot.context_id = current_context_id();  // 0 (look up again next time) if ids are unavailable
  slot.address = address;
  *out = address;
  return DSG_OK;
}

}  // namespace

unsigned long long dsg_current_context_id() { return current_context_id(); }

extern "C" int dsg_surfel_vjp_fixed_scratch(const DsgChirp* chirp, const float* positions,
                                            int32_t apertures, const float* centers,
                                            const float* normals, const float* weights,
                                            int32_t surfels, const float* upstream,
                                            float* grad_centers, float* grad_normals,
                                            float* grad_weights, void* stream) {
  if (!chirp_ok(chirp)) return DSG_ERR_UNSUPPORTED;
  if (apertures < 0 || surfels < 0) return DSG_ERR_ARGUMENT;
  if (surfels > 0 && (!weights || !grad_weights)) return DSG_ERR_ARGUMENT;
  // the exact form: its chunk partials are all the scratch it needs
  if (apertures > 0 && exact_workspace_bytes(apertures, surfels, 8) > DSG_VJP_SCRATCH_MAX_BYTES)
    return DSG_ERR_WORKSPACE;
  if (surfels == 0) return DSG_OK;
  void* scratch = nullptr;
  const int status = vjp_scratch_address(&scratch);
  if (status != DSG_OK) return status;
  return reduce_common(3, chirp, positions, apertures, centers, normals, weights, surfels,
                       upstream, grad_centers, grad_normals, grad_weights, nullptr, scratch,
                       DSG_VJP_SCRATCH_MAX_BYTES, stream, /*interp_allowed=*/false);
}
