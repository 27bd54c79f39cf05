// Backward elimination of the merged replacement on the device (reference:
// dsplat/replacement.py:104-140, backward_elimination). With W the regularized inverse of
// the pooled system and b = W q, removing unknown j raises the objective by
// |b_j|^2 / W_jj; each step removes the cheapest unknown that is still allowed and
// continues with W - w w^H / W_jj, w the current column j, kept as rank-one factors
// U[t] = w_t / sqrt(pivot_t) so a step costs O(n * step).
//
// Two kernels per step on the caller's stream, in float64 (real or complex):
//   pick_kernel   (one CTA) cost, masked argmin (first minimum; NaN counts as minimal, as
//                 torch.argmin), the pivot W_jj - sum_t |U[t][j]|^2 and the bookkeeping;
//   update_kernel (n / 32 CTAs) the column w_i = W_ij - sum_t U[t][i] conj(U[t][j]) with
//                 the sum split over 8 warps, then b, U[step] and the diagonal.
// The arithmetic is that of the reference's loop; only the order of the float64 sums in
// the column differs.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

struct Cplx {
  double x, y;
};

__device__ __forceinline__ double abs2(double v) { return v * v; }
__device__ __forceinline__ double abs2(Cplx v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ double real_part(double v) { return v; }
__device__ __forceinline__ double real_part(Cplx v) { return v.x; }
__device__ __forceinline__ double mul_conj(double a, double b) { return a * b; }
__device__ __forceinline__ Cplx mul_conj(Cplx a, Cplx b) {  // a * conj(b)
  return Cplx{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
__device__ __forceinline__ double add(double a, double b) { return a + b; }
__device__ __forceinline__ Cplx add(Cplx a, Cplx b) { return Cplx{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ double sub(double a, double b) { return a - b; }
__device__ __forceinline__ Cplx sub(Cplx a, Cplx b) { return Cplx{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ double divide(double a, double d) { return a / d; }
__device__ __forceinline__ Cplx divide(Cplx a, double d) { return Cplx{a.x / d, a.y / d}; }
__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ Cplx shfl_xor(Cplx v, int o) {
  return Cplx{__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)};
}
__device__ __forceinline__ double mul(double a, double b) { return a * b; }
__device__ __forceinline__ Cplx mul(Cplx a, Cplx b) {
  return Cplx{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__device__ __forceinline__ T zero();
template <>
__device__ __forceinline__ double zero<double>() { return 0.0; }
template <>
__device__ __forceinline__ Cplx zero<Cplx>() { return Cplx{0.0, 0.0}; }

// Shared state between the two kernels of a step.
struct Pick {
  long long index;  // the unknown removed this step
  double pivot;     // clamp(real(w_j), tiny)
  long long spent;  // removed unknowns marked in `limited`
  double pad;
};

constexpr int kPickThreads = 1024;
constexpr int kRows = 32;  // rows per update CTA
constexpr int kSplit = 8;  // warps sharing one row's sum over the earlier steps

// b = W q, diag = real(W_ii), alive = 1, spent = 0.
template <typename T>
__global__ void init_kernel(const T* __restrict__ W, const T* __restrict__ q, int n, T* __restrict__ b,
                            double* __restrict__ diag, uint8_t* __restrict__ alive,
                            Pick* __restrict__ pick) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;  // one row per warp
  if (i < n) {
    T acc = zero<T>();
    for (int k = lane; k < n; k += 32) acc = add(acc, mul(W[(size_t)i * n + k], q[k]));
    for (int o = 16; o > 0; o >>= 1) acc = add(acc, shfl_xor(acc, o));
    if (lane == 0) {
      b[i] = acc;
      diag[i] = real_part(W[(size_t)i * n + i]);
      alive[i] = 1;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) pick->spent = 0;
}

template <typename T>
__global__ void __launch_bounds__(kPickThreads) pick_kernel(
    const T* __restrict__ W, int n, int step, const T* __restrict__ b, const double* __restrict__ diag,
    const uint8_t* __restrict__ alive, const uint8_t* __restrict__ limited, long long limit,
    const T* __restrict__ U, Pick* __restrict__ pick, int64_t* __restrict__ removed) {
  __shared__ double s_cost[kPickThreads / 32];
  __shared__ int s_index[kPickThreads / 32];
  __shared__ double s_sum[kPickThreads / 32];
  __shared__ int s_choice;
  const double tiny = 2.2250738585072014e-308;  // smallest normal double (torch.finfo.tiny)
  const bool spent_out = limited != nullptr && pick->spent >= limit;
  // cost and the first minimal index (NaN first, then the smallest cost, then the lowest index)
  double best = INFINITY;
  int best_i = 0x7fffffff;
  bool best_nan = false;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const bool blocked = !alive[i] || (spent_out && limited[i]);
    double cost = blocked ? INFINITY : abs2(b[i]) / fmax(diag[i], tiny);
    const bool nan = cost != cost;
    if (best_i == 0x7fffffff || (nan && !best_nan) || (nan == best_nan && !nan && cost < best)) {
      best = cost;
      best_i = i;
      best_nan = nan;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const double oc = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, best_i, o);
    const bool on = __shfl_xor_sync(0xffffffffu, (int)best_nan, o) != 0;
    const bool take = oi != 0x7fffffff &&
                      (best_i == 0x7fffffff || (on && !best_nan) ||
                       (on == best_nan && (on ? oi < best_i : (oc < best || (oc == best && oi < best_i)))));
    if (take) {
      best = oc;
      best_i = oi;
      best_nan = on;
    }
  }
  if (lane == 0) {
    s_cost[warp] = best_nan ? NAN : best;
    s_index[warp] = best_i;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double c = INFINITY;
    int idx = 0x7fffffff;
    bool cn = false;
    for (int w = 0; w < kPickThreads / 32; ++w) {
      const int oi = s_index[w];
      if (oi == 0x7fffffff) continue;
      const double oc = s_cost[w];
      const bool on = oc != oc;
      if (idx == 0x7fffffff || (on && !cn) || (on == cn && (on ? oi < idx : (oc < c || (oc == c && oi < idx))))) {
        c = oc;
        idx = oi;
        cn = on;
      }
    }
    // Every cost infinite: torch.argmin of an all-inf vector returns 0.
    if (idx == 0x7fffffff || (!cn && c == INFINITY)) idx = 0;
    s_choice = idx;
  }
  __syncthreads();
  const int j = s_choice;
  // pivot = real(W_jj - sum_t U[t][j] conj(U[t][j]))
  double part = 0.0;
  for (int t = threadIdx.x; t < step; t += blockDim.x) part += abs2(U[(size_t)t * n + j]);
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if (lane == 0) s_sum[warp] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double total = 0.0;
    for (int w = 0; w < kPickThreads / 32; ++w) total += s_sum[w];
    const double pivot = real_part(W[(size_t)j * n + j]) - total;
    pick->index = j;
    pick->pivot = fmax(pivot, tiny);
    if (limited != nullptr && limited[j]) pick->spent += 1;
    removed[step] = j;
  }
}

template <typename T>
__global__ void __launch_bounds__(kRows * kSplit) update_kernel(
    const T* __restrict__ W, int n, int step, T* __restrict__ b_in, T* __restrict__ b_out,
    double* __restrict__ diag, uint8_t* __restrict__ alive, T* __restrict__ U,
    const Pick* __restrict__ pick) {
  __shared__ T s_part[kSplit][kRows];
  __shared__ T s_uj[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = (int)pick->index;
  const double pivot = pick->pivot;
  const int i = blockIdx.x * kRows + lane;
  T acc = zero<T>();
  for (int t0 = 0; t0 < step; t0 += 256) {
    const int len = min(256, step - t0);
    __syncthreads();
    for (int t = threadIdx.x; t < len; t += blockDim.x) s_uj[t] = U[(size_t)(t0 + t) * n + j];
    __syncthreads();
    if (i < n)
      for (int t = warp; t < len; t += kSplit) acc = add(acc, mul_conj(U[(size_t)(t0 + t) * n + i], s_uj[t]));
  }
  s_part[warp][lane] = acc;
  __syncthreads();
  if (warp == 0 && i < n) {
    T sum = s_part[0][lane];
    for (int w = 1; w < kSplit; ++w) sum = add(sum, s_part[w][lane]);
    const T column = step ? sub(W[(size_t)i * n + j], sum) : W[(size_t)i * n + j];
    const T bj = b_in[j];
    const T scaled = divide(column, sqrt(pivot));
    // b_i - w_i (b_j / pivot); the removed unknown keeps b = 0 and diag = 1 so that its
    // masked cost stays finite (as the reference's loop).
    T bi = sub(b_in[i], mul(column, divide(bj, pivot)));
    double di = diag[i] - abs2(scaled);
    if (i == j) {
      alive[i] = 0;
      di = 1.0;
      bi = zero<T>();
    }
    U[(size_t)step * n + i] = scaled;
    b_out[i] = bi;
    diag[i] = di;
  }
}

template <typename T>
int run(const void* inverse, const void* rhs, int n, int count, const uint8_t* limited, long long limit,
        void* workspace, int64_t* removed, cudaStream_t st) {
  uint8_t* w = reinterpret_cast<uint8_t*>(workspace);
  T* b0 = reinterpret_cast<T*>(w);
  T* b1 = b0 + n;
  double* diag = reinterpret_cast<double*>(b1 + n);
  T* U = reinterpret_cast<T*>(diag + n);
  Pick* pick = reinterpret_cast<Pick*>(U + (size_t)count * n);
  uint8_t* alive = reinterpret_cast<uint8_t*>(pick + 1);
  const T* W = reinterpret_cast<const T*>(inverse);
  init_kernel<T><<<(n + 7) / 8, 256, 0, st>>>(W, reinterpret_cast<const T*>(rhs), n, b0, diag, alive, pick);
  const int blocks = (n + kRows - 1) / kRows;
  for (int step = 0; step < count; ++step) {
    T* bi = (step & 1) ? b1 : b0;
    T* bo = (step & 1) ? b0 : b1;
    pick_kernel<T><<<1, kPickThreads, 0, st>>>(W, n, step, bi, diag, alive, limited, limit, U, pick, removed);
    update_kernel<T><<<blocks, kRows * kSplit, 0, st>>>(W, n, step, bi, bo, diag, alive, U, pick);
  }
  dsg_count_launches(1 + 2 * count);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // namespace

extern "C" {

size_t dsg_elimination_workspace_bytes(int32_t n, int32_t count, int32_t is_complex) {
  if (n <= 0 || count < 0) return 0;
  const size_t elem = is_complex ? 16 : 8;
  return elem * 2 * (size_t)n + 8 * (size_t)n + elem * (size_t)count * n + sizeof(Pick) + (size_t)n + 64;
}

int dsg_backward_elimination(const void* inverse, const void* rhs, int32_t n, int32_t count,
                             const uint8_t* limited, int64_t limit, int32_t is_complex, void* workspace,
                             size_t workspace_bytes, int64_t* removed, void* stream) {
  if (n < 0 || count < 0 || count > n) return DSG_ERR_ARGUMENT;
  if (count == 0 || n == 0) return DSG_OK;
  if (!inverse || !rhs || !removed) return DSG_ERR_ARGUMENT;
  if (!workspace || workspace_bytes < dsg_elimination_workspace_bytes(n, count, is_complex))
    return DSG_ERR_WORKSPACE;
  if (reinterpret_cast<uintptr_t>(workspace) & 15u) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  return is_complex ? run<Cplx>(inverse, rhs, n, count, limited, limit, workspace, removed, st)
                    : run<double>(inverse, rhs, n, count, limited, limit, workspace, removed, st);
}

}  // extern "C"
