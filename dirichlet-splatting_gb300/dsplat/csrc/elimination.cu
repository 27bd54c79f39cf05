// Backward elimination of the merged replacement on the device (reference:
// dsplat/replacement.py:104-140, backward_elimination). With W the regularized inverse of
// the pooled system and b = W q, removing unknown j raises the objective by
// |b_j|^2 / W_jj; each step removes the cheapest unknown that is still allowed and
// continues with W - w w^H / W_jj, w the current column j, kept as rank-one factors
// U[t] = w_t / sqrt(pivot_t) so a step costs O(n * step).
//
// One kernel per step on the caller's stream, in float64 (real or complex), after an
// initial pick of the first unknown:
//   step_kernel (n / 32 CTAs) the column w_i = W_ij - sum_t U[t][i] conj(U[t][j]) with the
//   sum split over 16 warps, then b, U[step] and the diagonal, and each CTA's masked argmin
//   of the next costs; the last CTA to finish (an atomic count, no waiting) reduces those,
//   computes the next pivot W_jj - sum_t |U[t][j]|^2 and writes the next pick.
// The argmin takes the first minimum and counts NaN as minimal, as torch.argmin. The
// arithmetic is that of the reference's loop; only the order of the float64 sums differs.
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
// Loads that bypass L1 (values written by another CTA of the same launch).
__device__ __forceinline__ double load_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ Cplx load_cg(const Cplx* p) { return Cplx{__ldcg(&p->x), __ldcg(&p->y)}; }

__device__ __forceinline__ double conj_of(double v) { return v; }
__device__ __forceinline__ Cplx conj_of(Cplx v) { return Cplx{v.x, -v.y}; }

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

struct Candidate {
  double cost;  // NaN allowed
  int index;    // 0x7fffffff: none
  int pad;
};

constexpr int kNone = 0x7fffffff;

// Whether (cost b, index ib) precedes (cost a, index ia) in torch.argmin order.
__device__ __forceinline__ bool precedes(double b, int ib, double a, int ia) {
  if (ib == kNone) return false;
  if (ia == kNone) return true;
  const bool nb = b != b, na = a != a;
  if (nb != na) return nb;
  if (nb) return ib < ia;
  return b < a || (b == a && ib < ia);
}

constexpr int kPickThreads = 1024;
constexpr int kRows = 32;  // rows per update CTA
constexpr int kSplit = 16;  // warps sharing one row's sums (over the factor's rows and the earlier steps)
// CTAs sharing one row block's factor-column sum (factor form): row block b sums over
// k >= max(j, 32 b), so the first blocks carry most of the triangle; splitting every
// block's k range into kParts shares bounds the longest CTA at a quarter of it.
constexpr int kParts = 4;

// b = W q, diag = real(W_ii), alive = 1, spent = 0.
template <typename T>
__global__ void init_kernel(const T* __restrict__ W, const T* __restrict__ q, int n, T* __restrict__ b,
                            double* __restrict__ diag, double* __restrict__ wdiag, uint8_t* __restrict__ alive,
                            Pick* __restrict__ pick, unsigned* __restrict__ counter) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;  // one row per warp
  if (i < n) {
    T acc = zero<T>();
    for (int k = lane; k < n; k += 32) acc = add(acc, mul(W[(size_t)i * n + k], q[k]));
    for (int o = 16; o > 0; o >>= 1) acc = add(acc, shfl_xor(acc, o));
    if (lane == 0) {
      b[i] = acc;
      diag[i] = wdiag[i] = real_part(W[(size_t)i * n + i]);
      alive[i] = 1;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    pick->spent = 0;
    *counter = 0;
  }
}

// Factor form, W = X^H X with X = L^-1 lower triangular (row-major): y = X q, one warp per
// row (this kernel), then b = X^H y and the diagonal sum_k |X_ki|^2 (factor_init_kernel).
template <typename T>
__global__ void factor_rows_kernel(const T* __restrict__ X, const T* __restrict__ q, int n, T* __restrict__ y) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= n) return;
  T acc = zero<T>();
  for (int k = lane; k <= i; k += 32) acc = add(acc, mul(X[(size_t)i * n + k], q[k]));
  for (int o = 16; o > 0; o >>= 1) acc = add(acc, shfl_xor(acc, o));
  if (lane == 0) y[i] = acc;
}

template <typename T>
__global__ void factor_init_kernel(const T* __restrict__ X, const T* __restrict__ y, int n, T* __restrict__ b,
                                   double* __restrict__ diag, double* __restrict__ wdiag,
                                   uint8_t* __restrict__ alive, Pick* __restrict__ pick,
                                   unsigned* __restrict__ counter) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    T acc = zero<T>();  // sum_k conj(X_ki) y_k = conj(sum_k X_ki conj(y_k))
    double d = 0.0;
    for (int k = i; k < n; ++k) {
      const T x = X[(size_t)k * n + i];
      acc = add(acc, mul_conj(x, y[k]));
      d += abs2(x);
    }
    b[i] = conj_of(acc);
    diag[i] = wdiag[i] = d;
    alive[i] = 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    pick->spent = 0;
    *counter = 0;
  }
}

template <typename T>
__global__ void __launch_bounds__(kPickThreads) pick_kernel(
    const T* __restrict__ W, int n, int step, const T* __restrict__ b, const double* __restrict__ diag,
    const uint8_t* __restrict__ alive, const uint8_t* __restrict__ limited, long long limit,
    const T* __restrict__ U, const double* __restrict__ wdiag, Pick* __restrict__ pick,
    int64_t* __restrict__ removed) {
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
    const double pivot = wdiag[j] - total;
    pick->index = j;
    pick->pivot = fmax(pivot, tiny);
    if (limited != nullptr && limited[j]) pick->spent += 1;
    removed[step] = j;
  }
}

// W is the inverse itself, or with FACTOR its lower-triangular factor X (W = X^H X): the
// column W_ij is then sum_k conj(X_ki) X_kj over k >= max(i, j), X's column j staged in
// shared memory.
template <typename T, bool FACTOR>
__global__ void __launch_bounds__(kRows * kSplit) step_kernel(
    const T* __restrict__ W, int n, int step, int count, const T* __restrict__ b_in, T* __restrict__ b_out,
    double* __restrict__ diag, const double* __restrict__ wdiag, uint8_t* __restrict__ alive,
    T* __restrict__ U, const uint8_t* __restrict__ limited, long long limit, const Pick* __restrict__ pick_in,
    Pick* __restrict__ pick_out, Candidate* __restrict__ partials, unsigned* __restrict__ counter,
    T* __restrict__ column_parts, unsigned* __restrict__ row_counter, int64_t* __restrict__ removed) {
  extern __shared__ uint8_t s_dyn[];
  __shared__ bool s_row_last;
  __shared__ T s_partw[FACTOR ? kSplit : 1][kRows];
  __shared__ T s_part[kSplit][kRows];
  __shared__ T s_uj[256];
  __shared__ double s_red[kRows * kSplit / 32];
  __shared__ Candidate s_best[kRows * kSplit / 32];
  __shared__ bool s_last;
  const double tiny = 2.2250738585072014e-308;  // smallest normal double (torch.finfo.tiny)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = (int)pick_in->index;
  const double pivot = pick_in->pivot;
  const long long spent = pick_in->spent;  // marked removals including j
  const bool spent_out = limited != nullptr && spent >= limit;
  const int i = blockIdx.x * kRows + lane;
  T accw = zero<T>();
  if (FACTOR) {
    // this CTA's share [kl, kh) of the row block's k range, X's column j staged for it
    T* s_xj = reinterpret_cast<T*>(s_dyn);
    const int parts = (int)gridDim.y;
    const int k0 = max(j, (int)blockIdx.x * kRows);
    const int share = (n - k0 + parts - 1) / parts;
    const int kl = min(n, k0 + (int)blockIdx.y * share), kh = min(n, kl + share);
    for (int k = kl + (int)threadIdx.x; k < kh; k += blockDim.x) s_xj[k - kl] = W[(size_t)k * n + j];
    __syncthreads();
    if (i < n)
      for (int k = kl + warp; k < kh; k += kSplit) accw = add(accw, mul_conj(W[(size_t)k * n + i], s_xj[k - kl]));
    s_partw[FACTOR ? warp : 0][lane] = accw;
    if (parts > 1) {
      // shares go to the row block's slots; the last CTA of the block adds them in share order
      __syncthreads();
      if (warp == 0) {
        T total = s_partw[0][lane];
        for (int w = 1; w < kSplit; ++w) total = add(total, s_partw[FACTOR ? w : 0][lane]);
        column_parts[((size_t)blockIdx.x * parts + blockIdx.y) * kRows + lane] = total;
        __threadfence();  // the share reaches L2 before the CTA is counted
      }
      __syncthreads();
      if (threadIdx.x == 0) s_row_last = atomicAdd(&row_counter[blockIdx.x], 1u) == (unsigned)parts - 1;
      __syncthreads();
      if (!s_row_last) return;
      __threadfence();
      if (threadIdx.x == 0) row_counter[blockIdx.x] = 0;
      if (warp == 0) {
        T total = zero<T>();
        for (int y = 0; y < parts; ++y) total = add(total, load_cg(&column_parts[((size_t)blockIdx.x * parts + y) * kRows + lane]));
        s_partw[0][lane] = total;
        for (int w = 1; w < kSplit; ++w) s_partw[FACTOR ? w : 0][lane] = zero<T>();
      }
    }
  }
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
  if (warp == 0) {
    double cost = INFINITY;
    int index = kNone;
    if (i < n) {
      T sum = s_part[0][lane];
      for (int w = 1; w < kSplit; ++w) sum = add(sum, s_part[w][lane]);
      T wij;
      if (FACTOR) {
        T total = s_partw[0][lane];
        for (int w = 1; w < kSplit; ++w) total = add(total, s_partw[FACTOR ? w : 0][lane]);
        wij = conj_of(total);
      } else {
        wij = W[(size_t)i * n + j];
      }
      const T column = step ? sub(wij, sum) : wij;
      const T bj = b_in[j];
      const T scaled = divide(column, sqrt(pivot));
      // b_i - w_i (b_j / pivot); the removed unknown keeps b = 0 and diag = 1 so that its
      // masked cost stays finite (as the reference's loop).
      T bi = sub(b_in[i], mul(column, divide(bj, pivot)));
      double di = diag[i] - abs2(scaled);
      bool live = alive[i] != 0;
      if (i == j) {
        alive[i] = 0;
        live = false;
        di = 1.0;
        bi = zero<T>();
      }
      U[(size_t)step * n + i] = scaled;
      b_out[i] = bi;
      diag[i] = di;
      const bool blocked = !live || (spent_out && limited[i]);
      cost = blocked ? INFINITY : abs2(bi) / fmax(di, tiny);
      index = i;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double oc = __shfl_xor_sync(0xffffffffu, cost, o);
      const int oi = __shfl_xor_sync(0xffffffffu, index, o);
      if (precedes(oc, oi, cost, index)) {
        cost = oc;
        index = oi;
      }
    }
    if (lane == 0) partials[blockIdx.x] = Candidate{cost, index, 0};
    __threadfence();  // this lane's writes reach L2 before the CTA is counted
  }
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  // The last CTA: every other CTA's writes are visible (they fenced before counting).
  __threadfence();
  if (threadIdx.x == 0) *counter = 0;
  if (step + 1 >= count) return;
  double cost = INFINITY;
  int index = kNone;
  for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x) {
    const double oc = __ldcg(&partials[c].cost);
    const int oi = __ldcg(&partials[c].index);
    if (precedes(oc, oi, cost, index)) {
      cost = oc;
      index = oi;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double oc = __shfl_xor_sync(0xffffffffu, cost, o);
    const int oi = __shfl_xor_sync(0xffffffffu, index, o);
    if (precedes(oc, oi, cost, index)) {
      cost = oc;
      index = oi;
    }
  }
  if (lane == 0) s_best[warp] = Candidate{cost, index, 0};
  __syncthreads();
  __shared__ int s_next;
  if (threadIdx.x == 0) {
    cost = INFINITY;
    index = kNone;
    for (int w = 0; w < kRows * kSplit / 32; ++w)
      if (precedes(s_best[w].cost, s_best[w].index, cost, index)) {
        cost = s_best[w].cost;
        index = s_best[w].index;
      }
    // Every cost infinite: torch.argmin of an all-inf vector returns 0.
    if (index == kNone || (cost == INFINITY)) index = 0;
    s_next = index;
  }
  __syncthreads();
  const int jn = s_next;
  double part = 0.0;
  for (int t = threadIdx.x; t <= step; t += blockDim.x) {
    const T u = t == step ? load_cg(&U[(size_t)t * n + jn]) : U[(size_t)t * n + jn];
    part += abs2(u);
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if (lane == 0) s_red[warp] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double total = 0.0;
    for (int w = 0; w < kRows * kSplit / 32; ++w) total += s_red[w];
    const double pv = wdiag[jn] - total;
    pick_out->index = jn;
    pick_out->pivot = fmax(pv, tiny);
    pick_out->spent = spent + (limited != nullptr && limited[jn] ? 1 : 0);
    removed[step + 1] = jn;
  }
}

template <typename T, bool FACTOR>
int run(const void* inverse, const void* rhs, int n, int count, const uint8_t* limited, long long limit,
        void* workspace, int64_t* removed, cudaStream_t st) {
  const int blocks = (n + kRows - 1) / kRows;
  uint8_t* w = reinterpret_cast<uint8_t*>(workspace);
  T* b0 = reinterpret_cast<T*>(w);
  T* b1 = b0 + n;
  double* diag = reinterpret_cast<double*>(b1 + n);
  double* wdiag = diag + n;
  T* U = reinterpret_cast<T*>(wdiag + n);
  Pick* picks = reinterpret_cast<Pick*>(U + (size_t)count * n);  // [2]
  Candidate* partials = reinterpret_cast<Candidate*>(picks + 2);
  unsigned* counter = reinterpret_cast<unsigned*>(partials + blocks);
  uint8_t* alive = reinterpret_cast<uint8_t*>(counter + 4);
  // after alive: the row blocks' counters and share slots (factor form), 16-byte aligned
  const size_t tail = (reinterpret_cast<uintptr_t>(alive + n) + 15) & ~(uintptr_t)15;
  unsigned* row_counter = reinterpret_cast<unsigned*>(tail);
  T* column_parts = reinterpret_cast<T*>(tail + (((size_t)blocks * sizeof(unsigned) + 15) & ~(size_t)15));
  const int parts = FACTOR ? kParts : 1;
  if (FACTOR && cudaMemsetAsync(row_counter, 0, (size_t)blocks * sizeof(unsigned), st) != cudaSuccess)
    return DSG_ERR_LAUNCH;
  const T* W = reinterpret_cast<const T*>(inverse);
  const T* q = reinterpret_cast<const T*>(rhs);
  size_t smem = 0;
  if (FACTOR) {
    smem = (size_t)n * sizeof(T);
    if (smem > 200 * 1024) return DSG_ERR_UNSUPPORTED;
    cudaFuncAttributes attributes;
    if (cudaFuncGetAttributes(&attributes, step_kernel<T, FACTOR>) != cudaSuccess) return DSG_ERR_LAUNCH;
    if (smem + attributes.sharedSizeBytes > 48 * 1024 &&  // dynamic plus static above the default
        cudaFuncSetAttribute(step_kernel<T, FACTOR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
      return DSG_ERR_LAUNCH;
    factor_rows_kernel<T><<<(n + 7) / 8, 256, 0, st>>>(W, q, n, b1);  // y = X q in b1
    factor_init_kernel<T><<<(n + 255) / 256, 256, 0, st>>>(W, b1, n, b0, diag, wdiag, alive, picks, counter);
  } else {
    init_kernel<T><<<(n + 7) / 8, 256, 0, st>>>(W, q, n, b0, diag, wdiag, alive, picks, counter);
  }
  pick_kernel<T><<<1, kPickThreads, 0, st>>>(W, n, 0, b0, diag, alive, limited, limit, U, wdiag, picks, removed);
  for (int step = 0; step < count; ++step) {
    const T* bi = (step & 1) ? b1 : b0;
    T* bo = (step & 1) ? b0 : b1;
    step_kernel<T, FACTOR><<<dim3(blocks, parts), kRows * kSplit, smem, st>>>(
        W, n, step, count, bi, bo, diag, wdiag, alive, U, limited, limit, picks + (step & 1),
        picks + ((step + 1) & 1), partials, counter, column_parts, row_counter, removed);
  }
  dsg_count_launches((FACTOR ? 3 : 2) + count);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // namespace

extern "C" {

size_t dsg_elimination_workspace_bytes(int32_t n, int32_t count, int32_t is_complex) {
  if (n <= 0 || count < 0) return 0;
  const size_t elem = is_complex ? 16 : 8;
  const size_t blocks = ((size_t)n + kRows - 1) / kRows;
  return elem * 2 * (size_t)n + 16 * (size_t)n + elem * (size_t)count * n + 2 * sizeof(Pick) +
         blocks * sizeof(Candidate) + 16 + (size_t)n + 64 + 16 + blocks * sizeof(unsigned) + 16 +
         blocks * kParts * kRows * elem;
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
  return is_complex ? run<Cplx, false>(inverse, rhs, n, count, limited, limit, workspace, removed, st)
                    : run<double, false>(inverse, rhs, n, count, limited, limit, workspace, removed, st);
}

int dsg_backward_elimination_factor(const void* factor_inverse, const void* rhs, int32_t n, int32_t count,
                                    const uint8_t* limited, int64_t limit, int32_t is_complex, void* workspace,
                                    size_t workspace_bytes, int64_t* removed, void* stream) {
  if (n < 0 || count < 0 || count > n) return DSG_ERR_ARGUMENT;
  if (count == 0 || n == 0) return DSG_OK;
  if (!factor_inverse || !rhs || !removed) return DSG_ERR_ARGUMENT;
  if (!workspace || workspace_bytes < dsg_elimination_workspace_bytes(n, count, is_complex))
    return DSG_ERR_WORKSPACE;
  if (reinterpret_cast<uintptr_t>(workspace) & 15u) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  return is_complex ? run<Cplx, true>(factor_inverse, rhs, n, count, limited, limit, workspace, removed, st)
                    : run<double, true>(factor_inverse, rhs, n, count, limited, limit, workspace, removed, st);
}

}  // extern "C"
