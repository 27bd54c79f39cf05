// Backward elimination of the merged replacement on the device (reference:
// dsplat/replacement.py:104-140, backward_elimination). With W the regularized inverse of
// the pooled system and b = W q, removing unknown j raises the objective by
// |b_j|^2 / W_jj; each step removes the cheapest unknown that is still allowed and
// continues with W - w w^H / W_jj, w the current column j, kept as rank-one factors
// U[t] = w_t / sqrt(pivot_t) so a step costs O(n * step).
//
// One kernel per removal on the caller's stream, in float64 (real or complex), after the
// initial pass and pick. Per row block of 32 unknowns the column
// w_i = W_ij - sum_t U[t][i] conj(U[t][j]) (in the factor form W_ij itself is a sum over X's
// rows k >= max(i, j)), then b, U[step], the diagonal and the block's masked argmin; the last
// CTA to finish (an atomic count, no waiting) reduces the blocks' candidates and writes the
// next pivot W_jj - sum_t |U[t][j]|^2. FP64 issues at a few lanes per clock on this part and
// a removal is set by its busiest SM, so the work is spread evenly: row blocks are paired (a
// long k range with a short one), each pair's sums are split over 8 CTAs, and the argmin
// compares integer keys instead of doubles. The argmin takes the first minimum and counts
// NaN as minimal, as torch.argmin. The arithmetic is that of the reference's loop; only the
// order of the float64 sums differs.
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

// State between two launches: the removal being applied.
struct Pick {
  long long index;  // the unknown removed this step
  double pivot;     // clamp(real(w_j), tiny)
  long long spent;  // removed unknowns marked in `limited`
  double pad;
};

// A row block's argmin candidate. key orders the costs as torch.argmin does (NaN first,
// then by value) with integer compares: the costs are never negative, so their bit
// patterns order as their values. index is the row, kNone for none.
struct Candidate {
  unsigned long long key;
  int index;
  int pad;
};

constexpr int kNone = 0x7fffffff;
constexpr unsigned long long kInfKey = 0x7ff0000000000001ull;  // cost_key(+inf)
constexpr double kTiny = 2.2250738585072014e-308;              // smallest normal double (torch.finfo.tiny)

__device__ __forceinline__ unsigned long long cost_key(double c) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(c);
  return (bits & 0x7fffffffffffffffull) > 0x7ff0000000000000ull ? 0ull : bits + 1ull;
}

// Whether (key kb, index ib) precedes (key ka, index ia): the first minimum wins.
__device__ __forceinline__ bool precedes(unsigned long long kb, int ib, unsigned long long ka, int ia) {
  if (ib == kNone) return false;
  if (ia == kNone) return true;
  return kb < ka || (kb == ka && ib < ia);
}

__device__ __forceinline__ void warp_argmin(unsigned long long& key, int& index) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
    const int oi = __shfl_xor_sync(0xffffffffu, index, o);
    if (precedes(ok, oi, key, index)) {
      key = ok;
      index = oi;
    }
  }
}

constexpr int kRows = 32;                 // rows per row block (one per lane)
constexpr int kSplit = 16;                // warps per CTA, sharing each row's sums
constexpr int kThreads = kRows * kSplit;  // 512
constexpr int kPickThreads = 512;
// FP64 issues at a few lanes per clock on this part, so a removal is set by the FP64 work of
// its busiest SM. The factor form's column sum for a row in block r runs over
// k >= max(j, 32 r): early blocks carry most of the triangle. Blocks are paired, r with its
// mirror B - 1 - r, whose k ranges together are about n long, and each pair is split into
// kPairParts CTAs of equal k work; the sum over the earlier removals is split the same way.
constexpr int kPairParts = 8;

// Share y of `parts` of the row-block pair p: blocks a = p and b = blocks - 1 - p (b < 0 when
// they coincide), whose k ranges [ka0, n) and [kb0, n) (k0 = max(first_k, 32 block)) are laid
// end to end and cut into equal shares; this share is k = ka0 + [sa0, sa1) of block a and
// k = kb0 + [sb0, sb1) of block b.
struct PairShare {
  int a, b, ka0, kb0, sa0, sa1, sb0, sb1;
};

__device__ __forceinline__ PairShare pair_share(int n, int blocks, int p, int y, int parts, int first_k) {
  PairShare s;
  s.a = p;
  s.b = blocks - 1 - p;
  if (s.b == s.a) s.b = -1;
  s.ka0 = max(first_k, s.a * kRows);
  s.kb0 = s.b >= 0 ? max(first_k, s.b * kRows) : n;
  const int la = n - s.ka0, total = la + (n - s.kb0);
  const int share = (total + parts - 1) / parts;
  const int s0 = min(total, y * share), s1 = min(total, s0 + share);
  s.sa0 = min(s0, la);
  s.sa1 = min(s1, la);
  s.sb0 = max(s0, la) - la;
  s.sb1 = max(s1, la) - la;
  return s;
}

__device__ __forceinline__ double to_real(double v) { return v; }
__device__ __forceinline__ double to_real(Cplx v) { return v.x; }
template <typename T>
__device__ __forceinline__ T from_real(double v);
template <>
__device__ __forceinline__ double from_real<double>(double v) { return v; }
template <>
__device__ __forceinline__ Cplx from_real<Cplx>(double v) { return Cplx{v, 0.0}; }

// Adds the 4 per-warp quantities in s_sum over the warps (warps 0-3, one quantity each, on
// separate SM sub-partitions); with parts > 1 the shares go to the pair's slots and the CTA
// that completes the pair adds them in share order. Returns whether this CTA holds the totals
// in s_tot.
template <typename T>
__device__ __forceinline__ bool combine_pair(T (*s_sum)[kSplit][kRows], T (*s_tot)[kRows], int p, int y, int parts,
                                             T* pair_parts, unsigned* pair_counter) {
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (warp < 4) {
    T total = s_sum[warp][0][lane];
    for (int w = 1; w < kSplit; ++w) total = add(total, s_sum[warp][w][lane]);
    if (parts > 1) {
      pair_parts[(((size_t)p * parts + y) * 4 + warp) * kRows + lane] = total;
      __threadfence();  // the share reaches L2 before the CTA is counted
    } else {
      s_tot[warp][lane] = total;
    }
  }
  if (parts > 1) {
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&pair_counter[p], 1u) == (unsigned)parts - 1;
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    if (threadIdx.x == 0) atomicExch(&pair_counter[p], 0u);
    if (warp < 4) {
      T total = zero<T>();
      for (int z = 0; z < parts; ++z) total = add(total, load_cg(&pair_parts[(((size_t)p * parts + z) * 4 + warp) * kRows + lane]));
      s_tot[warp][lane] = total;
    }
  }
  __syncthreads();
  return true;
}

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

// b_i = sum_{k >= i} conj(X_ki) y_k and diag_i = sum_{k >= i} |X_ki|^2 over the pair partition
// (one CTA per pair share; the pair's last CTA writes b, diag, wdiag and alive).
template <typename T>
__global__ void __launch_bounds__(kThreads) factor_init_kernel(const T* __restrict__ X, const T* __restrict__ y, int n,
                                                               int blocks, int parts, T* b, double* diag, double* wdiag,
                                                               uint8_t* alive, T* pair_parts, unsigned* pair_counter,
                                                               Pick* pick, unsigned* counter) {
  extern __shared__ __align__(16) uint8_t s_dyn[];
  __shared__ T s_sum[4][kSplit][kRows];  // per warp: X^H y and |X|^2 of block a, then of block b
  __shared__ T s_tot[4][kRows];
  T* s_y = reinterpret_cast<T*>(s_dyn);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p = blockIdx.x / parts, yy = blockIdx.x % parts;
  const PairShare s = pair_share(n, blocks, p, yy, parts, 0);
  const int na = s.sa1 - s.sa0, nb = s.sb1 - s.sb0;
  for (int m = threadIdx.x; m < na + nb; m += blockDim.x)
    s_y[m] = y[m < na ? s.ka0 + s.sa0 + m : s.kb0 + s.sb0 + (m - na)];
  __syncthreads();
  const int ia = s.a * kRows + lane, ib = s.b >= 0 ? s.b * kRows + lane : n;
  T sa = zero<T>(), sb = zero<T>();
  double da = 0.0, db = 0.0;
  if (ia < n)
    for (int m = warp; m < na; m += kSplit) {
      const T x = X[(size_t)(s.ka0 + s.sa0 + m) * n + ia];
      sa = add(sa, mul_conj(x, s_y[m]));
      da += abs2(x);
    }
  if (ib < n)
    for (int m = warp; m < nb; m += kSplit) {
      const T x = X[(size_t)(s.kb0 + s.sb0 + m) * n + ib];
      sb = add(sb, mul_conj(x, s_y[na + m]));
      db += abs2(x);
    }
  s_sum[0][warp][lane] = sa;
  s_sum[1][warp][lane] = from_real<T>(da);
  s_sum[2][warp][lane] = sb;
  s_sum[3][warp][lane] = from_real<T>(db);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    pick->spent = 0;
    *counter = 0;
  }
  if (!combine_pair<T>(s_sum, s_tot, p, yy, parts, pair_parts, pair_counter)) return;
  if (warp < 2) {
    const int blk = warp == 0 ? s.a : s.b;
    const int i = blk * kRows + lane;
    if (blk >= 0 && i < n) {
      b[i] = conj_of(s_tot[2 * warp][lane]);  // sum conj(X_ki) y_k = conj(sum X_ki conj(y_k))
      diag[i] = wdiag[i] = to_real(s_tot[2 * warp + 1][lane]);
      alive[i] = 1;
    }
  }
}

// The first removal: argmin of |b_i|^2 / W_ii over all unknowns (none removed or marked
// yet), its pivot W_jj and marked count (one CTA).
template <typename T>
__global__ void __launch_bounds__(kPickThreads) pick_kernel(int n, const T* __restrict__ b,
                                                            const double* __restrict__ diag,
                                                            const uint8_t* __restrict__ alive,
                                                            const uint8_t* __restrict__ limited, long long limit,
                                                            const double* __restrict__ wdiag, Pick* __restrict__ pick,
                                                            int64_t* __restrict__ removed) {
  __shared__ Candidate s_best[kPickThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool spent_out = limited != nullptr && pick->spent >= limit;
  unsigned long long key = ~0ull;
  int index = kNone;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const bool blocked = !alive[i] || (spent_out && limited[i]);
    const unsigned long long k = blocked ? kInfKey : cost_key(abs2(b[i]) / fmax(diag[i], kTiny));
    if (precedes(k, i, key, index)) {
      key = k;
      index = i;
    }
  }
  warp_argmin(key, index);
  if (lane == 0) s_best[warp] = Candidate{key, index, 0};
  __syncthreads();
  if (warp == 0) {
    key = lane < kPickThreads / 32 ? s_best[lane].key : ~0ull;
    index = lane < kPickThreads / 32 ? s_best[lane].index : kNone;
    warp_argmin(key, index);
    if (index == kNone || key == kInfKey) index = 0;  // every cost infinite: torch.argmin gives 0
    if (lane == 0) {
      pick->index = index;
      pick->pivot = fmax(wdiag[index], kTiny);
      if (limited != nullptr && limited[index]) pick->spent += 1;
      removed[0] = index;
    }
  }
}

// One removal per launch, one CTA per pair share. W is the inverse itself, or with FACTOR its
// lower-triangular factor X (W = X^H X): the column W_ij is then sum_k conj(X_ki) X_kj over
// k >= max(i, j), split over the pair partition with X's column j staged in shared memory.
// The sum over the earlier removals sum_t U[t][i] conj(U[t][j]) is split over the pair's CTAs
// by t. The CTA that completes the pair (the last of its parts) adds the shares in share
// order and applies the rank-one update to both blocks' rows (b_out, diag, alive, U[step];
// warp 0 block a, warp 1 block b) and their argmin candidates; the last such CTA of the grid
// (an atomic count, no waiting) reduces the candidates and writes the next pick. Everything
// another CTA of the same launch wrote is read from L2 (load_cg).
template <typename T, bool FACTOR>
__global__ void __launch_bounds__(kThreads) step_kernel(
    const T* __restrict__ W, int n, int blocks, int parts, int step, int count, const T* __restrict__ b_in,
    T* __restrict__ b_out, double* __restrict__ diag, const double* __restrict__ wdiag, uint8_t* __restrict__ alive,
    T* __restrict__ U, const uint8_t* __restrict__ limited, long long limit, const Pick* __restrict__ pick_in,
    Pick* __restrict__ pick_out, Candidate* __restrict__ block_best, unsigned* __restrict__ counter,
    T* __restrict__ pair_parts, unsigned* __restrict__ pair_counter, int64_t* __restrict__ removed) {
  extern __shared__ __align__(16) uint8_t s_dyn[];
  __shared__ T s_sum[4][kSplit][kRows];  // per warp: the k sum and the t sum of block a, then of block b
  __shared__ T s_tot[4][kRows];
  __shared__ T s_uj[256];
  __shared__ bool s_last;
  __shared__ Candidate s_best[kSplit];
  T* s_xj = reinterpret_cast<T*>(s_dyn);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = (int)pick_in->index;
  const double pivot = pick_in->pivot;
  const long long spent = pick_in->spent;  // marked removals including j
  const int p = blockIdx.x / parts, y = blockIdx.x % parts;
  const PairShare s = pair_share(n, blocks, p, y, parts, j);
  const int na = FACTOR ? s.sa1 - s.sa0 : 0, nb = FACTOR ? s.sb1 - s.sb0 : 0;
  const int ia = s.a * kRows + lane, ib = s.b >= 0 ? s.b * kRows + lane : n;
  const int tshare = (step + parts - 1) / parts;
  const int tl = min(step, y * tshare), th = min(step, tl + tshare);
  for (int m = threadIdx.x; m < na + nb; m += blockDim.x)
    s_xj[m] = W[(size_t)(m < na ? s.ka0 + s.sa0 + m : s.kb0 + s.sb0 + (m - na)) * n + j];
  T ka = zero<T>(), kb = zero<T>(), ta = zero<T>(), tb = zero<T>();
  for (int t0 = tl; t0 < th; t0 += 256) {
    const int len = min(256, th - t0);
    __syncthreads();
    for (int t = threadIdx.x; t < len; t += blockDim.x) s_uj[t] = U[(size_t)(t0 + t) * n + j];
    __syncthreads();
    for (int t = warp; t < len; t += kSplit) {
      const T uj = s_uj[t];
      if (ia < n) ta = add(ta, mul_conj(U[(size_t)(t0 + t) * n + ia], uj));
      if (ib < n) tb = add(tb, mul_conj(U[(size_t)(t0 + t) * n + ib], uj));
    }
  }
  __syncthreads();  // s_xj staged
  if (FACTOR) {
    if (ia < n)
      for (int m = warp; m < na; m += kSplit) ka = add(ka, mul_conj(W[(size_t)(s.ka0 + s.sa0 + m) * n + ia], s_xj[m]));
    if (ib < n)
      for (int m = warp; m < nb; m += kSplit)
        kb = add(kb, mul_conj(W[(size_t)(s.kb0 + s.sb0 + m) * n + ib], s_xj[na + m]));
  }
  s_sum[0][warp][lane] = ka;
  s_sum[1][warp][lane] = ta;
  s_sum[2][warp][lane] = kb;
  s_sum[3][warp][lane] = tb;
  if (!combine_pair<T>(s_sum, s_tot, p, y, parts, pair_parts, pair_counter)) return;
  if (warp < 2) {
    const int blk = warp == 0 ? s.a : s.b;
    if (blk >= 0) {  // warp-uniform
      const int i = blk * kRows + lane;
      const bool spent_out = limited != nullptr && spent >= limit;
      unsigned long long key = ~0ull;
      int index = kNone;
      if (i < n) {
        const T wij = FACTOR ? conj_of(s_tot[2 * warp][lane]) : W[(size_t)i * n + j];
        const T column = step ? sub(wij, s_tot[2 * warp + 1][lane]) : wij;
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
        key = blocked ? kInfKey : cost_key(abs2(bi) / fmax(di, kTiny));
        index = i;
      }
      warp_argmin(key, index);
      if (lane == 0) block_best[blk] = Candidate{key, index, 0};
      __threadfence();  // this lane's writes reach L2 before the CTA is counted
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == (unsigned)(gridDim.x / parts) - 1;
  __syncthreads();
  if (!s_last) return;
  // The last pair: every other CTA's writes are visible (they fenced before counting).
  __threadfence();
  if (threadIdx.x == 0) *counter = 0;
  if (step + 1 >= count) return;
  unsigned long long key = ~0ull;
  int index = kNone;
  for (int c = threadIdx.x; c < blocks; c += blockDim.x) {
    const unsigned long long ok = __ldcg(&block_best[c].key);
    const int oi = __ldcg(&block_best[c].index);
    if (precedes(ok, oi, key, index)) {
      key = ok;
      index = oi;
    }
  }
  warp_argmin(key, index);
  if (lane == 0) s_best[warp] = Candidate{key, index, 0};
  __syncthreads();
  if (warp == 0) {
    key = lane < kSplit ? s_best[lane].key : ~0ull;
    index = lane < kSplit ? s_best[lane].index : kNone;
    warp_argmin(key, index);
    if (index == kNone || key == kInfKey) index = 0;  // every cost infinite: torch.argmin gives 0
    double part = 0.0;  // sum_{t <= step} |U[t][jn]|^2
    for (int t = lane; t <= step; t += 32) part += abs2(load_cg(&U[(size_t)t * n + index]));
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) {
      pick_out->index = index;
      pick_out->pivot = fmax(wdiag[index] - part, kTiny);
      pick_out->spent = spent + (limited != nullptr && limited[index] ? 1 : 0);
      removed[step + 1] = index;
    }
  }
}

inline size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }
inline int blocks_of(int n) { return (n + kRows - 1) / kRows; }
inline int pairs_of(int n) { return (blocks_of(n) + 1) / 2; }

template <typename K>
int allow_smem(K kernel, size_t smem) {
  cudaFuncAttributes attributes;
  if (cudaFuncGetAttributes(&attributes, kernel) != cudaSuccess) return DSG_ERR_LAUNCH;
  if (smem + attributes.sharedSizeBytes > 48 * 1024 &&  // dynamic plus static above the default
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DSG_ERR_LAUNCH;
  return DSG_OK;
}

// The workspace, in order: b0, b1 [n] T; diag, wdiag [n] double; U [count][n] T; the two
// picks; the row blocks' candidates; the grid counter; alive [n]; then (16-byte aligned) the
// pairs' counters and their share slots (4 sums of 32 rows per share).
size_t elimination_bytes(int n, int count, bool is_complex) {
  const size_t elem = is_complex ? 16 : 8;
  const size_t blocks = blocks_of(n), pairs = pairs_of(n);
  return elem * 2 * (size_t)n + 16 * (size_t)n + elem * (size_t)count * n + 2 * sizeof(Pick) +
         blocks * sizeof(Candidate) + 16 + (size_t)n + 15 + align16(pairs * sizeof(unsigned)) +
         pairs * kPairParts * 4 * kRows * elem;
}

template <typename T, bool FACTOR>
int run(const void* inverse, const void* rhs, int n, int count, const uint8_t* limited, long long limit,
        void* workspace, int64_t* removed, cudaStream_t st) {
  const int blocks = blocks_of(n), pairs = pairs_of(n);
  const int parts = FACTOR ? kPairParts : 1;
  uint8_t* w = reinterpret_cast<uint8_t*>(workspace);
  T* b0 = reinterpret_cast<T*>(w);
  T* b1 = b0 + n;
  double* diag = reinterpret_cast<double*>(b1 + n);
  double* wdiag = diag + n;
  T* U = reinterpret_cast<T*>(wdiag + n);
  Pick* picks = reinterpret_cast<Pick*>(U + (size_t)count * n);  // [2]
  Candidate* best = reinterpret_cast<Candidate*>(picks + 2);
  unsigned* counter = reinterpret_cast<unsigned*>(best + blocks);
  uint8_t* alive = reinterpret_cast<uint8_t*>(counter + 4);
  const uintptr_t tail = align16(reinterpret_cast<uintptr_t>(alive + n));
  unsigned* pair_counter = reinterpret_cast<unsigned*>(tail);
  T* pair_parts = reinterpret_cast<T*>(tail + align16((size_t)pairs * sizeof(unsigned)));
  const size_t smem = FACTOR ? (size_t)((2 * n + parts - 1) / parts + 1) * sizeof(T) : 0;
  if (smem > 200 * 1024) return DSG_ERR_UNSUPPORTED;
  if (allow_smem(step_kernel<T, FACTOR>, smem) != DSG_OK) return DSG_ERR_LAUNCH;
  if (cudaMemsetAsync(pair_counter, 0, (size_t)pairs * sizeof(unsigned), st) != cudaSuccess) return DSG_ERR_LAUNCH;
  const T* W = reinterpret_cast<const T*>(inverse);
  const T* q = reinterpret_cast<const T*>(rhs);
  if (FACTOR) {
    const size_t init_smem = (size_t)((2 * n + kPairParts - 1) / kPairParts + 1) * sizeof(T);
    if (allow_smem(factor_init_kernel<T>, init_smem) != DSG_OK) return DSG_ERR_LAUNCH;
    factor_rows_kernel<T><<<(n + 7) / 8, 256, 0, st>>>(W, q, n, b1);  // y = X q in b1
    factor_init_kernel<T><<<pairs * kPairParts, kThreads, init_smem, st>>>(
        W, b1, n, blocks, kPairParts, b0, diag, wdiag, alive, pair_parts, pair_counter, picks, counter);
  } else {
    init_kernel<T><<<(n + 7) / 8, 256, 0, st>>>(W, q, n, b0, diag, wdiag, alive, picks, counter);
  }
  pick_kernel<T><<<1, kPickThreads, 0, st>>>(n, b0, diag, alive, limited, limit, wdiag, picks, removed);
  for (int step = 0; step < count; ++step) {
    const T* bi = (step & 1) ? b1 : b0;
    T* bo = (step & 1) ? b0 : b1;
    step_kernel<T, FACTOR><<<pairs * parts, kThreads, smem, st>>>(
        W, n, blocks, parts, step, count, bi, bo, diag, wdiag, alive, U, limited, limit, picks + (step & 1),
        picks + ((step + 1) & 1), best, counter, pair_parts, pair_counter, removed);
  }
  dsg_count_launches((FACTOR ? 3 : 2) + count);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // namespace

extern "C" {

size_t dsg_elimination_workspace_bytes(int32_t n, int32_t count, int32_t is_complex) {
  if (n <= 0 || count < 0) return 0;
  return elimination_bytes(n, count, is_complex != 0);
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
