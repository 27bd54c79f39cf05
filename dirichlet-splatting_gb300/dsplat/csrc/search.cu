// Candidate kernels of the spatial search: range gate, greedy separated peaks, the
// per-candidate quasi-Newton direction and the trial step, one fraction or all the
// backtracking fractions of an iteration (reference: dsplat/kernels/search.slang:1-109).
#include <cuda_runtime.h>
#include <math.h>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

__global__ void range_gate_kernel(const float* __restrict__ points, int count,
                                  const float* __restrict__ positions, int apertures,
                                  const int* __restrict__ intervals, int bins, float spacing,
                                  int required, int* __restrict__ output) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float px = points[3 * i], py = points[3 * i + 1], pz = points[3 * i + 2];
  int matches = 0;
  for (int a = 0; a < apertures; ++a) {
    const float dx = px - positions[3 * a], dy = py - positions[3 * a + 1],
                dz = pz - positions[3 * a + 2];
    const float x = sqrtf(dx * dx + dy * dy + dz * dz) / spacing;
    const int k = (int)rintf(x);  // round half to even
    if (k >= 0 && k < bins && intervals[(size_t)a * bins + k] != 0) ++matches;
  }
  output[i] = matches >= required ? 1 : 0;
}

constexpr int kPeakThreads = 1024;
constexpr int kMaxAccepted = 4096;  // peaks held in shared memory per launch
constexpr int kChunkSlots = 2048;   // cells of one chunk's survivors (at most kPeakThreads)

// Opt a kernel in to `dynamic` bytes of dynamic shared memory when that and its static
// arrays exceed the default 48 KB.
template <typename Kernel>
bool allow_shared(Kernel kernel, size_t dynamic) {
  cudaFuncAttributes attributes;
  if (cudaFuncGetAttributes(&attributes, kernel) != cudaSuccess) return false;
  if (dynamic + attributes.sharedSizeBytes <= 48 * 1024) return true;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dynamic) == cudaSuccess;
}

// Greedy separated peaks over candidates visited in descending-score order (ties in
// index order): a candidate is taken unless it lies within separation of one already
// taken. This selects the same indices in the same order as repeatedly taking the best
// remaining finite score (lowest index on ties) and suppressing its neighbourhood
// (reference: dsplat/kernels/search.slang:26-64). Chunks of 1024 candidates are first
// checked against the taken set in parallel; a chunk's survivors are then resolved in
// order, each taken one suppressing the later ones within separation.
//
// In one to three dimensions the taken peaks are also filed in a shared-memory hash of
// cells of side separation (1 + 2^-16), so a candidate looks only at the peaks of its own
// and the 3^d - 1 neighbouring cells (any peak nearer than separation lies there) instead
// of scanning every taken peak. A chunk's survivors are then filed in a second hash of the
// same cells and resolved in parallel rounds: a survivor is suppressed as soon as an
// earlier survivor within separation is taken, and taken once every earlier survivor
// within separation is suppressed. Each round settles at least the earliest open
// survivor (all of its earlier neighbours are settled), so the rounds end, and the
// decisions are those of the in-order greedy pass; the selection is the same.
constexpr unsigned long long kEmptyCell = ~0ull;

__device__ __forceinline__ int cell_of(float x, float inv_cell) {
  const float c = floorf(x * inv_cell);
  return (int)fminf(fmaxf(c, -1048000.0f), 1048000.0f);
}

__device__ __forceinline__ unsigned long long cell_key(int cx, int cy, int cz) {
  return ((unsigned long long)(cx + (1 << 20)) << 42) | ((unsigned long long)(cy + (1 << 20)) << 21) |
         (unsigned long long)(cz + (1 << 20));
}

__device__ __forceinline__ unsigned cell_slot(unsigned long long key, unsigned mask) {
  return (unsigned)((key * 0x9E3779B97F4A7C15ull) >> 40) & mask;
}

struct PeakCells {
  unsigned long long* keys;  // [slots], kEmptyCell when free
  int* heads;                // [slots] first taken peak filed in the cell
  int* next;                 // [peaks] next entry of the same cell, -1 at the end
  unsigned mask;             // slots - 1
  float inv_cell;
};

__device__ __forceinline__ void cell_coords(const PeakCells& h, const float* c, int dimension, int* cc) {
  cc[0] = cell_of(c[0], h.inv_cell);
  cc[1] = dimension > 1 ? cell_of(c[1], h.inv_cell) : 0;
  cc[2] = dimension > 2 ? cell_of(c[2], h.inv_cell) : 0;
}

// Whether a taken peak filed in the cell at offset (dx, dy, dz) from c's cell lies within
// separation of c (sep2 = separation^2).
__device__ bool cell_hit(const PeakCells& h, const float* c, int dimension, const int* cc, int dx, int dy, int dz,
                         const float* taken_xyz, float sep2) {
  const unsigned long long key = cell_key(cc[0] + dx, cc[1] + dy, cc[2] + dz);
  unsigned s = cell_slot(key, h.mask);
  for (unsigned probe = 0; probe <= h.mask; ++probe, s = (s + 1) & h.mask) {
    const unsigned long long k = h.keys[s];
    if (k == kEmptyCell) return false;
    if (k != key) continue;
    for (int t = h.heads[s]; t >= 0; t = h.next[t]) {
      float d2 = 0.0f;
      for (int j = 0; j < dimension; ++j) {
        const float d = c[j] - taken_xyz[t * dimension + j];
        d2 += d * d;
      }
      if (d2 < sep2) return true;
    }
    return false;
  }
  return false;
}

// Whether a taken peak lies within separation of c: its own and the neighbouring cells.
__device__ bool near_taken(const PeakCells& h, const float* c, int dimension, const float* taken_xyz,
                           float sep2) {
  int cc[3];
  cell_coords(h, c, dimension, cc);
  const int ry = dimension > 1 ? 1 : 0, rz = dimension > 2 ? 1 : 0;
  for (int dz = -rz; dz <= rz; ++dz)
    for (int dy = -ry; dy <= ry; ++dy)
      for (int dx = -1; dx <= 1; ++dx)
        if (cell_hit(h, c, dimension, cc, dx, dy, dz, taken_xyz, sep2)) return true;
  return false;
}

// Files taken peak `slot` under its cell; any number of threads at once.
__device__ __forceinline__ void file_peak_shared(const PeakCells& h, const float* c, int dimension, int slot) {
  int cc[3];
  cell_coords(h, c, dimension, cc);
  const unsigned long long key = cell_key(cc[0], cc[1], cc[2]);
  unsigned s = cell_slot(key, h.mask);
  for (unsigned probe = 0; probe <= h.mask; ++probe, s = (s + 1) & h.mask) {
    const unsigned long long seen = atomicCAS(&h.keys[s], kEmptyCell, key);
    if (seen == kEmptyCell || seen == key) {
      h.next[slot] = atomicExch(&h.heads[s], slot);
      return;
    }
  }
}

// Settles survivor q of a chunk (chunk cells `cc` of the survivors, coordinates xyz[q]):
// 1 taken, 2 suppressed, 0 still open (an earlier neighbour is open).
__device__ __forceinline__ int settle_survivor(const PeakCells& h, const float* xyz, int dimension, int q, float sep2,
                               const volatile int* state) {
  int cc[3];
  const float* c = xyz + q * 3;
  cell_coords(h, c, dimension, cc);
  const int ry = dimension > 1 ? 1 : 0, rz = dimension > 2 ? 1 : 0;
  bool open = false;
  for (int dz = -rz; dz <= rz; ++dz)
    for (int dy = -ry; dy <= ry; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const unsigned long long key = cell_key(cc[0] + dx, cc[1] + dy, cc[2] + dz);
        unsigned s = cell_slot(key, h.mask);
        for (unsigned probe = 0; probe <= h.mask; ++probe, s = (s + 1) & h.mask) {
          const unsigned long long k = h.keys[s];
          if (k == kEmptyCell) break;
          if (k != key) continue;
          for (int t = h.heads[s]; t >= 0; t = h.next[t]) {
            if (t >= q) continue;
            float d2 = 0.0f;
            for (int j = 0; j < dimension; ++j) {
              const float d = c[j] - xyz[t * 3 + j];
              d2 += d * d;
            }
            if (d2 < sep2) {
              const int st = state[t];
              if (st == 1) return 2;
              if (st == 0) open = true;
            }
          }
          break;
        }
      }
  return open ? 0 : 1;
}

__global__ void __launch_bounds__(kPeakThreads, 1) peaks_kernel(const float* __restrict__ scores,
                                                             const int* __restrict__ order,
                                                             const float* __restrict__ centers,
                                                             int count, int dimension, int peaks,
                                                             float separation, int slots,
                                                             int* __restrict__ output) {
  extern __shared__ unsigned long long peak_smem[];
  __shared__ float chunk_xyz[kPeakThreads * 3];  // hashed: the chunk's survivors' coordinates
  __shared__ int alive[kPeakThreads];
  __shared__ int alive_list[kPeakThreads];  // the chunk's survivors, in order
  __shared__ int warp_alive[2][kPeakThreads / 32];  // by chunk parity: no barrier before reuse
  __shared__ int warp_taken[kPeakThreads / 32];
  __shared__ int n_taken;
  const bool hashed = slots > 0;  // uniform
  PeakCells cells;
  cells.keys = peak_smem;
  cells.heads = reinterpret_cast<int*>(peak_smem + slots);
  cells.next = cells.heads + slots;
  cells.mask = (unsigned)slots - 1u;
  cells.inv_cell = 1.0f / (separation * (1.0f + 1.0f / 65536.0f));
  float* taken_xyz = reinterpret_cast<float*>(cells.next + (hashed ? peaks : 0));  // [peaks][dimension]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float sep2 = separation * separation;

  if (hashed) {
    // the chunk's survivors filed by cell (kChunkSlots keys and heads, next per survivor)
    PeakCells chunk_cells;
    chunk_cells.keys = reinterpret_cast<unsigned long long*>(
        (reinterpret_cast<uintptr_t>(taken_xyz + (size_t)peaks * dimension) + 7) & ~(uintptr_t)7);
    chunk_cells.heads = reinterpret_cast<int*>(chunk_cells.keys + kChunkSlots);
    chunk_cells.next = chunk_cells.heads + kChunkSlots;
    chunk_cells.mask = kChunkSlots - 1u;
    chunk_cells.inv_cell = cells.inv_cell;
    int* state = alive;  // per survivor: 0 open, 1 taken, 2 suppressed
    float* sxyz = chunk_xyz;
    for (int i = tid; i < slots; i += kPeakThreads) {
      cells.keys[i] = kEmptyCell;
      cells.heads[i] = -1;
    }
    for (int i = tid; i < kChunkSlots; i += kPeakThreads) {
      chunk_cells.keys[i] = kEmptyCell;
      chunk_cells.heads[i] = -1;
    }
    __syncthreads();
    int taken = 0;  // the same value in every thread
    for (int base = 0, chunk = 0; base < count && taken < peaks; base += kPeakThreads, ++chunk) {
      const int pos = base + tid;
      float c[3] = {0.f, 0.f, 0.f};
      bool ok = false;
      if (pos < count) {
        const int index = order[pos];
        ok = isfinite(scores[index]);
        for (int j = 0; j < dimension; ++j) c[j] = centers[(size_t)index * dimension + j];
      }
      if (ok && taken > 0) ok = !near_taken(cells, c, dimension, taken_xyz, sep2);
      int* wa = warp_alive[chunk & 1];
      const unsigned ballot = __ballot_sync(0xffffffffu, ok);
      if (lane == 0) wa[warp] = __popc(ballot);
      __syncthreads();
      int before = __popc(ballot & ((1u << lane) - 1u)), survivors = 0;
      for (int w = 0; w < kPeakThreads / 32; ++w) {
        before += w < warp ? wa[w] : 0;
        survivors += wa[w];
      }
      if (survivors == 0) continue;  // uniform: a chunk the taken peaks suppress entirely
      if (ok) {  // survivor `before`: its position, coordinates and state
        alive_list[before] = tid;
        for (int j = 0; j < 3; ++j) sxyz[before * 3 + j] = c[j];
        state[before] = 0;
      }
      __syncthreads();
      if (ok) file_peak_shared(chunk_cells, c, dimension, before);
      __syncthreads();
      // rounds: each settles at least the earliest open survivor, so survivors + 1 bound them
      for (int round = 0; round <= survivors; ++round) {
        int open = 0;
        if (tid < survivors && state[tid] == 0) {
          const int verdict = settle_survivor(chunk_cells, sxyz, dimension, tid, sep2, state);
          if (verdict != 0) state[tid] = verdict;
          open = verdict == 0;
        }
        if (!__syncthreads_or(open)) break;
      }
      // the taken survivors in order, up to the peaks still wanted
      const bool took = tid < survivors && state[tid] == 1;
      const unsigned tb = __ballot_sync(0xffffffffu, took);
      if (lane == 0) warp_taken[warp] = __popc(tb);
      __syncthreads();
      int rank = __popc(tb & ((1u << lane) - 1u)), total = 0;
      for (int w = 0; w < kPeakThreads / 32; ++w) {
        rank += w < warp ? warp_taken[w] : 0;
        total += warp_taken[w];
      }
      const int room = peaks - taken;
      if (took && rank < room) {
        const int slot = taken + rank;
        for (int j = 0; j < dimension; ++j) taken_xyz[slot * dimension + j] = sxyz[tid * 3 + j];
        output[slot] = order[base + alive_list[tid]];
        file_peak_shared(cells, sxyz + tid * 3, dimension, slot);
      }
      // the chunk hash was last read in the rounds: clear it for the next chunk
      for (int i = tid; i < kChunkSlots; i += kPeakThreads) {
        chunk_cells.keys[i] = kEmptyCell;
        chunk_cells.heads[i] = -1;
      }
      taken += min(total, room);
      __syncthreads();  // the new peaks are filed and the chunk hash is clear
    }
    return;
  }

  if (tid == 0) n_taken = 0;
  __syncthreads();
  for (int base = 0; base < count; base += kPeakThreads) {
    if (n_taken >= peaks) break;  // uniform: shared, stable between barriers
    const int pos = base + tid;
    int index = -1;
    float c[8];
    bool ok = false;
    if (pos < count) {
      index = order[pos];
      ok = isfinite(scores[index]);
      for (int j = 0; j < dimension; ++j) c[j] = centers[(size_t)index * dimension + j];
    }
    const int taken_now = n_taken;
    // Latest peaks first: a suppressed candidate mostly lies near a recent, slightly
    // better one, so its scan ends early (the outcome does not depend on the order).
    for (int t = taken_now - 1; ok && t >= 0; --t) {
      float d2 = 0.0f;
      for (int j = 0; j < dimension; ++j) {
        const float d = c[j] - taken_xyz[t * dimension + j];
        d2 += d * d;
      }
      if (d2 < sep2) ok = false;
    }
    alive[tid] = ok ? 1 : 0;
    const unsigned ballot = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) warp_alive[0][warp] = __popc(ballot);
    __syncthreads();
    int before = __popc(ballot & ((1u << lane) - 1u)), survivors = 0;
    for (int w = 0; w < kPeakThreads / 32; ++w) {
      before += w < warp ? warp_alive[0][w] : 0;
      survivors += warp_alive[0][w];
    }
    if (ok) alive_list[before] = tid;
    __syncthreads();
    const int limit = min(kPeakThreads, count - base);
    for (int q = 0; q < survivors; ++q) {
      const int k = alive_list[q];
      if (!alive[k]) continue;       // uniform
      const int slot = n_taken;      // uniform
      if (slot >= peaks) break;
      if (tid == k) {
        for (int j = 0; j < dimension; ++j) taken_xyz[slot * dimension + j] = c[j];
        output[slot] = index;
      }
      __syncthreads();
      if (tid > k && tid < limit && alive[tid]) {
        float d2 = 0.0f;
        for (int j = 0; j < dimension; ++j) {
          const float d = c[j] - taken_xyz[slot * dimension + j];
          d2 += d * d;
        }
        if (d2 < sep2) alive[tid] = 0;
      }
      if (tid == 0) n_taken = slot + 1;
      __syncthreads();
    }
    __syncthreads();  // the chunk's flags and lists are read by every thread before reuse
  }
}

// Best-scoring candidates that collide neither with an occupied point nor with a
// candidate kept before them (reference: dsplat/replacement.py:142-175 _distinct):
// candidates are visited in descending-score order (ties in index order, non-finite
// scores skipped); a distance below separation, or exactly zero, is a collision;
// distances fold periodic axes into [-period/2, period/2]. At most width are kept.
__device__ __forceinline__ float folded_distance(const float* a, const float* b, int dim,
                                                 const float* period) {
  float d2 = 0.0f;
  for (int j = 0; j < dim; ++j) {
    float d = a[j] - b[j];
    if (period != nullptr) d -= period[j] * rintf(d / period[j]);
    d2 += d * d;
  }
  return sqrtf(d2);
}

__global__ void __launch_bounds__(kPeakThreads) distinct_kernel(
    const float* __restrict__ scores, const int* __restrict__ order, const float* __restrict__ points,
    int count, int dimension, const float* __restrict__ occupied, int n_occupied,
    const float* __restrict__ period, float separation, int width, int* __restrict__ output,
    int* __restrict__ kept_count) {
  extern __shared__ float shared_xyz[];  // occupied [n_occupied][dim], then kept [width][dim]
  float* kept_xyz = shared_xyz + (size_t)n_occupied * dimension;
  __shared__ int alive[kPeakThreads];
  __shared__ int n_kept;
  __shared__ float per[8];
  const int tid = threadIdx.x;
  for (int i = tid; i < n_occupied * dimension; i += kPeakThreads) shared_xyz[i] = occupied[i];
  if (tid < dimension) per[tid] = period != nullptr ? period[tid] : 0.0f;
  if (tid == 0) n_kept = 0;
  __syncthreads();
  const float* pp = period != nullptr ? per : nullptr;
  for (int base = 0; base < count; base += kPeakThreads) {
    if (n_kept >= width) break;
    const int pos = base + tid;
    int index = -1;
    float c[8];
    bool ok = false;
    if (pos < count) {
      index = order[pos];
      ok = isfinite(scores[index]);
      for (int j = 0; j < dimension; ++j) c[j] = points[(size_t)index * dimension + j];
    }
    for (int o = 0; ok && o < n_occupied; ++o) {
      const float d = folded_distance(c, shared_xyz + o * dimension, dimension, pp);
      if (!(d >= separation) || !(d > 0.0f)) ok = false;
    }
    const int kept_now = n_kept;
    for (int t = 0; ok && t < kept_now; ++t) {
      const float d = folded_distance(c, kept_xyz + t * dimension, dimension, pp);
      if (!(d >= separation) || !(d > 0.0f)) ok = false;
    }
    alive[tid] = ok ? 1 : 0;
    __syncthreads();
    const int limit = min(kPeakThreads, count - base);
    for (int k = 0; k < limit; ++k) {
      if (!alive[k]) continue;  // uniform
      const int slot = n_kept;  // uniform
      if (slot >= width) break;
      if (tid == k) {
        for (int j = 0; j < dimension; ++j) kept_xyz[slot * dimension + j] = c[j];
        output[slot] = index;
      }
      __syncthreads();
      if (tid > k && tid < limit && alive[tid]) {
        const float d = folded_distance(c, kept_xyz + slot * dimension, dimension, pp);
        if (!(d >= separation) || !(d > 0.0f)) alive[tid] = 0;
      }
      if (tid == 0) n_kept = slot + 1;
      __syncthreads();
    }
    __syncthreads();  // the chunk's flags are read by every thread before reuse
  }
  if (tid == 0) *kept_count = n_kept;
}

__global__ void direction_kernel(const float* __restrict__ inverse,
                                 const float* __restrict__ gradient,
                                 const float* __restrict__ normals, const float* __restrict__ mask,
                                 int count, int width, float radius, float* __restrict__ output) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float d[6], g[6];
  for (int j = 0; j < width; ++j) g[j] = gradient[i * width + j];
  float descent = 0.0f;
  for (int j = 0; j < width; ++j) {
    float v = 0.0f;
    for (int k = 0; k < width; ++k) v -= inverse[((size_t)i * width + j) * width + k] * g[k];
    d[j] = v;
    descent += v * g[j];
  }
  for (int j = 0; j < width; ++j) d[j] = (descent >= 0.0f ? -g[j] : d[j]) * mask[j];
  if (width == 6) {
    float proj = 0.0f;
    for (int j = 0; j < 3; ++j) proj += d[3 + j] * normals[3 * i + j];
    for (int j = 0; j < 3; ++j) d[3 + j] -= proj * normals[3 * i + j];
  }
  float len2 = 0.0f;
  for (int j = 0; j < width; ++j) len2 += d[j] * d[j];
  const float scale = fminf(1.0f, radius / fmaxf(sqrtf(len2), 1e-30f));
  for (int j = 0; j < width; ++j) output[i * width + j] = d[j] * scale;
}

// One candidate's trial step: centers move by fraction * scale * direction on their
// free axes and are clamped to the box; normals (width 6) move and are renormalized.
__device__ __forceinline__ void trial_one(const float* __restrict__ centers, const float* __restrict__ normals,
                                          const float* __restrict__ direction,
                                          const float* __restrict__ controls, int i, int width, float fraction,
                                          float* __restrict__ out_centers, float* __restrict__ out_normals) {
  float n[3], len2 = 0.0f;
  for (int j = 0; j < 3; ++j) {
    const float c = centers[3 * i + j] + fraction * controls[j] * direction[i * width + j];
    const float lo = controls[12 + j], hi = controls[18 + j];
    out_centers[3 * i + j] = controls[6 + j] > 0.0f ? fminf(fmaxf(c, lo), hi) : centers[3 * i + j];
    n[j] = normals[3 * i + j] +
           (width == 6 ? fraction * controls[3 + j] * direction[i * width + 3 + j] : 0.0f);
    len2 += n[j] * n[j];
  }
  const float inv = width == 6 ? 1.0f / sqrtf(len2) : 1.0f;
  for (int j = 0; j < 3; ++j) out_normals[3 * i + j] = width == 6 ? n[j] * inv : normals[3 * i + j];
}

__global__ void trial_kernel(const float* __restrict__ centers, const float* __restrict__ normals,
                             const float* __restrict__ direction,
                             const float* __restrict__ controls, int count, int width,
                             float fraction, float* __restrict__ out_centers,
                             float* __restrict__ out_normals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  trial_one(centers, normals, direction, controls, i, width, fraction, out_centers, out_normals);
}

constexpr int kMaxFractions = 16;
struct Fractions {
  float value[kMaxFractions];
};

// Every backtracking fraction of an iteration in one launch: blockIdx.y picks the
// fraction, whose trials fill rows [y * count, (y + 1) * count) of the outputs.
__global__ void trials_kernel(const float* __restrict__ centers, const float* __restrict__ normals,
                              const float* __restrict__ direction, const float* __restrict__ controls,
                              int count, int width, Fractions fractions, float* __restrict__ out_centers,
                              float* __restrict__ out_normals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const size_t row = (size_t)blockIdx.y * count * 3;
  trial_one(centers, normals, direction, controls, i, width, fractions.value[blockIdx.y], out_centers + row,
            out_normals + row);
}

int status() { return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH; }

}  // namespace

extern "C" {

int dsg_range_gate(const float* points, int32_t count, const float* positions,
                   int32_t apertures, const int32_t* intervals, int32_t bins, float spacing,
                   int32_t required, int32_t* output, void* stream) {
  if (count < 0 || apertures < 0 || bins < 0 || !(spacing > 0.0f)) return DSG_ERR_ARGUMENT;
  if (count == 0) return DSG_OK;
  if (!points || !output || (apertures > 0 && (!positions || !intervals))) return DSG_ERR_ARGUMENT;
  range_gate_kernel<<<(count + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      points, count, positions, apertures, intervals, bins, spacing, required, output);
  dsg_count_launches(1);
  return status();
}

int dsg_peaks(const float* scores, const int32_t* order, const float* centers, int32_t count,
              int32_t dimension, int32_t peaks, float separation, int32_t* output, void* stream) {
  if (count < 0 || peaks < 0 || peaks > kMaxAccepted || dimension < 1 || dimension > 8)
    return DSG_ERR_ARGUMENT;
  if (peaks == 0) return DSG_OK;
  if (!output || (count > 0 && (!scores || !order || !centers))) return DSG_ERR_ARGUMENT;
  cudaMemsetAsync(output, 0xff, (size_t)peaks * sizeof(int32_t), (cudaStream_t)stream);
  if (count == 0) return status();
  // cell hash (1..3 dimensions, a finite positive separation): twice the peaks' slots
  int slots = 0;
  if (dimension <= 3 && separation > 0.0f && isfinite(separation)) {
    slots = 64;
    while (slots < 2 * peaks) slots <<= 1;
  }
  size_t smem = (size_t)slots * (sizeof(unsigned long long) + sizeof(int)) +
                (slots > 0 ? (size_t)peaks * sizeof(int) : 0) + (size_t)peaks * dimension * sizeof(float);
  if (slots > 0)  // the chunk's survivor hash, 8-byte aligned after the taken coordinates
    smem = (smem + 7) / 8 * 8 + (size_t)kChunkSlots * (sizeof(unsigned long long) + sizeof(int)) +
           (size_t)kPeakThreads * sizeof(int);
  if (!allow_shared(peaks_kernel, smem)) return DSG_ERR_LAUNCH;
  peaks_kernel<<<1, kPeakThreads, smem, (cudaStream_t)stream>>>(scores, order, centers, count, dimension,
                                                               peaks, separation, slots, output);
  dsg_count_launches(1);
  return status();
}

int dsg_distinct(const float* scores, const int32_t* order, const float* points, int32_t count,
                 int32_t dimension, const float* occupied, int32_t n_occupied, const float* period,
                 float separation, int32_t width, int32_t* output, int32_t* kept_count,
                 void* stream) {
  if (count < 0 || n_occupied < 0 || width < 0 || dimension < 1 || dimension > 8)
    return DSG_ERR_ARGUMENT;
  if (!kept_count || (width > 0 && !output)) return DSG_ERR_ARGUMENT;
  if ((count > 0 && (!scores || !order || !points)) || (n_occupied > 0 && !occupied))
    return DSG_ERR_ARGUMENT;
  const size_t smem = (size_t)(n_occupied + width) * dimension * sizeof(float);
  if (smem > 200 * 1024) return DSG_ERR_UNSUPPORTED;
  if (!allow_shared(distinct_kernel, smem)) return DSG_ERR_LAUNCH;
  distinct_kernel<<<1, kPeakThreads, smem, (cudaStream_t)stream>>>(
      scores, order, points, count, dimension, occupied, n_occupied, period, separation, width,
      output, kept_count);
  dsg_count_launches(1);
  return status();
}

int dsg_direction(const float* inverse, const float* gradient, const float* normals,
                  const float* mask, int32_t count, int32_t width, float radius, float* output,
                  void* stream) {
  if (count < 0 || (width != 3 && width != 6)) return DSG_ERR_ARGUMENT;
  if (count == 0) return DSG_OK;
  if (!inverse || !gradient || !normals || !mask || !output) return DSG_ERR_ARGUMENT;
  direction_kernel<<<(count + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      inverse, gradient, normals, mask, count, width, radius, output);
  dsg_count_launches(1);
  return status();
}

int dsg_trial(const float* centers, const float* normals, const float* direction,
              const float* controls, int32_t count, int32_t width, float fraction,
              float* out_centers, float* out_normals, void* stream) {
  if (count < 0 || (width != 3 && width != 6)) return DSG_ERR_ARGUMENT;
  if (count == 0) return DSG_OK;
  if (!centers || !normals || !direction || !controls || !out_centers || !out_normals)
    return DSG_ERR_ARGUMENT;
  trial_kernel<<<(count + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      centers, normals, direction, controls, count, width, fraction, out_centers, out_normals);
  dsg_count_launches(1);
  return status();
}

int dsg_trials(const float* centers, const float* normals, const float* direction,
               const float* controls, int32_t count, int32_t width, const float* fractions,
               int32_t fraction_count, float* out_centers, float* out_normals, void* stream) {
  if (count < 0 || (width != 3 && width != 6) || fraction_count < 1 || fraction_count > kMaxFractions ||
      !fractions)
    return DSG_ERR_ARGUMENT;
  if (count == 0) return DSG_OK;
  if (!centers || !normals || !direction || !controls || !out_centers || !out_normals)
    return DSG_ERR_ARGUMENT;
  Fractions f{};
  for (int b = 0; b < fraction_count; ++b) f.value[b] = fractions[b];
  const dim3 grid((unsigned)((count + 127) / 128), (unsigned)fraction_count);
  trials_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(centers, normals, direction, controls, count, width, f,
                                                        out_centers, out_normals);
  dsg_count_launches(1);
  return status();
}

}  // extern "C"
