// Fixed-order reductions, the float64 range response of the row basis, the plain FP32
// SYRK of the streamed normal equations, and the library's version and error strings.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <math.h>
#include <atomic>
#include <mutex>
#include "dsplat_gb300.h"

namespace {

constexpr int kEnergyBlocks = 512;
constexpr int kEnergyThreads = 256;

// Block b sums elements b, b + blocks, ... in double; lanes are combined in a fixed tree.
__global__ void energy_partial_kernel(const float2* __restrict__ v, const float2* __restrict__ r,
                                      int64_t count, double* __restrict__ partial) {
  __shared__ double sh[kEnergyThreads];
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const float2 a = v[i], b = r[i];
    const double dx = (double)a.x - (double)b.x, dy = (double)a.y - (double)b.y;
    acc += dx * dx + dy * dy;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kEnergyThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void energy_final_kernel(const double* __restrict__ partial, int n, double* out) {
  __shared__ double sh[kEnergyThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kEnergyThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

__global__ void range_response_kernel(double low, double high, int count, int bins, int samples,
                                      int nfft, double2* __restrict__ out) {
  const int64_t index = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (index >= (int64_t)count * bins) return;
  const int bin = (int)(index / count), peak = (int)(index % count);
  const double center = count > 1 ? low + (high - low) * (double)peak / (double)(count - 1) : low;
  double x = (double)bin - center;
  x -= (double)nfft * rint(x / (double)nfft);
  const double pi = 3.14159265358979323846;
  const double a = pi * samples / nfft, b = pi / nfft;
  double ratio;
  if (fabs(x) < 1e-3) {
    const double c2 = (b * b - a * a) / 6.0;
    const double c4 = (3.0 * a * a * a * a + 7.0 * b * b * b * b - 10.0 * a * a * b * b) / 360.0;
    ratio = 1.0 + c2 * x * x + c4 * x * x * x * x;
  } else {
    ratio = sinpi(x * samples / nfft) / (samples * sinpi(x / nfft));
  }
  double sp, cp;
  sincospi((double)(samples - 1) * x / nfft, &sp, &cp);
  out[index] = make_double2(ratio * cp, -ratio * sp);
}

std::mutex g_mutex;
std::atomic<unsigned long long> g_launches{0};
std::atomic<int> g_tuning[DSG_TUNE_COUNT] = {};
cublasHandle_t g_handles[64] = {};

}  // namespace

// Every launch site of the library adds its kernel count here (host side).
void dsg_count_launches(int kernels) { g_launches.fetch_add((unsigned long long)kernels); }

// Launch-shape knob for the launchers of this library; 0 means "choose automatically".
int dsg_tuning_value(int knob) { return knob >= 0 && knob < DSG_TUNE_COUNT ? g_tuning[knob].load() : 0; }

extern "C" {

uint64_t dsg_launch_count(void) { return g_launches.load(); }

int dsg_tuning_set(int32_t knob, int32_t value) {
  if (knob < 0 || knob >= DSG_TUNE_COUNT || value < 0) return DSG_ERR_ARGUMENT;
  static const int kMax[DSG_TUNE_COUNT] = {32, 8, 8, 2};
  if (value > kMax[knob]) return DSG_ERR_ARGUMENT;
  g_tuning[knob].store(value);
  return DSG_OK;
}

int32_t dsg_tuning_get(int32_t knob) {
  return knob >= 0 && knob < DSG_TUNE_COUNT ? g_tuning[knob].load() : -1;
}

const char* dsg_version(void) { return "dsplat-gb300 0.1.0 (sm_103a)"; }

const char* dsg_error_string(int code) {
  switch (code) {
    case DSG_OK: return "ok";
    case DSG_ERR_ARGUMENT: return "invalid argument";
    case DSG_ERR_UNSUPPORTED: return "unsupported configuration";
    case DSG_ERR_WORKSPACE: return "workspace missing or too small";
    case DSG_ERR_LAUNCH: return "kernel launch failed";
    case DSG_ERR_LIBRARY: return "cuBLAS call failed";
  }
  return "unknown error";
}

size_t dsg_energy_workspace_bytes(int64_t count) {
  (void)count;
  return kEnergyBlocks * sizeof(double);
}

int dsg_energy(const float* value, const float* reference, int64_t count, double* out,
               void* workspace, size_t workspace_bytes, void* stream) {
  if (count < 0 || !out) return DSG_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (count == 0) {
    cudaMemsetAsync(out, 0, sizeof(double), st);
    return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
  }
  if (!value || !reference) return DSG_ERR_ARGUMENT;
  if (!workspace || workspace_bytes < dsg_energy_workspace_bytes(count)) return DSG_ERR_WORKSPACE;
  double* part = reinterpret_cast<double*>(workspace);
  energy_partial_kernel<<<kEnergyBlocks, kEnergyThreads, 0, st>>>(
      reinterpret_cast<const float2*>(value), reinterpret_cast<const float2*>(reference), count,
      part);
  energy_final_kernel<<<1, kEnergyThreads, 0, st>>>(part, kEnergyBlocks, out);
  dsg_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

int dsg_range_response(double low, double high, int32_t count, int32_t bins, int32_t samples,
                       int32_t nfft, double* out, void* stream) {
  if (count <= 0 || bins <= 0 || samples <= 0 || nfft <= 0 || !out) return DSG_ERR_ARGUMENT;
  const int64_t n = (int64_t)count * bins;
  range_response_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      low, high, count, bins, samples, nfft, reinterpret_cast<double2*>(out));
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

static cublasHandle_t handle_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_handles[dev] && cublasCreate(&g_handles[dev]) != CUBLAS_STATUS_SUCCESS) g_handles[dev] = nullptr;
  return g_handles[dev];
}

int dsg_gemm_f32_bf16x9(int32_t m, int32_t n, int32_t k, const float* a, int32_t lda, const float* b,
                        int32_t ldb, float beta, float* c, int32_t ldc, void* stream) {
  if (m < 0 || n < 0 || k < 0 || lda < k || ldb < n || ldc < n) return DSG_ERR_ARGUMENT;
  if (m == 0 || n == 0) return DSG_OK;
  if (!a || !b || !c) return DSG_ERR_ARGUMENT;
  cublasHandle_t h = handle_for_current_device();
  if (!h) return DSG_ERR_LIBRARY;
  if (cublasSetStream(h, (cudaStream_t)stream) != CUBLAS_STATUS_SUCCESS) return DSG_ERR_LIBRARY;
  cublasSetEmulationStrategy(h, CUBLAS_EMULATION_STRATEGY_EAGER);
  const float one = 1.0f;
  // Row-major C = A B is column-major C^T = B^T A^T.
  cublasStatus_t st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, n, m, k, &one, b, CUDA_R_32F, ldb, a,
                                   CUDA_R_32F, lda, &beta, c, CUDA_R_32F, ldc,
                                   CUBLAS_COMPUTE_32F_EMULATED_16BFX9, CUBLAS_GEMM_DEFAULT);
  cublasSetEmulationStrategy(h, CUBLAS_EMULATION_STRATEGY_DEFAULT);
  return st == CUBLAS_STATUS_SUCCESS ? DSG_OK : DSG_ERR_LIBRARY;
}

int dsg_syrk_f32(const float* rows, int64_t m, int32_t n, float* out, void* stream) {
  if (m < 0 || n < 0 || m > 2147483647LL) return DSG_ERR_ARGUMENT;
  if (m == 0 || n == 0) return DSG_OK;
  if (!rows || !out) return DSG_ERR_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DSG_ERR_LIBRARY;
  cublasHandle_t h;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_handles[dev] && cublasCreate(&g_handles[dev]) != CUBLAS_STATUS_SUCCESS) {
      g_handles[dev] = nullptr;
      return DSG_ERR_LIBRARY;
    }
    h = g_handles[dev];
  }
  if (cublasSetStream(h, (cudaStream_t)stream) != CUBLAS_STATUS_SUCCESS) return DSG_ERR_LIBRARY;
  const float one = 1.0f;
  // The row-major [m, n] block is the column-major [n, m] matrix X; X X^T has in its
  // lower triangle (column-major) the upper triangle of the row-major result.
  cublasStatus_t s = cublasSsyrk(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, (int)m, &one, rows, n,
                                 &one, out, n);
  return s == CUBLAS_STATUS_SUCCESS ? DSG_OK : DSG_ERR_LIBRARY;
}

}  // extern "C"
