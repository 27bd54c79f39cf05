// Triangular inverse of a Cholesky factor in float64 (real or complex): the replacement's
// elimination then works from X = L^-1 (the inverse of the pooled system is X^H X)
// instead of forming the inverse with potri, which on this part costs about four times
// as much. Recursive halving in place,
//
//   [[A, 0], [B, C]]^-1 = [[A^-1, 0], [-C^-1 B A^-1, C^-1]],
//
// with the split points on multiples of kBlock rows: one launch first inverts every
// kBlock-row diagonal block (a CTA per block, forward substitution in shared memory, a
// thread per column), then the off-diagonal blocks are formed bottom-up by two cuBLAS trmm
// each (half the flops of general products).
#include <cublas_v2.h>
#include <cuComplex.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

constexpr int kBlock = 64;
constexpr int kNoZero = 0x7f7f7f7f;  // every byte 0x7f: set by one memset

std::mutex g_blas_mutex;
cublasHandle_t g_blas[64] = {};

cublasHandle_t blas_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_blas_mutex);
  if (!g_blas[dev] && cublasCreate(&g_blas[dev]) != CUBLAS_STATUS_SUCCESS) g_blas[dev] = nullptr;
  return g_blas[dev];
}

// Rows of the first diagonal block: about half, rounded up to a multiple of kBlock.
int64_t split(int64_t n) { return (n / 2 + kBlock - 1) / kBlock * kBlock; }

// The largest k x (n - k) product over every level of the halving: the top level's is not
// always the largest (n = 130 splits 128 + 2, and the 128-row half needs 64 x 64).
size_t scratch_bytes(int64_t n, bool complex_mode) {
  if (n <= kBlock) return 0;
  const int64_t k = split(n);
  const size_t here = (size_t)k * (size_t)(n - k) * (complex_mode ? 16 : 8);
  const size_t left = scratch_bytes(k, complex_mode), right = scratch_bytes(n - k, complex_mode);
  return here > left ? (here > right ? here : right) : (left > right ? left : right);
}

size_t align256(size_t bytes) { return (bytes + 255) / 256 * 256; }

__device__ __forceinline__ double mul_add(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ cuDoubleComplex mul_add(cuDoubleComplex a, cuDoubleComplex b, cuDoubleComplex c) {
  return make_cuDoubleComplex(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ double unit_minus(bool diagonal, double s) { return (diagonal ? 1.0 : 0.0) - s; }
__device__ __forceinline__ cuDoubleComplex unit_minus(bool diagonal, cuDoubleComplex s) {
  return make_cuDoubleComplex((diagonal ? 1.0 : 0.0) - s.x, -s.y);
}
__device__ __forceinline__ double divide(double a, double b) { return a / b; }
__device__ __forceinline__ cuDoubleComplex divide(cuDoubleComplex a, cuDoubleComplex b) { return cuCdiv(a, b); }
__device__ __forceinline__ bool is_zero(double a) { return a == 0.0; }
__device__ __forceinline__ bool is_zero(cuDoubleComplex a) { return a.x == 0.0 && a.y == 0.0; }
template <typename T>
__device__ __forceinline__ T zero_of();
template <>
__device__ __forceinline__ double zero_of<double>() { return 0.0; }
template <>
__device__ __forceinline__ cuDoubleComplex zero_of<cuDoubleComplex>() { return make_cuDoubleComplex(0.0, 0.0); }

// In place on the diagonal block of rows [kBlock * blockIdx.x, +kBlock) of a row-major
// lower-triangular matrix (leading dimension ld): the block becomes its inverse. Thread j
// owns column j; row i of the inverse is (e_i - sum_{k<i} L_ik X_k) / L_ii, so the block
// is overwritten row by row (rows above i already hold X, row i still holds L).
template <typename T>
__global__ void __launch_bounds__(kBlock) block_inverse_kernel(T* __restrict__ a, int n, int64_t ld,
                                                               int* __restrict__ first_zero) {
  extern __shared__ __align__(16) unsigned char raw[];
  T* x = reinterpret_cast<T*>(raw);  // [kBlock][kBlock]
  const int r0 = blockIdx.x * kBlock;
  const int size = min(kBlock, n - r0);
  const int j = threadIdx.x;
  const T zero = zero_of<T>();
  for (int i = 0; i < kBlock; ++i)
    x[i * kBlock + j] = (i < size && j <= i) ? a[(size_t)(r0 + i) * ld + r0 + j] : zero;
  __syncthreads();
  for (int i = 0; i < size; ++i) {
    T sum = zero;
    for (int k = 0; k < i; ++k) sum = mul_add(x[i * kBlock + k], x[k * kBlock + j], sum);
    const T diagonal = x[i * kBlock + i];
    __syncthreads();  // row i is read by every thread before it is overwritten
    if (j == 0 && is_zero(diagonal)) atomicMin(first_zero, r0 + i + 1);
    x[i * kBlock + j] = j <= i ? divide(unit_minus(i == j, sum), diagonal) : zero;
    __syncthreads();
  }
  for (int i = 0; i < size; ++i)
    if (j <= i) a[(size_t)(r0 + i) * ld + r0 + j] = x[i * kBlock + j];
}

__global__ void finish_info(const int* __restrict__ first_zero, int32_t* __restrict__ info) {
  *info = *first_zero == kNoZero ? 0 : *first_zero;
}

struct Inverter {
  cublasHandle_t blas;
  bool complex_mode;
  size_t element;
  void* scratch;  // the largest k x (n - k) product of the halving

  // The off-diagonal blocks of the n rows at a (leading dimension ld), bottom-up; the
  // diagonal blocks of kBlock rows are inverted already.
  bool combine(uint8_t* a, int64_t n, int64_t ld) const {
    if (n <= kBlock) return true;
    const int64_t k = split(n), m = n - k;
    uint8_t* lower = a + (size_t)k * ld * element;  // B: rows k.., columns ..k
    uint8_t* corner = lower + (size_t)k * element;  // C
    if (!combine(a, k, ld) || !combine(corner, m, ld)) return false;
    // Column-major views: A^-T (k x k upper), B^T (k x m), C^-T (m x m upper).
    // T^T = A^-T B^T into the scratch (k x m, leading dimension k), then
    // (-C^-1 B A^-1)^T = -T^T C^-T over B^T.
    dsg_count_launches(2);
    if (complex_mode) {
      const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), minus = make_cuDoubleComplex(-1.0, 0.0);
      auto A = reinterpret_cast<const cuDoubleComplex*>(a);
      auto B = reinterpret_cast<cuDoubleComplex*>(lower);
      auto C = reinterpret_cast<const cuDoubleComplex*>(corner);
      auto T = reinterpret_cast<cuDoubleComplex*>(scratch);
      return cublasZtrmm(blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, k, m,
                         &one, A, ld, B, ld, T, k) == CUBLAS_STATUS_SUCCESS &&
             cublasZtrmm(blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, k, m,
                         &minus, C, ld, T, k, B, ld) == CUBLAS_STATUS_SUCCESS;
    }
    const double one = 1.0, minus = -1.0;
    auto A = reinterpret_cast<const double*>(a);
    auto B = reinterpret_cast<double*>(lower);
    auto C = reinterpret_cast<const double*>(corner);
    auto T = reinterpret_cast<double*>(scratch);
    return cublasDtrmm(blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, k, m,
                       &one, A, ld, B, ld, T, k) == CUBLAS_STATUS_SUCCESS &&
           cublasDtrmm(blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, k, m,
                       &minus, C, ld, T, k, B, ld) == CUBLAS_STATUS_SUCCESS;
  }
};

template <typename T>
int invert_blocks(void* factor, int n, cudaStream_t stream, int* first_zero) {
  const size_t smem = (size_t)kBlock * kBlock * sizeof(T);
  if (smem > 48 * 1024 &&  // no static shared memory in this kernel
      cudaFuncSetAttribute(block_inverse_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return DSG_ERR_LAUNCH;
  block_inverse_kernel<T><<<(n + kBlock - 1) / kBlock, kBlock, smem, stream>>>(static_cast<T*>(factor), n, n,
                                                                              first_zero);
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // namespace

extern "C" {

size_t dsg_triangular_inverse_workspace_bytes(int32_t n, int32_t is_complex) {
  if (n <= 0) return 0;
  return align256(scratch_bytes(n, is_complex != 0)) + 256;
}

int dsg_triangular_inverse(void* factor, int32_t n, int32_t is_complex, void* workspace, size_t workspace_bytes,
                           int32_t* info, void* stream) {
  if (n < 0) return DSG_ERR_ARGUMENT;
  if (n == 0) return DSG_OK;
  if (!factor || !info) return DSG_ERR_ARGUMENT;
  const bool complex_mode = is_complex != 0;
  const size_t scratch = scratch_bytes(n, complex_mode);
  if (!workspace || workspace_bytes < align256(scratch) + sizeof(int)) return DSG_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* base = static_cast<uint8_t*>(workspace);
  int* first_zero = reinterpret_cast<int*>(base + align256(scratch));
  if (cudaMemsetAsync(first_zero, 0x7f, sizeof(int), st) != cudaSuccess) return DSG_ERR_LAUNCH;
  const int launched = complex_mode ? invert_blocks<cuDoubleComplex>(factor, n, st, first_zero)
                                    : invert_blocks<double>(factor, n, st, first_zero);
  if (launched != DSG_OK) return launched;
  if (n > kBlock) {
    cublasHandle_t b = blas_for_current_device();
    if (!b || cublasSetStream(b, st) != CUBLAS_STATUS_SUCCESS) return DSG_ERR_LIBRARY;
    const Inverter inverter{b, complex_mode, (size_t)(complex_mode ? 16 : 8), scratch ? base : nullptr};
    if (!inverter.combine(static_cast<uint8_t*>(factor), n, n)) return DSG_ERR_LIBRARY;
  }
  finish_info<<<1, 1, 0, st>>>(first_zero, info);
  dsg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? DSG_OK : DSG_ERR_LAUNCH;
}

}  // extern "C"
