// Triangular inverse of a Cholesky factor in float64 (real or complex): the replacement's
// elimination then works from X = L^-1 (the inverse of the pooled system is X^H X)
// instead of forming the inverse with potri, which on this part costs about four times
// as much. Recursive halving in place,
//
//   [[A, 0], [B, C]]^-1 = [[A^-1, 0], [-C^-1 B A^-1, C^-1]],
//
// with the off-diagonal block formed by two triangular products (cuBLAS trmm, half the
// flops of the general products) and diagonal blocks of at most kLeaf rows inverted by
// cuSOLVER's trtri.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <stdint.h>
#include <mutex>
#include <vector>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

constexpr int64_t kLeaf = 512;

std::mutex g_solver_mutex;
cusolverDnHandle_t g_solvers[64] = {};
cublasHandle_t g_blas[64] = {};

cusolverDnHandle_t solver_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_solver_mutex);
  if (!g_solvers[dev] && cusolverDnCreate(&g_solvers[dev]) != CUSOLVER_STATUS_SUCCESS) g_solvers[dev] = nullptr;
  return g_solvers[dev];
}

cublasHandle_t blas_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_solver_mutex);
  if (!g_blas[dev] && cublasCreate(&g_blas[dev]) != CUBLAS_STATUS_SUCCESS) g_blas[dev] = nullptr;
  return g_blas[dev];
}

// Rows of the first diagonal block: about half, rounded up to a multiple of 32.
int64_t split(int64_t n) { return (n / 2 + 31) / 32 * 32; }

// A row-major lower-triangular L is, read column-major, the upper-triangular L^T; trtri of
// that gives (L^-1)^T column-major, which is L^-1 row-major in the same buffer.
bool leaf_sizes(cusolverDnHandle_t h, void* a, int64_t n, int64_t ld, bool complex_mode, size_t* device,
                size_t* host) {
  return cusolverDnXtrtri_bufferSize(h, CUBLAS_FILL_MODE_UPPER, CUBLAS_DIAG_NON_UNIT, n,
                                     complex_mode ? CUDA_C_64F : CUDA_R_64F, a, ld, device, host) ==
         CUSOLVER_STATUS_SUCCESS;
}

size_t scratch_bytes(int64_t n, bool complex_mode) {
  if (n <= kLeaf) return 0;
  const int64_t k = split(n);
  return (size_t)k * (size_t)(n - k) * (complex_mode ? 16 : 8);
}

// The first nonzero status of the diagonal blocks, as the row of the whole factor.
__global__ void merge_info(int32_t* total, const int32_t* block, int64_t first_row) {
  if (*total == 0 && *block > 0) *total = (int32_t)(*block + first_row);
}

struct Inverter {
  cusolverDnHandle_t solver;
  cublasHandle_t blas;
  bool complex_mode;
  size_t element;
  uint8_t* leaf_workspace;
  size_t leaf_bytes;
  void* scratch;  // k x (n - k) of the top level, the largest product
  int32_t* info;        // of the whole factor
  int32_t* block_info;  // of one diagonal block
  cudaStream_t stream;
  std::vector<uint8_t>* host_buffer;

  // In place on the block at a (row-major, leading dimension ld) of n rows, whose first
  // row is row first of the whole factor.
  bool invert(uint8_t* a, int64_t n, int64_t ld, int64_t first) const {
    if (n <= kLeaf) {
      size_t device = 0, host = 0;
      if (!leaf_sizes(solver, a, n, ld, complex_mode, &device, &host) || device > leaf_bytes) return false;
      if (host_buffer->size() < host) host_buffer->resize(host);
      if (cusolverDnXtrtri(solver, CUBLAS_FILL_MODE_UPPER, CUBLAS_DIAG_NON_UNIT, n,
                           complex_mode ? CUDA_C_64F : CUDA_R_64F, a, ld, leaf_workspace, device,
                           host ? host_buffer->data() : nullptr, host, block_info) != CUSOLVER_STATUS_SUCCESS)
        return false;
      merge_info<<<1, 1, 0, stream>>>(info, block_info, first);
      dsg_count_launches(2);
      return cudaGetLastError() == cudaSuccess;
    }
    const int64_t k = split(n), m = n - k;
    uint8_t* lower = a + (size_t)k * ld * element;   // B: rows k.., columns ..k
    uint8_t* corner = lower + (size_t)k * element;   // C
    if (!invert(a, k, ld, first) || !invert(corner, m, ld, first + k)) return false;
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

size_t align256(size_t bytes) { return (bytes + 255) / 256 * 256; }

}  // namespace

extern "C" {

size_t dsg_triangular_inverse_workspace_bytes(int32_t n, int32_t is_complex) {
  if (n <= 0) return 0;
  cusolverDnHandle_t h = solver_for_current_device();
  size_t device = 0, host = 0;
  const int64_t leaf = n < kLeaf ? n : kLeaf;
  if (!h || !leaf_sizes(h, nullptr, leaf, n, is_complex != 0, &device, &host)) device = (size_t)1 << 20;
  return align256(device) + align256(scratch_bytes(n, is_complex != 0)) + 256;
}

int dsg_triangular_inverse(void* factor, int32_t n, int32_t is_complex, void* workspace, size_t workspace_bytes,
                           int32_t* info, void* stream) {
  if (n < 0) return DSG_ERR_ARGUMENT;
  if (n == 0) return DSG_OK;
  if (!factor || !info) return DSG_ERR_ARGUMENT;
  cusolverDnHandle_t h = solver_for_current_device();
  cublasHandle_t b = blas_for_current_device();
  if (!h || !b) return DSG_ERR_LIBRARY;
  const bool complex_mode = is_complex != 0;
  size_t device = 0, host = 0;
  const int64_t leaf = n < kLeaf ? n : kLeaf;
  if (!leaf_sizes(h, factor, leaf, n, complex_mode, &device, &host)) return DSG_ERR_LIBRARY;
  const size_t scratch = scratch_bytes(n, complex_mode);
  const size_t needed = align256(device) + align256(scratch) + sizeof(int32_t);
  if (!workspace || workspace_bytes < needed) return DSG_ERR_WORKSPACE;
  uint8_t* base = static_cast<uint8_t*>(workspace);
  thread_local std::vector<uint8_t> host_buffer;
  if (cusolverDnSetStream(h, (cudaStream_t)stream) != CUSOLVER_STATUS_SUCCESS ||
      cublasSetStream(b, (cudaStream_t)stream) != CUBLAS_STATUS_SUCCESS)
    return DSG_ERR_LIBRARY;
  int32_t* block_info = reinterpret_cast<int32_t*>(base + align256(device) + align256(scratch));
  if (cudaMemsetAsync(info, 0, sizeof(int32_t), (cudaStream_t)stream) != cudaSuccess) return DSG_ERR_LAUNCH;
  const Inverter inverter{h, b, complex_mode, (size_t)(complex_mode ? 16 : 8), base, align256(device),
                          scratch ? base + align256(device) : nullptr, info, block_info, (cudaStream_t)stream,
                          &host_buffer};
  return inverter.invert(static_cast<uint8_t*>(factor), n, n, 0) ? DSG_OK : DSG_ERR_LIBRARY;
}

}  // extern "C"
