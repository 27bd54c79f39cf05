// Triangular inverse of a Cholesky factor in float64 (real or complex) through cuSOLVER's
// trtri: the replacement's elimination then works from X = L^-1 (the inverse of the pooled
// system is X^H X) instead of forming the inverse with potri, which on this part costs
// about four times as much.
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <stdint.h>
#include <mutex>
#include <vector>
#include "dsplat_gb300.h"

void dsg_count_launches(int kernels);

namespace {

std::mutex g_solver_mutex;
cusolverDnHandle_t g_solvers[64] = {};

cusolverDnHandle_t solver_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_solver_mutex);
  if (!g_solvers[dev] && cusolverDnCreate(&g_solvers[dev]) != CUSOLVER_STATUS_SUCCESS) g_solvers[dev] = nullptr;
  return g_solvers[dev];
}

// A row-major lower-triangular L is, read column-major, the upper-triangular L^T; trtri of
// that gives (L^-1)^T column-major, which is L^-1 row-major in the same buffer.
bool sizes(cusolverDnHandle_t h, void* a, int64_t n, bool complex_mode, size_t* device, size_t* host) {
  return cusolverDnXtrtri_bufferSize(h, CUBLAS_FILL_MODE_UPPER, CUBLAS_DIAG_NON_UNIT, n,
                                     complex_mode ? CUDA_C_64F : CUDA_R_64F, a, n, device, host) ==
         CUSOLVER_STATUS_SUCCESS;
}

}  // namespace

extern "C" {

size_t dsg_triangular_inverse_workspace_bytes(int32_t n, int32_t is_complex) {
  if (n <= 0) return 0;
  cusolverDnHandle_t h = solver_for_current_device();
  size_t device = 0, host = 0;
  if (!h || !sizes(h, nullptr, n, is_complex != 0, &device, &host)) return (size_t)1 << 20;
  return device + 256;
}

int dsg_triangular_inverse(void* factor, int32_t n, int32_t is_complex, void* workspace, size_t workspace_bytes,
                           int32_t* info, void* stream) {
  if (n < 0) return DSG_ERR_ARGUMENT;
  if (n == 0) return DSG_OK;
  if (!factor || !info) return DSG_ERR_ARGUMENT;
  cusolverDnHandle_t h = solver_for_current_device();
  if (!h) return DSG_ERR_LIBRARY;
  size_t device = 0, host = 0;
  if (!sizes(h, factor, n, is_complex != 0, &device, &host)) return DSG_ERR_LIBRARY;
  if (device > 0 && (!workspace || workspace_bytes < device)) return DSG_ERR_WORKSPACE;
  thread_local std::vector<uint8_t> host_buffer;
  if (host_buffer.size() < host) host_buffer.resize(host);
  if (cusolverDnSetStream(h, (cudaStream_t)stream) != CUSOLVER_STATUS_SUCCESS) return DSG_ERR_LIBRARY;
  const cusolverStatus_t status =
      cusolverDnXtrtri(h, CUBLAS_FILL_MODE_UPPER, CUBLAS_DIAG_NON_UNIT, n, is_complex ? CUDA_C_64F : CUDA_R_64F,
                       factor, n, workspace, device, host ? host_buffer.data() : nullptr, host, info);
  dsg_count_launches(1);
  return status == CUSOLVER_STATUS_SUCCESS ? DSG_OK : DSG_ERR_LIBRARY;
}

}  // extern "C"
