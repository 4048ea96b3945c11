// pod.cu -- thin SVD of a snapshot matrix (the POD basis) in FP64 on the GPU.
//
// Reference: computeThinSVD, src/tools/main_eigen_svd.cc.  Method 1 (doThinSVDm0,
// :113-151) is Eigen's BDCSVD of the snapshot matrix S (n x t) with thin U; method 2
// (doThinSVDm1, :154-197) is a Householder QR S = Q R, the SVD R = U_R Sigma V^T of the
// t x t triangle and U = Q U_R.  Both give the same singular values and the same
// singular vectors up to the sign of each vector, so both run the QR route here:
//   n >= t : geqrf(S) -> gesvd(R) -> ormqr(Q, [U_R; 0])        U is n x t
//   n <  t : geqrf(S^T) = Q R -> S = R^T Q^T -> gesvd(R^T)      U is n x n
// (method 2 of the reference needs n >= t: its R block does not exist otherwise).
// The factorisations are cuSOLVER's; the layout kernels below are this file's.
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "shaw_internal.h"

namespace {

const char* cusolver_name(cusolverStatus_t s) {
  switch (s) {
    case CUSOLVER_STATUS_SUCCESS: return "success";
    case CUSOLVER_STATUS_NOT_INITIALIZED: return "not initialized";
    case CUSOLVER_STATUS_ALLOC_FAILED: return "allocation failed";
    case CUSOLVER_STATUS_INVALID_VALUE: return "invalid value";
    case CUSOLVER_STATUS_ARCH_MISMATCH: return "arch mismatch";
    case CUSOLVER_STATUS_EXECUTION_FAILED: return "execution failed";
    case CUSOLVER_STATUS_INTERNAL_ERROR: return "internal error";
    default: return "error";
  }
}

// At (cols x rows) = A^T, A rows x cols, both LayoutLeft.  32x32 tiles through shared memory.
__global__ void pod_transpose_kernel(const double* __restrict__ A, uint64_t rows, uint64_t cols,
                                     double* __restrict__ At) {
  __shared__ double tile[32][33];
  const uint64_t r0 = (uint64_t)blockIdx.x * 32, c0 = (uint64_t)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const uint64_t r = r0 + threadIdx.x, c = c0 + k;
    if (r < rows && c < cols) tile[k][threadIdx.x] = A[r + rows * c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const uint64_t c = c0 + threadIdx.x, r = r0 + k;
    if (r < rows && c < cols) At[c + cols * r] = tile[threadIdx.x][k];
  }
}

// R (k x k) = upper triangle of the QR factors (leading dimension ld), or its transpose.
__global__ void pod_extract_r_kernel(const double* __restrict__ qr, uint64_t ld, uint64_t k, int transpose,
                                     double* __restrict__ R) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= k) return;
  if (!transpose)
    R[i + k * j] = (i <= j) ? qr[i + ld * j] : 0.0;
  else
    R[i + k * j] = (j <= i) ? qr[j + ld * i] : 0.0;
}

// B (n x t) = [U_R; 0]
__global__ void pod_embed_kernel(const double* __restrict__ U, uint64_t n, uint64_t t, double* __restrict__ B) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i < n) B[i + n * j] = (i < t) ? U[i + t * j] : 0.0;
}

struct PodWork {
  cusolverDnHandle_t sol = nullptr;
  cudaStream_t s = nullptr;
  double *A = nullptr, *At = nullptr, *tau = nullptr, *R = nullptr, *U = nullptr, *S = nullptr, *work = nullptr,
         *B = nullptr;
  int* info = nullptr;
  ~PodWork() {
    if (s) cudaStreamSynchronize(s);
    double* bufs[] = {A, At, tau, R, U, S, work, B};
    for (double* p : bufs)
      if (p) cudaFree(p);
    if (info) cudaFree(info);
    if (sol) cusolverDnDestroy(sol);
    if (s) cudaStreamDestroy(s);
  }
};

int solver_fail(cusolverStatus_t st, const char* what) {
  return shaw::fail(SHAW_ERR_CUDA, std::string(what) + ": " + cusolver_name(st));
}

#define POD_CUDA(call)                                        \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return shaw::cuda_fail(e_, #call); \
  } while (0)
#define POD_SOLVER(call)                                                \
  do {                                                                  \
    cusolverStatus_t st_ = (call);                                      \
    if (st_ != CUSOLVER_STATUS_SUCCESS) return solver_fail(st_, #call); \
  } while (0)

int check_info(PodWork& w, const char* what) {
  int h_info = 0;
  POD_CUDA(cudaMemcpyAsync(&h_info, w.info, sizeof(int), cudaMemcpyDeviceToHost, w.s));
  POD_CUDA(cudaStreamSynchronize(w.s));
  if (h_info != 0)
    return shaw::fail(SHAW_ERR_CUDA, std::string(what) + " failed (info " + std::to_string(h_info) + ")");
  return SHAW_OK;
}

}  // namespace

extern "C" int shaw_pod(const double* snaps, uint64_t n, uint64_t t, int method, double* lsv, double* sv) {
  if (!snaps || !lsv || !sv) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (method != 1 && method != 2) return shaw::fail(SHAW_ERR_INVALID_ARG, "Invalid method");
  if (t == 0 || n == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "empty snapshot matrix");
  if (method == 2 && n < t)
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "method 2 (QR) needs at least as many rows as snapshots");
  // cuSOLVER's 32-bit interface; the k x k SVD bounds the smaller extent
  if (n > (uint64_t)INT32_MAX || t > (uint64_t)INT32_MAX || std::min(n, t) > 65535 ||
      (n < t && t > 65535ull * 32))
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "snapshot matrix too large");
  const bool tall = n >= t;
  const uint64_t m = tall ? n : t;  // rows of the factored matrix
  const uint64_t k = tall ? t : n;  // its columns = number of singular values
  PodWork w;
  POD_CUDA(cudaStreamCreateWithFlags(&w.s, cudaStreamNonBlocking));
  POD_SOLVER(cusolverDnCreate(&w.sol));
  POD_SOLVER(cusolverDnSetStream(w.sol, w.s));
  POD_CUDA(cudaMalloc(&w.A, n * t * sizeof(double)));
  POD_CUDA(cudaMalloc(&w.tau, k * sizeof(double)));
  POD_CUDA(cudaMalloc(&w.R, k * k * sizeof(double)));
  POD_CUDA(cudaMalloc(&w.U, k * k * sizeof(double)));
  POD_CUDA(cudaMalloc(&w.S, k * sizeof(double)));
  POD_CUDA(cudaMalloc(&w.info, sizeof(int)));
  POD_CUDA(cudaMemcpyAsync(w.A, snaps, n * t * sizeof(double), cudaMemcpyHostToDevice, w.s));
  double* F = w.A;  // the m x k matrix that is factored
  if (!tall) {
    POD_CUDA(cudaMalloc(&w.At, n * t * sizeof(double)));
    pod_transpose_kernel<<<dim3((unsigned)((n + 31) / 32), (unsigned)((t + 31) / 32)), dim3(32, 8), 0, w.s>>>(
        w.A, n, t, w.At);
    POD_CUDA(cudaGetLastError());
    F = w.At;
  }
  int lq = 0, ls = 0, lo = 0;
  POD_SOLVER(cusolverDnDgeqrf_bufferSize(w.sol, (int)m, (int)k, F, (int)m, &lq));
  POD_SOLVER(cusolverDnDgesvd_bufferSize(w.sol, (int)k, (int)k, &ls));
  if (tall)
    POD_SOLVER(cusolverDnDormqr_bufferSize(w.sol, CUBLAS_SIDE_LEFT, CUBLAS_OP_N, (int)n, (int)t, (int)t, F, (int)n,
                                           w.tau, F, (int)n, &lo));
  const int lwork = std::max(lq, std::max(ls, lo));
  POD_CUDA(cudaMalloc(&w.work, (size_t)std::max(lwork, 1) * sizeof(double)));
  // 1. F = Q R
  POD_SOLVER(cusolverDnDgeqrf(w.sol, (int)m, (int)k, F, (int)m, w.tau, w.work, lwork, w.info));
  if (int rc = check_info(w, "cusolverDnDgeqrf")) return rc;
  pod_extract_r_kernel<<<dim3((unsigned)((k + 255) / 256), (unsigned)k), 256, 0, w.s>>>(F, m, k, tall ? 0 : 1, w.R);
  POD_CUDA(cudaGetLastError());
  // 2. R (or R^T) = U_R Sigma V^T
  POD_SOLVER(cusolverDnDgesvd(w.sol, 'A', 'N', (int)k, (int)k, w.R, (int)k, w.S, w.U, (int)k, nullptr, 1, w.work,
                              lwork, nullptr, w.info));
  if (int rc = check_info(w, "cusolverDnDgesvd")) return rc;
  const double* Uout = w.U;
  if (tall) {
    // 3. U = Q [U_R; 0]
    POD_CUDA(cudaMalloc(&w.B, n * t * sizeof(double)));
    pod_embed_kernel<<<dim3((unsigned)((n + 255) / 256), (unsigned)t), 256, 0, w.s>>>(w.U, n, t, w.B);
    POD_CUDA(cudaGetLastError());
    POD_SOLVER(cusolverDnDormqr(w.sol, CUBLAS_SIDE_LEFT, CUBLAS_OP_N, (int)n, (int)t, (int)t, F, (int)n, w.tau, w.B,
                                (int)n, w.work, lwork, w.info));
    if (int rc = check_info(w, "cusolverDnDormqr")) return rc;
    Uout = w.B;
  }
  POD_CUDA(cudaMemcpyAsync(lsv, Uout, n * k * sizeof(double), cudaMemcpyDeviceToHost, w.s));
  POD_CUDA(cudaMemcpyAsync(sv, w.S, k * sizeof(double), cudaMemcpyDeviceToHost, w.s));
  POD_CUDA(cudaStreamSynchronize(w.s));
  return SHAW_OK;
}
