// pca.cu -- PCA preprocessing of the rows (scripts/data_prep/apply_pca.py:25-33):
// project onto the top `dims` principal components, L2-normalise every
// projected row, round to float16.
//
// The script fits sklearn's PCA on the float32 rows and normalises with
// sklearn.preprocessing.normalize before writing float16.  Here, on the GPU:
//   mean      mu = X^T 1 / n                         (cuBLAS gemv)
//   centre    X - 1 mu^T                              (kernel)
//   covariance C = Xc^T Xc / (n - 1)                 (cuBLAS syrk, fp32)
//   eigen     C = V diag(w) V^T, w ascending          (cuSOLVER syevd)
//   components the `dims` eigenvectors of the largest w, largest first; each
//             component's sign makes its largest-magnitude entry positive
//             (sklearn's svd_flip on the components)
//   project   Y = Xc V_k                               (cuBLAS gemm)
//   normalise y / ||y|| per row (zero rows stay zero), round to nearest f16.
// variance_kept = sum of the top `dims` w / sum of all w, sklearn's
// explained_variance_ratio_.sum().  The eigen-decomposition of the
// covariance finds the same subspace as sklearn's SVD of the centred rows;
// values agree to float32 precision, not bit for bit.
#include "knng_internal.cuh"

#include <cublas_v2.h>
#include <cuda_fp16.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace knng {
namespace {

__global__ void center_kernel(float* __restrict__ x, int64_t n, int d, const float* __restrict__ mu) {
  const int64_t tot = n * d;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < tot; q += int64_t(gridDim.x) * blockDim.x)
    x[q] -= mu[q % d];
}

// Components: column d-1-c of the eigenvector matrix (column-major, d x d)
// becomes column c of v (d x dims), sign-flipped so that its largest-magnitude
// entry is positive (first such entry on ties).  One block per component.
__global__ void components_kernel(const float* __restrict__ evec, int d, int dims, float* __restrict__ v) {
  const int c = blockIdx.x;
  if (c >= dims) return;
  const float* src = evec + int64_t(d - 1 - c) * d;
  __shared__ float best[256];
  __shared__ int besti[256];
  float b = -1.0f;
  int bi = d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    const float a = fabsf(src[j]);
    if (a > b || (a == b && j < bi)) {
      b = a;
      bi = j;
    }
  }
  best[threadIdx.x] = b;
  besti[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const float o = best[threadIdx.x + s];
      const int oi = besti[threadIdx.x + s];
      if (o > best[threadIdx.x] || (o == best[threadIdx.x] && oi < besti[threadIdx.x])) {
        best[threadIdx.x] = o;
        besti[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const float sign = src[besti[0]] < 0.0f ? -1.0f : 1.0f;
  for (int j = threadIdx.x; j < d; j += blockDim.x) v[int64_t(c) * d + j] = sign * src[j];
}

// One warp per projected row: divide by the row's L2 norm, round to f16.
__global__ void normalize_f16_kernel(const float* __restrict__ y, int64_t n, int dims, __half* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x / 32);
  for (int64_t r = int64_t(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5); r < n; r += warps) {
    const float* row = y + r * dims;
    float s = 0.0f;
    for (int j = lane; j < dims; j += 32) s += row[j] * row[j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float nrm = sqrtf(s);
    const float inv = nrm > 0.0f ? 1.0f / nrm : 0.0f;
    for (int j = lane; j < dims; j += 32) out[r * dims + j] = __float2half_rn(row[j] * inv);
  }
}

struct Handles {
  cublasHandle_t blas = nullptr;
  cusolverDnHandle_t solver = nullptr;
  ~Handles() {
    if (blas) cublasDestroy(blas);
    if (solver) cusolverDnDestroy(solver);
  }
};

}  // namespace
}  // namespace knng

extern "C" int knng_pca(const float* rows, int64_t n, int d, int dims, int device, uint16_t* out_f16,
                        double* variance_kept) {
  using namespace knng;
  if (!rows || !out_f16 || n < 2 || d < 1 || dims < 1 || dims > d) return KNNG_E_ARGS;
  int sms = 0;
  if (cudaSetDevice(device) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device))
    return KNNG_E_CUDA;
  const size_t nd = size_t(n) * d, nk = size_t(n) * dims;
  float *x = nullptr, *mu = nullptr, *ones = nullptr, *cov = nullptr, *w = nullptr, *v = nullptr, *y = nullptr,
        *work = nullptr;
  __half* h = nullptr;
  int* info = nullptr;
  int rc = KNNG_OK;
  Handles hd;
  auto cleanup = [&]() {
    cudaFree(x);
    cudaFree(mu);
    cudaFree(ones);
    cudaFree(cov);
    cudaFree(w);
    cudaFree(v);
    cudaFree(y);
    cudaFree(work);
    cudaFree(h);
    cudaFree(info);
  };
  do {
    if (cudaMalloc(&x, nd * 4) || cudaMalloc(&mu, size_t(d) * 4) || cudaMalloc(&ones, size_t(n) * 4) ||
        cudaMalloc(&cov, size_t(d) * d * 4) || cudaMalloc(&w, size_t(d) * 4) ||
        cudaMalloc(&v, size_t(d) * dims * 4) || cudaMalloc(&info, sizeof(int))) {
      rc = KNNG_E_OOM;
      break;
    }
    if (cudaMemcpy(x, rows, nd * 4, cudaMemcpyDefault)) {
      rc = KNNG_E_CUDA;
      break;
    }
    {
      std::vector<float> one;
      try {  // no exception leaves the library
        one.assign(static_cast<size_t>(n), 1.0f);
      } catch (...) {
        rc = KNNG_E_OOM;
        break;
      }
      if (cudaMemcpy(ones, one.data(), size_t(n) * 4, cudaMemcpyHostToDevice)) {
        rc = KNNG_E_CUDA;
        break;
      }
    }
    if (cublasCreate(&hd.blas) != CUBLAS_STATUS_SUCCESS || cusolverDnCreate(&hd.solver) != CUSOLVER_STATUS_SUCCESS) {
      rc = KNNG_E_CUDA;
      break;
    }
    // The row-major n x d rows are the column-major d x n matrix A (lda = d).
    const float inv_n = 1.0f / float(n), zero = 0.0f, one1 = 1.0f, inv_n1 = 1.0f / float(n - 1);
    if (cublasSgemv(hd.blas, CUBLAS_OP_N, d, int(n), &inv_n, x, d, ones, 1, &zero, mu, 1) != CUBLAS_STATUS_SUCCESS) {
      rc = KNNG_E_CUDA;
      break;
    }
    center_kernel<<<unsigned(std::min<size_t>((nd + 255) / 256, size_t(sms) * 64)), 256>>>(x, n, d, mu);
    if (cublasSsyrk(hd.blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, d, int(n), &inv_n1, x, d, &zero, cov, d) !=
        CUBLAS_STATUS_SUCCESS) {
      rc = KNNG_E_CUDA;
      break;
    }
    int lwork = 0;
    if (cusolverDnSsyevd_bufferSize(hd.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, d, cov, d, w,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS ||
        cudaMalloc(&work, size_t(std::max(lwork, 1)) * 4)) {
      rc = KNNG_E_CUDA;
      break;
    }
    if (cusolverDnSsyevd(hd.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, d, cov, d, w, work, lwork,
                         info) != CUSOLVER_STATUS_SUCCESS) {
      rc = KNNG_E_CUDA;
      break;
    }
    int hinfo = 0;
    std::vector<float> hw;
    try {
      hw.resize(static_cast<size_t>(d));
    } catch (...) {
      rc = KNNG_E_OOM;
      break;
    }
    if (cudaMemcpy(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost) ||
        cudaMemcpy(hw.data(), w, size_t(d) * 4, cudaMemcpyDeviceToHost) || hinfo != 0) {
      rc = KNNG_E_CUDA;
      break;
    }
    double total = 0.0, kept = 0.0;
    for (int j = 0; j < d; ++j) total += double(std::max(hw[size_t(j)], 0.0f));
    for (int j = d - dims; j < d; ++j) kept += double(std::max(hw[size_t(j)], 0.0f));
    if (variance_kept) *variance_kept = total > 0.0 ? kept / total : 0.0;
    components_kernel<<<unsigned(dims), 256>>>(cov, d, dims, v);
    cudaFree(ones);  // no longer needed
    ones = nullptr;
    if (cudaMalloc(&y, nk * 4) || cudaMalloc(&h, nk * 2)) {
      rc = KNNG_E_OOM;
      break;
    }
    // Y^T (dims x n, column-major) = V^T (dims x d) * A (d x n)
    if (cublasSgemm(hd.blas, CUBLAS_OP_T, CUBLAS_OP_N, dims, int(n), d, &one1, v, d, x, d, &zero, y, dims) !=
        CUBLAS_STATUS_SUCCESS) {
      rc = KNNG_E_CUDA;
      break;
    }
    normalize_f16_kernel<<<unsigned(std::min<int64_t>((n + 7) / 8, int64_t(sms) * 32)), 256>>>(y, n, dims, h);
    if (cudaMemcpy(out_f16, h, nk * 2, cudaMemcpyDefault) || cudaGetLastError()) {
      rc = KNNG_E_CUDA;
      break;
    }
  } while (false);
  cleanup();
  return rc;
}
