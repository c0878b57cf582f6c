// misc.cu -- small kernels: column normalisation, padded copies, signal norms, dense coefficients.
#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

// D <- D * diag(1/||d_k||): one warp per column.  The reference computes 1/sqrt(sum of squares)
// per column and multiplies (ReductionKernels.cu:179-190 + KSVD.cu:388-395).
__global__ void normcols_kernel(float* __restrict__ D, int n, int K) {
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (k >= K) return;
  float* d = D + (int64_t)k * n;
  float s = 0.f;
  for (int r = lane; r < n; r += 32) s = fmaf(d[r], d[r], s);
  s = warp_sum(s);
  const float c = 1.0f / sqrtf(s);
  for (int r = lane; r < n; r += 32) d[r] *= c;
}

__global__ void copy_pad_cols_kernel(const float* __restrict__ src, int n, int K,
                                     float* __restrict__ dst, int Kp) {
  const int64_t total = (int64_t)n * Kp;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = e / n;
    dst[e] = k < K ? src[e] : 0.f;
  }
}

__global__ void col_norm2_kernel(const float* __restrict__ X, int n, int64_t N,
                                 float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t s = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= N) return;
  const float* x = X + s * n;
  float acc = 0.f;
  for (int r = lane; r < n; r += 32) acc = fmaf(x[r], x[r], acc);
  acc = warp_sum(acc);
  if (lane == 0) out[s] = acc;
}

// gamma is K x N column-major and must be zeroed first.
__global__ void dense_gamma_kernel(const int32_t* __restrict__ idx, const float* __restrict__ coef,
                                   const int32_t* __restrict__ nnz, int64_t N, int T, int K,
                                   float* __restrict__ gamma) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N * T) return;
  const int64_t s = e / T;
  const int t = (int)(e - s * T);
  if (t >= nnz[s]) return;
  const int k = idx[e];
  if (k < 0 || k >= K) return;
  gamma[s * K + k] = coef[e];
}

__global__ void copy_matrix_kernel(const float* __restrict__ src, int64_t ld_src,
                                   float* __restrict__ dst, int64_t ld_dst, int rows,
                                   int64_t cols) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / rows;
    const int r = (int)(e - c * rows);
    dst[c * ld_dst + r] = src[c * ld_src + r];
  }
}

inline unsigned grid_for(int64_t work, int threads) {
  int64_t b = (work + threads - 1) / threads;
  if (b > 65535LL * 16) b = 65535LL * 16;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

cudaError_t launch_normcols(float* D, int n, int K, cudaStream_t st) {
  normcols_kernel<<<(K + 7) / 8, 256, 0, st>>>(D, n, K);
  return cudaGetLastError();
}

cudaError_t launch_copy_pad_cols(const float* src, int n, int K, float* dst, int Kp,
                                 cudaStream_t st) {
  copy_pad_cols_kernel<<<grid_for((int64_t)n * Kp, 256), 256, 0, st>>>(src, n, K, dst, Kp);
  return cudaGetLastError();
}

__global__ void advance_counter_kernel(int* c) { *c += 1; }

// Row means of X (n x N column-major): block b sums rows over its chunk of kRowChunk signals in
// FP64 (thread r owns rows r, r + blockDim, ...); partials land in part[b * n + r].
constexpr int kRowChunk = 2048;
__global__ void row_partial_kernel(const float* __restrict__ X, int n, int64_t N,
                                   double* __restrict__ part) {
  const int64_t s0 = (int64_t)blockIdx.x * kRowChunk;
  const int64_t s1 = min(N, s0 + kRowChunk);
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    double acc = 0.0;
    for (int64_t s = s0; s < s1; ++s) acc += (double)X[s * n + r];
    part[(int64_t)blockIdx.x * n + r] = acc;
  }
}

// mean[r] = (sum of the partials in block order) / N: deterministic, no atomics.
__global__ void row_mean_kernel(const double* __restrict__ part, int64_t nblk, int n, int64_t N,
                                float* __restrict__ mean) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double acc = 0.0;
  for (int64_t b = 0; b < nblk; ++b) acc += part[b * n + r];
  mean[r] = (float)(acc / (double)N);
}

__global__ void sub_row_mean_kernel(float* __restrict__ X, int n, int64_t N,
                                    const float* __restrict__ mean) {
  const int64_t total = (int64_t)n * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    X[e] -= mean[e % n];
}

cudaError_t launch_advance_counter(int* ctr, cudaStream_t st) {
  advance_counter_kernel<<<1, 1, 0, st>>>(ctr);
  return cudaGetLastError();
}

int64_t row_mean_blocks(int64_t N) { return (N + kRowChunk - 1) / kRowChunk; }

cudaError_t launch_remove_row_mean(float* X, int n, int64_t N, double* part, float* mean,
                                   cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  const int64_t nb = row_mean_blocks(N);
  if (nb > 0x7fffffffLL) return cudaErrorInvalidValue;
  row_partial_kernel<<<(unsigned)nb, 256, 0, st>>>(X, n, N, part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  row_mean_kernel<<<(n + 255) / 256, 256, 0, st>>>(part, nb, n, N, mean);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  sub_row_mean_kernel<<<1216, 256, 0, st>>>(X, n, N, mean);
  return cudaGetLastError();
}

cudaError_t launch_col_norm2(const float* X, int n, int64_t N, float* out, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  col_norm2_kernel<<<(unsigned)((N + 7) / 8), 256, 0, st>>>(X, n, N, out);
  return cudaGetLastError();
}

cudaError_t launch_dense_gamma(const int32_t* idx, const float* coef, const int32_t* nnz,
                               int64_t N, int T, int K, float* gamma, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(gamma, 0, sizeof(float) * (size_t)K * N, st);
  if (e != cudaSuccess) return e;
  const int64_t total = N * T;
  dense_gamma_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(idx, coef, nnz, N, T, K,
                                                                        gamma);
  return cudaGetLastError();
}

cudaError_t launch_copy_matrix(const float* src, int64_t ld_src, float* dst, int64_t ld_dst,
                               int rows, int64_t cols, cudaStream_t st) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  copy_matrix_kernel<<<grid_for((int64_t)rows * cols, 256), 256, 0, st>>>(src, ld_src, dst,
                                                                           ld_dst, rows, cols);
  return cudaGetLastError();
}

}  // namespace ksvd
