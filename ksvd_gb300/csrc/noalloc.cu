// noalloc.cu -- ksvd_rmse_noalloc: the reconstruction RMSE of a sparse code computed without any
// device allocation.
//
// Some callers cannot allocate device memory at the point where they need this number: a caller
// whose device memory is owned by another allocator (a framework's caching allocator, or a
// fixed memory budget handed to a plugin), or a caller on a latency-critical path where the
// implicit device synchronisation of cudaMalloc/cudaFree is not acceptable.  ksvd_error needs a
// handle, and a handle holds device workspace; this entry point needs neither.  The caller passes
// the inputs (D, X, the sparse code) and receives the RMSE on the host; the only scratch -- one
// FP64 partial sum per 256-signal block plus the result and a bad-index flag -- lives in the
// file-scope array below, which every GPU that loads this library holds until the process exits.
//
// Set-up: host code may not use the array's name as a device address, so every call that is not
// made under stream capture looks the address up with cudaGetSymbolAddress while the call's
// device is current (after a cudaDeviceReset the library's device code is loaded again and the
// array may move); a call under capture reuses the last address looked up on that device.  The
// first call on a device also makes the CUDA driver load this library's device code if nothing
// has yet, which makes the array resident; that first call should therefore come before any
// stream capture.  Calls share the array: two calls whose kernels overlap on the same GPU
// (different streams or threads) race on it.  Every slot a call reads is written earlier in the
// same call, so nothing has to be cleared between calls.
#include <mutex>
#include <string>

#include "../../include/ksvd_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace {

constexpr int kNoallocBlock = 256;       // signals per block (8 warps, one signal per warp)
constexpr int kNoallocBlocks = 65536;    // -> N <= 16,777,216

// [0, kNoallocBlocks): per-block partial sums (negative: the block met an atom index outside
// [0, K) in a used slot); [kNoallocBlocks]: the RMSE; [kNoallocBlocks + 1]: 1 if any block did
__device__ __align__(256) double g_rmse_scratch[kNoallocBlocks + 2];

// The RMSE half of the error kernel (clear.cu) with its per-block sums written to `part`:
// warp per signal reconstructs x - D gamma from the sparse code; no masked errors, no buckets.
template <int NPL>
__global__ void __launch_bounds__(256)
rmse_noalloc_partial_kernel(const float* __restrict__ X, const float* __restrict__ D, int n, int K,
                            int T, int64_t N, const int32_t* __restrict__ idx,
                            const float* __restrict__ coef, const int32_t* __restrict__ nnz,
                            double* __restrict__ part) {
  __shared__ double wsum[8];
  __shared__ int wbad[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t b = blockIdx.x;
  const int64_t s0 = b * kNoallocBlock, s1 = min(N, s0 + kNoallocBlock);
  double sum = 0.0;
  bool bad = false;
  for (int64_t s = s0 + w; s < s1; s += 8) {
    float acc[NPL];
    const float* x = X + s * n;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
      const int r = lane + 32 * i;
      acc[i] = r < n ? __ldcs(x + r) : 0.f;
    }
    const int nz = min(nnz[s], T);
    for (int t = 0; t < nz; ++t) {
      const int k = idx[s * T + t];
      if (k < 0 || k >= K) { bad = true; continue; }
      const float g = coef[s * T + t];
      const float* d = D + (int64_t)k * n;
#pragma unroll
      for (int i = 0; i < NPL; ++i) {
        const int r = lane + 32 * i;
        if (r < n) acc[i] = fmaf(-g, __ldg(d + r), acc[i]);
      }
    }
    float e = 0.f;
#pragma unroll
    for (int i = 0; i < NPL; ++i) e = fmaf(acc[i], acc[i], e);
    sum += (double)ksvd::warp_sum(e);
  }
  const bool wb = __any_sync(KSVD_FULL_MASK, bad);
  if (lane == 0) { wsum[w] = sum; wbad[w] = wb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    int nb = 0;
    for (int ww = 0; ww < 8; ++ww) { t += wsum[ww]; nb |= wbad[ww]; }
    part[b] = nb ? -1.0 : t;
  }
}

__global__ void rmse_noalloc_final_kernel(const double* __restrict__ part, int64_t nb,
                                          double denom, double* __restrict__ out) {
  __shared__ double red[32];
  double t = 0.0;
  bool bad = false;
  for (int64_t i = threadIdx.x; i < nb; i += blockDim.x) {
    const double v = part[i];
    bad |= v < 0.0;
    t += v;
  }
  bad = __syncthreads_or(bad);
  t = ksvd::warp_sum_d(t);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = t;
  __syncthreads();
  if (w == 0) {
    t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    t = ksvd::warp_sum_d(t);
    if (lane == 0) {
      out[0] = bad ? 0.0 : sqrt(t / denom);
      out[1] = bad ? 1.0 : 0.0;
    }
  }
}

cudaError_t launch_rmse_noalloc(const float* X, const float* D, int n, int K, int T, int64_t N,
                                const int32_t* idx, const float* coef, const int32_t* nnz,
                                double* part, int64_t nb, double* out, cudaStream_t st) {
  const int npl = (n + 31) / 32;
  const unsigned grid = (unsigned)nb;
  if (npl <= 2) rmse_noalloc_partial_kernel<2><<<grid, 256, 0, st>>>(X, D, n, K, T, N, idx, coef, nnz, part);
  else if (npl <= 4) rmse_noalloc_partial_kernel<4><<<grid, 256, 0, st>>>(X, D, n, K, T, N, idx, coef, nnz, part);
  else if (npl <= 8) rmse_noalloc_partial_kernel<8><<<grid, 256, 0, st>>>(X, D, n, K, T, N, idx, coef, nnz, part);
  else if (npl <= 16) rmse_noalloc_partial_kernel<16><<<grid, 256, 0, st>>>(X, D, n, K, T, N, idx, coef, nnz, part);
  else rmse_noalloc_partial_kernel<32><<<grid, 256, 0, st>>>(X, D, n, K, T, N, idx, coef, nnz, part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  rmse_noalloc_final_kernel<<<1, 1024, 0, st>>>(part, nb, (double)n * (double)N, out);
  return cudaGetLastError();
}

std::mutex g_mu;
double* g_scratch_ptr[128] = {nullptr};

ksvd_status fail(ksvd_status s, const char* msg) {
  ksvd::set_nohandle_error(msg);
  return s;
}

}  // namespace

extern "C" ksvd_status ksvd_rmse_noalloc(int32_t n, int32_t K, int32_t T, const float* D,
                                         const float* X, int64_t N, const int32_t* idx,
                                         const float* coef, const int32_t* nnz, double* rmse,
                                         void* stream) {
  using namespace ksvd;
  if (!D || !X || !idx || !coef || !nnz || !rmse)
    return fail(KSVD_ERR_INVALID_ARGUMENT, "ksvd_rmse_noalloc: null pointer");
  if (n < 1 || K < 1 || T < 1 || N < 1)
    return fail(KSVD_ERR_INVALID_ARGUMENT, "ksvd_rmse_noalloc: n, K, T and N must be >= 1");
  if (n > kMaxN || T > kMaxT || K > kMaxK)
    return fail(KSVD_ERR_UNSUPPORTED, "ksvd_rmse_noalloc: n <= 1024, K <= 1024, T <= 64");
  const int64_t nb = (N + kNoallocBlock - 1) / kNoallocBlock;
  if (nb > kNoallocBlocks)
    return fail(KSVD_ERR_UNSUPPORTED,
                "ksvd_rmse_noalloc: N exceeds the static scratch (at most 16,777,216 signals)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) {
    cudaGetLastError();
    return fail(KSVD_ERR_CUDA, "ksvd_rmse_noalloc: no current CUDA device");
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // look the address up again unless the stream is being captured (a reset device reloads the
  // library's device code); under capture the last address looked up on this device is used
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;
  }
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (cap == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_rmse_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return fail(KSVD_ERR_CUDA, "ksvd_rmse_noalloc: cudaGetSymbolAddress failed");
      }
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  double res[2] = {0.0, 0.0};
  e = launch_rmse_noalloc(X, D, n, K, T, N, idx, coef, nnz, scratch, nb,
                          scratch + kNoallocBlocks, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(res, scratch + kNoallocBlocks, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                        st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    const std::string msg = std::string("ksvd_rmse_noalloc: ") + cudaGetErrorString(e);
    cudaGetLastError();
    return fail(KSVD_ERR_CUDA, msg.c_str());
  }
  if (res[1] != 0.0)
    return fail(KSVD_ERR_INVALID_ARGUMENT,
                "ksvd_rmse_noalloc: sparse code holds an atom index outside [0, K)");
  *rmse = res[0];
  ksvd::set_nohandle_error("");
  return KSVD_OK;
}
