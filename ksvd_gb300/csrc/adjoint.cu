// adjoint.cu -- fixed-support coding and its adjoint (the differentiable form of the coding step).
//
// Forward, per signal s with fixed support S (the atoms idx[s*T + 0..nnz-1]):
//   A = D(:, S),  M = A'A = L L',  gamma = M^-1 A'x        (least squares on the support)
// the lower Cholesky factor L is saved, packed row by row (T(T+1)/2 floats per signal).
// Adjoint: given g = dL/dgamma,
//   u = M^-1 g                      (two triangular solves with the saved L)
//   dL/dx = A u
//   dL/dA = r u' - (A u) gamma',     r = x - A gamma
// so dL/dD(:, S_t) += r u_t - (A u) gamma_t  (accumulated with float atomics: the order of the
// additions, and so the last bits of dL/dD, vary from run to run).
// One warp per signal; the signal and the reconstruction live in registers (n/32 per lane), the
// factor in shared memory.  The reference has no differentiable path; this one gives the
// gradients w.r.t. D and X through the coding step (checked against FP64 finite differences).
#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

constexpr int kAdjWarps = 4;

__device__ __forceinline__ int packed(int i, int j) { return i * (i + 1) / 2 + j; }

// Cholesky of the t x t matrix in L (row stride LS, lower triangle used) in place; lanes own
// rows.  Returns false when a pivot is not positive (the support is linearly dependent).
template <int TMAX>
__device__ bool warp_cholesky(float* L, int LS, int t) {
  const int lane = threadIdx.x & 31;
  bool ok = true;
  for (int k = 0; k < t; ++k) {
    __syncwarp();
    const float piv = L[k * LS + k];
    if (!(piv > 0.f)) ok = false;
    const float d = sqrtf(fmaxf(piv, 1e-30f));
    __syncwarp();
    for (int i = lane; i < t; i += 32) {
      if (i == k) L[k * LS + k] = d;
      else if (i > k) L[i * LS + k] /= d;
    }
    __syncwarp();
    for (int i = lane; i < t; i += 32) {
      if (i > k) {
        const float lik = L[i * LS + k];
        for (int j = k + 1; j <= i; ++j) L[i * LS + j] = fmaf(-lik, L[j * LS + k], L[i * LS + j]);
      }
    }
  }
  __syncwarp();
  return ok;
}

// Solve L L' v = rhs in smem vector v (length t), lane 0 (t <= 64: cheap next to the gathers).
__device__ void chol_solve(const float* L, int LS, int t, float* v) {
  if ((threadIdx.x & 31) == 0) {
    for (int i = 0; i < t; ++i) {
      float a = v[i];
      for (int j = 0; j < i; ++j) a = fmaf(-L[i * LS + j], v[j], a);
      v[i] = a / L[i * LS + i];
    }
    for (int i = t - 1; i >= 0; --i) {
      float a = v[i];
      for (int j = i + 1; j < t; ++j) a = fmaf(-L[j * LS + i], v[j], a);
      v[i] = a / L[i * LS + i];
    }
  }
  __syncwarp();
}

template <int NPL, int TMAX>
__global__ void __launch_bounds__(kAdjWarps * 32)
code_fixed_kernel(const float* __restrict__ D, int n, int K, const float* __restrict__ G, int ldg,
                  const float* __restrict__ X, int64_t N, int T, const int32_t* __restrict__ idx,
                  const int32_t* __restrict__ nnz, float* __restrict__ coef,
                  float* __restrict__ chol, int* __restrict__ dev_err) {
  constexpr int LS = TMAX + 1;
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* L = smem + (size_t)w * (TMAX * LS + 2 * TMAX);
  float* v = L + TMAX * LS;
  int* at = reinterpret_cast<int*>(v + TMAX);
  bool bad = false;
  for (int64_t s = (int64_t)blockIdx.x * kAdjWarps + w; s < N; s += (int64_t)gridDim.x * kAdjWarps) {
    const int t = max(0, min(nnz[s], T));
    for (int j = lane; j < t; j += 32) {
      const int a = idx[s * T + j];
      at[j] = (a >= 0 && a < K) ? a : -1;
    }
    __syncwarp();
    bool okidx = true;
    for (int j = 0; j < t; ++j) okidx &= at[j] >= 0;
    float xr[NPL];
    const float* x = X + s * n;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
      const int r = lane + 32 * i;
      xr[i] = r < n ? x[r] : 0.f;
    }
    // M = G(S, S) (lower triangle) and b = A'x
    for (int e = lane; e < t * t; e += 32) {
      const int i = e / t, j = e - i * t;
      if (j <= i && okidx) L[i * LS + j] = G[(int64_t)at[j] * ldg + at[i]];
    }
    #pragma unroll 4
    for (int j = 0; j < t; ++j) {
      float acc = 0.f;
      if (okidx) {
        const float* d = D + (int64_t)at[j] * n;
#pragma unroll
        for (int i = 0; i < NPL; ++i) {
          const int r = lane + 32 * i;
          if (r < n) acc = fmaf(__ldg(d + r), xr[i], acc);
        }
      }
      acc = warp_sum(acc);
      if (lane == 0) v[j] = acc;
    }
    __syncwarp();
    const bool ok = okidx && warp_cholesky<TMAX>(L, LS, t);
    if (ok) chol_solve(L, LS, t, v);
    if (!ok) bad = true;
    const int TP = T * (T + 1) / 2;
    for (int j = lane; j < T; j += 32) coef[s * T + j] = (ok && j < t) ? v[j] : 0.f;
    if (chol)
      for (int e = lane; e < TP; e += 32) {
        int i = 0;
        while (packed(i + 1, 0) <= e) ++i;
        const int j = e - packed(i, 0);
        chol[s * TP + e] = (ok && i < t) ? L[i * LS + j] : 0.f;
      }
    __syncwarp();
  }
  if (__any_sync(KSVD_FULL_MASK, bad) && lane == 0) atomicOr(dev_err, kDevErrNumeric);
}

template <int NPL, int TMAX>
__global__ void __launch_bounds__(kAdjWarps * 32)
code_backward_kernel(const float* __restrict__ D, int n, int K, const float* __restrict__ X,
                     int64_t N, int T, const int32_t* __restrict__ idx,
                     const int32_t* __restrict__ nnz, const float* __restrict__ coef,
                     const float* __restrict__ chol, const float* __restrict__ dcoef,
                     float* __restrict__ dD, float* __restrict__ dX) {
  constexpr int LS = TMAX + 1;
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* L = smem + (size_t)w * (TMAX * LS + 2 * TMAX);
  float* u = L + TMAX * LS;
  int* at = reinterpret_cast<int*>(u + TMAX);
  const int TP = T * (T + 1) / 2;
  for (int64_t s = (int64_t)blockIdx.x * kAdjWarps + w; s < N; s += (int64_t)gridDim.x * kAdjWarps) {
    const int t = max(0, min(nnz[s], T));
    for (int j = lane; j < t; j += 32) {
      const int a = idx[s * T + j];
      at[j] = (a >= 0 && a < K) ? a : -1;
      u[j] = dcoef[s * T + j];
    }
    for (int e = lane; e < TP; e += 32) {
      int i = 0;
      while (packed(i + 1, 0) <= e) ++i;
      const int j = e - packed(i, 0);
      if (i < t) L[i * LS + j] = chol[s * TP + e];
    }
    __syncwarp();
    bool ok = t > 0;
    for (int j = 0; j < t; ++j) ok &= at[j] >= 0 && L[j * LS + j] > 0.f;
    if (ok) chol_solve(L, LS, t, u);                 // u = M^-1 g
    float r[NPL], au[NPL];
    const float* x = X + s * n;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
      const int rr = lane + 32 * i;
      r[i] = rr < n ? x[rr] : 0.f;
      au[i] = 0.f;
    }
    if (ok) {
      #pragma unroll 4
      for (int j = 0; j < t; ++j) {
        const float* d = D + (int64_t)at[j] * n;
        const float gj = coef[s * T + j], uj = u[j];
#pragma unroll
        for (int i = 0; i < NPL; ++i) {
          const int rr = lane + 32 * i;
          if (rr < n) {
            const float dv = __ldg(d + rr);
            r[i] = fmaf(-gj, dv, r[i]);
            au[i] = fmaf(uj, dv, au[i]);
          }
        }
      }
    }
    float* dx = dX ? dX + s * n : nullptr;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
      const int rr = lane + 32 * i;
      if (dx && rr < n) dx[rr] = ok ? au[i] : 0.f;
    }
    if (ok && dD) {
      #pragma unroll 4
      for (int j = 0; j < t; ++j) {
        float* dd = dD + (int64_t)at[j] * n;
        const float gj = coef[s * T + j], uj = u[j];
#pragma unroll
        for (int i = 0; i < NPL; ++i) {
          const int rr = lane + 32 * i;
          if (rr < n) atomicAdd(dd + rr, fmaf(r[i], uj, -au[i] * gj));
        }
      }
    }
    __syncwarp();
  }
}

// One step of mixed-precision iterative refinement of the least-squares coefficients on a fixed
// support: r = x - A gamma and b = A'r accumulated in FP64, delta = (L L')^-1 b with the FP32 Cholesky
// factor of G(S,S), gamma += delta in FP64.  One step takes the error from ~cond*eps32 to
// ~(cond*eps32)^2 (plus FP64 rounding).  coef is updated in place (rounded to FP32); coef64, when
// given, receives the FP64 values.
template <int NPL, int TMAX>
__global__ void __launch_bounds__(kAdjWarps * 32)
refine_kernel(const float* __restrict__ D, int n, int K, const float* __restrict__ G, int ldg,
              const float* __restrict__ X, int64_t N, int T, const int32_t* __restrict__ idx,
              const int32_t* __restrict__ nnz, float* __restrict__ coef,
              double* __restrict__ coef64, int* __restrict__ dev_err) {
  constexpr int LS = TMAX + 1;
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* L = smem + (size_t)w * (TMAX * LS + 2 * TMAX);
  float* v = L + TMAX * LS;
  int* at = reinterpret_cast<int*>(v + TMAX);
  bool bad = false;
  for (int64_t s = (int64_t)blockIdx.x * kAdjWarps + w; s < N; s += (int64_t)gridDim.x * kAdjWarps) {
    const int t = max(0, min(nnz[s], T));
    for (int j = lane; j < t; j += 32) {
      const int a = idx[s * T + j];
      at[j] = (a >= 0 && a < K) ? a : -1;
    }
    __syncwarp();
    bool okidx = true;
    for (int j = 0; j < t; ++j) okidx &= at[j] >= 0;
    double r[NPL];
    const float* x = X + s * n;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
      const int rr = lane + 32 * i;
      r[i] = rr < n ? (double)x[rr] : 0.0;
    }
    if (okidx)
      #pragma unroll 4
      for (int j = 0; j < t; ++j) {
        const float* d = D + (int64_t)at[j] * n;
        const double gj = (double)coef[s * T + j];
#pragma unroll
        for (int i = 0; i < NPL; ++i) {
          const int rr = lane + 32 * i;
          if (rr < n) r[i] = fma(-gj, (double)__ldg(d + rr), r[i]);
        }
      }
    for (int e = lane; e < t * t; e += 32) {
      const int i = e / t, j = e - i * t;
      if (j <= i && okidx) L[i * LS + j] = G[(int64_t)at[j] * ldg + at[i]];
    }
    // b = A'r in FP64 too: r is nearly orthogonal to the support columns, so an FP32 sum would
    // lose the small result to cancellation (error ~2^-24 ||r|| instead of ~2^-24 |b|)
    #pragma unroll 4
    for (int j = 0; j < t; ++j) {
      double acc = 0.0;
      if (okidx) {
        const float* d = D + (int64_t)at[j] * n;
#pragma unroll
        for (int i = 0; i < NPL; ++i) {
          const int rr = lane + 32 * i;
          if (rr < n) acc = fma((double)__ldg(d + rr), r[i], acc);
        }
      }
      acc = warp_sum_d(acc);
      if (lane == 0) v[j] = (float)acc;
    }
    __syncwarp();
    const bool ok = okidx && warp_cholesky<TMAX>(L, LS, t);
    if (ok) chol_solve(L, LS, t, v);
    if (!ok && t > 0) bad = true;
    for (int j = lane; j < t; j += 32) {
      const double g = (double)coef[s * T + j] + (ok ? (double)v[j] : 0.0);
      coef[s * T + j] = (float)g;
      if (coef64) coef64[s * T + j] = g;
    }
    if (coef64)
      for (int j = t + lane; j < T; j += 32) coef64[s * T + j] = 0.0;
    __syncwarp();
  }
  if (__any_sync(KSVD_FULL_MASK, bad) && lane == 0) atomicOr(dev_err, kDevErrNumeric);
}

template <int NPL, int TMAX>
cudaError_t launch_pair(int mode, const float* D, int n, int K, const float* G, int ldg,
                        const float* X, int64_t N, int T, const int32_t* idx,
                        const int32_t* nnz, float* coef_out, const float* coef_in, float* chol,
                        const float* dcoef, float* dD, float* dX, double* coef64, int* dev_err,
                        cudaStream_t st) {
  int64_t blocks = (N + kAdjWarps - 1) / kAdjWarps;
  if (blocks > 152 * 64) blocks = 152 * 64;
  const size_t smem = (size_t)kAdjWarps * (TMAX * (TMAX + 1) + 2 * TMAX) * sizeof(float);
  cudaError_t e;
  if (mode == 2) {
    e = cudaFuncSetAttribute(refine_kernel<NPL, TMAX>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    refine_kernel<NPL, TMAX><<<(unsigned)blocks, kAdjWarps * 32, smem, st>>>(
        D, n, K, G, ldg, X, N, T, idx, nnz, coef_out, coef64, dev_err);
  } else if (mode == 0) {
    e = cudaFuncSetAttribute(code_fixed_kernel<NPL, TMAX>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    code_fixed_kernel<NPL, TMAX><<<(unsigned)blocks, kAdjWarps * 32, smem, st>>>(
        D, n, K, G, ldg, X, N, T, idx, nnz, coef_out, chol, dev_err);
  } else {
    e = cudaFuncSetAttribute(code_backward_kernel<NPL, TMAX>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    code_backward_kernel<NPL, TMAX><<<(unsigned)blocks, kAdjWarps * 32, smem, st>>>(
        D, n, K, X, N, T, idx, nnz, coef_in, chol, dcoef, dD, dX);
  }
  return cudaGetLastError();
}

#define KSVD_ADJ_ARGS mode, D, n, K, G, ldg, X, N, T, idx, nnz, coef_out, coef_in, chol, dcoef, dD, dX, coef64, dev_err, st
template <int NPL>
cudaError_t launch_t(int mode, const float* D, int n, int K, const float* G, int ldg,
                     const float* X, int64_t N, int T, const int32_t* idx, const int32_t* nnz,
                     float* coef_out, const float* coef_in, float* chol, const float* dcoef,
                     float* dD, float* dX, double* coef64, int* dev_err, cudaStream_t st) {
  if (T <= 16) return launch_pair<NPL, 16>(KSVD_ADJ_ARGS);
  if (T <= 32) return launch_pair<NPL, 32>(KSVD_ADJ_ARGS);
  return launch_pair<NPL, 64>(KSVD_ADJ_ARGS);
}

cudaError_t dispatch(int mode, const float* D, int n, int K, const float* G, int ldg,
                     const float* X, int64_t N, int T, const int32_t* idx, const int32_t* nnz,
                     float* coef_out, const float* coef_in, float* chol, const float* dcoef,
                     float* dD, float* dX, double* coef64, int* dev_err, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  if (n < 1 || n > kMaxN || T < 1 || T > kMaxT) return cudaErrorInvalidValue;
  const int npl = (n + 31) / 32;
  if (npl <= 2) return launch_t<2>(KSVD_ADJ_ARGS);
  if (npl <= 4) return launch_t<4>(KSVD_ADJ_ARGS);
  if (npl <= 8) return launch_t<8>(KSVD_ADJ_ARGS);
  if (npl <= 16) return launch_t<16>(KSVD_ADJ_ARGS);
  return launch_t<32>(KSVD_ADJ_ARGS);
#undef KSVD_ADJ_ARGS
}

}  // namespace

cudaError_t launch_code_fixed(const float* D, int n, int K, const float* G, int ldg,
                              const float* X, int64_t N, int T, const int32_t* idx,
                              const int32_t* nnz, float* coef, float* chol, int* dev_err,
                              cudaStream_t st) {
  return dispatch(0, D, n, K, G, ldg, X, N, T, idx, nnz, coef, nullptr, chol, nullptr, nullptr,
                  nullptr, nullptr, dev_err, st);
}

cudaError_t launch_refine(const float* D, int n, int K, const float* G, int ldg, const float* X,
                          int64_t N, int T, const int32_t* idx, const int32_t* nnz, float* coef,
                          double* coef64, int* dev_err, cudaStream_t st) {
  return dispatch(2, D, n, K, G, ldg, X, N, T, idx, nnz, coef, nullptr, nullptr, nullptr, nullptr,
                  nullptr, coef64, dev_err, st);
}

cudaError_t launch_code_backward(const float* D, int n, int K, const float* X, int64_t N, int T,
                                 const int32_t* idx, const int32_t* nnz, const float* coef,
                                 const float* chol, const float* dcoef, float* dD, float* dX,
                                 cudaStream_t st) {
  return dispatch(1, D, n, K, nullptr, 0, X, N, T, idx, nnz, nullptr, coef,
                  const_cast<float*>(chol), dcoef, dD, dX, nullptr, nullptr, st);
}

}  // namespace ksvd
