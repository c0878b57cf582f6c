// common.cuh -- shared device helpers of the K-SVD engine (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define KSVD_FULL_MASK 0xffffffffu

namespace ksvd {

// Device error word bits (written with atomicOr, read by the host after a stage).
enum DeviceError : int {
  kDevErrNumeric = 1,   // NaN / Inf met
  kDevErrTimeout = 2,   // a bounded grid-barrier wait gave up
  kDevErrBounds = 4,    // an index failed its range check and the access was skipped
};

// Hardware limits of the kernels.
constexpr int kMaxK = 1024;      // atoms (the OMP kernel keeps K/32 coefficients per lane)
constexpr int kMaxT = 64;        // atoms per signal
constexpr int kMaxN = 1024;      // signal length for the block-per-signal kernels
constexpr int kKPad = 128;       // atom dimension padding of the internal buffers

__host__ __device__ inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(KSVD_FULL_MASK, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(KSVD_FULL_MASK, v, o);
  return v;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(KSVD_FULL_MASK, v, o));
  return v;
}

// (value, index) argmax with the lowest index winning ties; every lane gets the result.
__device__ __forceinline__ void warp_argmax(float& v, int& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float ov = __shfl_xor_sync(KSVD_FULL_MASK, v, o);
    int oi = __shfl_xor_sync(KSVD_FULL_MASK, i, o);
    if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
  }
}

// Block-wide argmax (lowest index on ties).  scratch holds >= 2*32 words.  All threads get it.
__device__ __forceinline__ void block_argmax(float& v, int& i, float* sv, int* si) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  warp_argmax(v, i);
  __syncthreads();
  if (lane == 0) { sv[wid] = v; si[wid] = i; }
  __syncthreads();
  v = lane < nw ? sv[lane] : -1.0f;
  i = lane < nw ? si[lane] : 0x7fffffff;
  warp_argmax(v, i);
}

__device__ __forceinline__ float block_sum(float v, float* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  v = lane < nw ? scratch[lane] : 0.0f;
  return warp_sum(v);
}

__device__ __forceinline__ bool finitef(float x) { return isfinite(x); }

}  // namespace ksvd
