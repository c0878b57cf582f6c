// clear.cu -- reconstruction error / RMSE (KSVD::errorComputation, KSVD.cu:235-262) and
// dictionary clearing (KSVD::clearDict, KSVD.cu:138-226).
//
// The error kernel reconstructs every signal from its sparse code (T atoms, warp per signal)
// instead of the reference's dense D*Gamma GEMM + RMSE_stage1..3 (ReductionKernels.cu:257-322);
// each 256-signal bucket records its error sum (FP64) and its largest masked error, which the
// clearDict kernel uses as a two-level argmax: each replacement takes the bucket maximum, zeroes
// that error and rescans only its bucket (device_max_err_STAGE1/2, ReductionKernels.cu:329-386).
//
// clearDict keeps G = D'D exact: per column the largest off-diagonal G(i,j)^2 and its row are
// precomputed in parallel; when atom j is replaced, G's row and column j are recomputed and
// only the later columns whose maximum involved row j are rescanned.
#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

constexpr int kErrWarps = 8;
constexpr int kBucket = 256;                 // signals per error block / bucket
constexpr int kClearThreads = 1024;

template <int NPL>
__global__ void __launch_bounds__(kErrWarps * 32)
error_kernel(ErrorArgs A) {
  __shared__ double wsum[kErrWarps];
  __shared__ float wval[kErrWarps];
  __shared__ int64_t widx[kErrWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = A.n, T = A.T;
  const int64_t b = blockIdx.x;
  const int64_t s0 = b * kBucket, s1 = min(A.N, s0 + kBucket);
  double sum = 0.0;
  float bv = -1.f;
  int64_t bi = INT64_MAX;
  bool bad = false;
  for (int64_t s = s0 + w; s < s1; s += kErrWarps) {
    float acc[NPL];
    const float* x = A.X + s * n;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
      const int r = lane + 32 * i;
      acc[i] = r < n ? __ldcs(x + r) : 0.f;
    }
    // the whole code row in registers first (lane t holds slots t and t + 32), so the support
    // columns' loads do not wait on one another
    const int nz = min(A.nnz[s], T);
    int kk[2];
    float gg[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int t = lane + 32 * u;
      const int k = t < nz ? A.idx[s * T + t] : -1;
      const bool ok = k >= 0 && k < A.K;
      bad |= t < nz && !ok;
      kk[u] = ok ? k : -1;
      gg[u] = ok ? A.coef[s * T + t] : 0.f;
    }
#pragma unroll 4
    for (int t = 0; t < nz; ++t) {
      const int k = __shfl_sync(KSVD_FULL_MASK, (t >> 5) == 0 ? kk[0] : kk[1], t & 31);
      const float g = __shfl_sync(KSVD_FULL_MASK, (t >> 5) == 0 ? gg[0] : gg[1], t & 31);
      if (k < 0) continue;
      const float* d = A.D + (int64_t)k * n;
#pragma unroll
      for (int i = 0; i < NPL; ++i) {
        const int r = lane + 32 * i;
        if (r < n) acc[i] = fmaf(-g, __ldg(d + r), acc[i]);
      }
    }
    float e = 0.f;
#pragma unroll
    for (int i = 0; i < NPL; ++i) e = fmaf(acc[i], acc[i], e);
    e = warp_sum(e);
    sum += (double)e;
    const float em = A.bitmap ? e * (float)A.bitmap[s] : e;
    if (lane == 0) A.err[s] = em;
    if (em > bv) { bv = em; bi = s; }       // s ascends within the warp: first maximum kept
  }
  if (__any_sync(KSVD_FULL_MASK, bad) && lane == 0 && A.dev_err) atomicOr(A.dev_err, kDevErrBounds);
  if (lane == 0) { wsum[w] = sum; wval[w] = bv; widx[w] = bi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    float v = -1.f;
    int64_t vi = INT64_MAX;
    for (int ww = 0; ww < kErrWarps; ++ww) {
      t += wsum[ww];
      if (wval[ww] > v || (wval[ww] == v && widx[ww] < vi)) { v = wval[ww]; vi = widx[ww]; }
    }
    A.part_sum[b] = t;
    A.bucket_val[b] = v;
    A.bucket_idx[b] = vi;
  }
}

// Half-warp variant for T <= 16, n % 4 == 0, n <= 64 NQ and 16-byte aligned X and D: each half
// of a warp reconstructs one signal (four consecutive rows per 16-byte load, slot lane & 15 of the
// code row per lane), so the per-column shuffles and address arithmetic are issued once for two
// signals.  The halves walk ascending signals and are combined at the end (sum, then the larger
// error with the lower signal on ties), so the results stay deterministic.
template <int NQ, bool FULLN>
__global__ void __launch_bounds__(kErrWarps * 32)
error_half_kernel(ErrorArgs A) {
  __shared__ double wsum[kErrWarps];
  __shared__ float wval[kErrWarps];
  __shared__ int64_t widx[kErrWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int hl = lane & 15, hbase = lane & 16;
  const int n = A.n, T = A.T;
  const int64_t b = blockIdx.x;
  const int64_t s0 = b * kBucket, s1 = min(A.N, s0 + kBucket);
  double sum = 0.0;
  float bv = -1.f;
  int64_t bi = INT64_MAX;
  bool bad = false;
  for (int64_t sp = s0 + 2 * w; sp < s1; sp += 2 * kErrWarps) {
    const int64_t s = sp + (lane >> 4);
    const bool live = s < s1;
    const float4* xp = reinterpret_cast<const float4*>(A.X + (live ? s : sp) * n) + hl;
    float4 acc[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k)
      acc[k] = (live && (FULLN || 4 * hl + 64 * k < n)) ? __ldcs(xp + 16 * k)
                                                        : make_float4(0.f, 0.f, 0.f, 0.f);
    const int nz = live ? min(A.nnz[s], T) : 0;
    const bool in = hl < nz;
    const int kraw = in ? A.idx[s * T + hl] : -1;
    const bool ok = (unsigned)kraw < (unsigned)A.K;
    bad |= in && !ok;
    const int kk = (in && ok) ? kraw : -1;
    const float gg = (in && ok) ? A.coef[s * T + hl] : 0.f;
    const int nzw = max(nz, __shfl_xor_sync(KSVD_FULL_MASK, nz, 16));
#pragma unroll 4
    for (int t = 0; t < nzw; ++t) {
      const int k = __shfl_sync(KSVD_FULL_MASK, kk, hbase | t);
      const float g = __shfl_sync(KSVD_FULL_MASK, gg, hbase | t);
      if (k < 0) continue;
      const float4* dp = reinterpret_cast<const float4*>(A.D + (int64_t)k * n) + hl;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        if (!FULLN && 4 * hl + 64 * q >= n) continue;
        const float4 d = __ldg(dp + 16 * q);
        acc[q].x = fmaf(-g, d.x, acc[q].x);
        acc[q].y = fmaf(-g, d.y, acc[q].y);
        acc[q].z = fmaf(-g, d.z, acc[q].z);
        acc[q].w = fmaf(-g, d.w, acc[q].w);
      }
    }
    float e = 0.f;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      e = fmaf(acc[k].x, acc[k].x, e);
      e = fmaf(acc[k].y, acc[k].y, e);
      e = fmaf(acc[k].z, acc[k].z, e);
      e = fmaf(acc[k].w, acc[k].w, e);
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) e += __shfl_xor_sync(KSVD_FULL_MASK, e, o);
    if (live) {
      sum += (double)e;
      const float em = A.bitmap ? e * (float)A.bitmap[s] : e;
      if (hl == 0) A.err[s] = em;
      if (em > bv) { bv = em; bi = s; }      // s ascends within the half: first maximum kept
    }
  }
  // half 1 into half 0
  sum += __shfl_down_sync(KSVD_FULL_MASK, sum, 16);
  {
    const float ov = __shfl_down_sync(KSVD_FULL_MASK, bv, 16);
    const long long oi = __shfl_down_sync(KSVD_FULL_MASK, (long long)bi, 16);
    if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
  }
  if (__any_sync(KSVD_FULL_MASK, bad) && lane == 0 && A.dev_err) atomicOr(A.dev_err, kDevErrBounds);
  if (lane == 0) { wsum[w] = sum; wval[w] = bv; widx[w] = bi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    float v = -1.f;
    int64_t vi = INT64_MAX;
    for (int ww = 0; ww < kErrWarps; ++ww) {
      t += wsum[ww];
      if (wval[ww] > v || (wval[ww] == v && widx[ww] < vi)) { v = wval[ww]; vi = widx[ww]; }
    }
    A.part_sum[b] = t;
    A.bucket_val[b] = v;
    A.bucket_idx[b] = vi;
  }
}

__global__ void rmse_kernel(const double* __restrict__ part, int64_t nb, double denom,
                            double* __restrict__ out, const int* __restrict__ iter_ctr) {
  __shared__ double red[32];
  double t = 0.0;
  for (int64_t i = threadIdx.x; i < nb; i += blockDim.x) t += part[i];
  t = warp_sum_d(t);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = t;
  __syncthreads();
  if (w == 0) {
    t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    t = warp_sum_d(t);
    if (lane == 0) out[iter_ctr ? *iter_ctr : 0] = sqrt(t / denom);
  }
}

// m[j] = max_{i != j, i < K} G(i,j)^2 and its row (lowest on ties); warp per column.
__global__ void coherence_kernel(const float* __restrict__ G, int K, int Kp, float* __restrict__ m,
                                 int* __restrict__ mi) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= K) return;
  float v = 0.f;
  int vi = 0x7fffffff;
  for (int i = lane; i < K; i += 32) {
    if (i == j) continue;
    const float g = G[(int64_t)j * Kp + i];
    const float g2 = g * g;
    if (g2 > v || (g2 == v && i < vi)) { v = g2; vi = i; }
  }
  warp_argmax(v, vi);
  if (lane == 0) { m[j] = v; mi[j] = vi; }
}

struct ClearSeqArgs {
  ClearArgs c;
  float* m;
  int* mi;
};

__device__ void bucket_rescan(const float* err, int64_t N, int64_t bkt, float* bucket_val,
                              int64_t* bucket_idx, float* rf, int* ri) {
  // threads of the block: one signal each (kBucket <= blockDim)
  const int64_t s = bkt * kBucket + threadIdx.x;
  float v = (threadIdx.x < kBucket && s < N) ? __ldcg(err + s) : -1.f;
  int i = (threadIdx.x < kBucket && s < N) ? (int)threadIdx.x : 0x7fffffff;
  block_argmax(v, i, rf, ri);
  if (threadIdx.x == 0) {
    bucket_val[bkt] = v;
    bucket_idx[bkt] = (i == 0x7fffffff) ? INT64_MAX : bkt * kBucket + i;
  }
}

__global__ void __launch_bounds__(kClearThreads, 1) clear_seq_kernel(ClearSeqArgs P) {
  const ClearArgs& A = P.c;
  __shared__ float rf[64];
  __shared__ int ri[64];
  __shared__ int64_t sbest;
  __shared__ float snorm;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int n = A.n, K = A.K, Kp = A.Kp;
  const float mu2 = A.mu_thresh * A.mu_thresh;
  int cleared = 0;
  int jstart = 0;
  while (true) {
    // first j >= jstart whose test fires
    int cand = 0x7fffffff;
    for (int j = jstart + tid; j < K; j += blockDim.x) {
      const bool fire = (P.m[j] > mu2 || A.usecount[j] < A.use_thresh) && A.replaced[j] == 0;
      if (fire && j < cand) cand = j;
    }
    float dummy = 0.f;
    {
      // block min via argmax machinery (all values equal -> lowest index wins)
      block_argmax(dummy, cand, rf, ri);
    }
    const int j = cand;
    __syncthreads();
    if (j >= K) break;
    // ---- the worst-represented signal: argmax over bucket maxima, lowest signal on ties
    {
      float v = -1.f;
      int bi = 0x7fffffff;
      for (int64_t bk = tid; bk < A.nbuckets; bk += blockDim.x) {
        const float bvv = __ldcg(A.bucket_val + bk);
        if (bvv > v) { v = bvv; bi = (int)bk; }   // buckets ascend per thread: first maximum
      }
      block_argmax(v, bi, rf, ri);
      if (tid == 0) sbest = (bi == 0x7fffffff) ? -1 : __ldcg(A.bucket_idx + bi);
      __syncthreads();
    }
    const int64_t s = sbest;
    if (s < 0 || s >= A.N) break;                  // no signal left to take
    const float* x = A.X + s * n;
    float nr = 0.f;
    for (int r = tid; r < n; r += blockDim.x) nr = fmaf(x[r], x[r], nr);
    nr = block_sum(nr, rf);
    if (tid == 0) snorm = sqrtf(nr);
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) A.D[(int64_t)j * n + r] = x[r] / snorm;
    if (tid == 0) A.err[s] = 0.f;
    __threadfence_block();
    __syncthreads();
    bucket_rescan(A.err, A.N, s / kBucket, A.bucket_val, A.bucket_idx, rf, ri);
    __syncthreads();
    // ---- G row/column j from the new atom (warp per atom i)
    const float* dj = A.D + (int64_t)j * n;
    for (int i = w; i < K; i += blockDim.x >> 5) {
      const float* di = A.D + (int64_t)i * n;
      float acc = 0.f;
      for (int r = lane; r < n; r += 32) acc = fmaf(__ldcg(di + r), __ldcg(dj + r), acc);
      acc = warp_sum(acc);
      if (lane == 0) {
        A.G[(int64_t)j * Kp + i] = acc;
        A.G[(int64_t)i * Kp + j] = acc;
      }
    }
    __syncthreads();
    // ---- later columns: fold in the new G(j, j') (rescan when the old maximum was row j)
    for (int jp = j + 1 + tid; jp < K; jp += blockDim.x) {
      const float g = A.G[(int64_t)jp * Kp + j];
      const float g2 = g * g;
      if (P.mi[jp] == j) {
        float v = 0.f;
        int vi = 0x7fffffff;
        for (int i = 0; i < K; ++i) {
          if (i == jp) continue;
          const float gg = A.G[(int64_t)jp * Kp + i];
          if (gg * gg > v) { v = gg * gg; vi = i; }
        }
        P.m[jp] = v;
        P.mi[jp] = vi;
      } else if (g2 > P.m[jp] || (g2 == P.m[jp] && j < P.mi[jp])) {
        P.m[jp] = g2;
        P.mi[jp] = j;
      }
    }
    __syncthreads();
    ++cleared;
    jstart = j + 1;
  }
  if (tid == 0) *A.cleared = cleared;
}

}  // namespace

int64_t error_block_count(int64_t N) { return (N + kBucket - 1) / kBucket; }

cudaError_t launch_error(const ErrorArgs& a, cudaStream_t st) {
  if (a.N <= 0) return cudaSuccess;
  if (a.n > kMaxN) return cudaErrorInvalidValue;
  const int64_t nb = error_block_count(a.N);
  const int npl = (a.n + 31) / 32;
  auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  const bool half = a.T <= 16 && a.n % 4 == 0 && a.n <= 256 && al16(a.X) && al16(a.D);
  const dim3 grid((unsigned)nb), blk(kErrWarps * 32);
  if (half && a.n == 64) error_half_kernel<1, true><<<grid, blk, 0, st>>>(a);
  else if (half && a.n < 64) error_half_kernel<1, false><<<grid, blk, 0, st>>>(a);
  else if (half && a.n == 128) error_half_kernel<2, true><<<grid, blk, 0, st>>>(a);
  else if (half && a.n < 128) error_half_kernel<2, false><<<grid, blk, 0, st>>>(a);
  else if (half && a.n == 256) error_half_kernel<4, true><<<grid, blk, 0, st>>>(a);
  else if (half) error_half_kernel<4, false><<<grid, blk, 0, st>>>(a);
  else if (npl <= 2) error_kernel<2><<<(unsigned)nb, kErrWarps * 32, 0, st>>>(a);
  else if (npl <= 4) error_kernel<4><<<(unsigned)nb, kErrWarps * 32, 0, st>>>(a);
  else if (npl <= 8) error_kernel<8><<<(unsigned)nb, kErrWarps * 32, 0, st>>>(a);
  else if (npl <= 16) error_kernel<16><<<(unsigned)nb, kErrWarps * 32, 0, st>>>(a);
  else error_kernel<32><<<(unsigned)nb, kErrWarps * 32, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  rmse_kernel<<<1, 1024, 0, st>>>(a.part_sum, nb, (double)a.n * (double)a.N, a.rmse_out,
                                  a.iter_ctr);
  return cudaGetLastError();
}

cudaError_t launch_clear_dict(const ClearArgs& a, float* m, int* mi, cudaStream_t st) {
  if (a.K <= 0) return cudaSuccess;
  coherence_kernel<<<(a.K + 7) / 8, 256, 0, st>>>(a.G, a.K, a.Kp, m, mi);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  ClearSeqArgs p;
  p.c = a;
  p.m = m;
  p.mi = mi;
  clear_seq_kernel<<<1, kClearThreads, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace ksvd
