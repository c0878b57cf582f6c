// omp.cu -- Batch-OMP (Rubinstein, Zibulevsky & Elad, CS-2008-08) on the GPU: one warp per
// signal, the K correlations of the signal held in registers (K/32 per lane), the incremental
// Cholesky factor of G restricted to the support in shared memory (one (TMAX) x (TMAX+1) tile
// per warp, padded against bank conflicts), and warp-shuffle argmax / reductions.
//
// Per step it does what the reference's parOMP does per thread (OMP.cu:254-405):
//   p = argmax |alpha| (first maximum, maxabs OMP.cu:201-213); stop if p is already selected or
//   alpha_p^2 < 1e-14 (OMP.cu:292,304); new row w of L from L w = G(I,p) (OMP.cu:321-326),
//   L_tt = sqrt(1 - ||w||^2), stop if <= 1e-14 (OMP.cu:329-335); forward/backward solves for the
//   coefficients (OMP.cu:347-357); alpha = alpha0 - G(:,I) gamma (addMul, OMP.cu:365-371).
// GPU-specific choices: the forward solve is incremental (only the new entry of y = L^-1
// alpha0_I is computed; the earlier entries do not change), the triangular solves run as
// column sweeps across the lanes that own the support slots, the final alpha update after the
// last atom is skipped (it is never read), and a failed pivot test does not add the atom.
// alpha0 is streamed once (evict-first loads); G stays L2-resident, and re-reading the support
// columns of G from L2 (N*K*T(T-1)/2 floats per sweep of all signals) is what bounds this kernel.
#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

constexpr int kOmpWarps = 8;

// Shared-memory layout of the Cholesky factor L (TMAX x TMAX, lower): rows of stride TMAX+1
// (bank-conflict padding) up to TMAX = 32; for TMAX = 64 packed by rows (row r at r(r+1)/2),
// half the space, so two CTAs fit on an SM.
template <int TMAX>
__host__ __device__ constexpr int l_floats() {
  return TMAX > 32 ? TMAX * (TMAX + 1) / 2 : TMAX * (TMAX + 1);
}
template <int TMAX>
__device__ __forceinline__ int lidx(int r, int q) {
  if constexpr (TMAX > 32) return r * (r + 1) / 2 + q;
  else return r * (TMAX + 1) + q;
}

// 16-byte read-only load that does not allocate in L1
__device__ __forceinline__ float4 ldg_f4_no_l1(const float* p) {
  float4 g;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(g.x), "=f"(g.y), "=f"(g.z), "=f"(g.w)
               : "l"(p));
  return g;
}

template <int SPL>
__device__ __forceinline__ float pick(const float (&a)[SPL], int j) {
  if constexpr (SPL == 1) return a[0];
  else return j == 0 ? a[0] : a[1];
}
template <int SPL>
__device__ __forceinline__ int pick(const int (&a)[SPL], int j) {
  if constexpr (SPL == 1) return a[0];
  else return j == 0 ? a[0] : a[1];
}
template <int SPL, typename V>
__device__ __forceinline__ void put(V (&a)[SPL], int j, V v) {
  if constexpr (SPL == 1) a[0] = v;
  else { if (j == 0) a[0] = v; else a[1] = v; }
}

// Batch-OMP of one signal by one warp.  a0p: the signal's alpha0 column (Kp = 32*KPL rows, rows
// >= K zero); L: (TMAX x TMAX+1) and a0s: (32*KPL) floats of this warp's shared memory.  emode:
// stop once ||x||^2 - ||y||^2 <= e2 (xn2 = ||x||^2).  Writes T slots of idx/coef and nnz.
template <int KPL, int TMAX>
__device__ __forceinline__ void omp_signal(const float* __restrict__ G, int64_t ldg,
                                           const float* __restrict__ a0col, int K, int T,
                                           bool emode, float e2, float xn2,
                                           int32_t* __restrict__ idx_s, float* __restrict__ coef_s,
                                           int32_t* __restrict__ nnz_s, float* L, float* a0s,
                                           bool& numeric_bad) {
  constexpr int M4 = KPL / 4;    // float4 groups per lane; lane owns rows 128*m + 4*lane + q
  constexpr int SPL = TMAX / 32; // support slots per lane; lane owns slots lane + 32*j
  const int lane = threadIdx.x & 31;
  {
    float al[M4][4];
    const float* a0p = a0col + 4 * lane;
    __syncwarp();                      // the previous signal's last reads of a0s are done
#pragma unroll
    for (int m = 0; m < M4; ++m) {
      const float4 v = __ldcs(reinterpret_cast<const float4*>(a0p + 128 * m));
      *reinterpret_cast<float4*>(a0s + 128 * m + 4 * lane) = v;
      al[m][0] = v.x; al[m][1] = v.y; al[m][2] = v.z; al[m][3] = v.w;
    }
    __syncwarp();
    int ind[SPL];
    float y[SPL], c[SPL];
#pragma unroll
    for (int j = 0; j < SPL; ++j) { ind[j] = -1; y[j] = 0.f; c[j] = 0.f; }

    float r2 = xn2;
    int i = 0;
    while (i < T) {
      if (emode && r2 <= e2) break;
      // ---- argmax |alpha| (first maximum) with alpha_p as payload
      float bv = -1.f, bal = 0.f;
      int bk = 0x7fffffff;
#pragma unroll
      for (int m = 0; m < M4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int k = 128 * m + 4 * lane + q;
          const float v = al[m][q] * al[m][q];
          if (k < K && v > bv) { bv = v; bk = k; bal = al[m][q]; }
        }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(KSVD_FULL_MASK, bv, o);
        const int ok = __shfl_xor_sync(KSVD_FULL_MASK, bk, o);
        const float oal = __shfl_xor_sync(KSVD_FULL_MASK, bal, o);
        if (ov > bv || (ov == bv && ok < bk)) { bv = ov; bk = ok; bal = oal; }
      }
      if (bk >= K) { numeric_bad = true; break; }   // every |alpha| was NaN
      const int p = bk;
      const float ba0 = a0s[p];
      bool dup = false;
#pragma unroll
      for (int j = 0; j < SPL; ++j) dup |= (lane + 32 * j < i) && ind[j] == p;
      if (__any_sync(KSVD_FULL_MASK, dup)) break;
      if (bal * bal < 1e-14f) break;

      float Lii = 1.f, ynew = ba0;
      if (i > 0) {
        // b = G(I, p); forward column sweep solves L w = b, lane q ends with w_q
        float b[SPL], w[SPL];
#pragma unroll
        for (int j = 0; j < SPL; ++j) {
          const int q = lane + 32 * j;
          b[j] = q < i ? __ldg(G + (int64_t)ind[j] * ldg + p) : 0.f;
          w[j] = 0.f;
        }
        for (int r = 0; r < i; ++r) {
          const int rl = r & 31, rj = r >> 5;
          const float wr = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(b, rj), rl) / L[lidx<TMAX>(r, r)];
          if (lane == rl) put<SPL>(w, rj, wr);
#pragma unroll
          for (int j = 0; j < SPL; ++j) {
            const int q = lane + 32 * j;
            if (q > r && q < i) b[j] = fmaf(-L[lidx<TMAX>(q, r)], wr, b[j]);
          }
        }
        float ss = 0.f, wy = 0.f;
#pragma unroll
        for (int j = 0; j < SPL; ++j) {
          if (lane + 32 * j < i) { ss = fmaf(w[j], w[j], ss); wy = fmaf(w[j], y[j], wy); }
        }
        ss = warp_sum(ss);
        const float l2 = 1.f - ss;
        if (l2 <= 1e-14f) break;               // pivot test failed: the atom is not added
        Lii = sqrtf(l2);
        wy = warp_sum(wy);
        ynew = (ba0 - wy) / Lii;
#pragma unroll
        for (int j = 0; j < SPL; ++j) {
          const int q = lane + 32 * j;
          if (q < i) L[lidx<TMAX>(i, q)] = w[j];
        }
      }
      if (lane == 0) L[lidx<TMAX>(i, i)] = Lii;
      if (lane == (i & 31)) { put<SPL>(ind, i >> 5, p); put<SPL>(y, i >> 5, ynew); }
      ++i;
      __syncwarp();

      if (emode) {
        float yy = 0.f;
#pragma unroll
        for (int j = 0; j < SPL; ++j)
          if (lane + 32 * j < i) yy = fmaf(y[j], y[j], yy);
        r2 = xn2 - warp_sum(yy);
      }
      // ---- backward column sweep: L' c = y
      {
        float t[SPL];
#pragma unroll
        for (int j = 0; j < SPL; ++j) t[j] = y[j];
        for (int r = i - 1; r >= 0; --r) {
          const int rl = r & 31, rj = r >> 5;
          const float cr = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(t, rj), rl) / L[lidx<TMAX>(r, r)];
          if (lane == rl) put<SPL>(c, rj, cr);
#pragma unroll
          for (int j = 0; j < SPL; ++j) {
            const int q = lane + 32 * j;
            if (q < r) t[j] = fmaf(-L[lidx<TMAX>(r, q)], cr, t[j]);
          }
        }
      }
      // ---- alpha = alpha0 - G(:, I) c   (not needed after the last atom)
      if (i < T && !(emode && r2 <= e2)) {
#pragma unroll
        for (int m = 0; m < M4; ++m)
#pragma unroll
          for (int q = 0; q < 4; ++q) al[m][q] = 0.f;
        // one support column per step (deeper unrolling measured slower: register pressure);
        // G's columns bypass L1 allocation -- they are reused from L2, not from L1
#pragma unroll 1
        for (int r = 0; r < i; ++r) {
          const int rl = r & 31, rj = r >> 5;
          const float cr = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(c, rj), rl);
          const int col = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(ind, rj), rl);
          const float* gp = G + (int64_t)col * ldg + 4 * lane;
#pragma unroll
          for (int m = 0; m < M4; ++m) {
            const float4 g = ldg_f4_no_l1(gp + 128 * m);
            al[m][0] = fmaf(g.x, cr, al[m][0]);
            al[m][1] = fmaf(g.y, cr, al[m][1]);
            al[m][2] = fmaf(g.z, cr, al[m][2]);
            al[m][3] = fmaf(g.w, cr, al[m][3]);
          }
        }
#pragma unroll
        for (int m = 0; m < M4; ++m) {
          const float4 a = *reinterpret_cast<const float4*>(a0s + 128 * m + 4 * lane);
          al[m][0] = a.x - al[m][0];
          al[m][1] = a.y - al[m][1];
          al[m][2] = a.z - al[m][2];
          al[m][3] = a.w - al[m][3];
        }
      }
    }
    // ---- outputs: slots in selection order, -1 / 0 padding
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int q = lane + 32 * j;
      if (q < T) {
        const bool used = q < i;
        idx_s[q] = used ? ind[j] : -1;
        coef_s[q] = used ? c[j] : 0.f;
        if (used && !finitef(c[j])) numeric_bad = true;
      }
    }
    if (lane == 0) *nnz_s = i;
  }
}

template <int KPL, int TMAX>
__global__ void __launch_bounds__(kOmpWarps * 32, (TMAX <= 32 ? 3 : 2))
omp_kernel(const float* __restrict__ G, int64_t ldg, const float* __restrict__ A0, int64_t lda,
           int K, int64_t N, int T, const float* __restrict__ xnorm2,
           const float* __restrict__ eps2, int32_t* __restrict__ idx_out,
           float* __restrict__ coef_out, int32_t* __restrict__ nnz_out, int* __restrict__ dev_err) {
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  float* L = smem + (size_t)wib * (l_floats<TMAX>() + 32 * KPL);   // Cholesky factor
  float* a0s = L + l_floats<TMAX>();                                // this warp's alpha0 column
  const int64_t warps_total = (int64_t)gridDim.x * kOmpWarps;
  bool numeric_bad = false;
  const bool emode = eps2 != nullptr;
  for (int64_t s = (int64_t)blockIdx.x * kOmpWarps + wib; s < N; s += warps_total)
    omp_signal<KPL, TMAX>(G, ldg, A0 + s * lda, K, T, emode, emode ? eps2[s] : 0.f,
                          emode ? xnorm2[s] : 0.f, idx_out + s * T, coef_out + s * T,
                          nnz_out + s, L, a0s, numeric_bad);
  if (__any_sync(KSVD_FULL_MASK, numeric_bad) && lane == 0) atomicOr(dev_err, kDevErrNumeric);
}

// Many independent Batch-OMP problems (different K, T, N; T-sparse or error-constrained) in one
// persistent launch.  Work queue: each warp takes the next chunk of kChunk signals with one
// atomicAdd on *queue (zeroed before the launch); chunk c belongs to the job whose range
// [chunk_begin, chunk_begin + ceil(N / kChunk)) holds it.  In error-constrained jobs ||x||^2
// comes from X in the same pass.
constexpr int kBatchChunk = 16;   // default signals per work-queue chunk

template <int TMAX>
__global__ void __launch_bounds__(kOmpWarps * 32, 2)
omp_batched_kernel(const OmpJob* __restrict__ jobs, int njobs, int64_t total_chunks,
                   int chunk, unsigned long long* __restrict__ queue, int* __restrict__ dev_err) {
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  float* L = smem + (size_t)wib * (l_floats<TMAX>() + 32 * 32);
  float* a0s = L + l_floats<TMAX>();
  bool numeric_bad = false;
  for (;;) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(queue, 1ull);
    c = __shfl_sync(KSVD_FULL_MASK, c, 0);
    if ((int64_t)c >= total_chunks) break;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].chunk_begin <= (int64_t)c) lo = mid; else hi = mid - 1;
    }
    const OmpJob& jb = jobs[lo];
    const int64_t s0 = ((int64_t)c - jb.chunk_begin) * chunk;
    const int64_t s1 = min(jb.N, s0 + chunk);
    const bool emode = jb.eps2 != nullptr;
    for (int64_t s = s0; s < s1; ++s) {
      float xn2 = 0.f, e2 = 0.f;
      if (emode) {
        const float* x = jb.X + s * jb.ldx;
        for (int r = lane; r < jb.n; r += 32) xn2 = fmaf(x[r], x[r], xn2);
        xn2 = warp_sum(xn2);
        e2 = jb.eps2[s];
      }
      const float* a0 = jb.A0 + s * jb.lda;
      int32_t* io = jb.idx + s * jb.T;
      float* co = jb.coef + s * jb.T;
      switch (jb.kpl) {
        case 4:
          omp_signal<4, TMAX>(jb.G, jb.ldg, a0, jb.K, jb.T, emode, e2, xn2, io, co, jb.nnz + s, L,
                              a0s, numeric_bad);
          break;
        case 8:
          omp_signal<8, TMAX>(jb.G, jb.ldg, a0, jb.K, jb.T, emode, e2, xn2, io, co, jb.nnz + s, L,
                              a0s, numeric_bad);
          break;
        case 16:
          omp_signal<16, TMAX>(jb.G, jb.ldg, a0, jb.K, jb.T, emode, e2, xn2, io, co, jb.nnz + s,
                               L, a0s, numeric_bad);
          break;
        default:
          omp_signal<32, TMAX>(jb.G, jb.ldg, a0, jb.K, jb.T, emode, e2, xn2, io, co, jb.nnz + s,
                               L, a0s, numeric_bad);
          break;
      }
    }
  }
  if (__any_sync(KSVD_FULL_MASK, numeric_bad) && lane == 0) atomicOr(dev_err, kDevErrNumeric);
}

template <int KPL, int TMAX>
cudaError_t launch_omp_t(const float* G, int64_t ldg, const float* A0, int64_t lda, int K,
                         int64_t N, int T, const float* xnorm2, const float* eps2, int32_t* idx,
                         float* coef, int32_t* nnz, int* dev_err, int grid_mult,
                         cudaStream_t st) {
  const size_t smem = (size_t)kOmpWarps * (l_floats<TMAX>() + 32 * KPL) * sizeof(float);
  auto kern = omp_kernel<KPL, TMAX>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kOmpWarps * 32, smem);
  if (per_sm < 1) per_sm = 1;
  int64_t blocks = (N + kOmpWarps - 1) / kOmpWarps;
  const int64_t cap = (int64_t)sms * per_sm * (grid_mult > 0 ? grid_mult : 8);
  if (blocks > cap) blocks = cap;
  kern<<<(unsigned)blocks, kOmpWarps * 32, smem, st>>>(G, ldg, A0, lda, K, N, T, xnorm2, eps2, idx,
                                                       coef, nnz, dev_err);
  return cudaGetLastError();
}

template <int TMAX>
cudaError_t launch_omp_batched_t(const OmpJob* jobs, int njobs, int64_t total_chunks, int chunk,
                                 unsigned long long* queue, int* dev_err, cudaStream_t st) {
  const size_t smem = (size_t)kOmpWarps * (l_floats<TMAX>() + 32 * 32) * sizeof(float);
  auto kern = omp_batched_kernel<TMAX>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kOmpWarps * 32, smem);
  if (per_sm < 1) per_sm = 1;
  const int64_t need = (total_chunks + kOmpWarps - 1) / kOmpWarps;
  int64_t blocks = (int64_t)sms * per_sm;
  if (blocks > need) blocks = need;
  e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  kern<<<(unsigned)blocks, kOmpWarps * 32, smem, st>>>(jobs, njobs, total_chunks, chunk, queue,
                                                       dev_err);
  return cudaGetLastError();
}

}  // namespace

int omp_batch_chunk() { return kBatchChunk; }

cudaError_t launch_omp_batched(const OmpJob* jobs_dev, int njobs, int64_t total_chunks, int tmax,
                               int chunk, unsigned long long* queue, int* dev_err,
                               cudaStream_t st) {
  if (njobs <= 0 || total_chunks <= 0) return cudaSuccess;
  if (tmax < 1 || tmax > kMaxT || chunk < 1) return cudaErrorInvalidValue;
  if (tmax <= 32)
    return launch_omp_batched_t<32>(jobs_dev, njobs, total_chunks, chunk, queue, dev_err, st);
  return launch_omp_batched_t<64>(jobs_dev, njobs, total_chunks, chunk, queue, dev_err, st);
}

int omp_padded_k(int K) {
  return K <= 128 ? 128 : K <= 256 ? 256 : K <= 512 ? 512 : 1024;
}

cudaError_t launch_omp(const float* G, int64_t ldg, const float* A0, int64_t lda, int K,
                       int64_t N, int T, const float* xnorm2, const float* eps2, int32_t* idx,
                       float* coef, int32_t* nnz, int* dev_err, cudaStream_t st, int grid_mult) {
  if (N <= 0) return cudaSuccess;
  if (K < 1 || K > kMaxK || T < 1 || T > kMaxT) return cudaErrorInvalidValue;
  const int kp = omp_padded_k(K);   // the lanes touch rows [0, kp) of every column
  if (ldg < kp || lda < kp || (ldg & 3) || (lda & 3)) return cudaErrorInvalidValue;
#define KSVD_OMP_ARGS G, ldg, A0, lda, K, N, T, xnorm2, eps2, idx, coef, nnz, dev_err, grid_mult, st
  if (T <= 32) {
    switch (kp) {
      case 128: return launch_omp_t<4, 32>(KSVD_OMP_ARGS);
      case 256: return launch_omp_t<8, 32>(KSVD_OMP_ARGS);
      case 512: return launch_omp_t<16, 32>(KSVD_OMP_ARGS);
      default: return launch_omp_t<32, 32>(KSVD_OMP_ARGS);
    }
  }
  switch (kp) {
    case 128: return launch_omp_t<4, 64>(KSVD_OMP_ARGS);
    case 256: return launch_omp_t<8, 64>(KSVD_OMP_ARGS);
    case 512: return launch_omp_t<16, 64>(KSVD_OMP_ARGS);
    default: return launch_omp_t<32, 64>(KSVD_OMP_ARGS);
  }
#undef KSVD_OMP_ARGS
}

}  // namespace ksvd
