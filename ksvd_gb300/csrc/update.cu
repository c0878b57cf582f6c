// update.cu -- approximate K-SVD dictionary sweep (DictionaryUpdate.cu:45-203 in the reference).
//
// Data flow per sweep:
//   1. per-atom signal lists (the reference's sprow, DictionaryUpdate.cu:210-230, 378-395):
//      a deterministic stable counting sort of the sparse code's (signal, slot) entries by atom,
//      so every list is in ascending signal order (count -> scan -> warp-ranked fill).
//   2. per-atom precompute, one CTA per atom (reduce1D_Batched_Sum_TOGETHER_collincomb,
//      Reduction.cu:80-93): ||gamma_j||^2, Y_j = X(:,I_j) gamma_j' and the co-occurrence column
//      C(:,j) = Gamma Gamma'(:,j).  C replaces the per-atom product v = Gamma(:,I_j) gamma_j'
//      (reduce2D_dot_products_modified, ReductionKernels.cu:105-168): v = C(:,j) as long as row
//      j of C is refreshed whenever atom j's coefficients change, which step 3 does.
//   3. one persistent cooperative kernel walks the K atoms in permutation order; per atom:
//        P1  a = Y_j - D v + d_j ||gamma_j||^2        (A_times_x_SUBTRACT, Multiplication.cu:177)
//        P2  ||a|| and a'D                             (rowlincomb, ReductionKernels.cu:196-250)
//        P3  gamma_j(s) = (a.x_s - Gamma(:,s).(a'D) + (a'd_j) gamma_j(s)) / ||a||, d_j = a/||a||,
//            C(j,:) refreshed                          (normal_x_times_A_modified, Mult.cu:198)
//      with a grid barrier between phases; an atom no signal uses takes the special case
//      (specialCase + SCase_*, DictionaryUpdate.cu:238-302, ReductionKernels.cu:436-539).
//      Barrier waits are bounded: on timeout the kernel records kDevErrTimeout and returns.
#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

constexpr int kSigPerBlock = 256;      // signals per list-building block
constexpr int kPrepThreads = 256;
constexpr int kSweepThreads = 512;
constexpr unsigned kBarrierSpinLimit = 1u << 24;   // x >= 64 ns sleeps: > 1 s before giving up

// ---- 1. atom lists --------------------------------------------------------------------------

__global__ void list_count_kernel(const int32_t* __restrict__ idx, const int32_t* __restrict__ nnz,
                                  int64_t N, int T, int K, int Kp, int64_t nblk,
                                  int32_t* __restrict__ block_hist, int* __restrict__ dev_err) {
  extern __shared__ int hist[];
  for (int k = threadIdx.x; k < Kp; k += blockDim.x) hist[k] = 0;
  __syncthreads();
  const int64_t b = blockIdx.x;
  const int64_t s0 = b * kSigPerBlock;
  const int64_t s1 = min(N, s0 + kSigPerBlock);
  const int64_t e0 = s0 * T, e1 = s1 * T;
  bool bad = false;
  for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int64_t s = e / T;
    const int t = (int)(e - s * T);
    if (t < nnz[s]) {
      const int a = idx[e];
      if (a >= 0 && a < K) atomicAdd(&hist[a], 1);
      else bad = true;
    }
  }
  if (bad) atomicOr(dev_err, kDevErrBounds);
  __syncthreads();
  for (int k = threadIdx.x; k < Kp; k += blockDim.x) block_hist[(int64_t)k * nblk + b] = hist[k];
}

// exclusive scan over blocks for every atom (warp per atom); atom totals to start[k + 1]
__global__ void list_scan_blocks_kernel(int32_t* __restrict__ block_hist, int64_t nblk, int Kp,
                                        int64_t* __restrict__ start) {
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (k >= Kp) return;
  int32_t* h = block_hist + (int64_t)k * nblk;
  int carry = 0;
  for (int64_t b0 = 0; b0 < nblk; b0 += 32) {
    const int64_t b = b0 + lane;
    const int v = b < nblk ? h[b] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(KSVD_FULL_MASK, incl, o);
      if (lane >= o) incl += u;
    }
    if (b < nblk) h[b] = carry + incl - v;
    carry += __shfl_sync(KSVD_FULL_MASK, incl, 31);
  }
  if (lane == 0) start[k + 1] = carry;
}

// exclusive scan of the atom totals (single block of 1024 threads, Kp <= 1024)
__global__ void list_scan_atoms_kernel(int64_t* __restrict__ start, int Kp) {
  __shared__ int64_t warp_tot[32];
  const int k = threadIdx.x, lane = k & 31, w = k >> 5;
  const int64_t v = k < Kp ? start[k + 1] : 0;
  int64_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t u = __shfl_up_sync(KSVD_FULL_MASK, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int64_t t = warp_tot[lane];
    int64_t ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t u = __shfl_up_sync(KSVD_FULL_MASK, ti, o);
      if (lane >= o) ti += u;
    }
    warp_tot[lane] = ti - t;
  }
  __syncthreads();
  const int64_t excl = warp_tot[w] + incl - v;
  __syncthreads();
  if (k < Kp) start[k] = excl;
  if (k == Kp - 1) start[Kp] = excl + v;
}

// Stable placement: one warp per block of signals walks its entries in signal-major order, 32
// at a time; lanes holding the same atom are ranked with __match_any_sync.
__global__ void list_fill_kernel(const int32_t* __restrict__ idx, const int32_t* __restrict__ nnz,
                                 int64_t N, int T, int K, int Kp, int64_t nblk,
                                 const int32_t* __restrict__ block_hist,
                                 const int64_t* __restrict__ start, int32_t* __restrict__ list) {
  extern __shared__ int64_t cursor[];
  const int lane = threadIdx.x;
  const int64_t b = blockIdx.x;
  for (int k = lane; k < Kp; k += 32) cursor[k] = start[k] + block_hist[(int64_t)k * nblk + b];
  __syncwarp();
  const int64_t s0 = b * kSigPerBlock;
  const int64_t s1 = min(N, s0 + kSigPerBlock);
  const int64_t e0 = s0 * T, e1 = s1 * T;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int64_t c0 = e0; c0 < e1; c0 += 32) {
    const int64_t e = c0 + lane;
    int a = -1;
    if (e < e1) {
      const int64_t s = e / T;
      const int t = (int)(e - s * T);
      if (t < nnz[s]) {
        const int v = idx[e];
        if (v >= 0 && v < K) a = v;
      }
    }
    const unsigned peers = __match_any_sync(KSVD_FULL_MASK, a);
    int64_t base = 0;
    if (a >= 0) base = cursor[a];
    __syncwarp();
    if (a >= 0) {
      const int rank = __popc(peers & lt_mask);
      list[base + rank] = (int32_t)e;
      if (rank == 0) cursor[a] = base + __popc(peers);
    }
    __syncwarp();
  }
}

// ---- 2. per-atom precompute -------------------------------------------------------------------

// CTA j: gn2[j], Y(:,j), C(:,j) from the atom's list.  Each warp walks every 8th entry and keeps
// private partials (deterministic), reduced in warp order at the end.
__global__ void __launch_bounds__(kPrepThreads)
prepare_kernel(const float* __restrict__ X, int n, int T, int Kp, const int32_t* __restrict__ idx,
               const float* __restrict__ coef, const int32_t* __restrict__ nnz,
               const int32_t* __restrict__ list, const int64_t* __restrict__ start,
               float* __restrict__ Y, float* __restrict__ gn2, float* __restrict__ C) {
  constexpr int NW = kPrepThreads / 32;
  extern __shared__ float sm[];
  float* Cw = sm;                        // NW x Kp
  float* Yw = sm + (size_t)NW * Kp;      // NW x n
  __shared__ float g2w[NW];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < NW * Kp; i += blockDim.x) Cw[i] = 0.f;
  for (int i = threadIdx.x; i < NW * n; i += blockDim.x) Yw[i] = 0.f;
  __syncthreads();
  const int64_t q0 = start[j], q1 = start[j + 1];
  float* cw = Cw + (size_t)w * Kp;
  float* yw = Yw + (size_t)w * n;
  float g2 = 0.f;
  for (int64_t q = q0 + w; q < q1; q += NW) {
    const int64_t e = list[q];
    const int64_t s = e / T;
    const float g = coef[e];
    g2 = fmaf(g, g, g2);
    const float* x = X + s * n;
    for (int r = lane; r < n; r += 32) yw[r] = fmaf(g, x[r], yw[r]);
    const int nz = min(nnz[s], T);
    for (int t = lane; t < nz; t += 32) {
      const int i = idx[s * T + t];
      if (i >= 0 && i < Kp) cw[i] = fmaf(g, coef[s * T + t], cw[i]);   // distinct per signal
    }
    __syncwarp();
  }
  if (lane == 0) g2w[w] = g2;
  __syncthreads();
  for (int i = threadIdx.x; i < Kp; i += blockDim.x) {
    float acc = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) acc += Cw[(size_t)ww * Kp + i];
    C[(int64_t)j * Kp + i] = acc;
  }
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    float acc = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) acc += Yw[(size_t)ww * n + r];
    Y[(int64_t)j * n + r] = acc;
  }
  if (threadIdx.x == 0) {
    float acc = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) acc += g2w[ww];
    gn2[j] = acc;
  }
}

__global__ void init_state_kernel(int64_t N, int Kp, int32_t* __restrict__ unused,
                                  int32_t* __restrict__ bitmap, int32_t* __restrict__ replaced,
                                  int32_t* __restrict__ usecount, int64_t* __restrict__ counter,
                                  float* __restrict__ avec, int n, unsigned* __restrict__ barrier) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = t; s < N; s += stride) { unused[s] = (int32_t)s; bitmap[s] = 1; }
  for (int64_t k = t; k < Kp; k += stride) { replaced[k] = 0; usecount[k] = 0; }
  for (int64_t r = t; r < 2 * n; r += stride) avec[r] = 0.f;
  if (t == 0) { *counter = 0; barrier[0] = 0; barrier[1] = 0; }
}

// ---- 3. the sweep -------------------------------------------------------------------------------

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Sense-free generation barrier over all CTAs of a cooperative launch.  Bounded: returns false
// (and records kDevErrTimeout) if the generation does not advance within the spin limit.
__device__ bool grid_barrier(unsigned* bar, unsigned nctas, int* dev_err, int* sflag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned gen = ld_acquire_gpu(bar + 1);
    const unsigned arrived = atomicAdd(bar, 1u) + 1u;
    if (arrived == nctas) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned spins = 0;
      while (ld_acquire_gpu(bar + 1) == gen) {
        if (++spins > kBarrierSpinLimit) { ok = 0; atomicOr(dev_err, kDevErrTimeout); break; }
        __nanosleep(64);
      }
    }
    __threadfence();
    *sflag = ok;
  }
  __syncthreads();
  const bool ok = *sflag != 0;
  __syncthreads();
  return ok;
}

struct SweepArgs {
  int n, K, Kp, T;
  int64_t N;
  const float* X;
  float* D;
  const int32_t* idx;
  float* coef;
  const int32_t* nnz;
  const int32_t* perm;
  int max_signals;
  const int32_t* list;
  const int64_t* start;
  const float* Y;
  const float* gn2;
  float* C;
  float* avec;
  float* aD;
  float* part;
  int32_t* unused;
  int32_t* bitmap;
  int32_t* replaced;
  int64_t* counter;
  int32_t* usecount;
  unsigned* barrier;
  int* dev_err;
};

__global__ void __launch_bounds__(kSweepThreads, 1) sweep_kernel(SweepArgs A) {
  constexpr int NW = kSweepThreads / 32;
  extern __shared__ float sm[];
  float* a_s = sm;                    // n
  float* aD_s = sm + A.n;             // Kp
  float* cpart = aD_s + A.Kp;         // Kp
  __shared__ float red_f[64];
  __shared__ int red_i[64];
  __shared__ int sflag;
  __shared__ int use_cnt;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int c = blockIdx.x, nctas = gridDim.x;
  const int n = A.n, K = A.K, Kp = A.Kp, T = A.T;
  // atom slice of this CTA (for P1 / P2 / zeroing)
  const int kper = (K + nctas - 1) / nctas;
  const int k0 = min(K, c * kper), k1 = min(K, k0 + kper);

  for (int jj = 0; jj < K; ++jj) {
    const int j = A.perm[jj];
    if (j < 0 || j >= K) {                       // not a permutation entry: skip the atom
      if (c == 0 && tid == 0) atomicOr(A.dev_err, kDevErrBounds);
      continue;
    }
    const int64_t q0 = A.start[j], q1 = A.start[j + 1];
    const int64_t cnt = q1 - q0;
    if (cnt == 0) {
      // ---- special case: replace the unused atom by the worst-represented unused signal
      const int64_t counter = *((volatile int64_t*)A.counter);
      const int64_t ncand = min((int64_t)A.max_signals, A.N - counter);
      if (ncand <= 0) continue;
      float best_v = -1.f;
      int best_b = 0x7fffffff;
      for (int64_t b = (int64_t)c * NW + w; b < ncand; b += (int64_t)nctas * NW) {
        const int64_t s = __ldcg(A.unused + b);
        const float* x = A.X + s * n;
        const int nz = min(A.nnz[s], T);
        float e = 0.f;
        for (int r = lane; r < n; r += 32) {
          float v = x[r];
          for (int t = 0; t < nz; ++t) {
            const int i = A.idx[s * T + t];
            if (i >= 0 && i < K)
              v = fmaf(-__ldcg(A.coef + s * T + t), __ldcg(A.D + (int64_t)i * n + r), v);
          }
          e = fmaf(v, v, e);
        }
        e = warp_sum(e);
        if (e > best_v) { best_v = e; best_b = (int)b; }
      }
      block_argmax(best_v, best_b, red_f, red_i);
      if (tid == 0) {
        A.part[c * 4 + 0] = best_v;
        reinterpret_cast<int*>(A.part)[c * 4 + 1] = best_b;
      }
      if (!grid_barrier(A.barrier, nctas, A.dev_err, &sflag)) return;
      if (c == 0) {
        float v = -1.f;
        int bi = 0x7fffffff;
        for (int cc = lane; cc < nctas; cc += 32) {
          const float pv = ((volatile float*)A.part)[cc * 4 + 0];
          const int pb = ((volatile int*)A.part)[cc * 4 + 1];
          if (pv > v || (pv == v && pb < bi)) { v = pv; bi = pb; }
        }
        if (w == 0) warp_argmax(v, bi);
        if (w == 0 && lane == 0) red_i[0] = bi;
        __syncthreads();
        const int bsel = red_i[0];
        if (bsel >= 0 && bsel < ncand) {
          const int64_t s = __ldcg(A.unused + bsel);
          const float* x = A.X + s * n;
          float nr = 0.f;
          for (int r = tid; r < n; r += blockDim.x) nr = fmaf(x[r], x[r], nr);
          nr = sqrtf(block_sum(nr, red_f));
          for (int r = tid; r < n; r += blockDim.x) A.D[(int64_t)j * n + r] = x[r] / nr;
          if (tid == 0) {
            A.unused[bsel] = __ldcg(A.unused + (A.N - counter - 1));
            *A.counter = counter + 1;
            A.replaced[j] = 1;
            A.bitmap[s] = 0;
          }
        } else if (tid == 0) {
          atomicOr(A.dev_err, kDevErrBounds);
        }
      }
      if (!grid_barrier(A.barrier, nctas, A.dev_err, &sflag)) return;
      continue;
    }

    // ---- P1: a += slice of (-D v), CTA 0 adds Y_j + d_j ||gamma_j||^2; zero C row j slice.
    // The accumulator avec is zero here: it starts zeroed and P3 clears it after use.
    float* acc_vec = A.avec;
    const float g2j = A.gn2[j];
    for (int r = tid; r < n; r += blockDim.x) {
      float acc = 0.f;
      for (int k = k0; k < k1; ++k) {
        const float vk = (k == j) ? g2j : __ldcg(A.C + (int64_t)j * Kp + k);
        acc = fmaf(-vk, __ldcg(A.D + (int64_t)k * n + r), acc);
      }
      if (c == 0)
        acc += A.Y[(int64_t)j * n + r] + __ldcg(A.D + (int64_t)j * n + r) * g2j;
      if (k1 > k0 || c == 0) atomicAdd(acc_vec + r, acc);
    }
    for (int k = k0 + tid; k < k1; k += blockDim.x) A.C[(int64_t)k * Kp + j] = 0.f;
    if (!grid_barrier(A.barrier, nctas, A.dev_err, &sflag)) return;

    // ---- P2: a to shared memory, ||a||, a'D for this CTA's atom slice
    for (int r = tid; r < n; r += blockDim.x) a_s[r] = __ldcg(acc_vec + r);
    __syncthreads();
    for (int k = k0 + w; k < k1; k += NW) {
      const float* d = A.D + (int64_t)k * n;
      float acc = 0.f;
      for (int r = lane; r < n; r += 32) acc = fmaf(__ldcg(d + r), a_s[r], acc);
      acc = warp_sum(acc);
      if (lane == 0) A.aD[k] = acc;
    }
    if (!grid_barrier(A.barrier, nctas, A.dev_err, &sflag)) return;

    // ---- P3: new coefficients of atom j, new d_j, refreshed C row j, use count of atom j
    float nr = 0.f;
    for (int r = tid; r < n; r += blockDim.x) nr = fmaf(a_s[r], a_s[r], nr);
    const float anorm = sqrtf(block_sum(nr, red_f));
    for (int k = tid; k < Kp; k += blockDim.x) {
      aD_s[k] = k < K ? __ldcg(A.aD + k) : 0.f;
      cpart[k] = 0.f;
    }
    if (tid == 0) use_cnt = 0;
    __syncthreads();
    if (c == 0)
      for (int r = tid; r < n; r += blockDim.x) {
        A.D[(int64_t)j * n + r] = a_s[r] / anorm;
        acc_vec[r] = 0.f;   // every CTA has read the accumulator (P2, before the barrier)
      }
    const float aDj = aD_s[j];
    const int64_t per = (cnt + nctas - 1) / nctas;
    const int64_t qa = q0 + min(cnt, (int64_t)c * per), qb = q0 + min(cnt, (int64_t)(c + 1) * per);
    int my_use = 0;
    for (int64_t q = qa + w; q < qb; q += NW) {
      const int64_t e = A.list[q];
      const int64_t s = e / T;
      const float* x = A.X + s * n;
      float ax = 0.f;
#pragma unroll 4
      for (int r = lane; r < n; r += 32) ax = fmaf(a_s[r], __ldcs(x + r), ax);
      const int nz = min(A.nnz[s], T);
      float gs = 0.f;
      for (int t = lane; t < nz; t += 32) {
        const int i = A.idx[s * T + t];
        if (i >= 0 && i < K) gs = fmaf(__ldcg(A.coef + s * T + t), aD_s[i], gs);
      }
      ax = warp_sum(ax);
      gs = warp_sum(gs);
      const float gold = __ldcg(A.coef + e);
      const float g = (ax - gs + aDj * gold) / anorm;
      for (int t = lane; t < nz; t += 32) {
        const int i = A.idx[s * T + t];
        if (i != j && i >= 0 && i < K) atomicAdd(cpart + i, g * __ldcg(A.coef + s * T + t));
      }
      __syncwarp();
      if (lane == 0) {
        A.coef[e] = g;
        if (g * g > 1e-7f) ++my_use;
      }
    }
    if (lane == 0 && my_use) atomicAdd(&use_cnt, my_use);
    __syncthreads();
    for (int k = tid; k < K; k += blockDim.x) {
      const float v = cpart[k];
      if (v != 0.f) atomicAdd(A.C + (int64_t)k * Kp + j, v);
    }
    if (tid == 0 && use_cnt) atomicAdd(A.usecount + j, use_cnt);
    if (!grid_barrier(A.barrier, nctas, A.dev_err, &sflag)) return;
  }
}

int sweep_grid_size() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

}  // namespace

int64_t update_block_count(int64_t N) { return (N + kSigPerBlock - 1) / kSigPerBlock; }

cudaError_t launch_update_prepare(const UpdateArgs& a, cudaStream_t st) {
  if (a.N <= 0) return cudaSuccess;
  if (a.Kp > 1024 || a.n > kMaxN) return cudaErrorInvalidValue;
  const int64_t nblk = update_block_count(a.N);
  cudaError_t e;
  init_state_kernel<<<256, 256, 0, st>>>(a.N, a.Kp, a.unused, a.bitmap, a.replaced, a.usecount,
                                         a.counter, a.avec, a.n, a.barrier);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  list_count_kernel<<<(unsigned)nblk, 256, a.Kp * sizeof(int), st>>>(
      a.idx, a.nnz, a.N, a.T, a.K, a.Kp, nblk, a.block_hist, a.dev_err);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  list_scan_blocks_kernel<<<(a.Kp + 7) / 8, 256, 0, st>>>(a.block_hist, nblk, a.Kp, a.start);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  list_scan_atoms_kernel<<<1, 1024, 0, st>>>(a.start, a.Kp);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  list_fill_kernel<<<(unsigned)nblk, 32, a.Kp * sizeof(int64_t), st>>>(
      a.idx, a.nnz, a.N, a.T, a.K, a.Kp, nblk, a.block_hist, a.start, a.list);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const size_t psm = sizeof(float) * ((size_t)(kPrepThreads / 32) * (a.Kp + a.n));
  e = cudaFuncSetAttribute(prepare_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm);
  if (e != cudaSuccess) return e;
  prepare_kernel<<<a.Kp, kPrepThreads, psm, st>>>(a.X, a.n, a.T, a.Kp, a.idx, a.coef, a.nnz,
                                                  a.list, a.start, a.Y, a.gn2, a.C);
  return cudaGetLastError();
}

cudaError_t launch_update_sweep(const UpdateArgs& a, cudaStream_t st) {
  if (a.N <= 0) return cudaSuccess;
  SweepArgs s;
  s.n = a.n; s.K = a.K; s.Kp = a.Kp; s.T = a.T; s.N = a.N; s.X = a.X; s.D = a.D; s.idx = a.idx;
  s.coef = a.coef; s.nnz = a.nnz; s.perm = a.perm; s.max_signals = a.max_signals;
  s.list = a.list; s.start = a.start; s.Y = a.Y; s.gn2 = a.gn2; s.C = a.C; s.avec = a.avec;
  s.aD = a.aD; s.part = a.part; s.unused = a.unused; s.bitmap = a.bitmap; s.replaced = a.replaced;
  s.counter = a.counter; s.usecount = a.usecount; s.barrier = a.barrier; s.dev_err = a.dev_err;
  const size_t smem = sizeof(float) * ((size_t)a.n + 2 * (size_t)a.Kp);
  cudaError_t e = cudaFuncSetAttribute(sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_kernel, kSweepThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorCooperativeLaunchTooLarge;
  const int grid = sweep_grid_size();
  void* args[] = {&s};
  return cudaLaunchCooperativeKernel((const void*)sweep_kernel, dim3(grid), dim3(kSweepThreads),
                                     args, smem, st);
}

int update_sweep_ctas() { return sweep_grid_size(); }

}  // namespace ksvd
