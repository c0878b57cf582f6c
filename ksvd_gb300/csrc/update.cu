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
#include <type_traits>

#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

constexpr int kSigPerBlock = 256;      // signals per list-building block
constexpr int kPrepThreads = 512;
constexpr int kPrepWinThreads = 256;   // windowed preparation: four CTAs per SM
constexpr int kSweepThreads = 512;
constexpr int kStageCap = 2048;   // list entries of the next atom staged per CTA (x2 buffers)
constexpr unsigned kBarrierSpinLimit = 1u << 24;   // x >= 64 ns sleeps: > 1 s before giving up

// e / T for list entries e = signal * T + slot as a 32-bit multiply-high and a shift.  With
// l = ceil(log2 T) and m = ceil(2^(31+l) / T) (< 2^32), m T - 2^(31+l) <= T - 1 < 2^l, so
// floor(e / T) = floor(e m / 2^(31+l)) for every 0 <= e < 2^31 (Granlund & Montgomery, "Division
// by invariant integers using multiplication", PLDI 1994, Thm 4.2 with 31-bit dividends);
// mulhi(2 e, m) = floor(e m / 2^31) leaves a shift by l.  The callers keep N * T < 2^31.
struct DivT {
  uint32_t m, l;
};
__host__ __device__ inline DivT div_t_magic(int T) {
  uint32_t l = 0;
  while ((1ll << l) < (long long)T) ++l;
  return {(uint32_t)((((uint64_t)1 << (31 + l)) + (uint64_t)T - 1) / (uint64_t)T), l};
}
__device__ __forceinline__ int div_t(int e, DivT d) {
  return (int)(__umulhi((uint32_t)e << 1, d.m) >> d.l);
}

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
  const DivT dt = div_t_magic(T);
  for (int64_t e64 = e0 + threadIdx.x; e64 < e1; e64 += blockDim.x) {
    const int e = (int)e64;                 // N * T < 2^31
    const int s = div_t(e, dt);
    const int t = e - s * T;
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
  const DivT dt = div_t_magic(T);
  for (int64_t c0 = e0; c0 < e1; c0 += 32) {
    const int e = (int)(c0 + lane);        // N * T < 2^31 (read only when c0 + lane < e1)
    int a = -1;
    if (c0 + lane < e1) {
      const int s = div_t(e, dt);
      const int t = e - s * T;
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

// Sums the NW warps' partials of C(:,j), Y(:,j) and ||gamma_j||^2 in warp order (deterministic).
template <int NW>
__device__ __forceinline__ void prepare_sum_warps(const float* Cw, const float* Yw,
                                                  const float* g2w, int n, int Kp, int j,
                                                  float* __restrict__ Y, float* __restrict__ gn2,
                                                  float* __restrict__ C) {
  for (int i = threadIdx.x; i < Kp; i += blockDim.x) {
    float a = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) a += Cw[(size_t)ww * Kp + i];
    C[(int64_t)j * Kp + i] = a;
  }
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    float a = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) a += Yw[(size_t)ww * n + r];
    Y[(int64_t)j * n + r] = a;
  }
  if (threadIdx.x == 0) {
    float a = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) a += g2w[ww];
    gn2[j] = a;
  }
}

// CTA j: gn2[j], Y(:,j), C(:,j) from the atom's list.  Each warp walks every 8th entry, two
// entries in flight, with its share of Y_j in registers (NPL rows per lane) and its share of
// C(:,j) in a private shared-memory vector; the warp partials are summed in warp order at the
// end, so the result is deterministic.
// CW: code-row words per lane (1 for T <= 32, else 2); FULLN: n == 32 NPL (no row test).
template <int NPL, int CW, bool FULLN>
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
  __syncthreads();
  const int64_t q0 = start[j], q1 = start[j + 1];
  float* cw = Cw + (size_t)w * Kp;
  float acc[NPL];
#pragma unroll
  for (int i = 0; i < NPL; ++i) acc[i] = 0.f;
  float g2 = 0.f;
  // entries per warp batch: 2 keeps the kernel at <= 64 registers, two 512-thread CTAs per SM
  // (measured faster than 4 or 6 entries with one CTA per SM)
  constexpr int EB = NPL <= 16 ? 2 : 1;
  const DivT dt = div_t_magic(T);
  // the list entries of the warp's next batch are loaded one batch ahead, so each batch costs
  // one round of loads (signals and code rows) instead of two
  int32_t ecur[EB];
#pragma unroll
  for (int b = 0; b < EB; ++b) {
    const int64_t q = q0 + (int64_t)w * EB + b;
    ecur[b] = q < q1 ? list[q] : 0;
  }
  for (int64_t qs = q0 + (int64_t)w * EB; qs < q1; qs += (int64_t)NW * EB) {
    const int ne = (int)min((int64_t)EB, q1 - qs);   // >= 1
    int sg[EB], ts[EB];
    bool live[EB];
#pragma unroll
    for (int b = 0; b < EB; ++b) {
      live[b] = b == 0 || b < ne;
      const int e = live[b] ? ecur[b] : 0;
      sg[b] = div_t(e, dt);                  // entries e = signal * T + slot < 2^31
      ts[b] = e - sg[b] * T;
    }
#pragma unroll
    for (int b = 0; b < EB; ++b) {
      const int64_t q = qs + (int64_t)NW * EB + b;
      ecur[b] = q < q1 ? list[q] : 0;
    }
    // the signals, their whole code rows and support sizes: one round of independent loads
    float xv[EB][NPL];
#pragma unroll
    for (int b = 0; b < EB; ++b) {
      const float* xp = X + (int64_t)sg[b] * n + lane;
#pragma unroll
      for (int i = 0; i < NPL; ++i)
        xv[b][i] = (live[b] && (FULLN || lane + 32 * i < n)) ? __ldg(xp + 32 * i) : 0.f;
    }
    float cf[EB][CW];
    int ix[EB][CW], nz[EB];
#pragma unroll
    for (int b = 0; b < EB; ++b) {
      nz[b] = live[b] ? nnz[sg[b]] : 0;
      const int cb = sg[b] * T;
#pragma unroll
      for (int u = 0; u < CW; ++u) {
        const int t = lane + 32 * u;
        const bool in = live[b] && t < T;
        ix[b][u] = in ? idx[cb + t] : -1;
        cf[b][u] = in ? coef[cb + t] : 0.f;
      }
    }
#pragma unroll
    for (int b = 0; b < EB; ++b) {
      // gamma_j(s) is slot ts of the code row
      const float cs = (CW == 1 || (ts[b] >> 5) == 0) ? cf[b][0] : cf[b][CW - 1];
      const float g = __shfl_sync(KSVD_FULL_MASK, cs, ts[b] & 31);
      if (!live[b]) continue;
#pragma unroll
      for (int i = 0; i < NPL; ++i) acc[i] = fmaf(g, xv[b][i], acc[i]);
      g2 = fmaf(g, g, g2);
      const int lim = min(nz[b], T);
#pragma unroll
      for (int u = 0; u < CW; ++u) {
        const int t = lane + 32 * u;
        const int i = ix[b][u];
        if (t < lim && i >= 0 && i < Kp) cw[i] = fmaf(g, cf[b][u], cw[i]);   // distinct per signal
      }
      __syncwarp();
    }
  }
#pragma unroll
  for (int i = 0; i < NPL; ++i) {
    const int r = lane + 32 * i;
    if (r < n) Yw[(size_t)w * n + r] = acc[i];
  }
  if (lane == 0) g2w[w] = g2;
  __syncthreads();
  prepare_sum_warps<NW>(Cw, Yw, g2w, n, Kp, j, Y, gn2, C);
}

// Half-warp preparation of list entries [q0, q1) of atom j, for T <= 16, n % 4 == 0, n <= 64 NQ
// and a 16-byte aligned X: each half-warp takes one list entry (a warp two consecutive entries),
// a lane gathers four consecutive rows per 16-byte load and holds slot (lane & 15) of the code
// row, so the per-entry bookkeeping (the division by T, the code-row loads, the shuffle for
// gamma_j(s)) is issued once for two entries.  The halves' C(:,j) updates go one after the other
// (two signals of atom j's list can share other atoms).  Leaves warp w's partials in
// Cw[w * Kp + .] (zeroed by the caller), Yw[w * n + .] and g2w[w]; the caller synchronises.
template <int NQ, bool FULLN, int NW>
__device__ __forceinline__ void prepare_half_range(
    const float* __restrict__ X, int n, int T, int Kp, const int32_t* __restrict__ idx,
    const float* __restrict__ coef, const int32_t* __restrict__ nnz,
    const int32_t* __restrict__ list, int64_t q0, int64_t q1, float* Cw, float* Yw, float* g2w) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int hl = lane & 15, half = lane >> 4;
  float* cw = Cw + (size_t)w * Kp;
  float4 acc[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  float g2 = 0.f;
  const DivT dt = div_t_magic(T);
  // this half's entry of the warp's next pair, loaded one pair ahead
  int ecur = 0;
  {
    const int64_t q = q0 + 2 * w + half;
    if (q < q1) ecur = list[q];
  }
  for (int64_t qs = q0 + 2 * w; qs < q1; qs += 2 * NW) {
    const bool live = qs + half < q1;
    const int e = live ? ecur : 0;
    const int s = div_t(e, dt);            // entries e = signal * T + slot < 2^31
    const int ts = e - s * T;
    {
      const int64_t qn = qs + 2 * NW + half;
      ecur = qn < q1 ? list[qn] : 0;
    }
    // the signal (4 consecutive rows per load), the code row slot and the support size
    const float4* xp = reinterpret_cast<const float4*>(X + (int64_t)s * n) + hl;
    float4 xv[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k)
      xv[k] = (live && (FULLN || 4 * hl + 64 * k < n)) ? __ldg(xp + 16 * k)
                                                       : make_float4(0.f, 0.f, 0.f, 0.f);
    const int nz = live ? nnz[s] : 0;
    const bool in = live && hl < T;
    const int ix = in ? idx[s * T + hl] : -1;
    const float cf = in ? coef[s * T + hl] : 0.f;
    // gamma_j(s) is slot ts (< T <= 16) of this half's code row; 0 for a dead half
    const float g = __shfl_sync(KSVD_FULL_MASK, cf, (lane & 16) | ts);
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      acc[k].x = fmaf(g, xv[k].x, acc[k].x);
      acc[k].y = fmaf(g, xv[k].y, acc[k].y);
      acc[k].z = fmaf(g, xv[k].z, acc[k].z);
      acc[k].w = fmaf(g, xv[k].w, acc[k].w);
    }
    g2 = fmaf(g, g, g2);
    const bool ok = hl < min(nz, T) && (unsigned)ix < (unsigned)Kp;
    if (half == 0 && ok) cw[ix] = fmaf(g, cf, cw[ix]);   // distinct atoms within one signal
    __syncwarp();
    if (half == 1 && ok) cw[ix] = fmaf(g, cf, cw[ix]);
    __syncwarp();
  }
  // half 1's partials into half 0
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    acc[k].x += __shfl_down_sync(KSVD_FULL_MASK, acc[k].x, 16);
    acc[k].y += __shfl_down_sync(KSVD_FULL_MASK, acc[k].y, 16);
    acc[k].z += __shfl_down_sync(KSVD_FULL_MASK, acc[k].z, 16);
    acc[k].w += __shfl_down_sync(KSVD_FULL_MASK, acc[k].w, 16);
  }
  g2 += __shfl_down_sync(KSVD_FULL_MASK, g2, 16);
  if (half == 0) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int r = 4 * hl + 64 * k;
      if (FULLN || r < n) *reinterpret_cast<float4*>(Yw + (size_t)w * n + r) = acc[k];
    }
  }
  if (lane == 0) g2w[w] = g2;
}

// One CTA per atom over its whole list (the half-warp layout of prepare_half_range).
template <int NQ, bool FULLN>
__global__ void __launch_bounds__(kPrepThreads)
prepare_half_kernel(const float* __restrict__ X, int n, int T, int Kp,
                    const int32_t* __restrict__ idx, const float* __restrict__ coef,
                    const int32_t* __restrict__ nnz, const int32_t* __restrict__ list,
                    const int64_t* __restrict__ start, float* __restrict__ Y,
                    float* __restrict__ gn2, float* __restrict__ C) {
  constexpr int NW = kPrepThreads / 32;
  extern __shared__ float sm[];
  float* Cw = sm;                        // NW x Kp
  float* Yw = sm + (size_t)NW * Kp;      // NW x n
  __shared__ float g2w[NW];
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < NW * Kp; i += blockDim.x) Cw[i] = 0.f;
  __syncthreads();
  prepare_half_range<NQ, FULLN, NW>(X, n, T, Kp, idx, coef, nnz, list, start[j], start[j + 1],
                                    Cw, Yw, g2w);
  __syncthreads();
  prepare_sum_warps<NW>(Cw, Yw, g2w, n, Kp, j, Y, gn2, C);
}

// Windowed preparation for X larger than L2: CTA b takes the entries of atom j = b % Kp whose
// signals lie in window w = b / Kp (bpw blocks of kSigPerBlock signals; the list's per-block
// offsets come from the count/scan kernels), so the CTAs resident at one time gather from one
// window of X, which stays in L2 while every atom of the window reads it.  Each CTA writes its
// partials [Y(:,j) (n) | C(:,j) (Kp) | ||gamma_j||^2 (1)] to part; prepare_win_reduce sums the
// windows in order (deterministic).
template <int NQ, bool FULLN>
__global__ void __launch_bounds__(kPrepWinThreads, 4)
prepare_win_kernel(const float* __restrict__ X, int n, int T, int Kp,
                   const int32_t* __restrict__ idx, const float* __restrict__ coef,
                   const int32_t* __restrict__ nnz, const int32_t* __restrict__ list,
                   const int64_t* __restrict__ start, const int32_t* __restrict__ block_hist,
                   int64_t nblk, int64_t bpw, float* __restrict__ part) {
  constexpr int NW = kPrepWinThreads / 32;
  extern __shared__ float sm[];
  float* Cw = sm;                        // NW x Kp
  float* Yw = sm + (size_t)NW * Kp;      // NW x n
  __shared__ float g2w[NW];
  const int j = (int)(blockIdx.x % (unsigned)Kp);
  const int64_t win = blockIdx.x / (unsigned)Kp;
  const int64_t b0 = win * bpw, b1 = b0 + bpw;
  const int64_t q0 = start[j] + block_hist[(int64_t)j * nblk + b0];
  const int64_t q1 = b1 < nblk ? start[j] + block_hist[(int64_t)j * nblk + b1] : start[j + 1];
  for (int i = threadIdx.x; i < NW * Kp; i += blockDim.x) Cw[i] = 0.f;
  __syncthreads();
  prepare_half_range<NQ, FULLN, NW>(X, n, T, Kp, idx, coef, nnz, list, q0, q1, Cw, Yw, g2w);
  __syncthreads();
  float* out = part + ((size_t)win * Kp + j) * (size_t)(n + Kp + 1);
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    float a = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) a += Yw[(size_t)ww * n + r];
    out[r] = a;
  }
  for (int i = threadIdx.x; i < Kp; i += blockDim.x) {
    float a = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) a += Cw[(size_t)ww * Kp + i];
    out[n + i] = a;
  }
  if (threadIdx.x == 0) {
    float a = 0.f;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) a += g2w[ww];
    out[n + Kp] = a;
  }
}

// Y, C and gn2 from the windows' partials, summed in window order.
__global__ void prepare_win_reduce(const float* __restrict__ part, int64_t nwin, int n, int Kp,
                                   float* __restrict__ Y, float* __restrict__ gn2,
                                   float* __restrict__ C) {
  const int64_t row = (int64_t)n + Kp + 1;
  const int64_t total = (int64_t)Kp * row;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    float a = 0.f;
    for (int64_t w = 0; w < nwin; ++w) a += part[w * total + t];
    const int64_t j = t / row, r = t - j * row;
    if (r < n) Y[j * n + r] = a;
    else if (r < n + Kp) C[j * Kp + (r - n)] = a;
    else gn2[j] = a;
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
  for (int64_t r = t; r < 3 * n; r += stride) avec[r] = 0.f;
  if (t == 0) { *counter = 0; barrier[0] = 0; barrier[1] = 0; }
}

// ---- 3. the sweep -------------------------------------------------------------------------------
//
// Pipelined schedule: one grid barrier per atom.  With j the current atom and j' the next one:
//   a(j') = Y_j' - sum_k v_k d_k + ||gamma_j'||^2 d_j',  v = C(:, j'), v_j' = ||gamma_j'||^2
//   a(j')'D = P(:, j') - G v + ||gamma_j'||^2 G(:, j')        (G = D'D, P = D'Y, both maintained)
// While atom j's coefficients are being recomputed, every CTA already accumulates its slice of
// a'(j') and a'(j')'D with the k = j term left out (d_j, C(j, j'), G(:, j), P(j, :) are being
// rewritten in that same phase).  After the barrier every CTA folds the missing term back in
// with the scalar c = C(j, j'):  a(j') = a'(j') - c d_j,  a(j')'d_i = a'(j')'d_i - c G(i, j)
// (i != j) and a(j')'d_j directly.  Rows of C, G, P that a phase rewrites are never read in it.

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Warp sum of M values per lane (M = 1, 2 or 4) in one shuffle tree: the first log2(M) levels
// exchange halves of the value set, so M values cost M - 1 + 5 - log2(M) shuffles instead of 5 M.
// Every lane returns the full sum of value (lane >> (5 - log2 M)).
template <int M>
__device__ __forceinline__ float warp_sum_multi(const float (&v)[M], int lane) {
  float b;
  if constexpr (M == 4) {
    const bool u16 = lane & 16, u8 = lane & 8;
    const float a0 = (u16 ? v[2] : v[0]) + __shfl_xor_sync(KSVD_FULL_MASK, u16 ? v[0] : v[2], 16);
    const float a1 = (u16 ? v[3] : v[1]) + __shfl_xor_sync(KSVD_FULL_MASK, u16 ? v[1] : v[3], 16);
    b = (u8 ? a1 : a0) + __shfl_xor_sync(KSVD_FULL_MASK, u8 ? a0 : a1, 8);
    b += __shfl_xor_sync(KSVD_FULL_MASK, b, 4);
  } else if constexpr (M == 2) {
    const bool u16 = lane & 16;
    b = (u16 ? v[1] : v[0]) + __shfl_xor_sync(KSVD_FULL_MASK, u16 ? v[0] : v[1], 16);
    b += __shfl_xor_sync(KSVD_FULL_MASK, b, 8);
    b += __shfl_xor_sync(KSVD_FULL_MASK, b, 4);
  } else {
    b = v[0];
#pragma unroll
    for (int o = 16; o >= 4; o >>= 1) b += __shfl_xor_sync(KSVD_FULL_MASK, b, o);
  }
  b += __shfl_xor_sync(KSVD_FULL_MASK, b, 2);
  b += __shfl_xor_sync(KSVD_FULL_MASK, b, 1);
  return b;
}

// Brings every 128-byte line of [p, p + bytes) into L2: one L2-only load per line whose value is
// never used (nothing waits for it).  Measured better than prefetch.global.L2, which the memory
// system may drop, and than bulk prefetches, which queue on the SM's single TMA unit.
__device__ __forceinline__ void prefetch_l2_lines(const void* p, uint32_t bytes) {
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(127);
  const uintptr_t a1 = reinterpret_cast<uintptr_t>(p) + bytes;
  for (uintptr_t a = a0; a < a1; a += 128) {
    // the load itself is the point: its result goes to a PTX-local register
    asm volatile("{\n .reg .b32 t;\n ld.global.cg.b32 t, [%0];\n}" ::"l"(a) : "memory");
  }
}

// Generation barrier over all CTAs of the cooperative launch.  Bounded: returns false (and
// records kDevErrTimeout) if the generation does not advance within the spin limit.
// Grid barrier on a monotonic arrival counter (zeroed by init_state_kernel before the launch):
// barrier number e of the launch is passed once e * nctas CTAs have arrived.  Arriving is one
// fire-and-forget atomic add, so the last CTA to arrive releases the others without a second
// round trip; a spin that runs past kBarrierSpinLimit polls records a timeout and gives up.
// `deferred` runs on every thread after this CTA has arrived and before it waits: work whose
// results no CTA reads before the following barrier overlaps the wait.
template <typename F>
__device__ bool grid_barrier_with(unsigned* bar, unsigned nctas, unsigned* epoch, int* dev_err,
                                  int* sflag, F deferred) {
  __syncthreads();
  const unsigned target = (*epoch + 1) * nctas;
  if (threadIdx.x == 0) {
    ++*epoch;
    // arrive with release semantics: the CTA barrier above orders every thread's writes before
    // it, and the release makes them visible to the CTAs whose acquire load sees the count
    // (cheaper than a sequentially consistent fence and a relaxed add: 10.0 -> 9.6 ms per sweep)
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
  }
  deferred();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned spins = 0;
    while (ld_acquire_gpu(bar) < target) {
      if (++spins > kBarrierSpinLimit) { ok = 0; atomicOr(dev_err, kDevErrTimeout); break; }
      if (spins > 4096) __nanosleep(100);
    }
    *sflag = ok;
  }
  __syncthreads();
  const bool ok = *sflag != 0;
  __syncthreads();
  return ok;
}

__device__ bool grid_barrier(unsigned* bar, unsigned nctas, unsigned* epoch, int* dev_err,
                             int* sflag) {
  return grid_barrier_with(bar, nctas, epoch, dev_err, sflag, [] {});
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
  const int* iter_ctr;
  int max_signals;
  const int32_t* list;
  const int64_t* start;
  const float* Y;
  const float* gn2;
  float* C;
  float* G;
  float* P;
  float* avec;     // 3 x n
  float* aDbuf;    // 2 x Kp
  float* part;
  int32_t* unused;
  int32_t* bitmap;
  int32_t* replaced;
  int64_t* counter;
  int32_t* usecount;
  unsigned* barrier;
  int* dev_err;
};

// HW: coefficient batches by half-warps (T <= 16, n % 4 == 0, n <= 64 (NPL / 2), X 16-byte
// aligned); FULLN: n == 32 NPL.
template <int NPL, bool HW = false, bool FULLN = false>
struct Sweep {
  static constexpr int NW = kSweepThreads / 32;
  static constexpr int HALF = kSweepThreads / 2;                  // threads per warp group
  static constexpr int EB = NPL <= 8 ? 4 : (NPL <= 16 ? 2 : 1);   // entries per warp batch
  const SweepArgs& A;
  float* a_s;      // n     current atom vector a(j)
  float* aD_s;     // Kp    a(j)'D
  float* cpart;    // Kp    this CTA's part of the new row j of C
  float* v_s;      // Kp    C(:, j') for the next atom (its left-out entry 0)
  int32_t* stage;  // 2 x kStageCap: this CTA's list entries of the current / next atom
  int32_t* pos;    // Kp: position of every atom in this sweep's order
  float* red_f;
  int* red_i;
  int* sflag;
  int tid, lane, w, c, nctas, k0, k1;

  __device__ Sweep(const SweepArgs& a, float* sm, float* rf, int* ri, int* sf)
      : A(a), red_f(rf), red_i(ri), sflag(sf) {
    a_s = sm;
    aD_s = a_s + round_up(A.n, 4);        // v_s is read as float4: 16-byte aligned for any n
    cpart = aD_s + A.Kp;
    v_s = cpart + A.Kp;
    stage = reinterpret_cast<int32_t*>(v_s + A.Kp);
    pos = stage + 2 * kStageCap;
    tid = threadIdx.x;
    lane = tid & 31;
    w = tid >> 5;
    c = blockIdx.x;
    nctas = gridDim.x;
    const int kper = (A.K + nctas - 1) / nctas;
    k0 = min(A.K, c * kper);
    k1 = min(A.K, k0 + kper);
  }

  unsigned epoch = 0;   // barriers passed (thread 0's copy is the one used)
  __device__ bool barrier() { return grid_barrier(A.barrier, nctas, &epoch, A.dev_err, sflag); }
  template <typename F>
  __device__ bool barrier_with(F deferred) {
    return grid_barrier_with(A.barrier, nctas, &epoch, A.dev_err, sflag, deferred);
  }

  __device__ float v_entry(int k, int jn, int jx) const {
    return (k >= A.K || k == jx) ? 0.f
                                 : (k == jn ? A.gn2[jn] : __ldcg(A.C + (int64_t)jn * A.Kp + k));
  }

  // Slices of a'(jn) and a'(jn)'D leaving out atom jx, from v_s (loaded and synchronised by
  // the caller), by the threads [gt0, gt0 + gsize) of this CTA.  The left-out atom has weight 0
  // in v_s; its column of D and entry of G may be rewritten concurrently by this phase, but any
  // value read there is finite and is multiplied by that 0.
  __device__ void next_partials(int jn, int jx, float* avec_slot, float* aD_slot, int gt,
                                int gsize) {
    const int n = A.n, Kp = A.Kp;
    const float g2 = A.gn2[jn];
    if (k1 > k0 || c == 0) {
      // two rows per thread at once (n <= 2 gsize in the usual split), so their loads share one
      // round trip
      for (int r0 = gt; r0 < n; r0 += 2 * gsize) {
        const int r1 = r0 + gsize;
        const bool two = r1 < n;
        float acc0 = 0.f, acc1 = 0.f;
#pragma unroll 8
        for (int k = k0; k < k1; ++k) {
          const float vk = v_s[k];
          acc0 = fmaf(-vk, __ldcg(A.D + (int64_t)k * n + r0), acc0);
          if (two) acc1 = fmaf(-vk, __ldcg(A.D + (int64_t)k * n + r1), acc1);
        }
        if (c == 0) {
          acc0 += A.Y[(int64_t)jn * n + r0] + g2 * __ldcg(A.D + (int64_t)jn * n + r0);
          if (two) acc1 += A.Y[(int64_t)jn * n + r1] + g2 * __ldcg(A.D + (int64_t)jn * n + r1);
        }
        atomicAdd(avec_slot + r0, acc0);
        if (two) atomicAdd(avec_slot + r1, acc1);
      }
    }
    const int k4n = Kp >> 2;                          // Kp is a multiple of 128
    const int gw = gt >> 5, gnw = gsize >> 5;
    for (int i = k0 + gw; i < k1; i += gnw) {
      if (i == jx) continue;                          // a(jn)'d_jx is formed after the barrier
      // P(i, jn) and G(i, jn) are loaded with the row of G, in the same round trip
      const float pij = __ldcg(A.P + (int64_t)jn * Kp + i);
      const float gij = __ldcg(A.G + (int64_t)jn * Kp + i);
      const float4* gi = reinterpret_cast<const float4*>(A.G + (int64_t)i * Kp);
      const float4* vv = reinterpret_cast<const float4*>(v_s);
      float acc = 0.f;
#pragma unroll
      for (int u = 0; u < 8; ++u) {                   // Kp <= 1024: at most 8 float4 per lane
        const int k4 = lane + 32 * u;
        if (k4 < k4n) {
          const float4 g = __ldcg(gi + k4);
          const float4 v = vv[k4];
          acc = fmaf(g.x, v.x, fmaf(g.y, v.y, fmaf(g.z, v.z, fmaf(g.w, v.w, acc))));
        }
      }
      acc = warp_sum(acc);
      if (lane == 0) aD_slot[i] = pij - acc + g2 * gij;
    }
  }

  // Row jn of C is rebuilt by atom jn's phase: clear this CTA's slice of it.
  __device__ void zero_row(int jn, int gt, int gsize) {
    for (int k = k0 + gt; k < k1; k += gsize) A.C[(int64_t)k * A.Kp + jn] = 0.f;
  }

  // G(:, j), G(j, :) and P(j, :) for this CTA's atom slice once d_j is final.  Regular path:
  // a_s holds the unnormalised atom and G(i, j) = a'd_i / ||a|| comes from aD_s.  Special case:
  // a_s holds d_j and G(i, j) is recomputed from D.
  __device__ void refresh_gp(int j, float inv_norm, bool from_aD, int gt, int gsize) {
    const int n = A.n, Kp = A.Kp;
    const int gw = gt >> 5, gnw = gsize >> 5;
    for (int i = k0 + gw; i < k1; i += gnw) {
      const float* yi = A.Y + (int64_t)i * n;
      float accp = 0.f, accg = 0.f;
#pragma unroll 8
      for (int r = lane; r < n; r += 32) {
        accp = fmaf(a_s[r], __ldg(yi + r), accp);
        if (!from_aD) accg = fmaf(a_s[r], __ldcg(A.D + (int64_t)i * n + r), accg);
      }
      accp = warp_sum(accp);
      if (!from_aD) accg = warp_sum(accg);
      float g = from_aD ? aD_s[i] * inv_norm : accg * inv_norm;
      if (i == j) g = 1.f;
      if (lane == 0) {
        A.G[(int64_t)j * Kp + i] = g;
        A.G[(int64_t)i * Kp + j] = g;
        A.P[(int64_t)i * Kp + j] = accp * inv_norm;
      }
    }
  }

  // Fold the left-out atom prev back into a(j) and a(j)'D, and load v_s for the next atom jn
  // (leaving out j): every load of the phase's start in one round.  Returns ||a(j)||.
  __device__ float correct(int j, int prev, int jn, const float* avec_slot, const float* aD_slot) {
    const int n = A.n, K = A.K, Kp = A.Kp;
    const float cp = prev >= 0 ? __ldcg(A.C + (int64_t)j * Kp + prev) : 0.f;
    float av[2], dv[2], ad[2], gp[2], vn[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {                     // n, Kp <= 1024 = 2 x 512 threads
      const int r = tid + u * kSweepThreads;
      av[u] = r < n ? __ldcg(avec_slot + r) : 0.f;
      dv[u] = (r < n && prev >= 0) ? __ldcg(A.D + (int64_t)prev * n + r) : 0.f;
      const int i = r;
      const bool ok = i < K && i != prev;
      ad[u] = ok ? __ldcg(aD_slot + i) : 0.f;
      gp[u] = (ok && prev >= 0) ? __ldcg(A.G + (int64_t)prev * Kp + i) : 0.f;
      vn[u] = (jn >= 0 && i < Kp) ? v_entry(i, jn, j) : 0.f;
    }
    float nn = 0.f, dp = 0.f;
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int r = tid + u * kSweepThreads;
      if (r < n) {
        const float a = fmaf(-cp, dv[u], av[u]);
        a_s[r] = a;
        nn = fmaf(a, a, nn);
        dp = fmaf(dv[u], a, dp);
      }
      if (r < Kp) {
        aD_s[r] = fmaf(-cp, gp[u], ad[u]);
        cpart[r] = 0.f;
        v_s[r] = vn[u];
      }
    }
    nn = warp_sum(nn);
    dp = warp_sum(dp);
    if (lane == 0) { red_f[w] = nn; red_f[32 + w] = dp; }
    __syncthreads();
    if (w == 0) {
      nn = lane < NW ? red_f[lane] : 0.f;
      dp = lane < NW ? red_f[32 + lane] : 0.f;
      nn = warp_sum(nn);
      dp = warp_sum(dp);
      if (lane == 0) {
        red_f[0] = nn;
        if (prev >= 0) aD_s[prev] = dp;
      }
    }
    __syncthreads();
    const float anorm = sqrtf(red_f[0]);
    __syncthreads();
    return anorm;
  }

  // Stage this CTA's list entries of the next atom in shared memory (buffer `buf`) and issue L2
  // prefetches of their signals and codes, so the next phase's loads start without a
  // dependent list read and hit L2.
  __device__ void prefetch_next(int jn, int buf, int gt, int gsize) {
    const int64_t q0 = A.start[jn], cnt = A.start[jn + 1] - q0;
    if (cnt == 0) return;
    const int64_t per = (cnt + nctas - 1) / nctas;
    const int64_t qa = q0 + min(cnt, (int64_t)c * per), qb = q0 + min(cnt, (int64_t)(c + 1) * per);
    int32_t* st = stage + buf * kStageCap;
    const DivT dt = div_t_magic(A.T);
    for (int64_t q = qa + gt; q < qb; q += gsize) {
      const int32_t e = A.list[q];
      if (q - qa < kStageCap) st[q - qa] = e;
      const int s = div_t(e, dt);
      prefetch_l2_lines(A.X + (int64_t)s * A.n, (uint32_t)A.n * 4);
      prefetch_l2_lines(A.coef + s * A.T, (uint32_t)A.T * 4);
      prefetch_l2_lines(A.idx + s * A.T, (uint32_t)A.T * 4);
    }
  }

  // update_coefs with half-warps: half h of a warp takes entries h, h + 2, ... of the batch,
  // loads its signal four rows per 16-byte load and slot (lane & 15) of its code row, so a warp
  // instruction serves two entries; the per-entry sums share one 16-lane shuffle tree.
  __device__ void update_coefs_half(int j, int64_t q0, int64_t cnt, float anorm, int buf,
                                    int* next, int* use_cnt) {
    constexpr int NQ = NPL / 2;            // float4 rows per lane
    constexpr int EH = EB / 2;             // entries per half
    static_assert(EB == 2 * EH && EH >= 1 && EH <= 2, "half-warp batches hold 2 or 4 entries");
    const int n = A.n, K = A.K, T = A.T;
    const int hl = lane & 15, hb = lane & 16, half = lane >> 4;
    const float aDj = aD_s[j];
    const int64_t per = (cnt + nctas - 1) / nctas;
    const int64_t qa = q0 + min(cnt, (int64_t)c * per), qb = q0 + min(cnt, (int64_t)(c + 1) * per);
    const int32_t* st = stage + buf * kStageCap;
    const DivT dt = div_t_magic(T);
    // this lane's rows of a(j), fixed through the phase (rows >= n are never read)
    float4 av[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k)
      av[k] = (FULLN || 4 * hl + 64 * k < n) ? reinterpret_cast<const float4*>(a_s)[hl + 16 * k]
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
    int my_use = 0;
    for (;;) {
      int bidx = 0;
      if (lane == 0) bidx = atomicAdd(next, 1);
      bidx = __shfl_sync(KSVD_FULL_MASK, bidx, 0);
      const int64_t qs = qa + (int64_t)bidx * EB;
      if (qs >= qb) break;
      const int ne = (int)min((int64_t)EB, qb - qs);
      int e[EH], s[EH];                      // entries e = signal * T + slot < 2^31
      bool live[EH];
#pragma unroll
      for (int m = 0; m < EH; ++m) {
        const int b = 2 * m + half;
        const int64_t q = qs + b;
        live[m] = b < ne;
        e[m] = live[m] ? (q - qa < kStageCap ? st[q - qa] : A.list[q]) : 0;
        s[m] = div_t(e[m], dt);
      }
      // the signal, its code row slot and its support size, all in one round of loads
      float4 xv[EH][NQ];
#pragma unroll
      for (int m = 0; m < EH; ++m) {
        const float4* xp = reinterpret_cast<const float4*>(A.X + (int64_t)s[m] * n) + hl;
#pragma unroll
        for (int k = 0; k < NQ; ++k)
          xv[m][k] = (live[m] && (FULLN || 4 * hl + 64 * k < n)) ? __ldcg(xp + 16 * k)
                                                                : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      float cf[EH];
      int ix[EH], nz[EH];
#pragma unroll
      for (int m = 0; m < EH; ++m) {
        nz[m] = live[m] ? A.nnz[s[m]] : 0;
        const bool in = live[m] && hl < T;
        ix[m] = in ? A.idx[s[m] * T + hl] : -1;
        cf[m] = in ? __ldcg(A.coef + s[m] * T + hl) : 0.f;
      }
      float dpart[EH], gold[EH];
#pragma unroll
      for (int m = 0; m < EH; ++m) {
        const bool ok = hl < min(nz[m], T) && (unsigned)ix[m] < (unsigned)K;
        ix[m] = ok ? ix[m] : -1;
        cf[m] = ok ? cf[m] : 0.f;
        // gamma_j(s) is slot e % T (< T <= 16) of the code row
        gold[m] = __shfl_sync(KSVD_FULL_MASK, cf[m], hb | (e[m] - s[m] * T));
        // this lane's part of a.x_s - Gamma(:,s).(a'D)
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
          acc = fmaf(av[k].x, xv[m][k].x, acc);
          acc = fmaf(av[k].y, xv[m][k].y, acc);
          acc = fmaf(av[k].z, xv[m][k].z, acc);
          acc = fmaf(av[k].w, xv[m][k].w, acc);
        }
        if (ix[m] >= 0) acc = fmaf(-cf[m], aD_s[ix[m]], acc);
        dpart[m] = acc;
      }
      // sums over each half: with EH = 2 the first level splits the entries (lanes with bit 8
      // keep entry 1), so lane holds the sum of entry (lane >> 3) & (EH - 1) of its half
      float dsum;
      if constexpr (EH == 2) {
        const bool u8 = lane & 8;
        dsum = (u8 ? dpart[1] : dpart[0]) +
               __shfl_xor_sync(KSVD_FULL_MASK, u8 ? dpart[0] : dpart[1], 8);
      } else {
        dsum = dpart[0] + __shfl_xor_sync(KSVD_FULL_MASK, dpart[0], 8);
      }
      dsum += __shfl_xor_sync(KSVD_FULL_MASK, dsum, 4);
      dsum += __shfl_xor_sync(KSVD_FULL_MASK, dsum, 2);
      dsum += __shfl_xor_sync(KSVD_FULL_MASK, dsum, 1);
      const int mm = (lane >> 3) & (EH - 1);
      const float go = (EH == 2 && mm == 1) ? gold[EH - 1] : gold[0];
      const float gmine = (dsum + aDj * go) / anorm;
#pragma unroll
      for (int m = 0; m < EH; ++m) {
        const float g = __shfl_sync(KSVD_FULL_MASK, gmine, hb | (m << 3));
        if (!live[m]) continue;
        if (ix[m] >= 0 && ix[m] != j) atomicAdd(cpart + ix[m], g * cf[m]);
        if (hl == 0) {
          A.coef[e[m]] = g;
          if (g * g > 1e-7f) ++my_use;
        }
      }
    }
    my_use += __shfl_down_sync(KSVD_FULL_MASK, my_use, 16);
    if (lane == 0 && my_use) atomicAdd(use_cnt, my_use);
  }

  // New coefficients of atom j for this CTA's share of its signals, by warps [0, gnw).  Adds
  // into cpart (C row j) and *use_cnt; the caller synchronises and flushes.
  // Warps pull batches of EB entries from a shared counter (*next, zeroed before the phase), so
  // the warps that finish their other work of the phase join in.
  __device__ void update_coefs(int j, int64_t q0, int64_t cnt, float anorm, int buf, int* next,
                               int* use_cnt) {
    if constexpr (HW) {
      update_coefs_half(j, q0, cnt, anorm, buf, next, use_cnt);
      return;
    }
    const int n = A.n, K = A.K, T = A.T;
    const float aDj = aD_s[j];
    const int64_t per = (cnt + nctas - 1) / nctas;
    const int64_t qa = q0 + min(cnt, (int64_t)c * per), qb = q0 + min(cnt, (int64_t)(c + 1) * per);
    const int32_t* st = stage + buf * kStageCap;
    const DivT dt = div_t_magic(T);
    int my_use = 0;
    for (;;) {
      int bidx = 0;
      if (lane == 0) bidx = atomicAdd(next, 1);
      bidx = __shfl_sync(KSVD_FULL_MASK, bidx, 0);
      const int64_t qs = qa + (int64_t)bidx * EB;
      if (qs >= qb) break;
      const int ne = (int)min((int64_t)EB, qb - qs);
      int e[EB], s[EB];                      // entries e = signal * T + slot < 2^31
#pragma unroll
      for (int b = 0; b < EB; ++b) {
        const int64_t q = qs + b;
        e[b] = b < ne ? (q - qa < kStageCap ? st[q - qa] : A.list[q]) : 0;
        s[b] = div_t(e[b], dt);
      }
      // the signal, its whole code row and its support size, all in one round of loads
      float xv[EB][NPL];
#pragma unroll
      for (int b = 0; b < EB; ++b) {
        const float* xp = A.X + (int64_t)s[b] * n + lane;
#pragma unroll
        for (int i = 0; i < NPL; ++i)
          xv[b][i] = (b < ne && lane + 32 * i < n) ? __ldcg(xp + 32 * i) : 0.f;
      }
      float cf[EB][2];
      int ix[EB][2], nz[EB];
#pragma unroll
      for (int b = 0; b < EB; ++b) {
        nz[b] = b < ne ? A.nnz[s[b]] : 0;
        const int cb = s[b] * T;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int t = lane + 32 * u;
          const bool in = b < ne && t < T;
          ix[b][u] = in ? A.idx[cb + t] : -1;
          cf[b][u] = in ? __ldcg(A.coef + cb + t) : 0.f;
        }
      }
#pragma unroll
      for (int b = 0; b < EB; ++b) {
        const int lim = min(nz[b], T);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int t = lane + 32 * u;
          const int v = ix[b][u];
          const bool ok = t < lim && v >= 0 && v < K;
          ix[b][u] = ok ? v : -1;
          cf[b][u] = ok ? cf[b][u] : 0.f;
        }
      }
      // this lane's part of a.x_s - Gamma(:,s).(a'D) per entry, summed over the warp in one tree
      float dpart[EB];
#pragma unroll
      for (int b = 0; b < EB; ++b) {
        float acc = 0.f;
#pragma unroll
        for (int i = 0; i < NPL; ++i) {
          const int r = lane + 32 * i;
          if (r < n) acc = fmaf(a_s[r], xv[b][i], acc);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
          if (ix[b][u] >= 0) acc = fmaf(-cf[b][u], aD_s[ix[b][u]], acc);
        dpart[b] = acc;
      }
      const float dsum = warp_sum_multi<EB>(dpart, lane);   // entry lane >> (5 - log2 EB)
      constexpr int SH = EB == 4 ? 3 : (EB == 2 ? 4 : 5);
      float gold[EB];
#pragma unroll
      for (int b = 0; b < EB; ++b) {
        // gamma_j(s) is slot e % T of the code row already in registers
        const int ts = e[b] - s[b] * T;
        gold[b] = __shfl_sync(KSVD_FULL_MASK, (ts >> 5) == 0 ? cf[b][0] : cf[b][1], ts & 31);
      }
      float gmine = 0.f;
      {
        const int mb = lane >> SH;
        float go = gold[0];
#pragma unroll
        for (int b = 1; b < EB; ++b)
          if (mb == b) go = gold[b];
        gmine = (dsum + aDj * go) / anorm;
      }
#pragma unroll
      for (int b = 0; b < EB; ++b) {
        const float g = __shfl_sync(KSVD_FULL_MASK, gmine, (b << SH) & 31);
        if (b >= ne) continue;
#pragma unroll
        for (int u = 0; u < 2; ++u)
          if (ix[b][u] >= 0 && ix[b][u] != j) atomicAdd(cpart + ix[b][u], g * cf[b][u]);
        if (lane == 0) {
          A.coef[e[b]] = g;
          if (g * g > 1e-7f) ++my_use;
        }
      }
    }
    if (lane == 0 && my_use) atomicAdd(use_cnt, my_use);
  }

  // After a CTA barrier: this CTA's part of C row j and of atom j's use count.
  // C(k, j) is read again only when atom k comes later in this sweep (its v = C(k, :)), so
  // the atoms already processed are skipped.
  // urgent: only the next two atoms' entries are read in the next phase (cp = C(j', j) and
  // v = C(j'', :)); the rest is flushed while the CTA waits at the grid barrier.
  __device__ void flush_row(int j, int jj, int k1n, int k2n, bool urgent, const int* use_cnt) {
    for (int k = tid; k < A.K; k += blockDim.x) {
      const bool next_two = k == k1n || k == k2n;
      if (next_two != urgent) continue;
      const float v = cpart[k];
      if (k != j && v != 0.f && pos[k] > jj) atomicAdd(A.C + (int64_t)k * A.Kp + j, v);
    }
    if (!urgent && tid == 0 && *use_cnt) atomicAdd(A.usecount + j, *use_cnt);
  }

  // The worst-represented of the first min(max_signals, N - counter) unused signals replaces
  // atom j (which no signal uses).  Leaves d_j in a_s.  Two grid barriers.
  __device__ bool special_case(int j) {
    const int n = A.n, T = A.T, K = A.K;
    const int64_t counter = *((volatile int64_t*)A.counter);
    const int64_t ncand = min((int64_t)A.max_signals, A.N - counter);
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
    if (!barrier()) return false;
    // every CTA reduces the partials the same way (first maximum) and reads the same signal
    float v = -1.f;
    int bi = 0x7fffffff;
    for (int cc = lane; cc < nctas; cc += 32) {
      const float pv = __ldcg(A.part + cc * 4);
      const int pb = __ldcg(reinterpret_cast<const int*>(A.part) + cc * 4 + 1);
      if (pv > v || (pv == v && pb < bi)) { v = pv; bi = pb; }
    }
    warp_argmax(v, bi);
    const bool have = ncand > 0 && bi >= 0 && bi < ncand;
    int64_t s = 0;
    if (have) s = __ldcg(A.unused + bi);
    float nr = 0.f;
    for (int r = tid; r < n; r += blockDim.x) {
      const float x = have ? A.X[s * n + r] : __ldcg(A.D + (int64_t)j * n + r);
      a_s[r] = x;
      nr = fmaf(x, x, nr);
    }
    nr = sqrtf(block_sum(nr, red_f));
    for (int r = tid; r < n; r += blockDim.x) a_s[r] = have ? a_s[r] / nr : a_s[r];
    __syncthreads();
    if (!barrier()) return false;       // every CTA has read the unused list entry
    if (c == 0 && have) {
      for (int r = tid; r < n; r += blockDim.x) A.D[(int64_t)j * n + r] = a_s[r];
      if (tid == 0) {
        A.unused[bi] = __ldcg(A.unused + (A.N - counter - 1));
        *A.counter = counter + 1;
        A.replaced[j] = 1;
        A.bitmap[s] = 0;
      }
    }
    return true;
  }
};

template <int NPL, bool HW, bool FULLN>
__global__ void __launch_bounds__(kSweepThreads, 1) sweep_kernel(SweepArgs A) {
  extern __shared__ float sm[];
  __shared__ float red_f[64];
  __shared__ int red_i[64];
  __shared__ int sflag;
  __shared__ int use_cnt;
  __shared__ int next_batch;
  Sweep<NPL, HW, FULLN> S(A, sm, red_f, red_i, &sflag);
  const int K = A.K, n = A.n, tid = threadIdx.x;
  constexpr int HALF = Sweep<NPL, HW, FULLN>::HALF;
  const int32_t* perm = A.perm + (A.iter_ctr ? (int64_t)(*A.iter_ctr) * K : 0);
  // every CTA checks the whole permutation itself, so all of them leave together or none does
  int bad = 0;
  for (int k = tid; k < A.Kp; k += blockDim.x) S.pos[k] = K;   // (an order with repeats: no skips)
  __syncthreads();
  for (int k = tid; k < K; k += blockDim.x) {
    const int j = perm[k];
    bad |= (j < 0 || j >= K);
    if (j >= 0 && j < K) S.pos[j] = k;
  }
  if (__syncthreads_or(bad)) {
    if (blockIdx.x == 0 && tid == 0) atomicOr(A.dev_err, kDevErrBounds);
    return;
  }
  // prologue: a(perm[0]) and a(perm[0])'D in full
  {
    const int j0 = perm[0];
    for (int k = tid; k < A.Kp; k += blockDim.x) S.v_s[k] = S.v_entry(k, j0, -1);
    __syncthreads();
    S.next_partials(j0, -1, A.avec, A.aDbuf, tid, blockDim.x);
    S.zero_row(j0, tid, blockDim.x);
    S.prefetch_next(j0, 0, tid, blockDim.x);
    if (!S.barrier()) return;
  }
  for (int jj = 0; jj < K; ++jj) {
    const int j = perm[jj];
    const int prev = jj > 0 ? perm[jj - 1] : -1;
    const int jn = jj + 1 < K ? perm[jj + 1] : -1;
    float* av_next = A.avec + ((jj + 1) % 3) * n;
    float* av_clear = A.avec + ((jj + 2) % 3) * n;
    float* ad_next = A.aDbuf + ((jj + 1) & 1) * A.Kp;
    if (tid == 0) { use_cnt = 0; next_batch = 0; }
    const float anorm = S.correct(j, prev, jn, A.avec + (jj % 3) * n, A.aDbuf + (jj & 1) * A.Kp);
    const int64_t q0 = A.start[j], cnt = A.start[j + 1] - q0;
    if (cnt == 0) {
      // special case: all warps, then the next atom's partials
      if (!S.special_case(j)) return;
      S.refresh_gp(j, 1.f, false, tid, blockDim.x);
      if (jn >= 0) {
        S.next_partials(jn, j, av_next, ad_next, tid, blockDim.x);
        S.zero_row(jn, tid, blockDim.x);
        S.prefetch_next(jn, (jj + 1) & 1, tid, blockDim.x);
      }
    } else if (tid < HALF) {
      // warps 0..7: atom j's new coefficients
      S.update_coefs(j, q0, cnt, anorm, jj & 1, &next_batch, &use_cnt);
    } else {
      // warps 8..15: d_j, G/P rows of j, the next atom's partials, prefetch; then they help
      // with the coefficients
      // two groups of four warps in parallel (the tasks are independent: next_partials gives
      // atom j weight 0, so it may read G/P entries refresh_gp is rewriting)
      const int gt = tid - HALF;
      constexpr int QUART = HALF / 2;
      if (S.c == 0)
        for (int r = gt; r < n; r += HALF) A.D[(int64_t)j * n + r] = S.a_s[r] / anorm;
      // The prefetch goes with the shorter refresh task: the next atom's partials (dependent
      // rounds of L2 loads and atomics) are the longer helper task (measured at n=256, K=1024,
      // N=1M, T=16: partials 6.1 us per atom, refresh 1.6 us, the coefficient warps 5.4 us
      // before the prefetch moved).
      if (gt < QUART) {
        S.refresh_gp(j, 1.f / anorm, true, gt, QUART);
        if (jn >= 0) S.prefetch_next(jn, (jj + 1) & 1, gt, QUART);
      } else if (jn >= 0) {
        S.next_partials(jn, j, av_next, ad_next, gt - QUART, QUART);
        S.zero_row(jn, gt - QUART, QUART);
      }
      S.update_coefs(j, q0, cnt, anorm, jj & 1, &next_batch, &use_cnt);
    }
    __syncthreads();
    const int jn2 = jj + 2 < K ? perm[jj + 2] : -1;
    if (cnt > 0) S.flush_row(j, jj, jn, jn2, true, &use_cnt);
    if (S.c == 0)
      for (int r = tid; r < n; r += blockDim.x) av_clear[r] = 0.f;
    if (!S.barrier_with([&] {
          if (cnt > 0) S.flush_row(j, jj, jn, jn2, false, &use_cnt);
        }))
      return;
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

// Windows of ~32 MB of signals once X exceeds 96 MB (L2 is 129 MB): a window's signals are read
// from HBM once and gathered from L2 by the T atoms of each signal's support.
int64_t prepare_window_signals(int64_t N, int n, int T) {
  constexpr int64_t kWindowBytes = 32ll << 20, kMinX = 96ll << 20;
  if (T > 16 || n % 4 != 0 || n > 256 || N * n * 4 <= kMinX) return 0;
  const int64_t w = std::max<int64_t>(1, kWindowBytes / (4ll * n) / kSigPerBlock) * kSigPerBlock;
  return w < N ? w : 0;
}

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
  const int npl = (a.n + 31) / 32;
  auto launch = [&](auto kern) -> cudaError_t {
    cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)psm);
    if (e2 != cudaSuccess) return e2;
    kern<<<a.Kp, kPrepThreads, psm, st>>>(a.X, a.n, a.T, a.Kp, a.idx, a.coef, a.nnz, a.list,
                                          a.start, a.Y, a.gn2, a.C);
    return cudaGetLastError();
  };
  const bool cw1 = a.T <= 32;
  auto launch_npl = [&](auto npl_c) -> cudaError_t {
    constexpr int P = decltype(npl_c)::value;
    const bool full = a.n == 32 * P;
    if (cw1) return full ? launch(prepare_kernel<P, 1, true>) : launch(prepare_kernel<P, 1, false>);
    return full ? launch(prepare_kernel<P, 2, true>) : launch(prepare_kernel<P, 2, false>);
  };
  auto launch_nq = [&](auto nq_c) -> cudaError_t {
    constexpr int Q = decltype(nq_c)::value;
    return a.n == 64 * Q ? launch(prepare_half_kernel<Q, true>)
                         : launch(prepare_half_kernel<Q, false>);
  };
  // the half-warp kernel when its layout fits (rows of X 16-byte aligned, one slot per lane)
  const bool half = a.T <= 16 && a.n % 4 == 0 && a.n <= 256 &&
                    (reinterpret_cast<uintptr_t>(a.X) & 15) == 0;
  if (half && a.prep_part && a.prep_win > 0 && a.prep_win % kSigPerBlock == 0 &&
      a.prep_win < a.N) {
    const int64_t nwin = (a.N + a.prep_win - 1) / a.prep_win;
    const int64_t bpw = a.prep_win / kSigPerBlock;
    const size_t wsm = sizeof(float) * ((size_t)(kPrepWinThreads / 32) * (a.Kp + a.n));
    auto launch_win = [&](auto kern) -> cudaError_t {
      cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)wsm);
      if (e2 != cudaSuccess) return e2;
      kern<<<(unsigned)(nwin * a.Kp), kPrepWinThreads, wsm, st>>>(
          a.X, a.n, a.T, a.Kp, a.idx, a.coef, a.nnz, a.list, a.start, a.block_hist, nblk, bpw,
          a.prep_part);
      if ((e2 = cudaGetLastError()) != cudaSuccess) return e2;
      prepare_win_reduce<<<1216, 256, 0, st>>>(a.prep_part, nwin, a.n, a.Kp, a.Y, a.gn2, a.C);
      return cudaGetLastError();
    };
    if (a.n <= 64) e = a.n == 64 ? launch_win(prepare_win_kernel<1, true>)
                                 : launch_win(prepare_win_kernel<1, false>);
    else if (a.n <= 128) e = a.n == 128 ? launch_win(prepare_win_kernel<2, true>)
                                        : launch_win(prepare_win_kernel<2, false>);
    else e = a.n == 256 ? launch_win(prepare_win_kernel<4, true>)
                        : launch_win(prepare_win_kernel<4, false>);
  } else if (half && a.n <= 64) e = launch_nq(std::integral_constant<int, 1>());
  else if (half && a.n <= 128) e = launch_nq(std::integral_constant<int, 2>());
  else if (half) e = launch_nq(std::integral_constant<int, 4>());
  else if (npl <= 2) e = launch_npl(std::integral_constant<int, 2>());
  else if (npl <= 4) e = launch_npl(std::integral_constant<int, 4>());
  else if (npl <= 8) e = launch_npl(std::integral_constant<int, 8>());
  else if (npl <= 16) e = launch_npl(std::integral_constant<int, 16>());
  else e = launch_npl(std::integral_constant<int, 32>());
  if (e != cudaSuccess) return e;
  // P = D'Y (P(i, j) = d_i . Y_j at P[j*Kp + i])
  return launch_gemm_tn_f32(a.D, a.n, a.Y, a.n, a.P, a.Kp, a.K, a.Kp, a.K, a.Kp, a.n, st);
}

cudaError_t launch_update_sweep(const UpdateArgs& a, cudaStream_t st) {
  if (a.N <= 0) return cudaSuccess;
  SweepArgs s;
  s.n = a.n; s.K = a.K; s.Kp = a.Kp; s.T = a.T; s.N = a.N; s.X = a.X; s.D = a.D; s.idx = a.idx;
  s.coef = a.coef; s.nnz = a.nnz; s.perm = a.perm; s.iter_ctr = a.iter_ctr; s.max_signals = a.max_signals;
  s.list = a.list; s.start = a.start; s.Y = a.Y; s.gn2 = a.gn2; s.C = a.C; s.G = a.G; s.P = a.P;
  s.avec = a.avec; s.aDbuf = a.aD; s.part = a.part; s.unused = a.unused; s.bitmap = a.bitmap;
  s.replaced = a.replaced; s.counter = a.counter; s.usecount = a.usecount; s.barrier = a.barrier;
  s.dev_err = a.dev_err;
  const size_t smem = sizeof(float) * ((size_t)round_up(a.n, 4) + 3 * (size_t)a.Kp) +
                      sizeof(int32_t) * (2 * kStageCap + (size_t)a.Kp);
  const int npl = (a.n + 31) / 32;
  auto launch = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSweepThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorCooperativeLaunchTooLarge;
    const int full = sweep_grid_size();
    const int grid = a.sweep_ctas > 0 && a.sweep_ctas < full ? a.sweep_ctas : full;
    void* args[] = {&s};
    return cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(kSweepThreads), args,
                                       smem, st);
  };
  // half-warp coefficient batches when their layout fits (as in the half-warp preparation)
  const bool hw = a.T <= 16 && a.n % 4 == 0 && a.n <= 256 &&
                  (reinterpret_cast<uintptr_t>(a.X) & 15) == 0;
  if (hw && a.n <= 64) return a.n == 64 ? launch(sweep_kernel<2, true, true>)
                                        : launch(sweep_kernel<2, true, false>);
  if (hw && a.n <= 128) return a.n == 128 ? launch(sweep_kernel<4, true, true>)
                                          : launch(sweep_kernel<4, true, false>);
  if (hw) return a.n == 256 ? launch(sweep_kernel<8, true, true>)
                            : launch(sweep_kernel<8, true, false>);
  if (npl <= 2) return launch(sweep_kernel<2, false, false>);
  if (npl <= 4) return launch(sweep_kernel<4, false, false>);
  if (npl <= 8) return launch(sweep_kernel<8, false, false>);
  if (npl <= 16) return launch(sweep_kernel<16, false, false>);
  return launch(sweep_kernel<32, false, false>);
}

int update_sweep_ctas() { return sweep_grid_size(); }

}  // namespace ksvd
