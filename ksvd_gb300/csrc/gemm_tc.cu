// gemm_tc.cu -- 5th-generation tensor-core GEMM for the mixed-precision path:
//   C[s*ldc + k] = sum_r A[k][r] * B[s][r]   (alpha0 = D'X and G = D'D)
// with A and B given as BF16 parts of FP32 matrices (x = hi + lo, hi = bf16(x),
// lo = bf16(x - hi)) and FP32 accumulation in tensor memory.  passes = 1 computes hi*hi;
// passes = 3 adds hi*lo + lo*hi, which keeps ~16 mantissa bits of every product (the lo*lo term,
// ~2^-16 relative, is dropped).
//
// One CTA computes a 128 (atoms) x 256 (signals) tile.  Warp 0 lane 0 streams 64-wide inner
// chunks of A and B with TMA (128-byte swizzle, zero fill outside the matrix) into a 2-stage
// ring; warp 1 lane 0 issues tcgen05.mma (M=128, N=256, K=16, kind::f16 with BF16 inputs) and
// frees each stage with tcgen05.commit; all four warps then drain the 128x256 FP32 accumulator
// with tcgen05.ld and store it column by column (128 contiguous bytes per warp and signal).
// 96 KB of shared memory and 256 TMEM columns per CTA let two CTAs share an SM, so one CTA's
// epilogue overlaps the other's MMAs.  Every mbarrier wait is bounded; on timeout the CTA
// records kDevErrTimeout, stops issuing work, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

constexpr int TM = 128, TN = 256, TK = 64;
constexpr int STAGES = 2;
constexpr int A_BYTES = TM * TK * 2;
constexpr int B_BYTES = TN * TK * 2;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 128;
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t kTmemCols = 256;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(const CUtensorMap* map, uint64_t* bar, void* dst, int x,
                                            int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
      "%4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile written by TMA with 128-byte
// swizzle: rows of 128 bytes, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);       // start address
  d |= (uint64_t)1 << 16;                         // leading byte offset (unused when swizzled)
  d |= (uint64_t)(1024 >> 4) << 32;               // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                         // descriptor version
  d |= (uint64_t)2 << 61;                         // 128-byte swizzle
  return d;
}

// kind::f16 instruction descriptor: BF16 A and B, FP32 D, both K-major, M = 128, N = 256.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

struct TcParams {
  float* C;
  int64_t ldc;
  int M;          // rows of C written (atoms)
  int64_t Ncols;  // columns of C written (signals)
  int nk;         // inner chunks of 64
  int passes;     // 1 or 3
  int mtiles;     // atom tiles (grid = mtiles x signal tiles, atom tile fastest)
  int* dev_err;
};

__global__ void __launch_bounds__(128, 2)
gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
               const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo,
               TcParams P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // atom tiles vary fastest, so the CTAs sharing a signal tile run together and the tile is read
  // from HBM once (the others hit L2)
  const int m0 = (int)(blockIdx.x % P.mtiles) * TM;
  const int64_t n0 = (int64_t)(blockIdx.x / P.mtiles) * TN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int items = P.nk * P.passes;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer
    for (int it = 0; it < items; ++it) {
      const int s = it % STAGES;
      const uint32_t use = it / STAGES;
      if (it >= STAGES && !mbar_wait(&empty[s], (use - 1) & 1)) {
        atomicOr(P.dev_err, kDevErrTimeout);
        *(volatile int*)abort_flag = 1;
        // before the CTA releases its shared memory: the loads still in flight land (bounded)
        for (int gg = it - STAGES; gg < it; ++gg) mbar_wait(&full[gg % STAGES], (gg / STAGES) & 1);
        break;
      }
      const int pass = it / P.nk, kc = it % P.nk;
      const CUtensorMap* ta = pass == 2 ? &tmA_lo : &tmA_hi;
      const CUtensorMap* tb = pass == 1 ? &tmB_lo : &tmB_hi;
      uint8_t* sa = smem + s * STAGE_BYTES;
      uint8_t* sb = sa + A_BYTES;
      mbar_expect_tx(&full[s], STAGE_BYTES);
      tma_load_2d(ta, &full[s], sa, kc * TK, m0);
      tma_load_2d(tb, &full[s], sb, kc * TK, (int)n0);
    }
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    bool ok = true;
    for (int it = 0; it < items; ++it) {
      const int s = it % STAGES;
      const uint32_t use = it / STAGES;
      if (!mbar_wait(&full[s], use & 1)) {
        atomicOr(P.dev_err, kDevErrTimeout);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
      const uint32_t sb = sa + A_BYTES;
      const uint64_t ad = sw128_desc(sa), bd = sw128_desc(sb);
#pragma unroll
      for (int j = 0; j < TK / 16; ++j)   // 16 BF16 = 32 bytes per MMA along K
        umma_bf16(tmem, ad + 2 * j, bd + 2 * j, (it > 0 || j > 0) ? 1u : 0u);
      umma_commit(&empty[s]);
    }
    if (!ok) *(volatile int*)abort_flag = 1;
    // done tracks every MMA issued so far: on an abort too, the epilogue's wait on it keeps
    // TMEM allocated until they have finished
    umma_commit(done);
  }
  __syncwarp();

  // ---- epilogue: every warp drains its 32 TMEM lanes (atoms m0 + 32*warp + lane)
  bool have = true;
  if (!mbar_wait(done, 0)) {
    have = false;
    if (lane == 0) atomicOr(P.dev_err, kDevErrTimeout);
  }
  have = have && (*(volatile int*)abort_flag == 0);
  have = __all_sync(KSVD_FULL_MASK, have);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (have) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
      uint32_t v[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
            "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
            "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
            "=r"(v[31])
          : "r"(taddr + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < P.M) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int64_t s = n0 + c0 + j;
          if (s < P.Ncols) __stcs(P.C + s * P.ldc + row, __uint_as_float(v[j]));
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// Persistent variant for many tiles: one CTA per SM walks tiles t = blockIdx.x, +gridDim.x, ...
// (atom tile fastest).  Warp 0 lane 0 streams the inner chunks through a 4-stage TMA ring,
// warp 1 lane 0 issues the MMAs into one of two 256-column TMEM accumulators, and warps 2-5
// drain the other accumulator (each warp the TMEM lane quarter warp % 4 allows it): the
// epilogue of tile t overlaps the MMAs of tile t+1.  Accumulator hand-off: tmem_full[b] (MMA
// commit -> epilogue) and tmem_empty[b] (one arrival per epilogue warp -> MMA).  Every wait is
// bounded; on a timeout the CTA records kDevErrTimeout, the roles stop and TMEM is freed.
constexpr int PSTAGES = 4;
constexpr int P_SMEM_BYTES = PSTAGES * STAGE_BYTES + 1024 + 256;
constexpr uint32_t kTmemColsP = 2 * TN;
constexpr int kEpiWarps = 4;

__global__ void __launch_bounds__(192, 1)
gemm_tc_persistent_kernel(const __grid_constant__ CUtensorMap tmA_hi,
                          const __grid_constant__ CUtensorMap tmA_lo,
                          const __grid_constant__ CUtensorMap tmB_hi,
                          const __grid_constant__ CUtensorMap tmB_lo, TcParams P,
                          int64_t ntiles) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + PSTAGES * STAGE_BYTES);
  uint64_t* empty = full + PSTAGES;
  uint64_t* tfull = empty + PSTAGES;
  uint64_t* tempty = tfull + 2;
  uint64_t* drain = tempty + 2;   // abort: completion of every MMA already issued
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(drain, 1);
    for (int s = 0; s < PSTAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], kEpiWarps);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemColsP)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int items = P.nk * P.passes;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer: one global item counter across the CTA's tiles
      int64_t g = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
        const int m0 = (int)(t % P.mtiles) * TM;
        const int n0 = (int)((t / P.mtiles) * TN);
        for (int it = 0; it < items; ++it, ++g) {
          const int s = (int)(g % PSTAGES);
          const uint32_t use = (uint32_t)(g / PSTAGES);
          if ((g >= PSTAGES && !mbar_wait(&empty[s], (use - 1) & 1)) ||
              *(volatile int*)abort_flag) {
            if (!*(volatile int*)abort_flag) atomicOr(P.dev_err, kDevErrTimeout);
            *(volatile int*)abort_flag = 1;
            ok = false;
            // before the CTA releases its shared memory: the loads still in flight land
            for (int64_t gg = g >= PSTAGES ? g - PSTAGES : 0; gg < g; ++gg)
              mbar_wait(&full[gg % PSTAGES], (uint32_t)(gg / PSTAGES) & 1);
            break;
          }
          const int pass = it / P.nk, kc = it % P.nk;
          const CUtensorMap* ta = pass == 2 ? &tmA_lo : &tmA_hi;
          const CUtensorMap* tb = pass == 1 ? &tmB_lo : &tmB_hi;
          uint8_t* sa = smem + s * STAGE_BYTES;
          uint8_t* sb = sa + A_BYTES;
          mbar_expect_tx(&full[s], STAGE_BYTES);
          tma_load_2d(ta, &full[s], sa, kc * TK, m0);
          tma_load_2d(tb, &full[s], sb, kc * TK, n0);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: tile lt of this CTA accumulates into buffer lt & 1
      int64_t g = 0;
      bool ok = true;
      int lt = 0;
      for (int64_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x, ++lt) {
        const int b = lt & 1;
        const uint32_t tuse = (uint32_t)(lt >> 1);
        if (lt >= 2 && !mbar_wait(&tempty[b], (tuse - 1) & 1)) {
          atomicOr(P.dev_err, kDevErrTimeout);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t tacc = tmem + (uint32_t)(b * TN);
        for (int it = 0; it < items; ++it, ++g) {
          const int s = (int)(g % PSTAGES);
          const uint32_t use = (uint32_t)(g / PSTAGES);
          if (!mbar_wait(&full[s], use & 1) || *(volatile int*)abort_flag) {
            if (!*(volatile int*)abort_flag) atomicOr(P.dev_err, kDevErrTimeout);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
          const uint32_t sb = sa + A_BYTES;
          const uint64_t ad = sw128_desc(sa), bd = sw128_desc(sb);
#pragma unroll
          for (int j = 0; j < TK / 16; ++j)
            umma_bf16(tacc, ad + 2 * j, bd + 2 * j, (it > 0 || j > 0) ? 1u : 0u);
          umma_commit(&empty[s]);
        }
        if (ok) umma_commit(&tfull[b]);
      }
      if (!ok) {
        *(volatile int*)abort_flag = 1;
        // the MMAs already issued finish before TMEM is released (bounded wait)
        umma_commit(drain);
        mbar_wait(drain, 0);
      }
    }
  } else {
    // ---- epilogue warps 2..5: TMEM lanes (atoms m0 + 32 * (warp % 4) + lane)
    const int q = warp & 3;
    int lt = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
      const int b = lt & 1;
      const uint32_t tuse = (uint32_t)(lt >> 1);
      const int m0 = (int)(t % P.mtiles) * TM;
      const int64_t n0 = (t / P.mtiles) * TN;
      bool have = mbar_wait(&tfull[b], tuse & 1);
      have = __all_sync(KSVD_FULL_MASK, have && *(volatile int*)abort_flag == 0);
      if (!have) {
        if (lane == 0) atomicOr(P.dev_err, kDevErrTimeout);
        *(volatile int*)abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int row = m0 + q * 32 + lane;
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * TN);
#pragma unroll 1
      for (int c0 = 0; c0 < TN; c0 += 32) {
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
            "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
              "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
              "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
              "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
              "=r"(v[31])
            : "r"(taddr + (uint32_t)c0));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row < P.M) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int64_t s = n0 + c0 + j;
            if (s < P.Ncols) __stcs(P.C + s * P.ldc + row, __uint_as_float(v[j]));
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);   // this warp is done with the accumulator
    }
  }
  __syncwarp();                        // warps 0 and 1: lane 0 rejoins the others
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemColsP)
                 : "memory");
  }
}

__global__ void split_bf16_kernel(const float* __restrict__ in, int64_t ld_in, int64_t rows,
                                  int inner, __nv_bfloat16* __restrict__ hi,
                                  __nv_bfloat16* __restrict__ lo, int64_t ld_out,
                                  int64_t rows_out) {
  const int64_t total = rows_out * ld_out;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / ld_out;
    const int c = (int)(e - r * ld_out);
    const float v = (r < rows && c < inner) ? in[r * ld_in + c] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    hi[e] = h;
    if (lo) lo[e] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    cudaGetLastError();
  }
  return fn;
}

// 2-D BF16 tensor map: inner dimension `inner` (elements), `rows` rows `ld` elements apart,
// box = 64 x box_rows, 128-byte swizzle, zero fill outside.
bool make_map(CUtensorMap* m, const uint16_t* base, int64_t ld, int64_t rows, int inner,
              int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || !base) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)TK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<uint16_t*>(base), dims, strides,
            box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t launch_split_bf16(const float* in, int64_t ld_in, int64_t rows, int inner,
                              uint16_t* hi, uint16_t* lo, int64_t ld_out, int64_t rows_out,
                              cudaStream_t st) {
  if (rows_out <= 0) return cudaSuccess;
  int64_t blocks = (rows_out * ld_out + 255) / 256;
  if (blocks > 65535LL * 32) blocks = 65535LL * 32;
  split_bf16_kernel<<<(unsigned)blocks, 256, 0, st>>>(
      in, ld_in, rows, inner, reinterpret_cast<__nv_bfloat16*>(hi),
      reinterpret_cast<__nv_bfloat16*>(lo), ld_out, rows_out);
  return cudaGetLastError();
}

int tc_tile_atoms() { return TM; }
int tc_tile_signals() { return TN; }

cudaError_t launch_gemm_tn_bf16(const TcOperand& A, const TcOperand& B, float* C, int64_t ldc,
                                int M, int64_t Ncols, int inner, int passes, int* dev_err,
                                cudaStream_t st) {
  if (M <= 0 || Ncols <= 0) return cudaSuccess;
  if ((passes != 1 && passes != 3) || inner < 1 || (A.ld & 7) || (B.ld & 7) ||
      ((uintptr_t)A.hi & 15) || ((uintptr_t)B.hi & 15) || A.rows % TM || A.rows < M)
    return cudaErrorInvalidValue;
  if (passes == 3 && (!A.lo || !B.lo || ((uintptr_t)A.lo & 15) || ((uintptr_t)B.lo & 15)))
    return cudaErrorInvalidValue;
  CUtensorMap ma_hi, ma_lo, mb_hi, mb_lo;
  if (!make_map(&ma_hi, A.hi, A.ld, A.rows, inner, TM) ||
      !make_map(&mb_hi, B.hi, B.ld, B.rows, inner, TN))
    return cudaErrorNotSupported;
  if (passes == 3) {
    if (!make_map(&ma_lo, A.lo, A.ld, A.rows, inner, TM) ||
        !make_map(&mb_lo, B.lo, B.ld, B.rows, inner, TN))
      return cudaErrorNotSupported;
  } else {
    ma_lo = ma_hi;
    mb_lo = mb_hi;
  }
  TcParams P;
  P.C = C;
  P.ldc = ldc;
  P.M = M;
  P.Ncols = Ncols;
  P.nk = (inner + TK - 1) / TK;
  P.passes = passes;
  P.dev_err = dev_err;
  const int64_t gx = (Ncols + TN - 1) / TN;
  const int gy = (M + TM - 1) / TM;
  if (gx * gy > 0x7fffffffLL) return cudaErrorInvalidValue;
  P.mtiles = gy;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t ntiles = gx * gy;
  cudaError_t e;
  if (ntiles > sms) {
    // many tiles: persistent CTAs, the epilogue of one tile under the MMAs of the next
    e = cudaFuncSetAttribute(gemm_tc_persistent_kernel,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, P_SMEM_BYTES);
    if (e != cudaSuccess) return e;
    gemm_tc_persistent_kernel<<<(unsigned)sms, 192, P_SMEM_BYTES, st>>>(ma_hi, ma_lo, mb_hi,
                                                                          mb_lo, P, ntiles);
    return cudaGetLastError();
  }
  e = cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           SMEM_BYTES);
  if (e != cudaSuccess) return e;
  gemm_tc_kernel<<<(unsigned)ntiles, 128, SMEM_BYTES, st>>>(ma_hi, ma_lo, mb_hi, mb_lo, P);
  return cudaGetLastError();
}

}  // namespace ksvd
