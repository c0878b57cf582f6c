// gemm_simt.cu -- FP32 CUDA-core GEMM for the plain-FP32 path:  C = A' B  with both operands
// stored "inner dimension contiguous" (column-major n x M and n x Ncols), i.e. the reference's
// AT_times_B (Multiplication.cu:40-63) used for G = D'D (KSVD.cu:64) and alpha0 = D'X
// (OMP.cu:44).  C is column-major M x Ncols with leading dimension ldc, so each signal's
// correlations are contiguous (the layout the OMP kernel streams).
//
// Tile 128 (atoms) x 128 (signals) x 8 (inner), 256 threads, 8x8 outputs per thread, register
// double buffering of the next inner slice.  Warp layout puts 16 threads along the atom axis so
// the epilogue writes 256 contiguous bytes per signal.
#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

constexpr int BM = 128, BN = 128, BK = 8, NT = 256;

// One 128 x 128 output tile at (m0 atoms, n0 signals).
__device__ __forceinline__ void gemm_tile(const float* __restrict__ A, int64_t lda,
                                          const float* __restrict__ B, int64_t ldb,
                                          float* __restrict__ C, int64_t ldc, int M, int Mst,
                                          int64_t Ncols, int64_t Nst, int inner, bool vec_a,
                                          bool vec_b, bool vec_c, int64_t m0, int64_t n0,
                                          float (&As)[2][BK][BM], float (&Bs)[2][BK][BN]) {
  const int tid = threadIdx.x;
  const int ty = tid & 15, tx = tid >> 4;

  // loader coordinates: row (atom or signal) and 4-wide inner offset
  const int lrow = tid >> 1, lc4 = (tid & 1) * 4;
  const int64_t arow = m0 + lrow, brow = n0 + lrow;
  const float* Ap = A + arow * lda;
  const float* Bp = B + brow * ldb;

  float ra[4], rb[4];
  auto load = [&](int r0) {
    const int r = r0 + lc4;
    if (arow < M && vec_a && r + 3 < inner) {
      float4 v = *reinterpret_cast<const float4*>(Ap + r);
      ra[0] = v.x; ra[1] = v.y; ra[2] = v.z; ra[3] = v.w;
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) ra[q] = (arow < M && r + q < inner) ? Ap[r + q] : 0.0f;
    }
    if (brow < Ncols && vec_b && r + 3 < inner) {
      float4 v = __ldcs(reinterpret_cast<const float4*>(Bp + r));
      rb[0] = v.x; rb[1] = v.y; rb[2] = v.z; rb[3] = v.w;
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) rb[q] = (brow < Ncols && r + q < inner) ? Bp[r + q] : 0.0f;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      As[buf][lc4 + q][lrow] = ra[q];
      Bs[buf][lc4 + q][lrow] = rb[q];
    }
  };

  // accumulators as packed pairs (acc2[i][jp] = outputs (i, 2jp) and (i, 2jp+1)): one packed
  // FP32 FMA per two outputs halves the issue slots of the inner product (same rounding as fmaf)
  float2 acc2[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc2[i][j] = make_float2(0.0f, 0.0f);

  const int nk = (inner + BK - 1) / BK;
  load(0);
  store(0);
  __syncthreads();
  for (int kt = 0; kt < nk; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < nk) load((kt + 1) * BK);
#pragma unroll
    for (int r = 0; r < BK; ++r) {
      float4 a0 = *reinterpret_cast<const float4*>(&As[buf][r][ty * 4]);
      float4 a1 = *reinterpret_cast<const float4*>(&As[buf][r][64 + ty * 4]);
      float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][r][tx * 4]);
      float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][r][64 + tx * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float2 b2[4] = {make_float2(b0.x, b0.y), make_float2(b0.z, b0.w),
                            make_float2(b1.x, b1.y), make_float2(b1.z, b1.w)};
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float2 ai = make_float2(a[i], a[i]);
#pragma unroll
        for (int j = 0; j < 4; ++j) acc2[i][j] = __ffma2_rn(ai, b2[j], acc2[i][j]);
      }
    }
    if (kt + 1 < nk) {
      store(buf ^ 1);
      __syncthreads();
    }
  }

  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      acc[i][2 * j] = acc2[i][j].x;
      acc[i][2 * j + 1] = acc2[i][j].y;
    }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int64_t s = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
    if (s >= Nst) continue;
    float* Cp = C + s * ldc;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t k = m0 + h * 64 + ty * 4;
      if (vec_c && k + 3 < Mst) {
        __stcs(reinterpret_cast<float4*>(Cp + k),
               make_float4(acc[h * 4 + 0][j], acc[h * 4 + 1][j], acc[h * 4 + 2][j],
                           acc[h * 4 + 3][j]));
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (k + q < Mst) Cp[k + q] = acc[h * 4 + q][j];
      }
    }
  }
}

__global__ void __launch_bounds__(NT, 2)
gemm_tn_f32_kernel(const float* __restrict__ A, int64_t lda, const float* __restrict__ B,
                   int64_t ldb, float* __restrict__ C, int64_t ldc, int M, int Mst, int64_t Ncols,
                   int64_t Nst, int inner, bool vec_a, bool vec_b, bool vec_c) {
  __shared__ __align__(16) float As[2][BK][BM];
  __shared__ __align__(16) float Bs[2][BK][BN];
  gemm_tile(A, lda, B, ldb, C, ldc, M, Mst, Ncols, Nst, inner, vec_a, vec_b, vec_c,
            (int64_t)blockIdx.y * BM, (int64_t)blockIdx.x * BN, As, Bs);
}

// Many independent products in one launch: block b works on the tile of the problem whose tile
// range [tile_begin, tile_begin + tiles_m * tiles_n) holds b (binary search over the table).
__global__ void __launch_bounds__(NT, 2)
gemm_tn_f32_grouped_kernel(const GemmDesc* __restrict__ descs, int ndesc) {
  __shared__ __align__(16) float As[2][BK][BM];
  __shared__ __align__(16) float Bs[2][BK][BN];
  const int64_t b = blockIdx.x;
  int lo = 0, hi = ndesc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (descs[mid].tile_begin <= b) lo = mid; else hi = mid - 1;
  }
  const GemmDesc& d = descs[lo];
  const int64_t t = b - d.tile_begin;
  if (t >= (int64_t)d.tiles_m * d.tiles_n) return;
  gemm_tile(d.A, d.lda, d.B, d.ldb, d.C, d.ldc, d.M_load, d.M_store, d.N_load, d.N_store,
            d.inner, d.vec_a, d.vec_b, d.vec_c, (t % d.tiles_m) * BM, (t / d.tiles_m) * BN, As,
            Bs);
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace

cudaError_t launch_gemm_tn_f32(const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                               int64_t ldc, int M_load, int M_store, int64_t N_load,
                               int64_t N_store, int inner, cudaStream_t st) {
  if (M_store <= 0 || N_store <= 0) return cudaSuccess;
  if (M_load > M_store || N_load > N_store) return cudaErrorInvalidValue;
  const int64_t gx = (N_store + BN - 1) / BN;
  const int64_t gy = (M_store + BM - 1) / BM;
  if (gy > 65535 || gx > 0x7fffffffLL) return cudaErrorInvalidValue;
  const bool va = (lda % 4 == 0) && aligned16(A);
  const bool vb = (ldb % 4 == 0) && aligned16(B);
  const bool vc = (ldc % 4 == 0) && aligned16(C);
  dim3 grid((unsigned)gx, (unsigned)gy);
  gemm_tn_f32_kernel<<<grid, NT, 0, st>>>(A, lda, B, ldb, C, ldc, M_load, M_store, N_load,
                                          N_store, inner, va, vb, vc);
  return cudaGetLastError();
}

int64_t gemm_desc_fill(GemmDesc& d, const float* A, int64_t lda, const float* B, int64_t ldb,
                       float* C, int64_t ldc, int M_load, int M_store, int64_t N_load,
                       int64_t N_store, int inner, int64_t tile_begin) {
  d.A = A; d.lda = lda; d.B = B; d.ldb = ldb; d.C = C; d.ldc = ldc;
  d.M_load = M_load; d.M_store = M_store; d.N_load = N_load; d.N_store = N_store;
  d.inner = inner;
  d.vec_a = (lda % 4 == 0) && aligned16(A);
  d.vec_b = (ldb % 4 == 0) && aligned16(B);
  d.vec_c = (ldc % 4 == 0) && aligned16(C);
  d.tiles_m = (int)((M_store + BM - 1) / BM);
  d.tiles_n = (N_store + BN - 1) / BN;
  d.tile_begin = tile_begin;
  return tile_begin + (int64_t)d.tiles_m * d.tiles_n;
}

cudaError_t launch_gemm_tn_f32_grouped(const GemmDesc* descs_dev, int ndesc, int64_t total_tiles,
                                       cudaStream_t st) {
  if (ndesc <= 0 || total_tiles <= 0) return cudaSuccess;
  if (total_tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  gemm_tn_f32_grouped_kernel<<<(unsigned)total_tiles, NT, 0, st>>>(descs_dev, ndesc);
  return cudaGetLastError();
}

}  // namespace ksvd
