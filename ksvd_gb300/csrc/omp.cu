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
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace ksvd {
namespace {

constexpr int kOmpWarps = 8;
constexpr int kOmpClaim = 4;   // signals per work-queue claim of the single-problem kernel

// Shared-memory layout of the Cholesky factor L (TMAX x TMAX, lower): rows of stride TMAX+1
// (bank-conflict padding) up to TMAX = 32; for TMAX = 64 packed by rows (row r at r(r+1)/2),
// half the space, so two CTAs fit on an SM.  The diagonal slots hold 1 / L_ii (the triangular
// solves multiply instead of dividing).
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
template <int SPL>
__device__ __forceinline__ unsigned pick(const unsigned (&a)[SPL], int j) {
  if constexpr (SPL == 1) return a[0];
  else return j == 0 ? a[0] : a[1];
}
template <int SPL, typename V>
__device__ __forceinline__ void put(V (&a)[SPL], int j, V v) {
  if constexpr (SPL == 1) a[0] = v;
  else { if (j == 0) a[0] = v; else a[1] = v; }
}

// 8-byte read-only load (four FP16 values) that does not allocate in L1
__device__ __forceinline__ uint2 ldg_u2_no_l1(const void* p) {
  uint2 g;
  asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0,%1}, [%2];"
               : "=r"(g.x), "=r"(g.y)
               : "l"(p));
  return g;
}

// 16-byte read-only load (eight FP16 values) that does not allocate in L1
__device__ __forceinline__ uint4 ldg_u4_no_l1(const void* p) {
  uint4 g;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(g.x), "=r"(g.y), "=r"(g.z), "=r"(g.w)
               : "l"(p));
  return g;
}

// a0 += lo(g) * c, a1 += hi(g) * c: FP16 products accumulated in FP32 (one mixed-precision FMA
// per element, no conversion instructions)
__device__ __forceinline__ void fma2_f16_f32(uint32_t g, unsigned short c, float& a0, float& a1) {
  asm("{\n .reg .f16 lo, hi;\n mov.b32 {lo, hi}, %2;\n fma.rn.f32.f16 %0, lo, %3, %0;\n"
      " fma.rn.f32.f16 %1, hi, %3, %1;\n}"
      : "+f"(a0), "+f"(a1)
      : "r"(g), "h"(c));
}

// Near-tie resolution of the FP16 alpha update: at most this many atoms are re-evaluated in FP32
// per step; more candidates (or a maximum too small to trust) recompute the whole alpha in FP32.
constexpr int kMaxCand = 8;

// Rigorous bound on |alpha~_k - alpha_k| for an atom k outside the support of i atoms, where
// alpha~_k = fl(alpha0_k - S acc_k), acc_k the FP32-accumulated sum of fp16(G(k, I_r)) c~_r with
// c~_r = fp16(c_r / S) (S = 2^ex > ||c||_1), and alpha_k = fl(alpha0_k - s_k) with s_k the FP32
// kernel's FMA chain over the same terms.  With |G(k, I_r)| <= mu_r (the coherence of support
// column I_r), w1 = sum_r mu_r |c_r| and cl1 = ||c||_1:
//   FP16 rounding: |fp16(g) - g| <= 2^-11 |g| + 2^-25, |c~ S - c| <= 2^-11 |c| + 2^-25 S, so
//   the products differ by <= 2^-10 |g c| + 2^-25 |c| (1 + 2^-11) + 2^-25 S |g| (1 + 2^-11),
//   and sum_r S mu_r <= 2 i cl1;
//   the two FMA chains of i terms add <= 2 i 2^-24 (1 + 2^-9) w1 (products exact in FP32);
//   the final subtractions add <= 2^-24 (|alpha~_k| + |alpha_k|) <= 2^-23 a (1 + 2^-9),
//   a = the largest |alpha~| over the atoms.
// Generous constants: eb = w1 (2^-10 + (i + 2) 2^-22) + cl1 (2^-24 + (i + 1) 2^-23) + a 2^-22.
// For a support atom k = I_q the column's own term has |G(k, k)| <= 1 + d_q (d_q = |G(k, k) - 1|)
// instead of mu_q: its bound is eb + 2^-9 (1 + d_q) |c_q|.
__device__ __forceinline__ float alpha_bound(float w1, float cl1, int i, float a) {
  return w1 * (ldexpf(1.f, -10) + (float)(i + 2) * ldexpf(1.f, -22)) +
         cl1 * (ldexpf(1.f, -24) + (float)(i + 1) * ldexpf(1.f, -23)) + a * ldexpf(1.f, -22);
}

// Batch-OMP of one signal by one warp.  a0col: the signal's alpha0 column (Kp = 32*KPL rows,
// rows >= K zero); L: the Cholesky factor (first T rows of the TMAX layout), a0s: 32*KPL floats
// and cand: kMaxCand ints of this warp's shared memory.  emode: stop once ||x||^2 - ||y||^2 <= e2
// (xn2 = ||x||^2).  Writes T slots of idx/coef and nnz.
//
// H16 (mixed path): alpha = alpha0 - G(:, I) c is formed from an FP16 copy Gh of G (half the L2
// bytes of the re-read support columns; c scaled by a power of two into FP16 range, products
// accumulated in FP32), with the rigorous per-atom error bound eb of alpha_bound() (mu_col: the
// per-column coherence).  The FP32 kernel's choice is provably among the atoms whose
// approximate |alpha| lies within 2 eb of the maximum (key truncation and the strictness of the
// squared comparison covered by a 2^-17 relative margin), provided no support atom can compete:
// a support atom's FP32 alpha is the residual of the FP32 Cholesky solve, at most
// (5 i + 4) 2^-24 ||c||_1 + max_q d_q |c_q| (backward error of Cholesky factorisation and solves,
// rows of L of unit norm; the pivot uses 1 for G(p, p)), plus its own approximation bound.  Those
// candidates are re-evaluated in FP32 with exactly the FP32 path's operations and the first
// maximum among them wins, so the selection, the stop tests and the coefficients are those of
// the FP32 Batch-OMP.  When the maximum does not stand clear of 4 eb, of the support atoms'
// reach or of the stop threshold, or more than kMaxCand atoms are candidates, the step's alpha
// is recomputed in FP32.
template <int KPL, int TMAX, bool H16>
__device__ __forceinline__ void omp_signal(const float* __restrict__ G,
                                           const uint16_t* __restrict__ Gh,
                                           const float* __restrict__ mu_col,
                                           int64_t ldg, const float* __restrict__ a0col, int K,
                                           int T, bool emode, float e2, float xn2,
                                           int32_t* __restrict__ idx_s, float* __restrict__ coef_s,
                                           int32_t* __restrict__ nnz_s, float* L, float* a0s,
                                           int* cand, bool& numeric_bad) {
  // lane layout of alpha: groups of V consecutive rows, lane owns rows 32*V*g + V*lane + q
  // (V = 8 lets the FP16 update read 16 bytes per load)
  constexpr int V = (H16 && KPL >= 8) ? 8 : 4;
  constexpr int NG = KPL / V;
  constexpr int SPL = TMAX / 32; // support slots per lane; lane owns slots lane + 32*j
  const int lane = threadIdx.x & 31;
  // H16: the dictionary's largest |G(k, k) - 1| (stored after the Kp column coherences)
  const float dmax = H16 ? __ldg(mu_col + 32 * KPL) : 0.f;
  // Rows >= K of G and alpha0 are zero (every caller pads them), so the padded atoms' alpha
  // stays 0 (or NaN) and never wins a strict comparison against the first real atom: the
  // per-element passes need no k < K test.
  {
    float al[NG][V];
    const float* a0p = a0col + V * lane;
    __syncwarp();                      // the previous signal's last reads of a0s are done
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
      for (int h = 0; h < V / 4; ++h) {
        const float4 v = __ldcs(reinterpret_cast<const float4*>(a0p + 32 * V * g + 4 * h));
        *reinterpret_cast<float4*>(a0s + 32 * V * g + V * lane + 4 * h) = v;
        al[g][4 * h] = v.x; al[g][4 * h + 1] = v.y; al[g][4 * h + 2] = v.z; al[g][4 * h + 3] = v.w;
      }
    __syncwarp();
    int ind[SPL];
    float y[SPL], c[SPL];
    float muq[SPL];            // H16: coherence of each support column
#pragma unroll
    for (int j = 0; j < SPL; ++j) { ind[j] = -1; y[j] = 0.f; c[j] = 0.f; muq[j] = 0.f; }

    // alpha = alpha0 - G(:, I) c in FP32: one support column per step, in slot order (deeper
    // unrolling measured slower: register pressure); G's columns bypass L1 allocation -- they
    // are reused from L2, not from L1
    auto exact_alpha = [&](int i) {
#pragma unroll
      for (int g = 0; g < NG; ++g)
#pragma unroll
        for (int q = 0; q < V; ++q) al[g][q] = 0.f;
#pragma unroll 1
      for (int r = 0; r < i; ++r) {
        const int rl = r & 31, rj = r >> 5;
        const float cr = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(c, rj), rl);
        const int col = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(ind, rj), rl);
        const float* gp = G + (int64_t)col * ldg + V * lane;
#pragma unroll
        for (int g = 0; g < NG; ++g)
#pragma unroll
          for (int h = 0; h < V / 4; ++h) {
            const float4 gv = ldg_f4_no_l1(gp + 32 * V * g + 4 * h);
            al[g][4 * h] = fmaf(gv.x, cr, al[g][4 * h]);
            al[g][4 * h + 1] = fmaf(gv.y, cr, al[g][4 * h + 1]);
            al[g][4 * h + 2] = fmaf(gv.z, cr, al[g][4 * h + 2]);
            al[g][4 * h + 3] = fmaf(gv.w, cr, al[g][4 * h + 3]);
          }
      }
#pragma unroll
      for (int g = 0; g < NG; ++g)
#pragma unroll
        for (int h = 0; h < V / 4; ++h) {
          const float4 a =
              *reinterpret_cast<const float4*>(a0s + 32 * V * g + V * lane + 4 * h);
          al[g][4 * h] = a.x - al[g][4 * h];
          al[g][4 * h + 1] = a.y - al[g][4 * h + 1];
          al[g][4 * h + 2] = a.z - al[g][4 * h + 2];
          al[g][4 * h + 3] = a.w - al[g][4 * h + 3];
        }
    };
    // argmax of alpha^2 (first maximum); alpha_p^2 is the stop test's value
    auto argmax = [&](float& bv, int& bk) {
      bv = -1.f; bk = 0x7fffffff;
#pragma unroll
      for (int g = 0; g < NG; ++g)
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const int k = 32 * V * g + V * lane + q;
          const float v = al[g][q] * al[g][q];
          if (v > bv) { bv = v; bk = k; }
        }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(KSVD_FULL_MASK, bv, o);
        const int ok = __shfl_xor_sync(KSVD_FULL_MASK, bk, o);
        if (ov > bv || (ov == bv && ok < bk)) { bv = ov; bk = ok; }
      }
    };

    float r2 = xn2;
    int i = 0;
    bool approx = false;   // al holds the FP16 update's alpha
    // this lane's two largest approximate |alpha| as keys, formed by the FP16 update's last pass:
    // the bits of |alpha| (positive floats order like unsigned integers) with the low five
    // mantissa bits replaced by 31 - (the element's slot in the lane), so one unsigned max tracks
    // value and atom together (the truncation, < 2^-18 relative, joins the tie allowance)
    unsigned hk1 = 0u, hk2 = 0u;
    while (i < T) {
      if (emode && r2 <= e2) break;
      float bv;
      int bk;
      if (!H16 || !approx) argmax(bv, bk);
      if constexpr (H16) {
        if (approx) {
          approx = false;
          // warp maximum and runner-up of the approximate |alpha|
          unsigned c1 = hk1, c2 = hk2;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const unsigned o1 = __shfl_xor_sync(KSVD_FULL_MASK, c1, o);
            const unsigned o2 = __shfl_xor_sync(KSVD_FULL_MASK, c2, o);
            c2 = max(max(c2, o2), min(c1, o1));
            c1 = max(c1, o1);
          }
          const int wl = __ffs(__ballot_sync(KSVD_FULL_MASK, hk1 == c1)) - 1;
          const int wb = 31 - (int)(c1 & 31u);
          bk = 32 * V * (wb / V) + V * wl + (wb % V);
          const float b1 = __uint_as_float(c1 & 0x7FFFFFE0u);
          const float b2 = __uint_as_float(c2 & 0x7FFFFFE0u);
          bv = b1 * b1;
          // the bound's inputs: ||c||_1, sum_r mu_r |c_r|, max |c_r|; the support atoms' reach
          // (5 i + 4) 2^-24 ||c||_1 + dmax max|c| (their FP32 alpha) + 2^-9 (1 + dmax) max|c|
          float cl1 = 0.f, w1 = 0.f, cm = 0.f;
#pragma unroll
          for (int j = 0; j < SPL; ++j)
            if (lane + 32 * j < i) {
              const float ac = fabsf(c[j]);
              cl1 += ac;
              w1 = fmaf(pick<SPL>(muq, j), ac, w1);
              cm = fmaxf(cm, ac);
            }
          cl1 = warp_sum(cl1);
          w1 = warp_sum(w1);
          cm = warp_max(cm);
          const float errb = alpha_bound(w1, cl1, i, b1);
          const float reach = (float)(5 * i + 4) * ldexpf(cl1, -24) * 1.01f +
                              cm * (dmax * 1.01f + ldexpf(1.f + dmax, -9));
          const float thr = b1 - 2.f * errb - ldexpf(b1, -17);
          bool full = !(b1 > 4.f * errb) || !(b1 > 1e-6f) || !(b1 <= 3.0e38f) ||
                      !(thr > reach + errb);
          if (!full && !(b2 < thr)) {
            // near tie: every atom within 2 errb of the maximum is a candidate
            unsigned mine = 0;
#pragma unroll
            for (int g = 0; g < NG; ++g)
#pragma unroll
              for (int q = 0; q < V; ++q)
                if (fabsf(al[g][q]) >= thr) mine |= 1u << (V * g + q);
            const int cnt = __popc(mine);
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const int t = __shfl_up_sync(KSVD_FULL_MASK, incl, o);
              if (lane >= o) incl += t;
            }
            const int total = __shfl_sync(KSVD_FULL_MASK, incl, 31);
            full = total > kMaxCand;
            if (!full) {
              // the candidates' alpha in FP32, in the FP32 update's order of operations
              int at = incl - cnt;
              while (mine) {
                const int b = __ffs(mine) - 1;
                mine &= mine - 1;
                cand[at++] = 32 * V * (b / V) + V * lane + (b % V);
              }
              __syncwarp();
              const bool mine_c = lane < total;
              const int kc = mine_c ? cand[lane] : 0;
              float ale = 0.f;
#pragma unroll 4
              for (int r = 0; r < i; ++r) {
                const int rl = r & 31, rj = r >> 5;
                const float cr = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(c, rj), rl);
                const int col = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(ind, rj), rl);
                if (mine_c) ale = fmaf(__ldg(G + (int64_t)col * ldg + kc), cr, ale);
              }
              const float ae = mine_c ? a0s[kc] - ale : 0.f;
              bv = mine_c ? ae * ae : -1.f;
              bk = mine_c ? kc : 0x7fffffff;
#pragma unroll
              for (int o = 16; o > 0; o >>= 1) {
                const float ov = __shfl_xor_sync(KSVD_FULL_MASK, bv, o);
                const int ok = __shfl_xor_sync(KSVD_FULL_MASK, bk, o);
                if (ov > bv || (ov == bv && ok < bk)) { bv = ov; bk = ok; }
              }
              __syncwarp();                    // cand is read before the next step writes it
            }
          }
          if (full) {
            exact_alpha(i);
            argmax(bv, bk);
          }
        }
      }
      if (bk >= K) { numeric_bad = true; break; }   // every |alpha| was NaN
      const int p = bk;
      const float ba0 = a0s[p];
      bool dup = false;
#pragma unroll
      for (int j = 0; j < SPL; ++j) dup |= (lane + 32 * j < i) && ind[j] == p;
      if (__any_sync(KSVD_FULL_MASK, dup)) break;
      if (bv < 1e-14f) break;                // alpha_p^2 (OMP.cu:304)

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
        // two rows per loop step, with the one-row sweep's operations in its order (row r + 1
        // takes row r's term before its own division), so the results are the same bits
        int r = 0;
        for (; r + 1 < i; r += 2) {
          const int rl = r & 31, rj = r >> 5, rl1 = (r + 1) & 31, rj1 = (r + 1) >> 5;
          const float br = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(b, rj), rl);
          const float br1 = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(b, rj1), rl1);
          const float wr = br * L[lidx<TMAX>(r, r)];
          const float wr1 = fmaf(-L[lidx<TMAX>(r + 1, r)], wr, br1) * L[lidx<TMAX>(r + 1, r + 1)];
          if (lane == rl) put<SPL>(w, rj, wr);
          if (lane == rl1) put<SPL>(w, rj1, wr1);
#pragma unroll
          for (int j = 0; j < SPL; ++j) {
            const int q = lane + 32 * j;
            if (q > r + 1 && q < i)
              b[j] = fmaf(-L[lidx<TMAX>(q, r + 1)], wr1, fmaf(-L[lidx<TMAX>(q, r)], wr, b[j]));
          }
        }
        if (r < i) {                         // the last row when i is odd
          const int rl = r & 31, rj = r >> 5;
          const float wr = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(b, rj), rl) * L[lidx<TMAX>(r, r)];
          if (lane == rl) put<SPL>(w, rj, wr);
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
      if (lane == 0) L[lidx<TMAX>(i, i)] = 1.f / Lii;   // the solves multiply by 1 / L_ii
      if (lane == (i & 31)) {
        put<SPL>(ind, i >> 5, p);
        put<SPL>(y, i >> 5, ynew);
        if constexpr (H16) put<SPL>(muq, i >> 5, __ldg(mu_col + p));
      }
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
        // two rows per loop step, in the one-row sweep's order of operations (same bits)
        int r = i - 1;
        for (; r >= 1; r -= 2) {
          const int rl = r & 31, rj = r >> 5, rl1 = (r - 1) & 31, rj1 = (r - 1) >> 5;
          const float tr = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(t, rj), rl);
          const float tr1 = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(t, rj1), rl1);
          const float cr = tr * L[lidx<TMAX>(r, r)];
          const float cr1 = fmaf(-L[lidx<TMAX>(r, r - 1)], cr, tr1) * L[lidx<TMAX>(r - 1, r - 1)];
          if (lane == rl) put<SPL>(c, rj, cr);
          if (lane == rl1) put<SPL>(c, rj1, cr1);
#pragma unroll
          for (int j = 0; j < SPL; ++j) {
            const int q = lane + 32 * j;
            if (q < r - 1)
              t[j] = fmaf(-L[lidx<TMAX>(r - 1, q)], cr1, fmaf(-L[lidx<TMAX>(r, q)], cr, t[j]));
          }
        }
        if (r == 0) {                        // row 0 when i is odd
          const float cr = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(t, 0), 0) * L[lidx<TMAX>(0, 0)];
          if (lane == 0) put<SPL>(c, 0, cr);
        }
      }
      // ---- alpha = alpha0 - G(:, I) c   (not needed after the last atom)
      if (i < T && !(emode && r2 <= e2)) {
        if constexpr (H16) {
          float cl1 = 0.f;
#pragma unroll
          for (int j = 0; j < SPL; ++j)
            if (lane + 32 * j < i) cl1 += fabsf(c[j]);
          cl1 = warp_sum(cl1);
          int ex = 0;
          frexpf(cl1, &ex);                    // |c| <= ||c||_1 < 2^ex: no FP16 overflow
          const float csc = ldexpf(1.f, ex), cisc = ldexpf(1.f, -ex);
#pragma unroll
          for (int g = 0; g < NG; ++g)
#pragma unroll
            for (int q = 0; q < V; ++q) al[g][q] = 0.f;
          // slot r's scaled FP16 coefficient and atom, packed for one shuffle per column
          unsigned pack[SPL];
#pragma unroll
          for (int j = 0; j < SPL; ++j)
            pack[j] = lane + 32 * j < i
                          ? ((unsigned)__half_as_ushort(__float2half_rn(c[j] * cisc)) << 16) |
                                (unsigned)ind[j]
                          : 0u;
#pragma unroll 1
          for (int r = 0; r < i; ++r) {
            const unsigned pk = __shfl_sync(KSVD_FULL_MASK, pick<SPL>(pack, r >> 5), r & 31);
            const unsigned short ch = (unsigned short)(pk >> 16);
            const int col = (int)(pk & 0xffffu);
            const uint16_t* gp = Gh + (int64_t)col * ldg + V * lane;
#pragma unroll
            for (int g = 0; g < NG; ++g) {
              if constexpr (V == 8) {
                const uint4 gv = ldg_u4_no_l1(gp + 256 * g);
                fma2_f16_f32(gv.x, ch, al[g][0], al[g][1]);
                fma2_f16_f32(gv.y, ch, al[g][2], al[g][3]);
                fma2_f16_f32(gv.z, ch, al[g][4], al[g][5]);
                fma2_f16_f32(gv.w, ch, al[g][6], al[g][7]);
              } else {
                const uint2 gv = ldg_u2_no_l1(gp + 128 * g);
                fma2_f16_f32(gv.x, ch, al[g][0], al[g][1]);
                fma2_f16_f32(gv.y, ch, al[g][2], al[g][3]);
              }
            }
          }
          hk1 = 0u; hk2 = 0u;
#pragma unroll
          for (int g = 0; g < NG; ++g)
#pragma unroll
            for (int h = 0; h < V / 4; ++h) {
              const float4 a =
                  *reinterpret_cast<const float4*>(a0s + 32 * V * g + V * lane + 4 * h);
              al[g][4 * h] = fmaf(-csc, al[g][4 * h], a.x);
              al[g][4 * h + 1] = fmaf(-csc, al[g][4 * h + 1], a.y);
              al[g][4 * h + 2] = fmaf(-csc, al[g][4 * h + 2], a.z);
              al[g][4 * h + 3] = fmaf(-csc, al[g][4 * h + 3], a.w);
            }
#pragma unroll
          for (int g = 0; g < NG; ++g)
#pragma unroll
            for (int q = 0; q < V; ++q) {
              const unsigned key = (__float_as_uint(al[g][q]) & 0x7FFFFFE0u) | (31u - (V * g + q));
              hk2 = max(hk2, min(hk1, key));
              hk1 = max(hk1, key);
            }
          approx = true;
        } else {
          exact_alpha(i);
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

// Shared memory of one warp: Cholesky factor, alpha0 column, near-tie candidates.
template <int KPL, int TMAX>
__host__ __device__ constexpr int warp_smem_floats() {
  return l_floats<TMAX>() + 32 * KPL + kMaxCand;
}
// The same for supports of at most T atoms: L needs only its first T rows (a multiple of four
// floats keeps the alpha0 column 16-byte aligned), so short supports leave room for more CTAs.
template <int TMAX>
__host__ __device__ constexpr int l_floats_for(int T) {
  return (int)round_up(TMAX > 32 ? T * (T + 1) / 2 : T * (TMAX + 1), 4);
}
template <int KPL, int TMAX>
__host__ __device__ constexpr int warp_smem_floats_for(int T) {
  return l_floats_for<TMAX>(T) + 32 * KPL + kMaxCand;
}

template <int KPL, int TMAX, bool H16, bool QUEUE>
__global__ void __launch_bounds__(kOmpWarps * 32, (TMAX <= 32 ? 3 : 2))
omp_kernel(const float* __restrict__ G, const uint16_t* __restrict__ Gh,
           const float* __restrict__ mu_col, int64_t ldg, const float* __restrict__ A0,
           int64_t lda, int K, int64_t N, int T, const float* __restrict__ xnorm2,
           const float* __restrict__ eps2, int32_t* __restrict__ idx_out,
           float* __restrict__ coef_out, int32_t* __restrict__ nnz_out, int* __restrict__ dev_err,
           unsigned long long* __restrict__ queue) {
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  float* L = smem + (size_t)wib * warp_smem_floats_for<KPL, TMAX>(T);   // Cholesky factor
  float* a0s = L + l_floats_for<TMAX>(T);                                // alpha0 column
  int* cand = reinterpret_cast<int*>(a0s + 32 * KPL);
  bool numeric_bad = false;
  const bool emode = eps2 != nullptr;
  if constexpr (QUEUE) {
    // resident grid: warps claim kOmpClaim signals at a time from *queue (a signal counter,
    // zeroed before the launch); early stops make signals uneven, and once fewer than
    // kOmpClaim signals per resident warp remain the claims shrink to one signal, so the last
    // warps finish close together (the size is chosen from a plain read of the counter; the
    // claimed ranges stay disjoint and cover [0, N) whatever the size)
    const unsigned long long tail =
        (unsigned long long)gridDim.x * kOmpWarps * kOmpClaim;
    for (;;) {
      unsigned long long cl = 0;
      int sz = kOmpClaim;
      if (lane == 0) {
        const unsigned long long seen = *((volatile unsigned long long*)queue);
        if (seen + tail >= (unsigned long long)N) sz = 1;
        cl = atomicAdd(queue, (unsigned long long)sz);
      }
      cl = __shfl_sync(KSVD_FULL_MASK, cl, 0);
      sz = __shfl_sync(KSVD_FULL_MASK, sz, 0);
      const int64_t s0 = (int64_t)cl;
      if (s0 >= N) break;
      const int64_t s1 = min(N, s0 + sz);
      for (int64_t s = s0; s < s1; ++s)
        omp_signal<KPL, TMAX, H16>(G, Gh, mu_col, ldg, A0 + s * lda, K, T, emode,
                                   emode ? eps2[s] : 0.f, emode ? xnorm2[s] : 0.f,
                                   idx_out + s * T, coef_out + s * T, nnz_out + s, L, a0s, cand,
                                   numeric_bad);
    }
  } else {
    const int64_t warps_total = (int64_t)gridDim.x * kOmpWarps;
    for (int64_t s = (int64_t)blockIdx.x * kOmpWarps + wib; s < N; s += warps_total)
      omp_signal<KPL, TMAX, H16>(G, Gh, mu_col, ldg, A0 + s * lda, K, T, emode,
                                 emode ? eps2[s] : 0.f, emode ? xnorm2[s] : 0.f, idx_out + s * T,
                                 coef_out + s * T, nnz_out + s, L, a0s, cand, numeric_bad);
  }
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
  float* L = smem + (size_t)wib * warp_smem_floats<32, TMAX>();
  float* a0s = L + l_floats<TMAX>();
  int* cand = reinterpret_cast<int*>(a0s + 32 * 32);
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
#define KSVD_BATCHED_SIGNAL(KPL)                                                              \
  omp_signal<KPL, TMAX, false>(jb.G, nullptr, nullptr, jb.ldg, a0, jb.K, jb.T, emode, e2, xn2, \
                               io, co, jb.nnz + s, L, a0s, cand, numeric_bad)
        case 4: KSVD_BATCHED_SIGNAL(4); break;
        case 8: KSVD_BATCHED_SIGNAL(8); break;
        case 16: KSVD_BATCHED_SIGNAL(16); break;
        default: KSVD_BATCHED_SIGNAL(32); break;
#undef KSVD_BATCHED_SIGNAL
      }
    }
  }
  if (__any_sync(KSVD_FULL_MASK, numeric_bad) && lane == 0) atomicOr(dev_err, kDevErrNumeric);
}

template <int KPL, int TMAX, bool H16>
cudaError_t launch_omp_t(const float* G, const uint16_t* Gh, const float* mu, int64_t ldg,
                         const float* A0, int64_t lda, int K, int64_t N, int T,
                         const float* xnorm2, const float* eps2, int32_t* idx, float* coef,
                         int32_t* nnz, int* dev_err, int grid_mult, unsigned long long* queue,
                         cudaStream_t st) {
  const size_t smem = (size_t)kOmpWarps * warp_smem_floats_for<KPL, TMAX>(T) * sizeof(float);
  // grid_mult 0 with a queue: one resident grid, signals claimed from the queue
  const bool use_queue = queue != nullptr && grid_mult == 0;
  auto kern = use_queue ? omp_kernel<KPL, TMAX, H16, true> : omp_kernel<KPL, TMAX, H16, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kOmpWarps * 32, smem);
  if (per_sm < 1) per_sm = 1;
  int64_t blocks = (N + kOmpWarps - 1) / kOmpWarps;
  const int64_t cap = (int64_t)sms * per_sm * (use_queue ? 1 : (grid_mult > 0 ? grid_mult : 8));
  if (blocks > cap) blocks = cap;
  if (use_queue) {
    e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
  }
  kern<<<(unsigned)blocks, kOmpWarps * 32, smem, st>>>(G, Gh, mu, ldg, A0, lda, K, N, T, xnorm2,
                                                       eps2, idx, coef, nnz, dev_err,
                                                       use_queue ? queue : nullptr);
  return cudaGetLastError();
}

template <int TMAX>
cudaError_t launch_omp_batched_t(const OmpJob* jobs, int njobs, int64_t total_chunks, int chunk,
                                 unsigned long long* queue, int* dev_err, cudaStream_t st) {
  const size_t smem = (size_t)kOmpWarps * warp_smem_floats<32, TMAX>() * sizeof(float);
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

// FP16 copy of G, elementwise.
__global__ void gram_half_kernel(const float* __restrict__ G, int64_t total,
                                 uint16_t* __restrict__ Gh) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    Gh[e] = __half_as_ushort(__float2half_rn(G[e]));
}

// Per-column coherence mu_col[c] = max_{k != c, k < K} |G(k, c)| (column c of the stored matrix,
// as the FP32 alpha update reads it), zero for padding columns; one warp per column.  Block 0
// also writes mu_col[kp] = max_{k < K} |G(k, k) - 1| (G's unit diagonal up to rounding).
__global__ void column_coherence_kernel(const float* __restrict__ G, int64_t ldg, int K, int kp,
                                        float* __restrict__ mu_col) {
  const int lane = threadIdx.x & 31;
  if (blockIdx.x == 0 && threadIdx.x < 32) {
    float dm = 0.f;
    for (int k = lane; k < K; k += 32) dm = fmaxf(dm, fabsf(G[(int64_t)k * ldg + k] - 1.f));
    dm = warp_max(dm);
    if (lane == 0) mu_col[kp] = dm;
  }
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= kp) return;
  float mx = 0.f;
  if (c < K)
    for (int k = lane; k < K; k += 32)
      if (k != c) mx = fmaxf(mx, fabsf(G[(int64_t)c * ldg + k]));
  mx = warp_max(mx);
  if (lane == 0) mu_col[c] = mx;
}

cudaError_t launch_gram_half(const float* G, int64_t ldg, int K, uint16_t* Gh, float* mu_col,
                             cudaStream_t st) {
  const int kp = omp_padded_k(K);
  if (K < 1 || K > kMaxK || ldg < kp) return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t total = ldg * kp;
  const unsigned blocks = (unsigned)std::min<int64_t>((total + 255) / 256, (int64_t)sms * 8);
  gram_half_kernel<<<blocks, 256, 0, st>>>(G, total, Gh);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  column_coherence_kernel<<<(kp + 7) / 8, 256, 0, st>>>(G, ldg, K, kp, mu_col);
  return cudaGetLastError();
}

cudaError_t launch_omp(const float* G, int64_t ldg, const float* A0, int64_t lda, int K,
                       int64_t N, int T, const float* xnorm2, const float* eps2, int32_t* idx,
                       float* coef, int32_t* nnz, int* dev_err, cudaStream_t st, int grid_mult,
                       const uint16_t* Gh, const float* mu, unsigned long long* queue) {
  if (N <= 0) return cudaSuccess;
  if (K < 1 || K > kMaxK || T < 1 || T > kMaxT) return cudaErrorInvalidValue;
  const int kp = omp_padded_k(K);   // the lanes touch rows [0, kp) of every column
  if (ldg < kp || lda < kp || (ldg & 3) || (lda & 3)) return cudaErrorInvalidValue;
  if ((Gh == nullptr) != (mu == nullptr)) return cudaErrorInvalidValue;
  if (Gh && (ldg & 7)) return cudaErrorInvalidValue;   // 16-byte rows of eight FP16 values
#define KSVD_OMP_ARGS G, Gh, mu, ldg, A0, lda, K, N, T, xnorm2, eps2, idx, coef, nnz, dev_err, \
                      grid_mult, queue, st
  if (T <= 32 && Gh) {
    switch (kp) {
      case 128: return launch_omp_t<4, 32, true>(KSVD_OMP_ARGS);
      case 256: return launch_omp_t<8, 32, true>(KSVD_OMP_ARGS);
      case 512: return launch_omp_t<16, 32, true>(KSVD_OMP_ARGS);
      default: return launch_omp_t<32, 32, true>(KSVD_OMP_ARGS);
    }
  }
  if (T <= 32) {
    switch (kp) {
      case 128: return launch_omp_t<4, 32, false>(KSVD_OMP_ARGS);
      case 256: return launch_omp_t<8, 32, false>(KSVD_OMP_ARGS);
      case 512: return launch_omp_t<16, 32, false>(KSVD_OMP_ARGS);
      default: return launch_omp_t<32, 32, false>(KSVD_OMP_ARGS);
    }
  }
  switch (kp) {
    case 128: return launch_omp_t<4, 64, false>(KSVD_OMP_ARGS);
    case 256: return launch_omp_t<8, 64, false>(KSVD_OMP_ARGS);
    case 512: return launch_omp_t<16, 64, false>(KSVD_OMP_ARGS);
    default: return launch_omp_t<32, 64, false>(KSVD_OMP_ARGS);
  }
#undef KSVD_OMP_ARGS
}

}  // namespace ksvd
