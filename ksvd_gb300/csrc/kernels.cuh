// kernels.cuh -- host launchers of the device kernels (internal interface of libksvd_gb300).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ksvd {

// ---- GEMM (gemm_simt.cu) --------------------------------------------------------------------
// C[s*ldc + k] = sum_{r<inner} A[k*lda + r] * B[s*ldb + r] for k < M_store, s < N_store, where
// rows k >= M_load of A and rows s >= N_load of B read as zero (zero padding of the outputs).
cudaError_t launch_gemm_tn_f32(const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                               int64_t ldc, int M_load, int M_store, int64_t N_load,
                               int64_t N_store, int inner, cudaStream_t st);

// ---- tensor-core GEMM (gemm_tc.cu) ------------------------------------------------------------
// Mixed precision C = A'B with A, B given as BF16 hi (+ optional lo) parts, FP32 accumulation
// in TMEM.  Returns cudaErrorNotSupported when the shape is outside the kernel's tiling.
struct TcOperand {
  const uint16_t* hi;   // bf16 bits, rows of `inner` contiguous elements, leading dim ld
  const uint16_t* lo;   // nullable: residual part for the split product
  int64_t ld;           // elements
  int64_t rows;         // rows available (multiple of the tile)
};
cudaError_t launch_gemm_tn_bf16(const TcOperand& A, const TcOperand& B, float* C, int64_t ldc,
                                int M, int64_t Ncols, int inner, int passes, int* dev_err,
                                cudaStream_t st);
int tc_tile_atoms();
int tc_tile_signals();
// hi/lo split of an FP32 matrix stored as `rows` rows of `inner` contiguous floats (ld_in),
// written with leading dimension ld_out (zero padded to ld_out and to rows_out).
cudaError_t launch_split_bf16(const float* in, int64_t ld_in, int64_t rows, int inner,
                              uint16_t* hi, uint16_t* lo, int64_t ld_out, int64_t rows_out,
                              cudaStream_t st);

// ---- Batch-OMP (omp.cu) -------------------------------------------------------------------------
// Atom-dimension padding used by every internal buffer: 128, 256, 512 or 1024 (K <= 1024).
int omp_padded_k(int K);
// G: Kp x Kp column-major (ldg >= Kp), zero padded; A0: Kp x N column-major (lda >= Kp), zero
// padded, with Kp = omp_padded_k(K).  T <= 64.
// grid_mult: resident CTAs per SM x grid_mult blocks at most, signals assigned grid-stride; 0 with
// a queue (one zeroed counter): one resident grid whose warps claim signals from the queue (0
// without a queue: 8; the autotuner's knob)
// Gh/mu (mixed path, T <= 32): FP16 copy of G and its per-column coherence from
// launch_gram_half; the alpha update then reads Gh and resolves near ties in FP32 (the selection
// is the FP32 Batch-OMP's).
cudaError_t launch_omp(const float* G, int64_t ldg, const float* A0, int64_t lda, int K,
                       int64_t N, int T, const float* xnorm2, const float* eps2, int32_t* idx,
                       float* coef, int32_t* nnz, int* dev_err, cudaStream_t st,
                       int grid_mult = 0, const uint16_t* Gh = nullptr,
                       const float* mu = nullptr, unsigned long long* queue = nullptr);
// Gh = FP16(G) (Kp x Kp, same ldg), mu_col[c] = max_{k != c, k < K} |G(k, c)| (zero past K) and
// mu_col[Kp] = max_k |G(k, k) - 1| (Kp + 1 floats): what the FP16 update's error bound uses.
cudaError_t launch_gram_half(const float* G, int64_t ldg, int K, uint16_t* Gh, float* mu_col,
                             cudaStream_t st);

// ---- misc (misc.cu) ---------------------------------------------------------------------------
cudaError_t launch_normcols(float* D, int n, int K, cudaStream_t st);
// copy an n x K column-major matrix into an n x Kp buffer (zero columns K..Kp-1)
cudaError_t launch_copy_pad_cols(const float* src, int n, int K, float* dst, int Kp,
                                 cudaStream_t st);
cudaError_t launch_col_norm2(const float* X, int n, int64_t N, float* out, cudaStream_t st);
cudaError_t launch_dense_gamma(const int32_t* idx, const float* coef, const int32_t* nnz,
                               int64_t N, int T, int K, float* gamma, cudaStream_t st);
cudaError_t launch_copy_matrix(const float* src, int64_t ld_src, float* dst, int64_t ld_dst,
                               int rows, int64_t cols, cudaStream_t st);

// ---- dictionary update (update.cu) ------------------------------------------------------------
struct UpdateArgs {
  int n, K, Kp, T;
  int64_t N;
  const float* X;        // n x N
  float* D;              // n x Kp (current dictionary, updated in place)
  const int32_t* idx;    // N x T
  float* coef;           // N x T (updated in place)
  const int32_t* nnz;    // N
  const int32_t* perm;   // K (or iters x K with iter_ctr)
  const int* iter_ctr;   // nullable: use perm + (*iter_ctr) * K (graph replays)
  int max_signals;
  int sweep_ctas;        // CTAs of the cooperative sweep (0: one per SM)
  // workspace
  int32_t* list;         // total entries (signal*T + slot), per-atom ascending signal order
  int64_t* start;        // Kp + 1
  int32_t* block_hist;   // nblk x Kp
  float* Y;              // n x Kp
  float* gn2;            // Kp
  float* C;              // Kp x Kp co-occurrence, C(i,j) = sum_s Gamma(i,s) Gamma(j,s)
  float* G;              // Kp x Kp, D'D of the current dictionary on entry, maintained
  float* P;              // Kp x Kp, D'Y (P(i,j) = d_i . Y_j), maintained
  float* avec;           // 3 x n rotating atom accumulators (zero on entry)
  float* aD;             // 2 x Kp alternating a'D slices
  float* part;           // nctas x 4 scratch
  int32_t* unused;       // N
  int32_t* bitmap;       // N
  int32_t* replaced;     // Kp
  int64_t* counter;      // 1
  int32_t* usecount;     // Kp
  unsigned int* barrier; // 2 words
  int* dev_err;
  // nullable: windowed list preparation (prep_win signals per window, partials in prep_part:
  // ceil(N / prep_win) x Kp x (n + Kp + 1) floats); see prepare_window_signals
  float* prep_part;
  int64_t prep_win;
};
cudaError_t launch_update_prepare(const UpdateArgs& a, cudaStream_t st);
// Signals per window of the windowed list preparation for this shape, or 0 when X fits L2 well
// enough (or the half-warp layout does not apply) and one pass over each atom's list is used.
int64_t prepare_window_signals(int64_t N, int n, int T);
cudaError_t launch_update_sweep(const UpdateArgs& a, cudaStream_t st);
int64_t update_block_count(int64_t N);
int update_sweep_ctas();

// ---- error + clearDict (clear.cu) -------------------------------------------------------------
struct ErrorArgs {
  int n, K, Kp, T;
  int64_t N;
  const float* X;
  const float* D;        // n x Kp
  const int32_t* idx;
  const float* coef;
  const int32_t* nnz;
  const int32_t* bitmap; // nullable
  float* err;            // N, masked error
  double* part_sum;      // per error block
  float* bucket_val;     // per error block: max masked error
  int64_t* bucket_idx;   // per error block: its signal (lowest on ties)
  double* rmse_out;      // device scalar (rmse_out[*iter_ctr] when iter_ctr is set)
  const int* iter_ctr;   // nullable
  int* dev_err;          // nullable: kDevErrBounds when a used slot holds an index outside [0, K)
};
int64_t error_block_count(int64_t N);
cudaError_t launch_error(const ErrorArgs& a, cudaStream_t st);

struct ClearArgs {
  int n, K, Kp;
  int64_t N;
  const float* X;
  float* D;              // n x Kp
  float* G;              // Kp x Kp, kept equal to D'D
  const int32_t* usecount;   // signals with gamma^2 > 1e-7 per atom (from the sweep)
  const int32_t* replaced;
  float* err;
  float* bucket_val;
  int64_t* bucket_idx;
  int64_t nbuckets;
  float mu_thresh;
  int use_thresh;
  int32_t* cleared;      // device scalar
};
// m, mi: Kp scratch floats / ints (per-column largest off-diagonal G^2 and its row)
cudaError_t launch_clear_dict(const ClearArgs& a, float* m, int* mi, cudaStream_t st);

// X(r, :) -= mean of row r over the N signals (Matlab/remmean.m:13-15), FP64 sums in a fixed order.
// part: row_mean_blocks(N) x n doubles of scratch; mean: n floats (out).
int64_t row_mean_blocks(int64_t N);
cudaError_t launch_remove_row_mean(float* X, int n, int64_t N, double* part, float* mean,
                                   cudaStream_t st);

// *ctr += 1 (one thread): the iteration counter that graph-replayed iterations index by.
cudaError_t launch_advance_counter(int* ctr, cudaStream_t st);

// ---- batched Batch-OMP: many problems in one persistent launch (omp.cu) ---------------------------
struct OmpJob {
  const float* G; int64_t ldg;      // Kp x Kp Gram (rows >= K zero)
  const float* A0; int64_t lda;     // Kp x N alpha0 (rows >= K zero)
  const float* X; int64_t ldx;      // n x N signals (read for ||x||^2 in error mode)
  const float* eps2;                // N error targets, or null (T-sparse)
  int32_t* idx; float* coef; int32_t* nnz;   // N x T slots, N
  int64_t N; int64_t chunk_begin;   // first work-queue chunk of this job
  int n, K, kpl, T;                 // kpl = Kp / 32 (4, 8, 16 or 32)
};
int omp_batch_chunk();              // default signals per work-queue chunk
// jobs_dev sorted by chunk_begin (chunk_begin in units of `chunk` signals); tmax = max T over
// the jobs.  Zeroes *queue on the stream.
cudaError_t launch_omp_batched(const OmpJob* jobs_dev, int njobs, int64_t total_chunks, int tmax,
                               int chunk, unsigned long long* queue, int* dev_err,
                               cudaStream_t st);

// ---- grouped FP32 GEMM: many C = A'B products (different sizes) in one launch -------------------
struct GemmDesc {
  const float* A; int64_t lda;
  const float* B; int64_t ldb;
  float* C; int64_t ldc;
  int M_load, M_store; int64_t N_load, N_store;
  int inner;
  int tiles_m; int64_t tiles_n; int64_t tile_begin;
  bool vec_a, vec_b, vec_c;
};
// Fills d (same meaning of the sizes as launch_gemm_tn_f32); returns tile_begin + its tiles.
int64_t gemm_desc_fill(GemmDesc& d, const float* A, int64_t lda, const float* B, int64_t ldb,
                       float* C, int64_t ldc, int M_load, int M_store, int64_t N_load,
                       int64_t N_store, int inner, int64_t tile_begin);
// descs_dev: device copy of the table, sorted by tile_begin (as gemm_desc_fill chains them).
cudaError_t launch_gemm_tn_f32_grouped(const GemmDesc* descs_dev, int ndesc, int64_t total_tiles,
                                       cudaStream_t st);

// ---- fixed-support coding and its adjoint (adjoint.cu) ---------------------------------------
// G: D'D with leading dimension ldg (>= K).  chol: N x T(T+1)/2 packed lower factors.
cudaError_t launch_code_fixed(const float* D, int n, int K, const float* G, int ldg,
                              const float* X, int64_t N, int T, const int32_t* idx,
                              const int32_t* nnz, float* coef, float* chol, int* dev_err,
                              cudaStream_t st);
// One FP64-residual refinement step of the coefficients on fixed supports (coef in place).
cudaError_t launch_refine(const float* D, int n, int K, const float* G, int ldg, const float* X,
                          int64_t N, int T, const int32_t* idx, const int32_t* nnz, float* coef,
                          double* coef64, int* dev_err, cudaStream_t st);
// dD (n x K, accumulated: zero it first) and dX (n x N, written); either may be null.
cudaError_t launch_code_backward(const float* D, int n, int K, const float* X, int64_t N, int T,
                                 const int32_t* idx, const int32_t* nnz, const float* coef,
                                 const float* chol, const float* dcoef, float* dD, float* dX,
                                 cudaStream_t st);

// The last failure of a call that had no handle to record it in (a null handle, a failed
// ksvd_create, ksvd_rmse_noalloc), per host thread; ksvd_last_error(NULL) returns it.
void set_nohandle_error(const char* msg);

}  // namespace ksvd
