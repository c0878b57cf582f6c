/*
 * ksvd_gb300.h -- C ABI of the GB300-native K-SVD engine (libksvd_gb300.so).
 *
 * The reference (patschris/KSVD) has no plugin or FFI layer: its in-process surface is the C++
 * class KSVD (K-SVD/K-SVD/KSVD.cuh:21-27) with ExecuteIterations(iternum) (KSVD.cu:55-131) and
 * its protected stages OMP::BatchOMP() (OMP.cuh:23, OMP.cu:42-59) and
 * DictionaryUpdate::updateDictionary(perm) (DictionaryUpdate.cuh:23, DictionaryUpdate.cu:45-203),
 * fed by enum-indexed device buffers (DeviceMemory.cuh:36-64) and the global sizes in Globals::
 * (Globals.cuh:10-20).  Each entry point below names the reference interface it replaces.
 *
 * Conventions
 *   - Matrices are column-major (MATLAB layout, as in the reference): X is n x N (signal s is the
 *     n contiguous floats at X + s*n), D is n x K, G is K x K.
 *   - Sparse codes use T slots per signal in selection order: idx[s*T + t] (atom index, -1 when
 *     unused) and coef[s*T + t] (0 when unused), plus nnz[s] = atoms used by signal s.  This
 *     replaces the reference's dense K x N slot map SELECTED_ATOMS plus the T x N array c
 *     (OMP.cu:373-400); ksvd_dense_gamma() expands it to the reference's K x N CUDA_Gamma.
 *   - Unless an entry point says "host", every array argument is a DEVICE pointer owned by the
 *     caller.  Work is enqueued on the stream given to ksvd_create(); entry points that return
 *     host results (rmse, counts) synchronise that stream.
 *   - Errors: every call returns a ksvd_status and never aborts or exits; ksvd_last_error()
 *     gives a message.  (The reference returns bool false and prints to cerr, e.g. main.cu:55-112.)
 *   - Threading: one handle must not be used from two threads at once; separate handles are
 *     independent.
 *   - Atoms must have unit l2 norm when calling ksvd_omp()/ksvd_omp_gram() directly, as in the
 *     reference's parOMP (OMP.cu:316-335 uses 1 - ||w||^2); ksvd_iterate() normalises D first
 *     (KSVD.cu:57).
 */
#ifndef KSVD_GB300_H
#define KSVD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KSVD_GB300_ABI_VERSION 1

#if defined(__GNUC__)
#define KSVD_API __attribute__((visibility("default")))
#else
#define KSVD_API
#endif

typedef enum ksvd_status {
  KSVD_OK = 0,
  KSVD_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, bad permutation            */
  KSVD_ERR_UNSUPPORTED = 2,      /* size beyond the kernels' limits (K > 1024, T > 64)  */
  KSVD_ERR_OUT_OF_MEMORY = 3,    /* device workspace allocation failed                  */
  KSVD_ERR_CUDA = 4,             /* a CUDA runtime call or kernel launch failed         */
  KSVD_ERR_NUMERIC = 5,          /* NaN/Inf met on the device                           */
  KSVD_ERR_TIMEOUT = 6,          /* a bounded device-side wait gave up                  */
  KSVD_ERR_STATE = 7             /* stage called out of order (e.g. clear before update)*/
} ksvd_status;

typedef enum ksvd_precision {
  KSVD_PREC_FP32 = 0,  /* plain FP32 everywhere (the correctness path)                       */
  KSVD_PREC_MIXED = 1  /* BF16 tensor-core Gram and D'X with FP32 accumulation, FP32 solve  */
} ksvd_precision;

/* Runtime parameters.  The reference fixes these at compile time:
 * Tdata, muTHRESH (ProgramParameters.cuh:17-23), USE_THRESH, MAX_SIGNALS
 * (GlobalDeclarations.cuh:54,63); n and K come from the input files (FileManager.cu:44-71). */
typedef struct ksvd_params {
  int32_t n;                   /* signal length: rows of X and D           (Globals::rowsX)  */
  int32_t K;                   /* atoms: columns of D                      (Globals::colsD)  */
  int32_t T;                   /* sparsity target = max atoms per signal   (Tdata)           */
  int32_t precision;           /* ksvd_precision                                             */
  float mu_thresh;             /* clearDict coherence threshold            (muTHRESH = 0.8)  */
  int32_t use_thresh;          /* clearDict minimum use count              (USE_THRESH = 4)  */
  int32_t max_replace_signals; /* candidates for an unused atom            (MAX_SIGNALS=5000)*/
  int32_t flags;               /* reserved, 0                                                */
  uint64_t seed;               /* atom-order seed used when no permutation is passed         */
} ksvd_params;

typedef struct ksvd_handle ksvd_handle;

/* params.flags bits */
#define KSVD_FLAG_PROFILE 1  /* record per-stage device time (CUDA events on the handle's stream) */
#define KSVD_FLAG_REFINE_FINAL 2 /* ksvd_iterate ends with ksvd_refine_coefs on the final D:
                                    the returned coefficients are then the least-squares ones on
                                    the final supports (the reference returns the sweep's) */
#define KSVD_FLAG_GRAPH 4        /* ksvd_iterate captures one K-SVD iteration in a CUDA graph and
                                    replays it for iterations 2..iters (on a private stream,
                                    fenced to the handle's stream); the graph is cached while
                                    the buffers stay the same.  Ignored with KSVD_FLAG_PROFILE. */

/* Stages of one K-SVD iteration, for ksvd_read_stage_times(). */
typedef enum ksvd_stage {
  KSVD_STAGE_GRAM = 0,   /* G = D'D                                  */
  KSVD_STAGE_DTX = 1,    /* alpha0 = D'X                             */
  KSVD_STAGE_OMP = 2,    /* Batch-OMP kernel                         */
  KSVD_STAGE_LISTS = 3,  /* per-atom lists, Y, ||gamma||^2, Gamma Gamma' */
  KSVD_STAGE_SWEEP = 4,  /* the sequential atom sweep                */
  KSVD_STAGE_ERROR = 5,  /* reconstruction error and RMSE            */
  KSVD_STAGE_CLEAR = 6,  /* clearDict                                */
  KSVD_STAGE_COUNT = 7
} ksvd_stage;

typedef struct ksvd_stage_times {
  double ms[8];          /* accumulated device milliseconds per ksvd_stage */
  int64_t calls[8];      /* number of timed executions per stage          */
} ksvd_stage_times;

/* ---- handle ------------------------------------------------------------------------------ */

/* Fills the reference's defaults: T=6, mu_thresh=0.8, use_thresh=4, max_replace_signals=5000. */
KSVD_API void ksvd_default_params(ksvd_params* params);

/* Replaces the KSVD/OMP/DictionaryUpdate constructors and the DeviceMemory pool
 * (KSVD.cu:42-44, CudaAlgorithm.cu:23-33, DeviceMemory.cu:19-138).  stream is a cudaStream_t
 * (NULL = legacy default stream).  Workspace is allocated lazily and grows with N. */
KSVD_API ksvd_status ksvd_create(ksvd_handle** out, const ksvd_params* params, void* stream);
KSVD_API void ksvd_destroy(ksvd_handle* handle);
KSVD_API const char* ksvd_status_string(ksvd_status status);
KSVD_API const char* ksvd_last_error(const ksvd_handle* handle);
KSVD_API int32_t ksvd_abi_version(void);
/* Bytes of device workspace the handle holds now. */
KSVD_API int64_t ksvd_workspace_bytes(const ksvd_handle* handle);

/* Host-only: the atom visiting order of one dictionary sweep, a permutation of 0..K-1 drawn
 * from (seed, iteration).  Replaces RandomPermutation::generateRandPerm (RandPermutation.cu:
 * 35-42), which shuffles with an unseeded std::random_shuffle.  perm is a HOST array. */
KSVD_API ksvd_status ksvd_random_permutation(uint64_t seed, int64_t iteration, int32_t K, int32_t* perm);

/* ---- stages ------------------------------------------------------------------------------ */

/* D <- D * diag(1/||d_k||), in place.  Replaces KSVD::normcols (KSVD.cu:267-286). */
KSVD_API ksvd_status ksvd_normcols(ksvd_handle* handle, float* D);

/* Preprocessing of the fMRI workflow: subtract from every row of X (n x N, device, in place) its
 * mean over the N signals; mean (nullable, device, n floats) receives the means.  Sums are FP64
 * in a fixed order (deterministic).  Replaces Matlab/remmean.m:13-15 run before the executable. */
KSVD_API ksvd_status ksvd_remove_row_mean(ksvd_handle* handle, float* X, int64_t N, float* mean);

/* Checkpoint/resume of the atom-order stream: ksvd_iterate without explicit permutations draws
 * iteration i's order as ksvd_random_permutation(seed, draws + i, K) and then advances draws by
 * the iteration count.  Saving draws with D and restoring it (with the same seed) continues a
 * run with exactly the orders it would have used.  No reference counterpart (its orders come
 * from unseeded std::random_shuffle, S/RandPermutation.cu:35-42). */
KSVD_API int64_t ksvd_perm_draws(const ksvd_handle* handle);
KSVD_API ksvd_status ksvd_set_perm_draws(ksvd_handle* handle, int64_t draws);

/* G = D'D (K x K).  Replaces Multiplication::AT_times_B at KSVD.cu:64-73. */
KSVD_API ksvd_status ksvd_gram(ksvd_handle* handle, const float* D, float* G);

/* alpha0 = D'X (K x N).  Replaces Multiplication::AT_times_B at OMP.cu:44-53. */
KSVD_API ksvd_status ksvd_dtx(ksvd_handle* handle, const float* D, const float* X, int64_t N, float* A0);

/* Batch-OMP from precomputed G (K x K) and alpha0 = D'X (K x N).  Replaces the parOMP launch
 * (OMP.cu:65-113, 254-405).  eps2 (nullable, N entries): per-signal squared error target; when
 * given, a signal stops once ||x - D gamma||^2 <= eps2[s] (T is then the atom cap) and xnorm2
 * (N entries, ||x_s||^2) is required.  Outputs idx/coef (T x N slots) and nnz (N). */
KSVD_API ksvd_status ksvd_omp_gram(ksvd_handle* handle, const float* G, const float* A0, int64_t N,
                          const float* xnorm2, const float* eps2, int32_t* idx, float* coef,
                          int32_t* nnz);

/* Sparse coding of X over D: Gram, D'X and Batch-OMP.  Replaces OMP::BatchOMP (OMP.cu:42-59)
 * together with the Gram at KSVD.cu:64.  eps2 as in ksvd_omp_gram (xnorm2 is computed). */
KSVD_API ksvd_status ksvd_omp(ksvd_handle* handle, const float* D, const float* X, int64_t N,
                     const float* eps2, int32_t* idx, float* coef, int32_t* nnz);

/* One approximate K-SVD dictionary sweep over the atoms in the order perm (DEVICE array of K
 * atom indices, or NULL to draw one from the handle's seed).  Updates D and coef in place;
 * idx/nnz are unchanged.  Also resets the unused-signal bookkeeping first, as
 * ExecuteIterations does with its init kernel.  Replaces initialize() + updateDictionary(perm)
 * (KSVD.cu:97-114, DictionaryUpdate.cu:45-203).
 * Speed (not results): with T <= 16, n % 4 == 0, n <= 256 and X 16-byte aligned the sweep and
 * its list preparation use their half-warp kernels (and, once X exceeds 96 MiB, the windowed
 * preparation, which needs about ceil(N / W) * Kp * (n + Kp + 1) floats of workspace, W the
 * signals in 32 MB); other inputs take the warp-per-entry kernels.  The same holds for
 * ksvd_error (with D 16-byte aligned too) and for the stages inside ksvd_iterate. */
KSVD_API ksvd_status ksvd_update_dictionary(ksvd_handle* handle, float* D, const float* X, int64_t N,
                                   const int32_t* idx, float* coef, const int32_t* nnz,
                                   const int32_t* perm);

/* err[s] = ||x_s - D gamma_s||^2 masked by the unused-signal bitmap left by the last
 * ksvd_update_dictionary on this handle (unmasked if none), and *rmse (HOST) =
 * sqrt(sum_s ||x_s - D gamma_s||^2 / (n N)).  err is nullable.  Replaces
 * KSVD::errorComputation (KSVD.cu:235-262). */
KSVD_API ksvd_status ksvd_error(ksvd_handle* handle, const float* D, const float* X, int64_t N,
                       const int32_t* idx, const float* coef, const int32_t* nnz, float* err,
                       double* rmse);

/* Replace atoms that are too coherent with another atom or used by fewer than use_thresh
 * signals by the worst-represented signals (errors from the last ksvd_error on this handle).
 * *cleared (HOST, nullable) = number of atoms replaced.  Replaces KSVD::clearDict
 * (KSVD.cu:138-226). */
KSVD_API ksvd_status ksvd_clear_dict(ksvd_handle* handle, float* D, const float* X, int64_t N,
                            const int32_t* idx, const float* coef, const int32_t* nnz,
                            int32_t* cleared);

/* Fixed-support coding, the differentiable form of the coding step: for every signal the least
 * squares coefficients on the support given by idx/nnz (T slots per signal, e.g. from ksvd_omp),
 * gamma_S = (D_S'D_S)^-1 D_S'x.  chol (nullable) receives each signal's lower Cholesky factor of
 * D_S'D_S, packed row by row, T(T+1)/2 floats per signal, for ksvd_code_backward.  coef gets the
 * coefficients (0 in unused slots).  No counterpart in the reference (its coding is OMP only). */
KSVD_API ksvd_status ksvd_code_fixed(ksvd_handle* handle, const float* D, const float* X, int64_t N,
                                     const int32_t* idx, const int32_t* nnz, float* coef,
                                     float* chol);

/* One step of mixed-precision iterative refinement of least-squares coefficients on the fixed
 * supports idx/nnz: r = x - D_S gamma accumulated in FP64, delta = (D_S'D_S)^-1 D_S'r with the FP32
 * Cholesky factor, gamma += delta.  coef (N x T slots) is updated in place, rounded to FP32;
 * coef64 (nullable, N x T doubles) receives the FP64 result.  Starting from any coefficients on
 * the support this gives the least-squares solution to ~(cond * 2^-24)^2 relative error.
 * No counterpart in the reference (its coefficients are never refined). */
KSVD_API ksvd_status ksvd_refine_coefs(ksvd_handle* handle, const float* D, const float* X,
                                       int64_t N, const int32_t* idx, const int32_t* nnz,
                                       float* coef, double* coef64);

/* Adjoint of ksvd_code_fixed: given dcoef = dL/dgamma (T slots per signal), adds the gradient
 * through the coding step, dL/dD(:, S_t) += r u_t - (D_S u) gamma_t with u = (D_S'D_S)^-1 dcoef
 * and r = x - D_S gamma, into dD (n x K, accumulated: zero it for a fresh gradient; nullable),
 * and writes dL/dX = D_S u into dX (n x N; nullable).  Uses the Cholesky factors saved by
 * ksvd_code_fixed.  No counterpart in the reference. */
KSVD_API ksvd_status ksvd_code_backward(ksvd_handle* handle, const float* D, const float* X,
                                        int64_t N, const int32_t* idx, const int32_t* nnz,
                                        const float* coef, const float* chol, const float* dcoef,
                                        float* dD, float* dX);

/* Number of iterations ksvd_iterate and ksvd_batched_iterate have run as CUDA-graph replays on
 * this handle (0 when the flag is off or capture was refused, in which case the iterations ran
 * as plain launches). */
KSVD_API int64_t ksvd_graph_replays(const ksvd_handle* handle);

/* ---- autotuning --------------------------------------------------------------------------- */

/* Launch shapes chosen per handle (0 = the built-in default). */
typedef struct ksvd_tuning {
  int32_t omp_grid_mult; /* Batch-OMP blocks = resident CTA slots x this (grid-stride); 0 (the
                            default): one resident grid, warps claim signals from a queue      */
  int32_t sweep_ctas;    /* CTAs of the cooperative atom sweep (0: one per SM)                  */
  int32_t batch_chunk;   /* signals per work-queue chunk of the batched Batch-OMP (default 16)  */
  int32_t batch_concurrent; /* ksvd_batched_iterate: 1 = per-problem updates concurrently on
                               their own streams with SM shares; 0 (default) = one after
                               another, each sweep on the whole GPU                            */
  int32_t tuned;         /* 1 after an autotune call                                           */
  int32_t omp_fp16;      /* mixed precision, T <= 32: Batch-OMP's alpha update from an FP16 copy
                            of G with FP32 near-tie re-evaluation (same selections as FP32):
                            1 on, 0 off, -1 automatic (on for T >= 14)                        */
} ksvd_tuning;

/* Times Batch-OMP grid sizes (and, for a mixed-precision handle, the FP16 alpha update on and
 * off) and sweep CTA counts on this problem (D n x K, X n x N, device) and
 * keeps the fastest for the handle's later calls; D, X and the atom-order stream are not
 * changed.  Costs a few OMP and dictionary-update passes.  No reference counterpart. */
KSVD_API ksvd_status ksvd_autotune(ksvd_handle* handle, const float* D, const float* X, int64_t N,
                                   ksvd_tuning* out);
/* Times the batched work-queue chunk (ksvd_batched_omp) and the batched update mode (one
 * iteration of ksvd_batched_iterate; the dictionaries are restored afterwards) on these
 * problems. */
KSVD_API ksvd_status ksvd_autotune_batched(ksvd_handle* handle, const struct ksvd_problem* probs,
                                           int32_t nprob, ksvd_tuning* out);
KSVD_API ksvd_status ksvd_get_tuning(const ksvd_handle* handle, ksvd_tuning* out);
KSVD_API ksvd_status ksvd_set_tuning(ksvd_handle* handle, const ksvd_tuning* tuning);

/* ---- many independent problems ------------------------------------------------------------- */

/* One problem of a batched call.  Device pointers, column-major like the single-problem calls. */
typedef struct ksvd_problem {
  int32_t n;          /* signal length, 1..1024                                              */
  int32_t K;          /* atoms, 1..1024                                                      */
  int32_t T;          /* coefficient slots per signal (maximum support), 1..min(K, 64)        */
  int32_t reserved;   /* 0                                                                   */
  int64_t N;          /* signals (0 = skip this problem)                                     */
  float* D;           /* n x K dictionary, unit-norm columns (ksvd_batched_iterate updates it) */
  const float* X;     /* n x N signals                                                       */
  const float* eps2;  /* N error targets ||x - D gamma||^2 <= eps2 (nullable: T atoms each)   */
  int32_t* idx;       /* N x T atom slots (out)                                              */
  float* coef;        /* N x T coefficients (out)                                            */
  int32_t* nnz;       /* N atoms used per signal (out)                                       */
} ksvd_problem;

/* Batch-OMP of every problem: one grouped GEMM launch for all G = D'D and alpha0 = D'X, then ONE
 * persistent launch in which warps take chunks of signals of any problem from a device work
 * queue (uneven supports from the error targets balance themselves).  FP32; the handle's
 * n/K/T are not used, only its stream and workspace.  Asynchronous on the handle's stream.
 * Replaces a loop of OMP::BatchOMP calls (S/OMP.cu:42-59), one per dictionary. */
KSVD_API ksvd_status ksvd_batched_omp(ksvd_handle* handle, const ksvd_problem* probs,
                                      int32_t nprob);

/* iters K-SVD iterations of every problem (each N >= 1): per iteration ONE persistent Batch-OMP
 * launch over all problems (as ksvd_batched_omp), then every problem's dictionary update, error
 * and clearDict -- one after another with each sweep on the whole GPU, or (tuning
 * batch_concurrent) concurrently on their own streams with the cooperative sweeps sharing the
 * SMs in proportion to N*T.  D is normalised first and updated in place; idx/coef/nnz hold the last
 * iteration's code; rmse (host, nullable) gets nprob x iters values, problem-major.  The
 * handle's mu_thresh, use_thresh, max_replace_signals and seed apply to every problem (FP32).
 * With KSVD_FLAG_GRAPH on the handle, iterations 2..iters replay one CUDA graph of the whole
 * batched iteration (captured once per set of buffers and shapes).
 * Replaces a host loop of KSVD::ExecuteIterations calls (S/KSVD.cu:55-131), one per dictionary. */
KSVD_API ksvd_status ksvd_batched_iterate(ksvd_handle* handle, ksvd_problem* probs,
                                          int32_t nprob, int32_t iters, double* rmse);

/* ---- whole algorithm ----------------------------------------------------------------------- */

/* iters K-SVD iterations: normcols(D) once, then per iteration Gram, D'X, Batch-OMP, dictionary
 * sweep, error, clearDict.  D (n x K) is updated in place; idx/coef/nnz receive the last
 * iteration's sparse code; rmse (HOST, nullable, iters entries) the per-iteration RMSE printed
 * by the reference.  perms: HOST array of iters*K atom orders, or NULL to draw them from
 * (seed, iteration).  Replaces KSVD::ExecuteIterations (KSVD.cu:55-131). */
KSVD_API ksvd_status ksvd_iterate(ksvd_handle* handle, float* D, const float* X, int64_t N, int32_t iters,
                         const int32_t* perms, int32_t* idx, float* coef, int32_t* nnz,
                         double* rmse);

/* ksvd_iterate with error-constrained coding: signal s stops taking atoms once
 * ||x_s - D gamma_s||^2 <= eps2[s] (device, N floats) or after T atoms (Rubinstein et al.'s
 * Batch-OMP stopping rule; the reference codes to sparsity T only). */
KSVD_API ksvd_status ksvd_iterate_eps(ksvd_handle* handle, float* D, const float* X, int64_t N,
                                      int32_t iters, const int32_t* perms, const float* eps2,
                                      int32_t* idx, float* coef, int32_t* nnz, double* rmse);

/* Same as ksvd_iterate with every array in HOST memory: X and D are copied to the device, the
 * iterations run, and D, idx, coef, nnz are copied back.  This is the whole-program contract of
 * the reference executable (main.cu:42-159) minus its MAT-file I/O. */
KSVD_API ksvd_status ksvd_iterate_host(ksvd_handle* handle, float* D, const float* X, int64_t N,
                              int32_t iters, const int32_t* perms, int32_t* idx, float* coef,
                              int32_t* nnz, double* rmse);

/* Dense K x N coefficients from the sparse code (zeros elsewhere): the reference's CUDA_Gamma
 * output (main.cu:133-142). */
KSVD_API ksvd_status ksvd_dense_gamma(ksvd_handle* handle, int64_t N, const int32_t* idx,
                             const float* coef, const int32_t* nnz, float* gamma);

/* Per-stage device times accumulated since the last reset (needs KSVD_FLAG_PROFILE in
 * params.flags; zeros otherwise).  Synchronises the stream.  No counterpart in the reference,
 * which times only the whole run (main.cu:108-113). */
KSVD_API ksvd_status ksvd_read_stage_times(ksvd_handle* handle, ksvd_stage_times* out,
                                           int32_t reset);

/* sqrt(sum_s ||x_s - D gamma_s||^2 / (n N)) -- the RMSE of ksvd_error -- without allocating any
 * device memory and without a handle, for callers that cannot call cudaMalloc where they need
 * the number: their device memory is owned by another allocator (a framework's caching
 * allocator, a fixed budget given to a plugin), or they run on a latency-critical path where
 * cudaMalloc's implicit device synchronisation is not acceptable.  All arrays are DEVICE arrays
 * (D n x K, X n x N, the sparse code); *rmse is written on the HOST and the stream is
 * synchronised.  The scratch is a static device array of 65,538 doubles: N <= 16,777,216
 * (KSVD_ERR_UNSUPPORTED beyond), n <= 1024, K <= 1024, T <= 64.  The first call on a device
 * resolves the array's address (make it before any stream capture); concurrent calls on one
 * device race on the shared array.  ksvd_last_error(NULL) describes the last failure.  No
 * counterpart in the reference. */
KSVD_API ksvd_status ksvd_rmse_noalloc(int32_t n, int32_t K, int32_t T, const float* D,
                                       const float* X, int64_t N, const int32_t* idx,
                                       const float* coef, const int32_t* nnz, double* rmse,
                                       void* stream);

/* Block until all work enqueued by this handle has finished; reports device-side errors. */
KSVD_API ksvd_status ksvd_synchronize(ksvd_handle* handle);

#ifdef __cplusplus
}
#endif

#endif /* KSVD_GB300_H */
