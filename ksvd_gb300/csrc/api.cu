// api.cu -- the C ABI (include/ksvd_gb300.h): handle, device workspace and the host-side
// orchestration of the K-SVD iteration.  Replaces the reference's KSVD / OMP /
// DictionaryUpdate classes (KSVD.cu, OMP.cu, DictionaryUpdate.cu), its enum-indexed
// DeviceMemory pool (DeviceMemory.cu:19-138) and its cuBLAS handle base (CudaAlgorithm.cu).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "../../include/ksvd_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

using namespace ksvd;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

}  // namespace

struct ksvd_handle {
  ksvd_params p{};
  int Kp = 0;
  cudaStream_t stream = nullptr;
  int device = 0;
  std::string err;
  std::vector<DevBuf> bufs;
  // stage state (what the last update / error call left behind)
  int64_t update_N = -1;
  int64_t error_N = -1;
  int64_t perm_draws = 0;
  // BF16 hi/lo copy of X for the mixed path (valid for one call: X may change between calls)
  const float* xsplit_src = nullptr;
  int64_t xsplit_N = -1;
  // stage profiling (KSVD_FLAG_PROFILE)
  struct Pending { int stage; cudaEvent_t a, b; };
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<Pending> pending;
  double stage_ms[8] = {0};
  int64_t stage_calls[8] = {0};
  bool profiling() const { return (p.flags & KSVD_FLAG_PROFILE) != 0; }
  // CUDA graphs of one K-SVD iteration (KSVD_FLAG_GRAPH): captured on a side stream, replayed.
  // One cache for ksvd_iterate, one for ksvd_batched_iterate; a key lists every pointer and size
  // the captured launches bake in.
  struct GraphCache {
    cudaGraphExec_t exec = nullptr;
    std::vector<const void*> key;
  };
  cudaStream_t gstream = nullptr;
  cudaEvent_t gev[2] = {nullptr, nullptr};
  GraphCache graphs[2];
  bool graph_broken = false;
  int64_t graph_replays = 0;
  // batched K-SVD: one child handle (own stream and workspace) per problem
  std::vector<ksvd_handle*> kids;
  std::vector<cudaStream_t> kid_streams;
  std::vector<cudaEvent_t> kid_events;
  cudaEvent_t fork_ev = nullptr;
  int sweep_ctas = 0;   // CTAs of this handle's cooperative sweep (0: one per SM)
  // error-constrained iterations (ksvd_iterate_eps): per-signal ||x||^2 and targets, for the call
  const float* it_xn2 = nullptr;
  const float* it_eps2 = nullptr;
  // ksvd_iterate_host: X arrives in chunks on a copy stream; the first iteration's D'X and
  // Batch-OMP start on each chunk as soon as its copy event fires
  static constexpr int kMaxInflow = 16;
  struct Inflow {
    bool active = false;
    int nchunks = 0;
    int64_t bounds[kMaxInflow + 1] = {};
    cudaEvent_t ev[kMaxInflow] = {};
    cudaStream_t cstream = nullptr;
    // results drained to the host while the last iteration finishes (ksvd_iterate_host):
    // idx/nnz after its Batch-OMP, coef after its sweep, on cstream
    bool drain = false;
    int32_t* h_idx = nullptr;
    float* h_coef = nullptr;
    int32_t* h_nnz = nullptr;
    cudaEvent_t dev_ev[2] = {};
  } inflow;
  int omp_grid_mult = 0;  // Batch-OMP blocks per resident CTA slot (0: default)
  int omp_fp16 = -1;      // mixed path's FP16 alpha update: 1 on, 0 off, -1 automatic
  int batch_chunk = 0;    // signals per batched work-queue chunk (0: default)
  int batch_concurrent = 0;  // batched updates: 1 = concurrent streams with SM shares,
                             // 0 = one after another, each sweep on the whole GPU
  bool tuned = false;
  // host copies of the batched call's tables (kept alive for the asynchronous uploads)
  std::vector<ksvd::GemmDesc> batch_descs;
  std::vector<ksvd::OmpJob> batch_jobs;
  std::vector<const float*> batch_dicts;   // every job's dictionary (n x K), for the mixed path
};

namespace {

enum BufId {
  B_DPAD, B_G, B_A0, B_XN2, B_LIST, B_START, B_BHIST, B_Y, B_GN2, B_C, B_AVEC, B_AD, B_PART,
  B_UNUSED, B_BITMAP, B_REPLACED, B_COUNTER, B_USE, B_BARRIER, B_ERR, B_PSUM, B_BVAL, B_BIDX,
  B_RMSE, B_M, B_MI, B_CLEARED, B_DEVERR, B_PERM, B_GPAD_IN, B_HX, B_HD, B_HIDX, B_HCOEF, B_HNNZ,
  B_XHI, B_XLO, B_DHI, B_DLO, B_P, B_BG, B_BA0, B_BDESC, B_BJOB, B_BQUEUE, B_ITER, B_RPART, B_RMEAN, B_TUNE_D, B_TUNE_C, B_GH, B_MU, B_OMPQ, B_PREP_PART, B_COUNT
};

ksvd_status fail(ksvd_handle* h, ksvd_status s, const char* fmt, const char* detail = nullptr) {
  if (h) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), fmt, detail ? detail : "");
    h->err = buf;
  }
  return s;
}

ksvd_status cuda_fail(ksvd_handle* h, cudaError_t e, const char* where) {
  if (h) h->err = std::string(where) + ": " + cudaGetErrorString(e);
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return KSVD_ERR_OUT_OF_MEMORY;
  return KSVD_ERR_CUDA;
}

#define KSVD_CK(h, call)                                   \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

#define KSVD_TRY(expr)                     \
  do {                                     \
    ksvd_status s_ = (expr);               \
    if (s_ != KSVD_OK) return s_;          \
  } while (0)

template <typename T>
ksvd_status ensure(ksvd_handle* h, BufId id, size_t count, T** out) {
  DevBuf& b = h->bufs[id];
  const size_t bytes = count * sizeof(T) + 256;
  if (b.cap < bytes) {
    if (b.p) {
      cudaStreamSynchronize(h->stream);
      cudaFree(b.p);
      b.p = nullptr;
      b.cap = 0;
    }
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc(workspace)");
    b.cap = bytes;
  }
  *out = reinterpret_cast<T*>(b.p);
  return KSVD_OK;
}

ksvd_status check_params(const ksvd_params* p, ksvd_handle* h) {
  if (!p) return fail(h, KSVD_ERR_INVALID_ARGUMENT, "null params%s");
  if (p->n < 1 || p->K < 1 || p->T < 1) return fail(h, KSVD_ERR_INVALID_ARGUMENT, "n, K, T must be >= 1%s");
  if (p->K > kMaxK) return fail(h, KSVD_ERR_UNSUPPORTED, "K > 1024 is not supported%s");
  if (p->T > kMaxT) return fail(h, KSVD_ERR_UNSUPPORTED, "T > 64 is not supported%s");
  if (p->n > kMaxN) return fail(h, KSVD_ERR_UNSUPPORTED, "n > 1024 is not supported%s");
  if (p->T > p->K) return fail(h, KSVD_ERR_INVALID_ARGUMENT, "T must be <= K%s");
  if (p->precision != KSVD_PREC_FP32 && p->precision != KSVD_PREC_MIXED)
    return fail(h, KSVD_ERR_INVALID_ARGUMENT, "unknown precision%s");
  if (p->max_replace_signals < 1) return fail(h, KSVD_ERR_INVALID_ARGUMENT, "max_replace_signals must be >= 1%s");
  return KSVD_OK;
}

ksvd_status check_dev_err(ksvd_handle* h) {
  int* de = nullptr;
  KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
  int v = 0;
  KSVD_CK(h, cudaMemcpyAsync(&v, de, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  KSVD_CK(h, cudaStreamSynchronize(h->stream));
  if (v == 0) return KSVD_OK;
  KSVD_CK(h, cudaMemsetAsync(de, 0, sizeof(int), h->stream));
  if (v & kDevErrTimeout) return fail(h, KSVD_ERR_TIMEOUT, "a device-side grid barrier timed out%s");
  if (v & kDevErrBounds) return fail(h, KSVD_ERR_INVALID_ARGUMENT, "sparse code holds an atom index outside [0, K)%s");
  return fail(h, KSVD_ERR_NUMERIC, "NaN or Inf met on the device%s");
}

uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

cudaEvent_t next_event(ksvd_handle* h) {
  if (h->ev_used == h->ev_pool.size()) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    h->ev_pool.push_back(e);
  }
  return h->ev_pool[h->ev_used++];
}

// Brackets one stage with events on the handle's stream when profiling is on.
struct StageScope {
  ksvd_handle* h;
  int stage;
  cudaEvent_t a = nullptr;
  StageScope(ksvd_handle* hh, int s) : h(hh), stage(s) {
    if (h->profiling() && (a = next_event(h))) cudaEventRecord(a, h->stream);
  }
  ~StageScope() {
    if (!a) return;
    cudaEvent_t b = next_event(h);
    if (!b) return;
    cudaEventRecord(b, h->stream);
    h->pending.push_back({stage, a, b});
  }
};

void collect_stage_times(ksvd_handle* h) {
  for (const auto& p : h->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      h->stage_ms[p.stage] += ms;
      h->stage_calls[p.stage] += 1;
    }
  }
  h->pending.clear();
  h->ev_used = 0;
  cudaGetLastError();
}

// Working copy of a user dictionary (n x K) in the zero-padded n x Kp buffer.
ksvd_status load_dict(ksvd_handle* h, const float* D, float** Dp) {
  const int n = h->p.n, K = h->p.K, Kp = h->Kp;
  KSVD_TRY(ensure(h, B_DPAD, (size_t)n * Kp, Dp));
  KSVD_CK(h, launch_copy_pad_cols(D, n, K, *Dp, Kp, h->stream));
  return KSVD_OK;
}

ksvd_status store_dict(ksvd_handle* h, const float* Dp, float* D) {
  const size_t bytes = sizeof(float) * (size_t)h->p.n * h->p.K;
  KSVD_CK(h, cudaMemcpyAsync(D, Dp, bytes, cudaMemcpyDeviceToDevice, h->stream));
  return KSVD_OK;
}

// Row length of the BF16 parts: at least one 64-element TMA box (the columns past n are zero),
// a multiple of 8 (16-byte rows).  tc_inner(n) is the inner extent the tensor-core GEMM reads.
int64_t bf16_ld(int n) { return n < 64 ? 64 : round_up(n, 8); }
int tc_inner(int n) { return n < 64 ? 64 : n; }

bool mixed(const ksvd_handle* h) { return h->p.precision == KSVD_PREC_MIXED; }

// BF16 hi/lo parts of the padded working dictionary (Kp rows of n).
ksvd_status split_dict(ksvd_handle* h, const float* Dp, TcOperand* op) {
  const int n = h->p.n, Kp = h->Kp;
  const int64_t ld = bf16_ld(n);
  uint16_t *hi = nullptr, *lo = nullptr;
  KSVD_TRY(ensure(h, B_DHI, (size_t)Kp * ld, &hi));
  KSVD_TRY(ensure(h, B_DLO, (size_t)Kp * ld, &lo));
  KSVD_CK(h, launch_split_bf16(Dp, n, Kp, n, hi, lo, ld, Kp, h->stream));
  op->hi = hi; op->lo = lo; op->ld = ld; op->rows = Kp;
  return KSVD_OK;
}

// BF16 hi/lo parts of X (N rows of n); made once per call and reused by every iteration.
ksvd_status split_signals(ksvd_handle* h, const float* X, int64_t N, TcOperand* op) {
  const int n = h->p.n;
  const int64_t ld = bf16_ld(n);
  uint16_t *hi = nullptr, *lo = nullptr;
  KSVD_TRY(ensure(h, B_XHI, (size_t)N * ld, &hi));
  KSVD_TRY(ensure(h, B_XLO, (size_t)N * ld, &lo));
  if (h->xsplit_src != X || h->xsplit_N != N) {
    StageScope sc(h, KSVD_STAGE_DTX);
    KSVD_CK(h, launch_split_bf16(X, n, N, n, hi, lo, ld, N, h->stream));
    h->xsplit_src = X;
    h->xsplit_N = N;
  }
  op->hi = hi; op->lo = lo; op->ld = ld; op->rows = N;
  return KSVD_OK;
}

// Forget the cached X split (called at the end of every public call).
void drop_xsplit(ksvd_handle* h) { h->xsplit_src = nullptr; h->xsplit_N = -1; }

// G = D'D for the padded working dictionary (Kp x Kp, zero padded)
ksvd_status gram_padded(ksvd_handle* h, const float* Dp, float* G) {
  StageScope sc(h, KSVD_STAGE_GRAM);
  const int n = h->p.n, K = h->p.K, Kp = h->Kp;
  if (mixed(h)) {
    TcOperand d;
    int* de = nullptr;
    KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
    KSVD_TRY(split_dict(h, Dp, &d));
    KSVD_CK(h, launch_gemm_tn_bf16(d, d, G, Kp, Kp, Kp, tc_inner(n), 3, de, h->stream));
    return KSVD_OK;
  }
  KSVD_CK(h, launch_gemm_tn_f32(Dp, n, Dp, n, G, Kp, K, Kp, K, Kp, n, h->stream));
  return KSVD_OK;
}

// alpha0 = D'X into the Kp x N buffer (rows K..Kp-1 zero)
ksvd_status dtx_padded(ksvd_handle* h, const float* Dp, const float* X, int64_t N, float* A0) {
  const int n = h->p.n, K = h->p.K, Kp = h->Kp;
  if (mixed(h)) {
    TcOperand d, x;
    int* de = nullptr;
    KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
    KSVD_TRY(split_signals(h, X, N, &x));
    StageScope sc(h, KSVD_STAGE_DTX);
    KSVD_TRY(split_dict(h, Dp, &d));
    KSVD_CK(h, launch_gemm_tn_bf16(d, x, A0, Kp, Kp, N, tc_inner(n), 3, de, h->stream));
    return KSVD_OK;
  }
  StageScope sc(h, KSVD_STAGE_DTX);
  KSVD_CK(h, launch_gemm_tn_f32(Dp, n, X, n, A0, Kp, K, Kp, N, N, n, h->stream));
  return KSVD_OK;
}

// alpha0 columns [s0, s1) (signals s0..s1-1 of X; for the mixed path their BF16 parts are
// made first, into the call's cached split of X).
ksvd_status dtx_padded_range(ksvd_handle* h, const float* Dp, const float* X, int64_t N,
                             int64_t s0, int64_t s1, float* A0) {
  const int n = h->p.n, K = h->p.K, Kp = h->Kp;
  const int64_t Nc = s1 - s0;
  if (Nc <= 0) return KSVD_OK;
  if (mixed(h)) {
    const int64_t ld = bf16_ld(n);
    uint16_t *hi = nullptr, *lo = nullptr;
    int* de = nullptr;
    KSVD_TRY(ensure(h, B_XHI, (size_t)N * ld, &hi));
    KSVD_TRY(ensure(h, B_XLO, (size_t)N * ld, &lo));
    KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
    StageScope sc(h, KSVD_STAGE_DTX);
    KSVD_CK(h, launch_split_bf16(X + s0 * n, n, Nc, n, hi + s0 * ld, lo + s0 * ld, ld, Nc,
                                 h->stream));
    TcOperand d, x;
    KSVD_TRY(split_dict(h, Dp, &d));
    x.hi = hi + s0 * ld; x.lo = lo + s0 * ld; x.ld = ld; x.rows = Nc;
    KSVD_CK(h, launch_gemm_tn_bf16(d, x, A0 + s0 * Kp, Kp, Kp, Nc, tc_inner(n), 3, de, h->stream));
    return KSVD_OK;
  }
  StageScope sc(h, KSVD_STAGE_DTX);
  KSVD_CK(h, launch_gemm_tn_f32(Dp, n, X + s0 * n, n, A0 + s0 * Kp, Kp, K, Kp, Nc, Nc, n,
                                h->stream));
  return KSVD_OK;
}

ksvd_status run_omp(ksvd_handle* h, const float* G, const float* A0, int64_t N,
                    const float* xnorm2, const float* eps2, int32_t* idx, float* coef,
                    int32_t* nnz, bool make_gh = true) {
  int* de = nullptr;
  KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
  // mixed path: the alpha update reads an FP16 copy of G (made here, G may have changed since
  // the last call) and resolves near ties in FP32.  It pays once the re-read support columns
  // dominate the step (measured: slower at T = 8 and 10, faster at T = 16); the autotuner
  // times both.
  uint16_t* gh = nullptr;
  float* mu = nullptr;
  const int T = h->p.T;
  if (mixed(h) && T <= 32 && (h->omp_fp16 > 0 || (h->omp_fp16 < 0 && T >= 14))) {
    KSVD_TRY(ensure(h, B_GH, (size_t)h->Kp * h->Kp, &gh));
    KSVD_TRY(ensure(h, B_MU, (size_t)h->Kp + 1, &mu));
  }
  unsigned long long* q = nullptr;     // grid_mult 0: signals claimed from a work queue
  if (h->omp_grid_mult == 0) KSVD_TRY(ensure(h, B_OMPQ, 1, &q));
  StageScope sc(h, KSVD_STAGE_OMP);
  if (gh && make_gh) KSVD_CK(h, launch_gram_half(G, h->Kp, h->p.K, gh, mu, h->stream));
  KSVD_CK(h, launch_omp(G, h->Kp, A0, h->Kp, h->p.K, N, h->p.T, xnorm2, eps2, idx, coef, nnz, de,
                        h->stream, h->omp_grid_mult, gh, mu, q));
  return KSVD_OK;
}

ksvd_status update_ws(ksvd_handle* h, int64_t N, UpdateArgs& u) {
  const int n = h->p.n, Kp = h->Kp;
  const int64_t nblk = update_block_count(N);
  const int nctas = update_sweep_ctas();
  std::memset(&u, 0, sizeof(u));
  KSVD_TRY(ensure(h, B_LIST, (size_t)N * h->p.T, &u.list));
  KSVD_TRY(ensure(h, B_START, (size_t)Kp + 1, &u.start));
  KSVD_TRY(ensure(h, B_BHIST, (size_t)Kp * nblk, &u.block_hist));
  KSVD_TRY(ensure(h, B_Y, (size_t)n * Kp, &u.Y));
  KSVD_TRY(ensure(h, B_GN2, (size_t)Kp, &u.gn2));
  KSVD_TRY(ensure(h, B_C, (size_t)Kp * Kp, &u.C));
  KSVD_TRY(ensure(h, B_AVEC, (size_t)3 * n, &u.avec));
  KSVD_TRY(ensure(h, B_AD, (size_t)2 * Kp, &u.aD));
  KSVD_TRY(ensure(h, B_G, (size_t)Kp * Kp, &u.G));
  KSVD_TRY(ensure(h, B_P, (size_t)Kp * Kp, &u.P));
  KSVD_TRY(ensure(h, B_PART, (size_t)4 * (nctas + 1), &u.part));
  KSVD_TRY(ensure(h, B_UNUSED, (size_t)N, &u.unused));
  KSVD_TRY(ensure(h, B_BITMAP, (size_t)N, &u.bitmap));
  KSVD_TRY(ensure(h, B_REPLACED, (size_t)Kp, &u.replaced));
  KSVD_TRY(ensure(h, B_COUNTER, 1, &u.counter));
  KSVD_TRY(ensure(h, B_USE, (size_t)Kp, &u.usecount));
  KSVD_TRY(ensure(h, B_BARRIER, 2, &u.barrier));
  KSVD_TRY(ensure(h, B_DEVERR, 1, &u.dev_err));
  u.prep_win = prepare_window_signals(N, n, h->p.T);
  if (u.prep_win > 0) {
    const int64_t nwin = (N + u.prep_win - 1) / u.prep_win;
    KSVD_TRY(ensure(h, B_PREP_PART, (size_t)nwin * Kp * (n + Kp + 1), &u.prep_part));
  }
  u.n = n; u.K = h->p.K; u.Kp = Kp; u.T = h->p.T; u.N = N;
  u.max_signals = h->p.max_replace_signals;
  u.sweep_ctas = h->sweep_ctas;
  return KSVD_OK;
}

ksvd_status run_update(ksvd_handle* h, float* Dp, const float* X, int64_t N, const int32_t* idx,
                       float* coef, const int32_t* nnz, const int32_t* perm_dev,
                       const int* iter_ctr = nullptr) {
  UpdateArgs u;
  KSVD_TRY(update_ws(h, N, u));
  u.X = X; u.D = Dp; u.idx = idx; u.coef = coef; u.nnz = nnz; u.perm = perm_dev;
  u.iter_ctr = iter_ctr;
  KSVD_TRY(gram_padded(h, Dp, u.G));          // the sweep maintains G = D'D from here on
  {
    StageScope sc(h, KSVD_STAGE_LISTS);
    KSVD_CK(h, launch_update_prepare(u, h->stream));
  }
  {
    StageScope sc(h, KSVD_STAGE_SWEEP);
    KSVD_CK(h, launch_update_sweep(u, h->stream));
  }
  h->update_N = N;
  return KSVD_OK;
}

ksvd_status run_error(ksvd_handle* h, const float* Dp, const float* X, int64_t N,
                      const int32_t* idx, const float* coef, const int32_t* nnz,
                      double* rmse_dev_slot, const int* iter_ctr = nullptr) {
  ErrorArgs a;
  std::memset(&a, 0, sizeof(a));
  const int64_t nb = error_block_count(N);
  KSVD_TRY(ensure(h, B_ERR, (size_t)N, &a.err));
  KSVD_TRY(ensure(h, B_PSUM, (size_t)nb, &a.part_sum));
  KSVD_TRY(ensure(h, B_BVAL, (size_t)nb, &a.bucket_val));
  KSVD_TRY(ensure(h, B_BIDX, (size_t)nb, &a.bucket_idx));
  a.n = h->p.n; a.K = h->p.K; a.Kp = h->Kp; a.T = h->p.T; a.N = N;
  a.X = X; a.D = Dp; a.idx = idx; a.coef = coef; a.nnz = nnz;
  int32_t* bm = nullptr;
  if (h->update_N == N) KSVD_TRY(ensure(h, B_BITMAP, (size_t)N, &bm));
  a.bitmap = bm;
  a.rmse_out = rmse_dev_slot;
  a.iter_ctr = iter_ctr;
  KSVD_TRY(ensure(h, B_DEVERR, 1, &a.dev_err));
  StageScope sc(h, KSVD_STAGE_ERROR);
  KSVD_CK(h, launch_error(a, h->stream));
  h->error_N = N;
  return KSVD_OK;
}

ksvd_status run_clear(ksvd_handle* h, float* Dp, float* G, const float* X, int64_t N,
                      int32_t* cleared_dev) {
  ClearArgs c;
  std::memset(&c, 0, sizeof(c));
  const int Kp = h->Kp;
  c.n = h->p.n; c.K = h->p.K; c.Kp = Kp; c.N = N; c.X = X; c.D = Dp; c.G = G;
  int32_t *use = nullptr, *rep = nullptr;
  KSVD_TRY(ensure(h, B_USE, (size_t)Kp, &use));
  KSVD_TRY(ensure(h, B_REPLACED, (size_t)Kp, &rep));
  c.usecount = use; c.replaced = rep;
  const int64_t nb = error_block_count(N);
  KSVD_TRY(ensure(h, B_ERR, (size_t)N, &c.err));
  KSVD_TRY(ensure(h, B_BVAL, (size_t)nb, &c.bucket_val));
  KSVD_TRY(ensure(h, B_BIDX, (size_t)nb, &c.bucket_idx));
  c.nbuckets = nb;
  c.mu_thresh = h->p.mu_thresh;
  c.use_thresh = h->p.use_thresh;
  c.cleared = cleared_dev;
  float* m = nullptr;
  int* mi = nullptr;
  KSVD_TRY(ensure(h, B_M, (size_t)Kp, &m));
  KSVD_TRY(ensure(h, B_MI, (size_t)Kp, &mi));
  StageScope sc(h, KSVD_STAGE_CLEAR);
  KSVD_CK(h, launch_clear_dict(c, m, mi, h->stream));
  return KSVD_OK;
}

ksvd_status upload_perm(ksvd_handle* h, const int32_t* perms_host, int32_t iters, int32_t** out) {
  const int K = h->p.K;
  std::vector<int32_t> tmp;
  if (!perms_host) {
    tmp.resize((size_t)iters * K);
    for (int32_t it = 0; it < iters; ++it)
      ksvd_random_permutation(h->p.seed, h->perm_draws + it, K, tmp.data() + (size_t)it * K);
    h->perm_draws += iters;
    perms_host = tmp.data();
  } else {
    std::vector<char> seen(K);
    for (int32_t it = 0; it < iters; ++it) {
      std::fill(seen.begin(), seen.end(), 0);
      for (int k = 0; k < K; ++k) {
        const int32_t v = perms_host[(size_t)it * K + k];
        if (v < 0 || v >= K || seen[v])
          return fail(h, KSVD_ERR_INVALID_ARGUMENT, "perms must hold permutations of 0..K-1%s");
        seen[v] = 1;
      }
    }
  }
  int32_t* d = nullptr;
  KSVD_TRY(ensure(h, B_PERM, (size_t)iters * K, &d));
  KSVD_CK(h, cudaMemcpyAsync(d, perms_host, sizeof(int32_t) * (size_t)iters * K,
                             cudaMemcpyHostToDevice, h->stream));
  KSVD_CK(h, cudaStreamSynchronize(h->stream));   // perms_host may be a temporary
  *out = d;
  return KSVD_OK;
}

bool bad_ptr(const void* p) { return p == nullptr; }

// A public call given a null handle records that in the no-handle error slot.
bool null_handle(const ksvd_handle* h) {
  if (h) return false;
  ksvd::set_nohandle_error("a ksvd_* call was given a null handle");
  return true;
}


}  // namespace

namespace ksvd {
thread_local std::string g_nohandle_err;
void set_nohandle_error(const char* msg) { g_nohandle_err = msg ? msg : ""; }
}  // namespace ksvd

// ============================================================================================
extern "C" {

void ksvd_default_params(ksvd_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->T = 6;                        // ProgramParameters.cuh:20
  p->precision = KSVD_PREC_FP32;
  p->mu_thresh = 0.8f;             // ProgramParameters.cuh:23
  p->use_thresh = 4;               // GlobalDeclarations.cuh:54
  p->max_replace_signals = 5000;   // GlobalDeclarations.cuh:63
  p->seed = 0x4B535644ull;
}

int32_t ksvd_abi_version(void) { return KSVD_GB300_ABI_VERSION; }

const char* ksvd_status_string(ksvd_status s) {
  switch (s) {
    case KSVD_OK: return "ok";
    case KSVD_ERR_INVALID_ARGUMENT: return "invalid argument";
    case KSVD_ERR_UNSUPPORTED: return "unsupported size";
    case KSVD_ERR_OUT_OF_MEMORY: return "out of device memory";
    case KSVD_ERR_CUDA: return "CUDA error";
    case KSVD_ERR_NUMERIC: return "NaN or Inf encountered";
    case KSVD_ERR_TIMEOUT: return "device-side wait timed out";
    case KSVD_ERR_STATE: return "stage called out of order";
  }
  return "unknown status";
}

const char* ksvd_last_error(const ksvd_handle* h) {
  return h ? h->err.c_str() : ksvd::g_nohandle_err.c_str();
}

int64_t ksvd_workspace_bytes(const ksvd_handle* h) {
  if (!h) return 0;
  int64_t t = 0;
  for (const auto& b : h->bufs) t += (int64_t)b.cap;
  return t;
}

ksvd_status ksvd_random_permutation(uint64_t seed, int64_t iteration, int32_t K, int32_t* perm) {
  if (!perm || K < 1) return KSVD_ERR_INVALID_ARGUMENT;
  uint64_t st = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(iteration + 1));
  for (int32_t k = 0; k < K; ++k) perm[k] = k;
  for (int32_t k = K - 1; k > 0; --k) {       // Fisher-Yates
    const uint64_t r = splitmix64(st) % (uint64_t)(k + 1);
    const int32_t t = perm[k];
    perm[k] = perm[r];
    perm[r] = t;
  }
  return KSVD_OK;
}

ksvd_status ksvd_create(ksvd_handle** out, const ksvd_params* params, void* stream) {
  if (!out) {
    ksvd::set_nohandle_error("ksvd_create: null output pointer");
    return KSVD_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  ksvd_status s = check_params(params, nullptr);
  if (s != KSVD_OK) {
    ksvd::set_nohandle_error("ksvd_create: invalid or unsupported parameters");
    return s;
  }
  ksvd_handle* h = new (std::nothrow) ksvd_handle();
  if (!h) {
    ksvd::set_nohandle_error("ksvd_create: out of host memory");
    return KSVD_ERR_OUT_OF_MEMORY;
  }
  h->p = *params;
  h->Kp = omp_padded_k(params->K);
  h->stream = reinterpret_cast<cudaStream_t>(stream);
  h->bufs.resize(B_COUNT);
  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) {
    delete h;
    cudaGetLastError();
    ksvd::set_nohandle_error("ksvd_create: no current CUDA device");
    return KSVD_ERR_CUDA;
  }
  int* de = nullptr;
  if ((s = ensure(h, B_DEVERR, 1, &de)) != KSVD_OK) {
    ksvd::set_nohandle_error(("ksvd_create: " + h->err).c_str());
    delete h;
    return s;
  }
  if (cudaMemsetAsync(de, 0, sizeof(int), h->stream) != cudaSuccess) {
    ksvd_destroy(h);
    cudaGetLastError();
    ksvd::set_nohandle_error("ksvd_create: cudaMemsetAsync failed");
    return KSVD_ERR_CUDA;
  }
  *out = h;
  return KSVD_OK;
}

void ksvd_destroy(ksvd_handle* h) {
  if (!h) return;
  cudaStreamSynchronize(h->stream);
  for (auto& b : h->bufs)
    if (b.p) cudaFree(b.p);
  for (auto e : h->ev_pool) cudaEventDestroy(e);
  if (h->inflow.cstream) {
    cudaStreamSynchronize(h->inflow.cstream);
    cudaStreamDestroy(h->inflow.cstream);
  }
  for (auto e : h->inflow.ev)
    if (e) cudaEventDestroy(e);
  for (auto e : h->inflow.dev_ev)
    if (e) cudaEventDestroy(e);
  for (auto k : h->kids) ksvd_destroy(k);
  for (auto st : h->kid_streams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  for (auto e : h->kid_events) cudaEventDestroy(e);
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  for (auto& g : h->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (h->gstream) {
    cudaStreamSynchronize(h->gstream);
    cudaStreamDestroy(h->gstream);
  }
  for (auto e : h->gev)
    if (e) cudaEventDestroy(e);
  delete h;
}

int64_t ksvd_graph_replays(const ksvd_handle* h) { return h ? h->graph_replays : -1; }

ksvd_status ksvd_read_stage_times(ksvd_handle* h, ksvd_stage_times* out, int32_t reset) {
  if (null_handle(h) || !out) return KSVD_ERR_INVALID_ARGUMENT;
  KSVD_CK(h, cudaStreamSynchronize(h->stream));
  collect_stage_times(h);
  for (int i = 0; i < 8; ++i) {
    out->ms[i] = h->stage_ms[i];
    out->calls[i] = h->stage_calls[i];
    if (reset) { h->stage_ms[i] = 0; h->stage_calls[i] = 0; }
  }
  // a batched call's per-problem stages (their streams overlap: the sums exceed wall time)
  for (auto k : h->kids) {
    if (!k) continue;
    ksvd_stage_times kt;
    KSVD_TRY(ksvd_read_stage_times(k, &kt, reset));
    for (int i = 0; i < 8; ++i) {
      out->ms[i] += kt.ms[i];
      out->calls[i] += kt.calls[i];
    }
  }
  return KSVD_OK;
}

ksvd_status ksvd_synchronize(ksvd_handle* h) {
  if (null_handle(h)) return KSVD_ERR_INVALID_ARGUMENT;
  KSVD_CK(h, cudaStreamSynchronize(h->stream));
  collect_stage_times(h);
  KSVD_CK(h, cudaGetLastError());
  return check_dev_err(h);
}

ksvd_status ksvd_normcols(ksvd_handle* h, float* D) {
  if (null_handle(h) || bad_ptr(D)) return KSVD_ERR_INVALID_ARGUMENT;
  KSVD_CK(h, launch_normcols(D, h->p.n, h->p.K, h->stream));
  return KSVD_OK;
}

ksvd_status ksvd_remove_row_mean(ksvd_handle* h, float* X, int64_t N, float* mean) {
  if (null_handle(h) || bad_ptr(X) || N < 1) return KSVD_ERR_INVALID_ARGUMENT;
  double* part = nullptr;
  float* m = nullptr;
  KSVD_TRY(ensure(h, B_RPART, (size_t)row_mean_blocks(N) * h->p.n, &part));
  KSVD_TRY(ensure(h, B_RMEAN, (size_t)h->p.n, &m));
  KSVD_CK(h, launch_remove_row_mean(X, h->p.n, N, part, m, h->stream));
  if (mean)
    KSVD_CK(h, cudaMemcpyAsync(mean, m, sizeof(float) * h->p.n, cudaMemcpyDeviceToDevice,
                               h->stream));
  return KSVD_OK;
}

int64_t ksvd_perm_draws(const ksvd_handle* h) { return h ? h->perm_draws : -1; }

ksvd_status ksvd_set_perm_draws(ksvd_handle* h, int64_t draws) {
  if (null_handle(h) || draws < 0) return KSVD_ERR_INVALID_ARGUMENT;
  h->perm_draws = draws;
  return KSVD_OK;
}

ksvd_status ksvd_gram(ksvd_handle* h, const float* D, float* G) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(G)) return KSVD_ERR_INVALID_ARGUMENT;
  const int n = h->p.n, K = h->p.K;
  if (mixed(h)) {
    float *Dp = nullptr;
    TcOperand d;
    int* de = nullptr;
    KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
    KSVD_TRY(load_dict(h, D, &Dp));
    KSVD_TRY(split_dict(h, Dp, &d));
    KSVD_CK(h, launch_gemm_tn_bf16(d, d, G, K, K, K, tc_inner(n), 3, de, h->stream));
    return KSVD_OK;
  }
  KSVD_CK(h, launch_gemm_tn_f32(D, n, D, n, G, K, K, K, K, K, n, h->stream));
  return KSVD_OK;
}

ksvd_status ksvd_dtx(ksvd_handle* h, const float* D, const float* X, int64_t N, float* A0) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(A0) || N < 0) return KSVD_ERR_INVALID_ARGUMENT;
  const int n = h->p.n, K = h->p.K;
  if (mixed(h)) {
    float* Dp = nullptr;
    TcOperand d, x;
    int* de = nullptr;
    KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
    KSVD_TRY(load_dict(h, D, &Dp));
    KSVD_TRY(split_dict(h, Dp, &d));
    KSVD_TRY(split_signals(h, X, N, &x));
    drop_xsplit(h);
    KSVD_CK(h, launch_gemm_tn_bf16(d, x, A0, K, K, N, tc_inner(n), 3, de, h->stream));
    return KSVD_OK;
  }
  KSVD_CK(h, launch_gemm_tn_f32(D, n, X, n, A0, K, K, K, N, N, n, h->stream));
  return KSVD_OK;
}

ksvd_status ksvd_omp_gram(ksvd_handle* h, const float* G, const float* A0, int64_t N,
                          const float* xnorm2, const float* eps2, int32_t* idx, float* coef,
                          int32_t* nnz) {
  if (null_handle(h) || bad_ptr(G) || bad_ptr(A0) || bad_ptr(idx) || bad_ptr(coef) || bad_ptr(nnz) || N < 0)
    return KSVD_ERR_INVALID_ARGUMENT;
  if (eps2 && !xnorm2) return fail(h, KSVD_ERR_INVALID_ARGUMENT, "eps2 needs xnorm2%s");
  if (N == 0) return KSVD_OK;
  const int K = h->p.K, Kp = h->Kp;
  float *Gp = nullptr, *Ap = nullptr;
  KSVD_TRY(ensure(h, B_GPAD_IN, (size_t)Kp * Kp, &Gp));
  KSVD_TRY(ensure(h, B_A0, (size_t)Kp * N, &Ap));
  KSVD_CK(h, cudaMemsetAsync(Gp, 0, sizeof(float) * (size_t)Kp * Kp, h->stream));
  KSVD_CK(h, launch_copy_matrix(G, K, Gp, Kp, K, K, h->stream));
  if (Kp != K) KSVD_CK(h, cudaMemsetAsync(Ap, 0, sizeof(float) * (size_t)Kp * N, h->stream));
  KSVD_CK(h, launch_copy_matrix(A0, K, Ap, Kp, K, N, h->stream));
  return run_omp(h, Gp, Ap, N, xnorm2, eps2, idx, coef, nnz);
}

ksvd_status ksvd_omp(ksvd_handle* h, const float* D, const float* X, int64_t N, const float* eps2,
                     int32_t* idx, float* coef, int32_t* nnz) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(idx) || bad_ptr(coef) || bad_ptr(nnz) || N < 0)
    return KSVD_ERR_INVALID_ARGUMENT;
  if (N == 0) return KSVD_OK;
  drop_xsplit(h);
  float *Dp = nullptr, *G = nullptr, *A0 = nullptr, *xn2 = nullptr;
  KSVD_TRY(load_dict(h, D, &Dp));
  KSVD_TRY(ensure(h, B_G, (size_t)h->Kp * h->Kp, &G));
  KSVD_TRY(ensure(h, B_A0, (size_t)h->Kp * N, &A0));
  KSVD_TRY(gram_padded(h, Dp, G));
  KSVD_TRY(dtx_padded(h, Dp, X, N, A0));
  if (eps2) {
    KSVD_TRY(ensure(h, B_XN2, (size_t)N, &xn2));
    KSVD_CK(h, launch_col_norm2(X, h->p.n, N, xn2, h->stream));
  }
  drop_xsplit(h);
  return run_omp(h, G, A0, N, xn2, eps2, idx, coef, nnz);
}

// Many independent problems: one grouped GEMM launch for every G_p = D_p'D_p and alpha0_p =
// D_p'X_p, then one persistent Batch-OMP launch whose warps pull signal chunks of all problems
// from a device work queue.
namespace {

// The device tables of one batched Batch-OMP call: the grouped GEMM's tile table (G_i = D_i'D_i
// and alpha0_i = D_i'X_i) and the work queue's job table.
struct BatchPlan {
  GemmDesc* ddev = nullptr;
  int nd = 0;
  int64_t tiles = 0;
  OmpJob* jdev = nullptr;
  int nj = 0;
  int64_t chunks = 0;
  int tmax = 1;
  int chunk = 1;
  unsigned long long* queue = nullptr;
  int* de = nullptr;
};

// Checks the problems, sizes the shared workspace and uploads the tables (asynchronously, from
// host copies kept in the handle).  The tables depend only on the problems' sizes and pointers,
// so a batched K-SVD call uploads them once and launches them every iteration.
ksvd_status batched_omp_plan(ksvd_handle* h, const ksvd_problem* probs, int32_t nprob,
                             BatchPlan* pl) {
  int64_t g_off = 0, a_off = 0;
  int tmax = 1;
  std::vector<int64_t> goff(nprob), aoff(nprob);
  for (int32_t i = 0; i < nprob; ++i) {
    const ksvd_problem& q = probs[i];
    if (q.n < 1 || q.n > kMaxN || q.K < 1 || q.K > kMaxK || q.T < 1 || q.T > kMaxT || q.T > q.K ||
        q.N < 0)
      return fail(h, KSVD_ERR_INVALID_ARGUMENT,
                  "batched problem sizes out of range (1<=n<=1024, 1<=T<=min(K,64), K<=1024)%s");
    if (q.N > 0 && (bad_ptr(q.D) || bad_ptr(q.X) || bad_ptr(q.idx) || bad_ptr(q.coef) ||
                    bad_ptr(q.nnz)))
      return fail(h, KSVD_ERR_INVALID_ARGUMENT, "batched problem with a null pointer%s");
    if (q.N * q.T > 0x7fffffffLL)
      return fail(h, KSVD_ERR_UNSUPPORTED, "N*T must stay below 2^31 per problem%s");
    const int kp = omp_padded_k(q.K);
    goff[i] = g_off;
    aoff[i] = a_off;
    g_off += round_up((int64_t)kp * kp, 64);
    a_off += round_up((int64_t)kp * q.N, 64);
    tmax = std::max(tmax, (int)q.T);
  }
  float *Gall = nullptr, *Aall = nullptr;
  GemmDesc* ddev = nullptr;
  OmpJob* jdev = nullptr;
  unsigned long long* queue = nullptr;
  int* de = nullptr;
  KSVD_TRY(ensure(h, B_BG, (size_t)g_off, &Gall));
  KSVD_TRY(ensure(h, B_BA0, (size_t)a_off, &Aall));
  KSVD_TRY(ensure(h, B_BDESC, (size_t)2 * nprob, &ddev));
  KSVD_TRY(ensure(h, B_BJOB, (size_t)nprob, &jdev));
  KSVD_TRY(ensure(h, B_BQUEUE, 1, &queue));
  KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
  auto& descs = h->batch_descs;
  auto& jobs = h->batch_jobs;
  descs.assign(2 * (size_t)nprob, GemmDesc{});
  jobs.assign((size_t)nprob, OmpJob{});
  h->batch_dicts.assign((size_t)nprob, nullptr);
  int64_t tiles = 0, chunks = 0;
  int nd = 0, nj = 0;
  const int chunk = h->batch_chunk > 0 ? h->batch_chunk : omp_batch_chunk();
  for (int32_t i = 0; i < nprob; ++i) {
    const ksvd_problem& q = probs[i];
    if (q.N == 0) continue;
    const int kp = omp_padded_k(q.K);
    float* G = Gall + goff[i];
    float* A0 = Aall + aoff[i];
    tiles = gemm_desc_fill(descs[nd++], q.D, q.n, q.D, q.n, G, kp, q.K, kp, q.K, kp, q.n, tiles);
    tiles = gemm_desc_fill(descs[nd++], q.D, q.n, q.X, q.n, A0, kp, q.K, kp, q.N, q.N, q.n, tiles);
    h->batch_dicts[nj] = q.D;
    OmpJob& j = jobs[nj++];
    j.G = G; j.ldg = kp; j.A0 = A0; j.lda = kp; j.X = q.X; j.ldx = q.n; j.eps2 = q.eps2;
    j.idx = q.idx; j.coef = q.coef; j.nnz = q.nnz; j.N = q.N; j.chunk_begin = chunks;
    j.n = q.n; j.K = q.K; j.kpl = kp / 32; j.T = q.T;
    chunks += (q.N + chunk - 1) / chunk;
  }
  *pl = BatchPlan{ddev, nd, tiles, jdev, nj, chunks, tmax, chunk, queue, de};
  if (nj == 0) return KSVD_OK;
  // the host tables live in the handle, so the asynchronous copies read valid memory
  KSVD_CK(h, cudaMemcpyAsync(ddev, descs.data(), sizeof(GemmDesc) * nd, cudaMemcpyHostToDevice,
                             h->stream));
  KSVD_CK(h, cudaMemcpyAsync(jdev, jobs.data(), sizeof(OmpJob) * nj, cudaMemcpyHostToDevice,
                             h->stream));
  return KSVD_OK;
}

// Mixed precision: every problem's G = D'D and alpha0 = D'X on the tensor cores (BF16 hi/lo
// parts, three passes, FP32 accumulation, as the single-problem mixed path), one problem after
// another on the handle's stream; the split buffers are shared by the problems in turn.
ksvd_status batched_gemms_tc(ksvd_handle* h, const BatchPlan& pl) {
  int64_t dmax = 0, xmax = 0;
  for (int j = 0; j < pl.nj; ++j) {
    const OmpJob& jb = h->batch_jobs[j];
    const int64_t ld = bf16_ld(jb.n);
    dmax = std::max<int64_t>(dmax, (int64_t)jb.ldg * ld);
    xmax = std::max<int64_t>(xmax, jb.N * ld);
  }
  uint16_t *dhi = nullptr, *dlo = nullptr, *xhi = nullptr, *xlo = nullptr;
  KSVD_TRY(ensure(h, B_DHI, (size_t)dmax, &dhi));
  KSVD_TRY(ensure(h, B_DLO, (size_t)dmax, &dlo));
  KSVD_TRY(ensure(h, B_XHI, (size_t)xmax, &xhi));
  KSVD_TRY(ensure(h, B_XLO, (size_t)xmax, &xlo));
  drop_xsplit(h);                       // the X split buffers now hold other signals
  for (int j = 0; j < pl.nj; ++j) {
    const OmpJob& jb = h->batch_jobs[j];
    const int kp = (int)jb.ldg, n = jb.n;
    const int64_t ld = bf16_ld(n);
    KSVD_CK(h, launch_split_bf16(h->batch_dicts[j], n, jb.K, n, dhi, dlo, ld, kp, h->stream));
    KSVD_CK(h, launch_split_bf16(jb.X, jb.ldx, jb.N, n, xhi, xlo, ld, jb.N, h->stream));
    const TcOperand d{dhi, dlo, ld, kp}, x{xhi, xlo, ld, jb.N};
    KSVD_CK(h, launch_gemm_tn_bf16(d, d, const_cast<float*>(jb.G), kp, kp, kp, tc_inner(n), 3,
                                   pl.de, h->stream));
    KSVD_CK(h, launch_gemm_tn_bf16(d, x, const_cast<float*>(jb.A0), kp, kp, jb.N, tc_inner(n), 3,
                                   pl.de, h->stream));
  }
  return KSVD_OK;
}

// The GEMMs (grouped FP32 launch, or per-problem tensor-core products for the mixed path) and
// the persistent Batch-OMP launch of an uploaded plan.
ksvd_status batched_omp_launch(ksvd_handle* h, const BatchPlan& pl) {
  if (pl.nj == 0) return KSVD_OK;
  {
    StageScope sc(h, KSVD_STAGE_DTX);
    if (mixed(h)) KSVD_TRY(batched_gemms_tc(h, pl));
    else KSVD_CK(h, launch_gemm_tn_f32_grouped(pl.ddev, pl.nd, pl.tiles, h->stream));
  }
  StageScope sc(h, KSVD_STAGE_OMP);
  KSVD_CK(h, launch_omp_batched(pl.jdev, pl.nj, pl.chunks, pl.tmax, pl.chunk, pl.queue, pl.de,
                                h->stream));
  return KSVD_OK;
}

}  // namespace

ksvd_status ksvd_batched_omp(ksvd_handle* h, const ksvd_problem* probs, int32_t nprob) {
  if (null_handle(h) || nprob < 0 || (nprob > 0 && !probs)) return KSVD_ERR_INVALID_ARGUMENT;
  if (nprob == 0) return KSVD_OK;
  BatchPlan pl;
  KSVD_TRY(batched_omp_plan(h, probs, nprob, &pl));
  return batched_omp_launch(h, pl);
}

namespace {

// Child handle i of a batched call: sizes (n, K, T) of problem i, the parent's other parameters,
// its own non-blocking stream and completion event.  Reused while the sizes stay the same.
ksvd_status batch_child(ksvd_handle* h, int i, const ksvd_problem& q, ksvd_handle** out) {
  while ((int)h->kids.size() <= i) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    KSVD_CK(h, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    h->kid_streams.push_back(st);
    KSVD_CK(h, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    h->kid_events.push_back(ev);
    h->kids.push_back(nullptr);
  }
  ksvd_handle*& k = h->kids[i];
  if (k && (k->p.n != q.n || k->p.K != q.K || k->p.T != q.T)) {
    ksvd_destroy(k);
    k = nullptr;
  }
  if (!k) {
    ksvd_params p = h->p;
    p.n = q.n; p.K = q.K; p.T = q.T;
    p.precision = KSVD_PREC_FP32;
    p.flags = h->p.flags & KSVD_FLAG_PROFILE;
    p.seed = h->p.seed + 0x9E3779B97F4A7C15ULL * (uint64_t)(i + 1);
    const ksvd_status st = ksvd_create(&k, &p, h->kid_streams[i]);
    if (st != KSVD_OK) return fail(h, st, "creating a batched problem's handle failed%s");
  }
  *out = k;
  return KSVD_OK;
}

// Parent stream -> every child stream (fork) and back (join).
ksvd_status batch_fork(ksvd_handle* h, int n) {
  if (!h->fork_ev) KSVD_CK(h, cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming));
  KSVD_CK(h, cudaEventRecord(h->fork_ev, h->stream));
  for (int i = 0; i < n; ++i) KSVD_CK(h, cudaStreamWaitEvent(h->kid_streams[i], h->fork_ev, 0));
  return KSVD_OK;
}
ksvd_status batch_join(ksvd_handle* h, int n) {
  for (int i = 0; i < n; ++i) {
    KSVD_CK(h, cudaEventRecord(h->kid_events[i], h->kid_streams[i]));
    KSVD_CK(h, cudaStreamWaitEvent(h->stream, h->kid_events[i], 0));
  }
  return KSVD_OK;
}

ksvd_status kid_error(ksvd_handle* h, ksvd_handle* k, ksvd_status s) {
  if (s != KSVD_OK && h != k) h->err = "batched problem: " + k->err;
  return s;
}

}  // namespace

}  // extern "C"

namespace {

// Median of `reps` timings (ms) of fn() on the handle's stream, after one untimed run.
template <typename F>
ksvd_status time_on_stream(ksvd_handle* h, int reps, F fn, double* ms_out) {
  cudaEvent_t a = nullptr, b = nullptr;
  KSVD_CK(h, cudaEventCreate(&a));
  KSVD_CK(h, cudaEventCreate(&b));
  std::vector<float> t;
  ksvd_status st = fn();
  for (int r = 0; r < reps && st == KSVD_OK; ++r) {
    cudaEventRecord(a, h->stream);
    st = fn();
    cudaEventRecord(b, h->stream);
    float ms = 0.f;
    if (st == KSVD_OK && cudaEventSynchronize(b) == cudaSuccess &&
        cudaEventElapsedTime(&ms, a, b) == cudaSuccess)
      t.push_back(ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (st != KSVD_OK) return st;
  if (t.empty()) return fail(h, KSVD_ERR_CUDA, "autotune timing failed%s");
  std::sort(t.begin(), t.end());
  *ms_out = t[t.size() / 2];
  return KSVD_OK;
}

void fill_tuning(const ksvd_handle* h, ksvd_tuning* out) {
  if (!out) return;
  std::memset(out, 0, sizeof(*out));
  out->omp_grid_mult = h->omp_grid_mult;
  out->sweep_ctas = h->sweep_ctas;
  out->batch_chunk = h->batch_chunk;
  out->batch_concurrent = h->batch_concurrent;
  out->tuned = h->tuned ? 1 : 0;
  out->omp_fp16 = h->omp_fp16;
}

}  // namespace

extern "C" {

// Times the launch shapes that have no single best value across problem sizes on this GPU and
// this problem, and keeps the fastest for the handle's later calls:
//   * Batch-OMP grid: resident CTA slots x {1, 2, 4, 8, 16} blocks (grid-stride over signals);
//   * the cooperative sweep's CTAs: {SMs, SMs/2, SMs/4} (fewer CTAs make the per-atom grid
//     barrier cheaper, more spread each atom's signals wider).
// The inputs are not modified: the sweep runs on scratch copies of D and the coefficients, and
// the handle's atom-order stream and stage state are restored.
ksvd_status ksvd_autotune(ksvd_handle* h, const float* D, const float* X, int64_t N,
                          ksvd_tuning* out) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || N < 1) return KSVD_ERR_INVALID_ARGUMENT;
  if ((int64_t)N * h->p.T > 0x7fffffffLL)
    return fail(h, KSVD_ERR_UNSUPPORTED, "N*T must stay below 2^31%s");
  const int n = h->p.n, Kp = h->Kp, T = h->p.T;
  drop_xsplit(h);
  float *Dp = nullptr, *G = nullptr, *A0 = nullptr, *Dt = nullptr, *Ct = nullptr, *coef = nullptr;
  int32_t *idx = nullptr, *nnz = nullptr, *pd = nullptr;
  KSVD_TRY(load_dict(h, D, &Dp));
  KSVD_CK(h, launch_normcols(Dp, n, h->p.K, h->stream));
  KSVD_TRY(ensure(h, B_G, (size_t)Kp * Kp, &G));
  KSVD_TRY(ensure(h, B_A0, (size_t)Kp * N, &A0));
  KSVD_TRY(ensure(h, B_HIDX, (size_t)N * T, &idx));
  KSVD_TRY(ensure(h, B_HCOEF, (size_t)N * T, &coef));
  KSVD_TRY(ensure(h, B_HNNZ, (size_t)N, &nnz));
  KSVD_TRY(ensure(h, B_TUNE_D, (size_t)n * Kp, &Dt));
  KSVD_TRY(ensure(h, B_TUNE_C, (size_t)N * T, &Ct));
  KSVD_TRY(gram_padded(h, Dp, G));
  KSVD_TRY(dtx_padded(h, Dp, X, N, A0));
  const bool prof = h->profiling();
  h->p.flags &= ~KSVD_FLAG_PROFILE;        // no stage events while tuning
  ksvd_status st = KSVD_OK;
  double best = 1e30;
  int best_mult = 8, best_fp16 = h->omp_fp16;
  const bool try_fp16 = mixed(h) && T <= 32;
  for (int fp16 : {0, 1}) {
    if (!try_fp16 && fp16 == 1) break;
    if (try_fp16) h->omp_fp16 = fp16;
    for (int mult : {0, 1, 2, 4, 8, 16}) {
      h->omp_grid_mult = mult;
      double ms = 0;
      st = time_on_stream(h, 3, [&] {
        return run_omp(h, G, A0, N, nullptr, nullptr, idx, coef, nnz);
      }, &ms);
      if (st != KSVD_OK) break;
      if (ms < best) { best = ms; best_mult = mult; best_fp16 = h->omp_fp16; }
    }
    if (st != KSVD_OK) break;
  }
  h->omp_grid_mult = best_mult;
  h->omp_fp16 = best_fp16;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  const int64_t draws = h->perm_draws;
  if (st == KSVD_OK) st = upload_perm(h, nullptr, 1, &pd);
  best = 1e30;
  int best_ctas = 0;
  for (int div : {1, 2, 4, 8, 16}) {
    if (st != KSVD_OK) break;
    const int ctas = std::max(1, sms / div);
    h->sweep_ctas = ctas;
    double ms = 0;
    st = time_on_stream(h, 2, [&]() -> ksvd_status {
      KSVD_CK(h, cudaMemcpyAsync(Dt, Dp, sizeof(float) * (size_t)n * Kp,
                                 cudaMemcpyDeviceToDevice, h->stream));
      KSVD_CK(h, cudaMemcpyAsync(Ct, coef, sizeof(float) * (size_t)N * T,
                                 cudaMemcpyDeviceToDevice, h->stream));
      return run_update(h, Dt, X, N, idx, Ct, nnz, pd);
    }, &ms);
    if (st == KSVD_OK && ms < best) { best = ms; best_ctas = div == 1 ? 0 : ctas; }
  }
  h->sweep_ctas = best_ctas;
  h->perm_draws = draws;
  h->update_N = -1;
  h->error_N = -1;
  if (prof) h->p.flags |= KSVD_FLAG_PROFILE;
  drop_xsplit(h);
  if (st != KSVD_OK) return st;
  KSVD_CK(h, cudaStreamSynchronize(h->stream));
  KSVD_TRY(check_dev_err(h));
  h->tuned = true;
  fill_tuning(h, out);
  return KSVD_OK;
}

// Work-queue chunk of the batched Batch-OMP ({4, 16, 64} signals) and the batched update mode,
// timed on the given problems.
ksvd_status ksvd_autotune_batched(ksvd_handle* h, const ksvd_problem* probs, int32_t nprob,
                                  ksvd_tuning* out) {
  if (null_handle(h) || nprob < 1 || !probs) return KSVD_ERR_INVALID_ARGUMENT;
  const bool prof = h->profiling();
  h->p.flags &= ~KSVD_FLAG_PROFILE;
  ksvd_status st = KSVD_OK;
  double best = 1e30;
  int best_chunk = 16;
  for (int chunk : {4, 16, 64}) {
    h->batch_chunk = chunk;
    double ms = 0;
    st = time_on_stream(h, 2, [&] { return ksvd_batched_omp(h, probs, nprob); }, &ms);
    if (st != KSVD_OK) break;
    if (ms < best) { best = ms; best_chunk = chunk; }
  }
  h->batch_chunk = best_chunk;
  // updates: concurrent streams with SM shares vs one after another on the whole GPU, timed
  // on one K-SVD iteration; the dictionaries and the children's atom-order streams are restored
  std::vector<float*> saved(nprob, nullptr);
  std::vector<ksvd_problem> work(probs, probs + nprob);
  bool all_n = true;
  for (int32_t i = 0; i < nprob; ++i) all_n &= probs[i].N >= 1;
  for (int32_t i = 0; i < nprob && st == KSVD_OK && all_n; ++i) {
    const size_t bytes = sizeof(float) * (size_t)probs[i].n * probs[i].K;
    if (cudaMalloc(&saved[i], bytes) != cudaSuccess ||
        cudaMemcpyAsync(saved[i], probs[i].D, bytes, cudaMemcpyDeviceToDevice, h->stream) !=
            cudaSuccess)
      st = cuda_fail(h, cudaGetLastError(), "autotune scratch");
  }
  if (st == KSVD_OK && all_n) {
    std::vector<int64_t> draws;
    for (auto k : h->kids) draws.push_back(k ? k->perm_draws : 0);
    best = 1e30;
    int best_mode = 0;
    for (int mode : {0, 1}) {
      h->batch_concurrent = mode;
      double ms = 0;
      st = time_on_stream(h, 1, [&]() -> ksvd_status {
        for (int32_t i = 0; i < nprob; ++i)
          KSVD_CK(h, cudaMemcpyAsync(work[i].D, saved[i],
                                     sizeof(float) * (size_t)probs[i].n * probs[i].K,
                                     cudaMemcpyDeviceToDevice, h->stream));
        return ksvd_batched_iterate(h, work.data(), nprob, 1, nullptr);
      }, &ms);
      if (st != KSVD_OK) break;
      if (ms < best) { best = ms; best_mode = mode; }
    }
    h->batch_concurrent = best_mode;
    for (int32_t i = 0; i < nprob; ++i)
      cudaMemcpyAsync(work[i].D, saved[i], sizeof(float) * (size_t)probs[i].n * probs[i].K,
                      cudaMemcpyDeviceToDevice, h->stream);
    for (size_t i = 0; i < h->kids.size(); ++i)
      if (h->kids[i]) h->kids[i]->perm_draws = i < draws.size() ? draws[i] : 0;
  }
  cudaStreamSynchronize(h->stream);
  for (auto p : saved)
    if (p) cudaFree(p);
  if (prof) h->p.flags |= KSVD_FLAG_PROFILE;
  if (st != KSVD_OK) return st;
  KSVD_TRY(check_dev_err(h));
  h->tuned = true;
  fill_tuning(h, out);
  return KSVD_OK;
}

ksvd_status ksvd_get_tuning(const ksvd_handle* h, ksvd_tuning* out) {
  if (null_handle(h) || !out) return KSVD_ERR_INVALID_ARGUMENT;
  fill_tuning(h, out);
  return KSVD_OK;
}

ksvd_status ksvd_set_tuning(ksvd_handle* h, const ksvd_tuning* t) {
  if (null_handle(h) || !t || t->omp_grid_mult < 0 || t->omp_grid_mult > 64 || t->sweep_ctas < 0 ||
      t->batch_chunk < 0 || t->batch_chunk > 4096 || t->omp_fp16 < -1 || t->omp_fp16 > 1)
    return KSVD_ERR_INVALID_ARGUMENT;
  h->omp_fp16 = t->omp_fp16;
  h->omp_grid_mult = t->omp_grid_mult;
  h->sweep_ctas = t->sweep_ctas;
  h->batch_chunk = t->batch_chunk;
  h->batch_concurrent = t->batch_concurrent != 0;
  h->tuned = t->tuned != 0;
  return KSVD_OK;
}

ksvd_status ksvd_update_dictionary(ksvd_handle* h, float* D, const float* X, int64_t N,
                                   const int32_t* idx, float* coef, const int32_t* nnz,
                                   const int32_t* perm) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(idx) || bad_ptr(coef) || bad_ptr(nnz) || N < 1)
    return KSVD_ERR_INVALID_ARGUMENT;
  if ((int64_t)N * h->p.T > 0x7fffffffLL)
    return fail(h, KSVD_ERR_UNSUPPORTED, "N*T must stay below 2^31%s");
  float* Dp = nullptr;
  KSVD_TRY(load_dict(h, D, &Dp));
  const int32_t* pd = perm;
  if (!pd) {
    int32_t* tmp = nullptr;
    KSVD_TRY(upload_perm(h, nullptr, 1, &tmp));
    pd = tmp;
  }
  KSVD_TRY(run_update(h, Dp, X, N, idx, coef, nnz, pd));
  KSVD_TRY(store_dict(h, Dp, D));
  return KSVD_OK;
}

ksvd_status ksvd_error(ksvd_handle* h, const float* D, const float* X, int64_t N,
                       const int32_t* idx, const float* coef, const int32_t* nnz, float* err,
                       double* rmse) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(idx) || bad_ptr(coef) || bad_ptr(nnz) || N < 1)
    return KSVD_ERR_INVALID_ARGUMENT;
  float* Dp = nullptr;
  double* rd = nullptr;
  KSVD_TRY(load_dict(h, D, &Dp));
  KSVD_TRY(ensure(h, B_RMSE, 1024, &rd));
  KSVD_TRY(run_error(h, Dp, X, N, idx, coef, nnz, rd));
  if (err) {
    float* e = nullptr;
    KSVD_TRY(ensure(h, B_ERR, (size_t)N, &e));
    KSVD_CK(h, cudaMemcpyAsync(err, e, sizeof(float) * N, cudaMemcpyDeviceToDevice, h->stream));
  }
  if (rmse) {
    KSVD_CK(h, cudaMemcpyAsync(rmse, rd, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    KSVD_CK(h, cudaStreamSynchronize(h->stream));
    return check_dev_err(h);
  }
  return KSVD_OK;
}

ksvd_status ksvd_clear_dict(ksvd_handle* h, float* D, const float* X, int64_t N,
                            const int32_t* idx, const float* coef, const int32_t* nnz,
                            int32_t* cleared) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || N < 1) return KSVD_ERR_INVALID_ARGUMENT;
  (void)idx; (void)coef; (void)nnz;
  if (h->update_N != N || h->error_N != N)
    return fail(h, KSVD_ERR_STATE,
                "clear_dict needs ksvd_update_dictionary and ksvd_error on the same N first%s");
  float *Dp = nullptr, *G = nullptr;
  int32_t* cd = nullptr;
  KSVD_TRY(load_dict(h, D, &Dp));
  KSVD_TRY(ensure(h, B_G, (size_t)h->Kp * h->Kp, &G));
  KSVD_TRY(ensure(h, B_CLEARED, 1, &cd));
  KSVD_TRY(gram_padded(h, Dp, G));
  KSVD_TRY(run_clear(h, Dp, G, X, N, cd));
  KSVD_TRY(store_dict(h, Dp, D));
  if (cleared) {
    KSVD_CK(h, cudaMemcpyAsync(cleared, cd, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    KSVD_CK(h, cudaStreamSynchronize(h->stream));
    return check_dev_err(h);
  }
  return KSVD_OK;
}

namespace {

// One K-SVD iteration (S/KSVD.cu:55-131 loop body) on the handle's stream.  The permutation and
// the RMSE slot are indexed by the device iteration counter, which the iteration advances last,
// so the same launches serve every iteration and a captured graph can be replayed.
ksvd_status iteration_body(ksvd_handle* h, float* Dp, float* G, float* A0, const float* X,
                           int64_t N, int32_t* idx, float* coef, int32_t* nnz,
                           const int32_t* pd, double* rd, int32_t* cd, int* ctr) {
  if (h->inflow.active) {
    // X is still arriving: code each chunk as soon as it has landed
    auto& in = h->inflow;
    in.active = false;
    for (int c = 0; c < in.nchunks; ++c) {
      const int64_t s0 = in.bounds[c], s1 = in.bounds[c + 1];
      KSVD_CK(h, cudaStreamWaitEvent(h->stream, in.ev[c], 0));
      KSVD_TRY(dtx_padded_range(h, Dp, X, N, s0, s1, A0));
      if (h->it_eps2)
        KSVD_CK(h, launch_col_norm2(X + s0 * h->p.n, h->p.n, s1 - s0,
                                    const_cast<float*>(h->it_xn2) + s0, h->stream));
      KSVD_TRY(run_omp(h, G, A0 + s0 * h->Kp, s1 - s0, h->it_eps2 ? h->it_xn2 + s0 : nullptr,
                       h->it_eps2 ? h->it_eps2 + s0 : nullptr, idx + s0 * h->p.T,
                       coef + s0 * h->p.T, nnz + s0, c == 0));   // G's FP16 copy: once
    }
    if (mixed(h)) { h->xsplit_src = X; h->xsplit_N = N; }   // every chunk's split is made
  } else {
    KSVD_TRY(dtx_padded(h, Dp, X, N, A0));                             // OMP.cu:44
    KSVD_TRY(run_omp(h, G, A0, N, h->it_xn2, h->it_eps2, idx, coef, nnz));  // OMP.cu:55
  }
  auto& dr = h->inflow;
  const bool drain = dr.drain;   // this is the call's last iteration and its results go to the host
  if (drain) {
    dr.drain = false;
    const int T = h->p.T;
    KSVD_CK(h, cudaEventRecord(dr.dev_ev[0], h->stream));
    KSVD_CK(h, cudaStreamWaitEvent(dr.cstream, dr.dev_ev[0], 0));
    KSVD_CK(h, cudaMemcpyAsync(dr.h_idx, idx, sizeof(int32_t) * (size_t)N * T,
                               cudaMemcpyDeviceToHost, dr.cstream));
    KSVD_CK(h, cudaMemcpyAsync(dr.h_nnz, nnz, sizeof(int32_t) * (size_t)N, cudaMemcpyDeviceToHost,
                               dr.cstream));
  }
  KSVD_TRY(run_update(h, Dp, X, N, idx, coef, nnz, pd, ctr));       // KSVD.cu:97-114
  if (drain) {
    KSVD_CK(h, cudaEventRecord(dr.dev_ev[1], h->stream));
    KSVD_CK(h, cudaStreamWaitEvent(dr.cstream, dr.dev_ev[1], 0));
    KSVD_CK(h, cudaMemcpyAsync(dr.h_coef, coef, sizeof(float) * (size_t)N * h->p.T,
                               cudaMemcpyDeviceToHost, dr.cstream));
  }
  KSVD_TRY(run_error(h, Dp, X, N, idx, coef, nnz, rd, ctr));        // KSVD.cu:119
  KSVD_TRY(gram_padded(h, Dp, G));                                   // G of the updated D
  KSVD_TRY(run_clear(h, Dp, G, X, N, cd));                           // KSVD.cu:126
  KSVD_CK(h, launch_advance_counter(ctr, h->stream));
  return KSVD_OK;
}

// Runs the calls in between on the handle's private non-blocking stream, fenced to the
// caller's stream on entry and on exit (stream capture is not allowed on the legacy stream).
struct SideStream {
  ksvd_handle* h;
  cudaStream_t user = nullptr;
  bool active = false;
  explicit SideStream(ksvd_handle* hh) : h(hh) {}
  ksvd_status enter() {
    if (!h->gstream) {
      KSVD_CK(h, cudaStreamCreateWithFlags(&h->gstream, cudaStreamNonBlocking));
      for (auto& e : h->gev) KSVD_CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    user = h->stream;
    KSVD_CK(h, cudaEventRecord(h->gev[0], user));
    KSVD_CK(h, cudaStreamWaitEvent(h->gstream, h->gev[0], 0));
    h->stream = h->gstream;
    active = true;
    return KSVD_OK;
  }
  ~SideStream() {
    if (!active) return;
    cudaEventRecord(h->gev[1], h->gstream);
    cudaStreamWaitEvent(user, h->gev[1], 0);
    h->stream = user;
  }
};

// Replays `count` iterations from the graph in `cache`, capturing `body` (one iteration) first
// when the cached graph was made for another key.  Returns false (nothing launched) when
// capture is refused; the caller then runs the iterations eagerly.
bool replay_graph(ksvd_handle* h, ksvd_handle::GraphCache& cache,
                  const std::vector<const void*>& key, int32_t count,
                  const std::function<ksvd_status()>& body) {
  if (h->graph_broken) return false;
  if (!cache.exec || cache.key != key) {
    if (cache.exec) {
      cudaGraphExecDestroy(cache.exec);
      cache.exec = nullptr;
    }
    if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      h->graph_broken = true;
      return false;
    }
    const ksvd_status st = body();
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    cudaGraphExec_t ex = nullptr;
    const bool ok = st == KSVD_OK && ec == cudaSuccess && g &&
                    cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (!ok) {
      if (ex) cudaGraphExecDestroy(ex);
      h->graph_broken = true;
      h->err.clear();
      return false;
    }
    cache.exec = ex;
    cache.key = key;
  }
  for (int32_t r = 0; r < count; ++r)
    if (cudaGraphLaunch(cache.exec, h->stream) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
  h->graph_replays += count;
  return true;
}

}  // namespace

namespace {
ksvd_status iterate_impl(ksvd_handle* h, float* D, const float* X, int64_t N, int32_t iters,
                         const int32_t* perms, const float* eps2, int32_t* idx, float* coef,
                         int32_t* nnz, double* rmse);
}

ksvd_status ksvd_iterate(ksvd_handle* h, float* D, const float* X, int64_t N, int32_t iters,
                         const int32_t* perms, int32_t* idx, float* coef, int32_t* nnz,
                         double* rmse) {
  return iterate_impl(h, D, X, N, iters, perms, nullptr, idx, coef, nnz, rmse);
}

ksvd_status ksvd_iterate_eps(ksvd_handle* h, float* D, const float* X, int64_t N, int32_t iters,
                             const int32_t* perms, const float* eps2, int32_t* idx, float* coef,
                             int32_t* nnz, double* rmse) {
  if (bad_ptr(eps2)) return KSVD_ERR_INVALID_ARGUMENT;
  return iterate_impl(h, D, X, N, iters, perms, eps2, idx, coef, nnz, rmse);
}

namespace {
// The call's error targets live in the handle while it runs (the iteration body and a captured
// graph read them from there); cleared on every exit.
struct EpsScope {
  ksvd_handle* h;
  ~EpsScope() { h->it_xn2 = nullptr; h->it_eps2 = nullptr; }
};

ksvd_status iterate_impl(ksvd_handle* h, float* D, const float* X, int64_t N, int32_t iters,
                         const int32_t* perms, const float* eps2, int32_t* idx, float* coef,
                         int32_t* nnz, double* rmse) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(idx) || bad_ptr(coef) || bad_ptr(nnz) || N < 1 ||
      iters < 0)
    return KSVD_ERR_INVALID_ARGUMENT;
  EpsScope eps_scope{h};
  if (iters > 1024) return fail(h, KSVD_ERR_UNSUPPORTED, "at most 1024 iterations per call%s");
  if ((int64_t)N * h->p.T > 0x7fffffffLL)
    return fail(h, KSVD_ERR_UNSUPPORTED, "N*T must stay below 2^31%s");
  const int Kp = h->Kp;
  const bool graph = (h->p.flags & KSVD_FLAG_GRAPH) && !h->profiling() && iters > 1;
  SideStream side(h);
  if (graph) KSVD_TRY(side.enter());
  drop_xsplit(h);
  float *Dp = nullptr, *G = nullptr, *A0 = nullptr;
  double* rd = nullptr;
  int32_t *pd = nullptr, *cd = nullptr;
  int* ctr = nullptr;
  KSVD_TRY(load_dict(h, D, &Dp));
  KSVD_TRY(ensure(h, B_G, (size_t)Kp * Kp, &G));
  KSVD_TRY(ensure(h, B_A0, (size_t)Kp * N, &A0));
  KSVD_TRY(ensure(h, B_RMSE, 1024, &rd));
  KSVD_TRY(ensure(h, B_CLEARED, 1, &cd));
  KSVD_TRY(ensure(h, B_ITER, 1, &ctr));
  KSVD_CK(h, cudaMemsetAsync(ctr, 0, sizeof(int), h->stream));
  if (eps2) {
    float* xn2 = nullptr;
    KSVD_TRY(ensure(h, B_XN2, (size_t)N, &xn2));
    if (!h->inflow.active) KSVD_CK(h, launch_col_norm2(X, h->p.n, N, xn2, h->stream));
    h->it_xn2 = xn2;          // (with X still arriving, per chunk in the first iteration)
    h->it_eps2 = eps2;
  }
  if (iters > 0) KSVD_TRY(upload_perm(h, perms, iters, &pd));
  KSVD_CK(h, launch_normcols(Dp, h->p.n, h->p.K, h->stream));         // KSVD.cu:57
  KSVD_TRY(gram_padded(h, Dp, G));                                     // KSVD.cu:64
  int32_t done = 0;
  if (iters > 0) {
    // the first iteration runs eagerly: it sizes every workspace buffer (no allocation may
    // happen under capture) and makes the mixed path's BF16 copy of X for this call
    KSVD_TRY(iteration_body(h, Dp, G, A0, X, N, idx, coef, nnz, pd, rd, cd, ctr));
    done = 1;
  }
  if (graph && done < iters) {
    const std::vector<const void*> key{
        Dp, G, A0, X, idx, coef, nnz, pd, rd, cd, ctr,
        reinterpret_cast<const void*>((intptr_t)h->p.precision), h->it_eps2,
        reinterpret_cast<const void*>((intptr_t)N)};
    if (replay_graph(h, h->graphs[0], key, iters - done, [&] {
          return iteration_body(h, Dp, G, A0, X, N, idx, coef, nnz, pd, rd, cd, ctr);
        }))
      done = iters;
  }
  for (; done < iters; ++done)
    KSVD_TRY(iteration_body(h, Dp, G, A0, X, N, idx, coef, nnz, pd, rd, cd, ctr));
  if (iters > 0 && (h->p.flags & KSVD_FLAG_REFINE_FINAL)) {
    int* de = nullptr;
    KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
    KSVD_CK(h, launch_refine(Dp, h->p.n, h->p.K, G, Kp, X, N, h->p.T, idx, nnz, coef, nullptr, de,
                             h->stream));                            // G is D'D after clearDict
  }
  drop_xsplit(h);
  KSVD_TRY(store_dict(h, Dp, D));
  if (rmse && iters > 0)
    KSVD_CK(h, cudaMemcpyAsync(rmse, rd, sizeof(double) * iters, cudaMemcpyDeviceToHost,
                               h->stream));
  KSVD_CK(h, cudaStreamSynchronize(h->stream));
  collect_stage_times(h);
  return check_dev_err(h);
}
}  // namespace

// K-SVD on many independent problems.  Per iteration: ONE persistent Batch-OMP launch over all
// problems (the batched plan's tables are uploaded once per call), then every problem's
// dictionary update, error and clearDict -- one after another on the parent stream, each sweep
// on the whole GPU (sequential mode), or on the problems' own streams at once with the SMs
// shared in proportion to each problem's work N*T (concurrent mode).  Every problem has a
// device iteration counter that selects its permutation and RMSE slot, so with KSVD_FLAG_GRAPH
// the second and later iterations replay one captured graph of the whole batched iteration.
ksvd_status ksvd_batched_iterate(ksvd_handle* h, ksvd_problem* probs, int32_t nprob,
                                 int32_t iters, double* rmse) {
  if (null_handle(h) || nprob < 0 || (nprob > 0 && !probs) || iters < 0) return KSVD_ERR_INVALID_ARGUMENT;
  if (nprob == 0 || iters == 0) return KSVD_OK;
  if (iters > 1024) return fail(h, KSVD_ERR_UNSUPPORTED, "at most 1024 iterations per call%s");
  for (int32_t i = 0; i < nprob; ++i)
    if (probs[i].N < 1)
      return fail(h, KSVD_ERR_INVALID_ARGUMENT, "every batched K-SVD problem needs N >= 1%s");
  const bool graph = (h->p.flags & KSVD_FLAG_GRAPH) && !h->profiling() && iters > 1;
  SideStream side(h);
  if (graph) KSVD_TRY(side.enter());
  // workspace of the children first: the sweep CTA shares, dictionaries, permutations
  int sms = 0;
  KSVD_CK(h, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
  double work = 0;
  for (int32_t i = 0; i < nprob; ++i) work += (double)probs[i].N * probs[i].T;
  std::vector<ksvd_handle*> ks(nprob);
  std::vector<float*> Dp(nprob);
  std::vector<int32_t*> pd(nprob);
  std::vector<double*> rd(nprob);
  std::vector<int32_t*> cd(nprob);
  std::vector<int*> ctr(nprob);
  std::vector<ksvd_problem> inner(probs, probs + nprob);
  const bool conc = h->batch_concurrent != 0;
  int budget = sms - nprob;   // every problem has one CTA; the rest go by work
  for (int32_t i = 0; i < nprob; ++i) {
    KSVD_TRY(batch_child(h, i, probs[i], &ks[i]));
    ksvd_handle* k = ks[i];
    const int extra = budget > 0 ? (int)((double)budget * probs[i].N * probs[i].T / work) : 0;
    // concurrent: shares that fit on the GPU together; sequential: every sweep gets all SMs
    k->sweep_ctas = conc ? std::max(1, 1 + extra) : 0;
  }
  KSVD_TRY(batch_fork(h, nprob));
  for (int32_t i = 0; i < nprob; ++i) {
    ksvd_handle* k = ks[i];
    if (bad_ptr(probs[i].D) || bad_ptr(probs[i].X))
      return fail(h, KSVD_ERR_INVALID_ARGUMENT, "batched problem with a null pointer%s");
    KSVD_TRY(kid_error(h, k, load_dict(k, probs[i].D, &Dp[i])));
    KSVD_TRY(kid_error(h, k, ensure(k, B_RMSE, 1024, &rd[i])));
    KSVD_TRY(kid_error(h, k, ensure(k, B_CLEARED, 1, &cd[i])));
    KSVD_TRY(kid_error(h, k, ensure(k, B_ITER, 1, &ctr[i])));
    KSVD_TRY(kid_error(h, k, upload_perm(k, nullptr, iters, &pd[i])));
    KSVD_CK(h, cudaMemsetAsync(ctr[i], 0, sizeof(int), k->stream));
    KSVD_CK(h, launch_normcols(Dp[i], k->p.n, k->p.K, k->stream));   // KSVD.cu:57
    inner[i].D = Dp[i];             // OMP codes with the children's working dictionaries
  }
  KSVD_TRY(batch_join(h, nprob));
  BatchPlan plan;
  KSVD_TRY(batched_omp_plan(h, inner.data(), nprob, &plan));
  auto one_iteration = [&]() -> ksvd_status {
    KSVD_TRY(batched_omp_launch(h, plan));
    if (conc) KSVD_TRY(batch_fork(h, nprob));
    for (int32_t i = 0; i < nprob; ++i) {
      ksvd_handle* k = ks[i];
      const ksvd_problem& q = probs[i];
      // sequential mode runs every problem's stages on the parent stream, in order
      const cudaStream_t own = k->stream;
      if (!conc) k->stream = h->stream;
      float* G = nullptr;
      ksvd_status s2 = ensure(k, B_G, (size_t)k->Kp * k->Kp, &G);
      if (s2 == KSVD_OK)
        s2 = run_update(k, Dp[i], q.X, q.N, q.idx, q.coef, q.nnz, pd[i], ctr[i]);
      if (s2 == KSVD_OK) s2 = run_error(k, Dp[i], q.X, q.N, q.idx, q.coef, q.nnz, rd[i], ctr[i]);
      if (s2 == KSVD_OK) s2 = gram_padded(k, Dp[i], G);
      if (s2 == KSVD_OK) s2 = run_clear(k, Dp[i], G, q.X, q.N, cd[i]);
      if (s2 == KSVD_OK) {
        const cudaError_t e = launch_advance_counter(ctr[i], k->stream);
        if (e != cudaSuccess) s2 = cuda_fail(k, e, "launch_advance_counter");
      }
      k->stream = own;
      KSVD_TRY(kid_error(h, k, s2));
    }
    if (conc) KSVD_TRY(batch_join(h, nprob));
    return KSVD_OK;
  };
  // the first iteration runs eagerly: it sizes every child's workspace (nothing may be
  // allocated under capture)
  KSVD_TRY(one_iteration());
  int32_t done = 1;
  if (graph && done < iters) {
    std::vector<const void*> key{reinterpret_cast<const void*>((intptr_t)conc),
                                 plan.ddev, plan.jdev,
                                 reinterpret_cast<const void*>((intptr_t)plan.chunk)};
    for (int32_t i = 0; i < nprob; ++i) {
      const ksvd_problem& q = probs[i];
      key.insert(key.end(), {ks[i], Dp[i], q.X, q.idx, q.coef, q.nnz, pd[i], rd[i], cd[i],
                             ctr[i], reinterpret_cast<const void*>((intptr_t)q.N),
                             reinterpret_cast<const void*>((intptr_t)ks[i]->sweep_ctas)});
    }
    if (replay_graph(h, h->graphs[1], key, iters - done, one_iteration)) done = iters;
  }
  for (; done < iters; ++done) KSVD_TRY(one_iteration());
  KSVD_TRY(batch_fork(h, nprob));
  for (int32_t i = 0; i < nprob; ++i) {
    KSVD_TRY(kid_error(h, ks[i], store_dict(ks[i], Dp[i], probs[i].D)));
    if (rmse)
      KSVD_CK(h, cudaMemcpyAsync(rmse + (size_t)i * iters, rd[i], sizeof(double) * iters,
                                 cudaMemcpyDeviceToHost, ks[i]->stream));
  }
  KSVD_TRY(batch_join(h, nprob));
  KSVD_CK(h, cudaStreamSynchronize(h->stream));
  for (int32_t i = 0; i < nprob; ++i) KSVD_TRY(kid_error(h, ks[i], check_dev_err(ks[i])));
  return check_dev_err(h);
}

// Body of ksvd_iterate_host; a return before its final synchronisation may leave copies that
// read X or write idx/coef/nnz queued on the handle's stream or the copy stream.
static ksvd_status iterate_host_body(ksvd_handle* h, float* D, const float* X, int64_t N,
                                     int32_t iters, const int32_t* perms, int32_t* idx,
                                     float* coef, int32_t* nnz, double* rmse) {
  const int n = h->p.n, K = h->p.K, T = h->p.T;
  float *dX = nullptr, *dD = nullptr, *dC = nullptr;
  int32_t *dI = nullptr, *dN = nullptr;
  KSVD_TRY(ensure(h, B_HX, (size_t)n * N, &dX));
  KSVD_TRY(ensure(h, B_HD, (size_t)n * K, &dD));
  KSVD_TRY(ensure(h, B_HIDX, (size_t)N * T, &dI));
  KSVD_TRY(ensure(h, B_HCOEF, (size_t)N * T, &dC));
  KSVD_TRY(ensure(h, B_HNNZ, (size_t)N, &dN));
  KSVD_CK(h, cudaMemcpyAsync(dD, D, sizeof(float) * (size_t)n * K, cudaMemcpyHostToDevice, h->stream));
  // X in chunks on a copy stream (after the work already queued on the handle's stream), so the
  // first iteration's D'X and Batch-OMP overlap the rest of the transfer
  auto& in = h->inflow;
  // Chunks growing fourfold from 65,536 signals: the first lands after a short wait, and each
  // later one lands while Batch-OMP codes the one before (a signal's coding takes ~4x its copy),
  // with few launches -- every Batch-OMP launch ends in a tail where SMs idle.
  int64_t cb[ksvd_handle::kMaxInflow + 1];
  int nch = 0;
  cb[0] = 0;
  for (int64_t sz = 65536; cb[nch] < N && nch < ksvd_handle::kMaxInflow; sz *= 4) {
    cb[nch + 1] = (nch + 1 == ksvd_handle::kMaxInflow || cb[nch] + sz >= N) ? N : cb[nch] + sz;
    ++nch;
  }
  if (nch >= 2 && N - cb[nch - 1] < 65536) {   // no tiny last chunk: fold it into the one before
    cb[nch - 1] = N;
    --nch;
    cb[nch] = N;
  }
  if (iters >= 1 && nch >= 2) {
    if (!in.cstream) {
      KSVD_CK(h, cudaStreamCreateWithFlags(&in.cstream, cudaStreamNonBlocking));
      for (auto& e : in.ev) KSVD_CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    KSVD_CK(h, cudaEventRecord(in.ev[0], h->stream));
    KSVD_CK(h, cudaStreamWaitEvent(in.cstream, in.ev[0], 0));
    in.nchunks = nch;
    for (int c = 0; c <= nch; ++c) in.bounds[c] = cb[c];
    for (int c = 0; c < nch; ++c) {
      const int64_t s0 = in.bounds[c], s1 = in.bounds[c + 1];
      KSVD_CK(h, cudaMemcpyAsync(dX + s0 * n, X + s0 * n, sizeof(float) * (size_t)n * (s1 - s0),
                                 cudaMemcpyHostToDevice, in.cstream));
      KSVD_CK(h, cudaEventRecord(in.ev[c], in.cstream));
    }
    in.active = true;
  } else {
    KSVD_CK(h, cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * N, cudaMemcpyHostToDevice,
                               h->stream));
  }
  // a single eager iteration drains its code to the host while it finishes
  const bool drain = iters == 1 && in.cstream != nullptr;
  if (drain) {
    for (auto& e : in.dev_ev)
      if (!e) KSVD_CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    in.drain = true;
    in.h_idx = idx; in.h_coef = coef; in.h_nnz = nnz;
  }
  const ksvd_status st = ksvd_iterate(h, dD, dX, N, iters, perms, dI, dC, dN, rmse);
  if (in.active) {   // not consumed (an early error): the copy must still finish before reuse
    in.active = false;
    cudaStreamWaitEvent(h->stream, in.ev[in.nchunks - 1], 0);
  }
  const bool drained = drain && !in.drain;
  in.drain = false;
  if (in.cstream) {
    // the host copies on the copy stream are complete before the call returns
    cudaEvent_t e = in.ev[0];
    cudaEventRecord(e, in.cstream);
    cudaStreamWaitEvent(h->stream, e, 0);
  }
  KSVD_TRY(st);
  KSVD_CK(h, cudaMemcpyAsync(D, dD, sizeof(float) * (size_t)n * K, cudaMemcpyDeviceToHost, h->stream));
  if (!drained) {
    KSVD_CK(h, cudaMemcpyAsync(idx, dI, sizeof(int32_t) * (size_t)N * T, cudaMemcpyDeviceToHost, h->stream));
    KSVD_CK(h, cudaMemcpyAsync(coef, dC, sizeof(float) * (size_t)N * T, cudaMemcpyDeviceToHost, h->stream));
    KSVD_CK(h, cudaMemcpyAsync(nnz, dN, sizeof(int32_t) * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
  }
  KSVD_CK(h, cudaStreamSynchronize(h->stream));
  return KSVD_OK;
}

ksvd_status ksvd_iterate_host(ksvd_handle* h, float* D, const float* X, int64_t N, int32_t iters,
                              const int32_t* perms, int32_t* idx, float* coef, int32_t* nnz,
                              double* rmse) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(idx) || bad_ptr(coef) || bad_ptr(nnz) || N < 1)
    return KSVD_ERR_INVALID_ARGUMENT;
  const ksvd_status st = iterate_host_body(h, D, X, N, iters, perms, idx, coef, nnz, rmse);
  if (st != KSVD_OK) {
    // no copy may touch the caller's host buffers after the call returns: drain both streams
    // (their own errors are already reported by st)
    cudaStreamSynchronize(h->stream);
    if (h->inflow.cstream) cudaStreamSynchronize(h->inflow.cstream);
    cudaGetLastError();
    h->inflow.active = false;
    h->inflow.drain = false;
  }
  return st;
}

ksvd_status ksvd_code_fixed(ksvd_handle* h, const float* D, const float* X, int64_t N,
                            const int32_t* idx, const int32_t* nnz, float* coef, float* chol) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(idx) || bad_ptr(nnz) || bad_ptr(coef) || N < 0)
    return KSVD_ERR_INVALID_ARGUMENT;
  if (N == 0) return KSVD_OK;
  float *Dp = nullptr, *G = nullptr;
  int* de = nullptr;
  KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
  KSVD_TRY(load_dict(h, D, &Dp));
  KSVD_TRY(ensure(h, B_G, (size_t)h->Kp * h->Kp, &G));
  KSVD_TRY(gram_padded(h, Dp, G));
  KSVD_CK(h, launch_code_fixed(D, h->p.n, h->p.K, G, h->Kp, X, N, h->p.T, idx, nnz, coef, chol,
                               de, h->stream));
  return KSVD_OK;
}

ksvd_status ksvd_refine_coefs(ksvd_handle* h, const float* D, const float* X, int64_t N,
                              const int32_t* idx, const int32_t* nnz, float* coef, double* coef64) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(idx) || bad_ptr(nnz) || bad_ptr(coef) || N < 0)
    return KSVD_ERR_INVALID_ARGUMENT;
  if (N == 0) return KSVD_OK;
  float *Dp = nullptr, *G = nullptr;
  int* de = nullptr;
  KSVD_TRY(ensure(h, B_DEVERR, 1, &de));
  KSVD_TRY(load_dict(h, D, &Dp));
  KSVD_TRY(ensure(h, B_G, (size_t)h->Kp * h->Kp, &G));
  KSVD_TRY(gram_padded(h, Dp, G));
  KSVD_CK(h, launch_refine(D, h->p.n, h->p.K, G, h->Kp, X, N, h->p.T, idx, nnz, coef, coef64,
                           de, h->stream));
  return KSVD_OK;
}

ksvd_status ksvd_code_backward(ksvd_handle* h, const float* D, const float* X, int64_t N,
                               const int32_t* idx, const int32_t* nnz, const float* coef,
                               const float* chol, const float* dcoef, float* dD, float* dX) {
  if (null_handle(h) || bad_ptr(D) || bad_ptr(X) || bad_ptr(idx) || bad_ptr(nnz) || bad_ptr(coef) ||
      bad_ptr(chol) || bad_ptr(dcoef) || N < 0)
    return KSVD_ERR_INVALID_ARGUMENT;
  if (N == 0) return KSVD_OK;
  KSVD_CK(h, launch_code_backward(D, h->p.n, h->p.K, X, N, h->p.T, idx, nnz, coef, chol, dcoef,
                                  dD, dX, h->stream));
  return KSVD_OK;
}

ksvd_status ksvd_dense_gamma(ksvd_handle* h, int64_t N, const int32_t* idx, const float* coef,
                             const int32_t* nnz, float* gamma) {
  if (null_handle(h) || bad_ptr(idx) || bad_ptr(coef) || bad_ptr(nnz) || bad_ptr(gamma) || N < 0)
    return KSVD_ERR_INVALID_ARGUMENT;
  KSVD_CK(h, launch_dense_gamma(idx, coef, nnz, N, h->p.T, h->p.K, gamma, h->stream));
  return KSVD_OK;
}

}  // extern "C"
