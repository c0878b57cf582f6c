// ksvd -- command-line K-SVD on one GPU through libksvd_gb300, with the reference executable's
// stdout contract (S/main.cu:47-129: banner, one "Iteration %02d / %d complete, RMSE = %.5f"
// line per iteration as printed by S/ReductionKernels.cu:294, "Final Execution Time" and memory
// lines), so Matlab/fmriKSVD.m:54-69, which parses "RMSE = " from stdout, keeps working.
//
// Files are "raw" matrices (the reference reads MAT-files through the MATLAB SDK,
// S/FileManager.cu:98-160, which is proprietary; ksvd_gb300/matio.py converts .mat <-> raw):
//   8 bytes "KSVDRAW1", uint32 dtype (0 float32, 1 float64), uint32 0, uint64 rows, uint64 cols,
//   then rows x cols values, column-major, little-endian.
//
//   ksvd [options] X.raw D.raw Gamma.raw [Dout.raw]
//     -T t                 atoms per signal (required; with --eps, the most per signal)
//     --eps E              error-constrained coding: a signal stops once ||x - D gamma|| <= E
//     --iters N            K-SVD iterations (default 10)
//     --precision P        fp32 | mixed (default fp32)
//     --seed S             atom-order seed (default 0x4B535644)
//     --remove-row-mean    subtract each row's mean over the signals first (Matlab/remmean.m)
//     --refine             FP64-refined least-squares coefficients on the final supports
//     --graph              replay iterations 2..N of each call as a CUDA graph
//     --checkpoint F       write D, the iteration count and the atom-order state to F ...
//     --checkpoint-every k ... every k iterations (default 1 when --checkpoint is given)
//     --resume F           continue the run saved in F (its D replaces D.raw's)
// Gamma.raw receives the dense K x N code (float64, the reference's CUDA_Gamma,
// S/main.cu:133-142); Dout.raw, when given, the final dictionary (float64, S/FileManager.cu:76-82).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cinttypes>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ksvd_gb300.h"

namespace {

struct Matrix {
  uint64_t rows = 0, cols = 0;
  std::vector<float> v;  // column-major
};

const char kRawMagic[8] = {'K', 'S', 'V', 'D', 'R', 'A', 'W', '1'};
const char kCkpMagic[8] = {'K', 'S', 'V', 'D', 'C', 'K', 'P', '1'};

bool read_raw(const char* path, Matrix* m) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char magic[8];
  uint32_t dtype = 0, pad = 0;
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kRawMagic, 8) == 0 &&
            std::fread(&dtype, 4, 1, f) == 1 && std::fread(&pad, 4, 1, f) == 1 &&
            std::fread(&m->rows, 8, 1, f) == 1 && std::fread(&m->cols, 8, 1, f) == 1 &&
            (dtype == 0 || dtype == 1) && m->rows > 0 && m->cols > 0 &&
            m->rows * m->cols < (1ull << 40);
  if (ok) {
    const size_t count = m->rows * m->cols;
    m->v.resize(count);
    if (dtype == 0) {
      ok = std::fread(m->v.data(), 4, count, f) == count;
    } else {
      std::vector<double> tmp(count);
      ok = std::fread(tmp.data(), 8, count, f) == count;
      for (size_t i = 0; ok && i < count; ++i) m->v[i] = (float)tmp[i];
    }
  }
  std::fclose(f);
  return ok;
}

bool write_raw_f64(const char* path, uint64_t rows, uint64_t cols, const std::vector<double>& v) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return false;
  const uint32_t dtype = 1, pad = 0;
  bool ok = std::fwrite(kRawMagic, 1, 8, f) == 8 && std::fwrite(&dtype, 4, 1, f) == 1 &&
            std::fwrite(&pad, 4, 1, f) == 1 && std::fwrite(&rows, 8, 1, f) == 1 &&
            std::fwrite(&cols, 8, 1, f) == 1 &&
            std::fwrite(v.data(), 8, v.size(), f) == v.size();
  return std::fclose(f) == 0 && ok;
}

// checkpoint: magic, int32 n, K, iterations done, pad, uint64 seed, int64 perm draws, D (n x K f32)
bool write_checkpoint(const char* path, int32_t n, int32_t K, int32_t done, uint64_t seed,
                      int64_t draws, const std::vector<float>& D) {
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return false;
  const int32_t pad = 0;
  bool ok = std::fwrite(kCkpMagic, 1, 8, f) == 8 && std::fwrite(&n, 4, 1, f) == 1 &&
            std::fwrite(&K, 4, 1, f) == 1 && std::fwrite(&done, 4, 1, f) == 1 &&
            std::fwrite(&pad, 4, 1, f) == 1 && std::fwrite(&seed, 8, 1, f) == 1 &&
            std::fwrite(&draws, 8, 1, f) == 1 &&
            std::fwrite(D.data(), 4, D.size(), f) == D.size();
  ok = std::fclose(f) == 0 && ok;
  return ok && std::rename(tmp.c_str(), path) == 0;
}

bool read_checkpoint(const char* path, int32_t n, int32_t K, int32_t* done, uint64_t* seed,
                     int64_t* draws, std::vector<float>* D) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char magic[8];
  int32_t cn = 0, cK = 0, pad = 0;
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kCkpMagic, 8) == 0 &&
            std::fread(&cn, 4, 1, f) == 1 && std::fread(&cK, 4, 1, f) == 1 &&
            std::fread(done, 4, 1, f) == 1 && std::fread(&pad, 4, 1, f) == 1 &&
            std::fread(seed, 8, 1, f) == 1 && std::fread(draws, 8, 1, f) == 1 && cn == n &&
            cK == K && *done >= 0 && *draws >= 0;
  if (ok) {
    D->resize((size_t)n * K);
    ok = std::fread(D->data(), 4, D->size(), f) == D->size();
  }
  std::fclose(f);
  return ok;
}

void usage() {
  std::printf(
      "usage: ksvd [options] X.raw D.raw Gamma.raw [Dout.raw]\n"
      "  -T t                 atoms per signal (required; with --eps, the most per signal)\n"
      "  --eps E              error-constrained coding: stop once ||x - D gamma|| <= E\n"
      "  --iters N            K-SVD iterations (default 10)\n"
      "  --precision P        fp32 | mixed (default fp32)\n"
      "  --seed S             atom-order seed (default 0x4B535644)\n"
      "  --remove-row-mean    subtract each row's mean over the signals first\n"
      "  --refine             FP64-refined least-squares coefficients on the final supports\n"
      "  --graph              replay iterations as a CUDA graph\n"
      "  --checkpoint F       save D, iteration count and atom-order state to F\n"
      "  --checkpoint-every k save every k iterations (default 1)\n"
      "  --resume F           continue the run saved in F\n");
}

#define CUDA_OR_DIE(call)                                                       \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      std::fprintf(stderr, "%s: %s\n", #call, cudaGetErrorString(e_));          \
      return 1;                                                                 \
    }                                                                           \
  } while (0)

#define KSVD_OR_DIE(h, call)                                                    \
  do {                                                                          \
    ksvd_status s_ = (call);                                                    \
    if (s_ != KSVD_OK) {                                                        \
      std::fprintf(stderr, "An error occured while executing KSVD!...Aborting\n%s: %s\n", \
                   ksvd_status_string(s_), ksvd_last_error(h));                 \
      return 1;                                                                 \
    }                                                                           \
  } while (0)

}  // namespace

int main(int argc, char** argv) {
  int T = 0, iters = 10, every = 0;
  double eps = -1.0;
  int precision = KSVD_PREC_FP32;
  uint64_t seed = 0x4B535644ULL;
  bool remove_mean = false, refine = false, graph = false;
  const char *ckp = nullptr, *resume = nullptr;
  std::vector<const char*> pos;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> const char* { return i + 1 < argc ? argv[++i] : nullptr; };
    const char* v = nullptr;
    if (a == "-h" || a == "--help") { usage(); return 0; }
    else if (a == "-T" && (v = next())) T = std::atoi(v);
    else if (a == "--iters" && (v = next())) iters = std::atoi(v);
    else if (a == "--eps" && (v = next())) eps = std::atof(v);
    else if (a == "--precision" && (v = next()))
      precision = std::string(v) == "mixed" ? KSVD_PREC_MIXED : KSVD_PREC_FP32;
    else if (a == "--seed" && (v = next())) seed = std::strtoull(v, nullptr, 0);
    else if (a == "--remove-row-mean") remove_mean = true;
    else if (a == "--refine") refine = true;
    else if (a == "--graph") graph = true;
    else if (a == "--checkpoint" && (v = next())) ckp = v;
    else if (a == "--checkpoint-every" && (v = next())) every = std::atoi(v);
    else if (a == "--resume" && (v = next())) resume = v;
    else if (!a.empty() && a[0] == '-') { usage(); return 2; }
    else pos.push_back(argv[i]);
  }
  if (pos.size() < 3 || T < 1 || iters < 0) { usage(); return 2; }
  if (ckp && every < 1) every = 1;

  std::printf("Initializing! Please wait...\n");
  Matrix X, D;
  if (!read_raw(pos[0], &X)) { std::fprintf(stderr, "cannot read %s\n", pos[0]); return 1; }
  if (!read_raw(pos[1], &D)) { std::fprintf(stderr, "cannot read %s\n", pos[1]); return 1; }
  if (X.rows != D.rows) { std::fprintf(stderr, "X and D must have the same rows\n"); return 1; }
  const int n = (int)D.rows, K = (int)D.cols;
  const int64_t N = (int64_t)X.cols;
  int32_t done = 0;
  int64_t draws = 0;
  if (resume && !read_checkpoint(resume, n, K, &done, &seed, &draws, &D.v)) {
    std::fprintf(stderr, "cannot resume from %s (missing, or made for other sizes)\n", resume);
    return 1;
  }
  std::printf(precision == KSVD_PREC_MIXED ? "Mixed (BF16/FP32) precision mode.\n"
                                           : "Single precision mode.\n");
  std::printf("Dictionary size: %d x %d\n", n, K);
  std::printf("Input data size: %d x %" PRId64 "\n", n, N);

  ksvd_params p;
  ksvd_default_params(&p);
  p.n = n; p.K = K; p.T = T; p.precision = precision; p.seed = seed;
  p.flags = (refine ? KSVD_FLAG_REFINE_FINAL : 0) | (graph ? KSVD_FLAG_GRAPH : 0);
  ksvd_handle* h = nullptr;
  cudaStream_t st = nullptr;
  CUDA_OR_DIE(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  KSVD_OR_DIE(h, ksvd_create(&h, &p, st));
  KSVD_OR_DIE(h, ksvd_set_perm_draws(h, draws));
  float *dX = nullptr, *dD = nullptr, *dC = nullptr, *dG = nullptr, *dE = nullptr;
  int32_t *dI = nullptr, *dN = nullptr;
  CUDA_OR_DIE(cudaMalloc(&dX, sizeof(float) * X.v.size()));
  CUDA_OR_DIE(cudaMalloc(&dD, sizeof(float) * D.v.size()));
  CUDA_OR_DIE(cudaMalloc(&dI, sizeof(int32_t) * (size_t)N * T));
  CUDA_OR_DIE(cudaMalloc(&dC, sizeof(float) * (size_t)N * T));
  CUDA_OR_DIE(cudaMalloc(&dN, sizeof(int32_t) * (size_t)N));
  CUDA_OR_DIE(cudaMemcpyAsync(dX, X.v.data(), sizeof(float) * X.v.size(), cudaMemcpyHostToDevice, st));
  CUDA_OR_DIE(cudaMemcpyAsync(dD, D.v.data(), sizeof(float) * D.v.size(), cudaMemcpyHostToDevice, st));
  if (remove_mean) KSVD_OR_DIE(h, ksvd_remove_row_mean(h, dX, N, nullptr));
  if (eps >= 0) {
    std::vector<float> e2((size_t)N, (float)(eps * eps));
    CUDA_OR_DIE(cudaMalloc(&dE, sizeof(float) * (size_t)N));
    CUDA_OR_DIE(cudaMemcpy(dE, e2.data(), sizeof(float) * e2.size(), cudaMemcpyHostToDevice));
  }
  std::printf("Running...\n\n");

  cudaEvent_t e0, e1;
  CUDA_OR_DIE(cudaEventCreate(&e0));
  CUDA_OR_DIE(cudaEventCreate(&e1));
  CUDA_OR_DIE(cudaEventRecord(e0, st));
  const int chunk = ckp ? every : (iters > 0 ? iters : 1);
  std::vector<double> rmse(chunk > 0 ? chunk : 1);
  for (int it = done; it < iters;) {
    const int m = std::min(chunk, iters - it);
    if (dE)
      KSVD_OR_DIE(h, ksvd_iterate_eps(h, dD, dX, N, m, nullptr, dE, dI, dC, dN, rmse.data()));
    else
      KSVD_OR_DIE(h, ksvd_iterate(h, dD, dX, N, m, nullptr, dI, dC, dN, rmse.data()));
    for (int k = 0; k < m; ++k)
      std::printf("Iteration %02d / %d complete, RMSE = %.5f\n", it + k + 1, iters, rmse[k]);
    it += m;
    if (ckp) {
      std::vector<float> Dh((size_t)n * K);
      CUDA_OR_DIE(cudaMemcpy(Dh.data(), dD, sizeof(float) * Dh.size(), cudaMemcpyDeviceToHost));
      if (!write_checkpoint(ckp, n, K, it, seed, ksvd_perm_draws(h), Dh)) {
        std::fprintf(stderr, "cannot write checkpoint %s\n", ckp);
        return 1;
      }
    }
  }
  CUDA_OR_DIE(cudaEventRecord(e1, st));
  CUDA_OR_DIE(cudaEventSynchronize(e1));
  float ms = 0.f;
  CUDA_OR_DIE(cudaEventElapsedTime(&ms, e0, e1));

  // dense K x N code (CUDA_Gamma) and final dictionary, both float64
  CUDA_OR_DIE(cudaMalloc(&dG, sizeof(float) * (size_t)K * N));
  KSVD_OR_DIE(h, ksvd_dense_gamma(h, N, dI, dC, dN, dG));
  std::vector<float> G32((size_t)K * N), D32((size_t)n * K);
  KSVD_OR_DIE(h, ksvd_synchronize(h));
  CUDA_OR_DIE(cudaMemcpy(G32.data(), dG, sizeof(float) * G32.size(), cudaMemcpyDeviceToHost));
  CUDA_OR_DIE(cudaMemcpy(D32.data(), dD, sizeof(float) * D32.size(), cudaMemcpyDeviceToHost));
  if (!write_raw_f64(pos[2], K, N, std::vector<double>(G32.begin(), G32.end()))) {
    std::fprintf(stderr, "cannot write %s\n", pos[2]);
    return 1;
  }
  if (pos.size() > 3 &&
      !write_raw_f64(pos[3], n, K, std::vector<double>(D32.begin(), D32.end()))) {
    std::fprintf(stderr, "cannot write %s\n", pos[3]);
    return 1;
  }
  size_t freeb = 0, total = 0;
  cudaMemGetInfo(&freeb, &total);
  const double mb = 1024.0 * 1024.0;
  const double used_prog = (double)ksvd_workspace_bytes(h) +
                           sizeof(float) * ((double)X.v.size() + D.v.size() + (double)K * N +
                                            (double)N * T) +
                           sizeof(int32_t) * ((double)N * T + N);
  std::printf("\nFinal Execution Time =>\t\t%.3f ms (%.2f sec)\n", ms, ms / 1000.0);
  std::printf("Total Memory Used (program) =>\t%.2f MB\n", used_prog / mb);
  std::printf("Total Available Memory =>\t%.2f MB\n", total / mb);
  std::printf("Total Memory Used (OS) =>\t%.2f MB\n", (total - freeb) / mb);
  std::printf("Total Free Memory =>\t\t%.2f MB\n", freeb / mb);
  std::printf("Memory Utilization =>\t\t%.1f %%\n", 100.0 * used_prog / (double)total);
  ksvd_destroy(h);
  cudaFree(dX); cudaFree(dD); cudaFree(dI); cudaFree(dC); cudaFree(dN); cudaFree(dG);
  if (dE) cudaFree(dE);
  cudaStreamDestroy(st);
  std::printf("----------------------------------------------------\n# Exiting!\n");
  return 0;
}
