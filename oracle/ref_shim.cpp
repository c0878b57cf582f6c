// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY: a host harness that compiles the reference's own
// per-thread device code unchanged and runs it on the CPU, so that the oracle can be checked
// against the reference's arithmetic.
//
// The reference's parOMP kernel and its helpers (K-SVD/K-SVD/OMP.cu:126-404) and its two
// per-atom update kernels device_A_times_x_modified / device_normal_x_times_A_modified
// (K-SVD/K-SVD/Multiplication.cu:177-224) are plain per-thread C with no warp-level code.
// oracle/ref_build.py copies those line ranges, untouched, from a reference checkout into the
// git-ignored build folder oracle/_ref/ (ref_omp_src.inc, ref_mult_src.inc) and compiles this
// file against them.  Nothing of the reference is kept in the repository.
//
// The shim supplies what the reference's headers would: `datatype` (double, its default:
// GlobalDeclarations.cuh:27-35), SQR (GlobalDeclarations.cuh:84), the compile-time sparsity
// Tdata (ProgramParameters.cuh:20; one copy of the code per T in 1-8, 10, 12), CUDA qualifiers
// defined away and the thread coordinates as host variables.  A kernel "launch" is a loop that
// sets those coordinates for every thread of the reference's grid, one thread at a time.
#include <cmath>
#include <cstdint>

typedef double datatype;
#define SQR(x) (x) * (x)
#define __inline__ inline
#define __device__
#define __global__

namespace {
struct RefDim { unsigned int x; };
RefDim threadIdx{0}, blockIdx{0}, blockDim{1};
}  // namespace

// the reference's parOMP and helpers, once per T (Tdata is a compile-time constant there)
namespace ref_t1 { constexpr int Tdata = 1;
#include "ref_omp_src.inc"
}
namespace ref_t2 { constexpr int Tdata = 2;
#include "ref_omp_src.inc"
}
namespace ref_t3 { constexpr int Tdata = 3;
#include "ref_omp_src.inc"
}
namespace ref_t4 { constexpr int Tdata = 4;
#include "ref_omp_src.inc"
}
namespace ref_t5 { constexpr int Tdata = 5;
#include "ref_omp_src.inc"
}
namespace ref_t6 { constexpr int Tdata = 6;
#include "ref_omp_src.inc"
}
namespace ref_t7 { constexpr int Tdata = 7;
#include "ref_omp_src.inc"
}
namespace ref_t8 { constexpr int Tdata = 8;
#include "ref_omp_src.inc"
}
namespace ref_t10 { constexpr int Tdata = 10;
#include "ref_omp_src.inc"
}
namespace ref_t12 { constexpr int Tdata = 12;
#include "ref_omp_src.inc"
}
namespace ref_mult {
#include "ref_mult_src.inc"
}

namespace {
template <void (*KERNEL)(datatype*, datatype*, datatype*, datatype*, int, int)>
void run_paromp(datatype* DtX, datatype* sel, datatype* G, datatype* c, int K, int N) {
  // parOMP<<<ceil(N / 512), 512>>> (OMP.cu:110-112): thread signum = blockIdx.x * 512 + tid
  blockDim.x = 512;
  for (int s = 0; s < N; ++s) {
    blockIdx.x = (unsigned)(s / 512);
    threadIdx.x = (unsigned)(s % 512);
    KERNEL(DtX, sel, G, c, K, N);
  }
}
}  // namespace

// Batch-OMP of N signals with the reference's parOMP (K <= 32: its alpha[32], OMP.cu:270).
// DtX K x N, G K x K (column-major, FP64); outputs: sel K x N (slot number + 1 of each chosen
// atom, 0 elsewhere; OMP.cu:313) and c T x N (coefficients by slot).  Returns -1 for an
// unsupported T or K.
extern "C" int ref_paromp(int T, datatype* DtX, datatype* sel, datatype* G, datatype* c, int K,
                          int N) {
  if (K < 1 || K > 32 || N < 0) return -1;
  switch (T) {
    case 1: run_paromp<ref_t1::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 2: run_paromp<ref_t2::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 3: run_paromp<ref_t3::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 4: run_paromp<ref_t4::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 5: run_paromp<ref_t5::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 6: run_paromp<ref_t6::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 7: run_paromp<ref_t7::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 8: run_paromp<ref_t8::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 10: run_paromp<ref_t10::parOMP>(DtX, sel, G, c, K, N); return 0;
    case 12: run_paromp<ref_t12::parOMP>(DtX, sel, G, c, K, N); return 0;
    default: return -1;
  }
}

// out = out - A x + d gammaJ (rows < n) with the reference's device_A_times_x_modified
// (Multiplication.cu:177-193; launched <<<1, recommended>>> with recommended >= n).  `count` is
// the atom's list length, stored as an int in the first bytes of a datatype as the reference does.
extern "C" void ref_a_times_x(datatype* A, datatype* x, datatype* out, int n, int K, datatype* d,
                              datatype* gammaJ, int count) {
  datatype counters[1] = {0};
  *reinterpret_cast<int*>(counters) = count;
  blockDim.x = (unsigned)n;
  blockIdx.x = 0;
  for (int t = 0; t < n; ++t) {
    threadIdx.x = (unsigned)t;
    ref_mult::device_A_times_x_modified(A, x, out, (unsigned)n, (unsigned)K, d, gammaJ, counters);
  }
}

// New coefficients Gamma(pJ, columns[m]) for the m < count list entries and the new atom
// D = in / norm (n rows) with the reference's device_normal_x_times_A_modified
// (Multiplication.cu:198-224; launched over colsX + n threads in blocks of 512).
extern "C" void ref_normal_x_times_a(datatype* aD, datatype* Gamma, datatype* columns, int K,
                                     datatype* gammaJ, datatype* rowlincomb, datatype* constant,
                                     datatype* norm, int pJ, int count, datatype* D, datatype* in,
                                     int n, int colsX) {
  datatype counter[1] = {0};
  *reinterpret_cast<int*>(counter) = count;
  blockDim.x = 512;
  const int total = colsX + n;
  for (int t = 0; t < total; ++t) {
    blockIdx.x = (unsigned)(t / 512);
    threadIdx.x = (unsigned)(t % 512);
    ref_mult::device_normal_x_times_A_modified(aD, Gamma, columns, (unsigned)K, gammaJ,
                                               rowlincomb, constant, norm, (unsigned)pJ, counter,
                                               D, in, (unsigned)n, (unsigned)colsX);
  }
}
