// cpu_gemm.cpp -- register-blocked FP64 matrix product for the timed CPU baseline (test infrastructure:
// used by the oracle's cached-AO engine when it is timed as CalChem's CPU path, never by the product).
//
// CalChem's RksVxcEngine::evaluate does its two contractions per 128-point batch with faer's blocked,
// SIMD, fused-multiply-add GEMM (gemm_nn_into / gemm_nt_into, crates/calchem-tensor/src/lib.rs:114-135,
// called at crates/calchem-dft/src/vxc.rs:860-949).  The oracle's checker keeps plain triple loops
// without fused multiply-adds; this unit is the fast form of the same products for timing.  It is
// portable C++ (no intrinsics): a 4 x 8 block of C is held in local accumulators across the whole
// K loop, so the compiler keeps it in vector registers and emits vector FMAs on both x86-64 and
// AArch64, and the 8-column panel of B it streams stays in L1 across the row blocks.
#include <algorithm>

namespace orc {

// C (M x N, row stride ldc) += A B, where A(i, k) = A[i * ars + k * acs] and B is row-major (row
// stride ldb).  Summation over k runs in order for every element.
void gemm_acc(int M, int N, int K, const double* A, long ars, long acs, const double* B, long ldb, double* C,
              long ldc) {
  constexpr int MR = 4, NR = 8;
  int j = 0;
  for (; j + NR <= N; j += NR) {
    int i = 0;
    for (; i + MR <= M; i += MR) {
      double acc[MR][NR] = {};
      for (int k = 0; k < K; ++k) {
        const double* b = B + (long)k * ldb + j;
        double x[MR];
#pragma GCC unroll 4
        for (int r = 0; r < MR; ++r) x[r] = A[(long)(i + r) * ars + (long)k * acs];
#pragma GCC unroll 4
        for (int r = 0; r < MR; ++r)
#pragma GCC unroll 8
          for (int jj = 0; jj < NR; ++jj) acc[r][jj] += x[r] * b[jj];
      }
      for (int r = 0; r < MR; ++r) {
        double* c = C + (long)(i + r) * ldc + j;
#pragma GCC unroll 8
        for (int jj = 0; jj < NR; ++jj) c[jj] += acc[r][jj];
      }
    }
    for (; i < M; ++i) {  // remaining rows
      double acc[NR] = {};
      const double* a = A + (long)i * ars;
      for (int k = 0; k < K; ++k) {
        const double* b = B + (long)k * ldb + j;
        const double x = a[(long)k * acs];
#pragma GCC unroll 8
        for (int jj = 0; jj < NR; ++jj) acc[jj] += x * b[jj];
      }
      double* c = C + (long)i * ldc + j;
      for (int jj = 0; jj < NR; ++jj) c[jj] += acc[jj];
    }
  }
  for (; j < N; ++j)  // remaining columns
    for (int i = 0; i < M; ++i) {
      double s = 0.0;
      const double* a = A + (long)i * ars;
      for (int k = 0; k < K; ++k) s += a[(long)k * acs] * B[(long)k * ldb + j];
      C[(long)i * ldc + j] += s;
    }
}

}  // namespace orc
