// FP64 GEMM building block (gemm_fp64.cu) and the FP64 hot-path helpers built
// on it (transforms.cu).
#pragma once

#include <cuda_runtime.h>

#include "abi_internal.h"

namespace corr {

struct GemmF64 {
  const double* A;
  const double* B;
  double* C;
  int M, N, K;
  long long lda, ldb, ldc;
  long long sa, sb, sc;  // batch strides (elements), 0 = shared operand
  int batch;
  int ta, tb;
  double alpha, beta;
};

// Enqueue C = alpha op(A) op(B) + beta C on stream s.
int gemm_f64(const GemmF64& g, int* status, cudaStream_t s);

inline GemmF64 gemm_args(const double* A, const double* B, double* C, int M, int N, int K,
                         long long lda, long long ldb, long long ldc, int ta, int tb) {
  GemmF64 g;
  g.A = A;
  g.B = B;
  g.C = C;
  g.M = M;
  g.N = N;
  g.K = K;
  g.lda = lda;
  g.ldb = ldb;
  g.ldc = ldc;
  g.sa = g.sb = g.sc = 0;
  g.batch = 1;
  g.ta = ta;
  g.tb = tb;
  g.alpha = 1.0;
  g.beta = 0.0;
  return g;
}

}  // namespace corr
