// FP64-accurate GEMM on the tensor cores (dgemm_tc.cu): exact digit slicing
// of both FP64 operands, integer-exact level sums on tcgen05 (kind::f16, BF16
// digits, FP32 accumulation in TMEM), integer recombination to FP64.
#pragma once

#include <cuda_runtime.h>

#include "abi_internal.h"

namespace corr {

// An FP64 matrix read as `rows` x K: element (r, k) at
//   p[(r / rdiv) * rs_hi + (r % rdiv) * rs_lo + k * ks]
// (rdiv = rows, rs_hi = 0 for a plain strided matrix; a two-level row index
// for row sets such as (P, nu) of a 3-index tensor).
struct MatView {
  const double* p;
  long long rs_hi, rs_lo, ks, rdiv;
};
// Output element (m, n) at p[(m / rdiv) * rs_hi + (m % rdiv) * rs_lo + n * cs].
struct OutView {
  double* p;
  long long rs_hi, rs_lo, cs, rdiv;
};

inline MatView mat_view(const double* p, long long rs, long long ks) {
  return MatView{p, 0, rs, ks, 1LL << 62};
}
inline OutView out_view(double* p, long long rs, long long cs) {
  return OutView{p, 0, rs, cs, 1LL << 62};
}

// C[m][n] = alpha sum_k A(m, k) B(n, k) (+ C[m][n] when accumulate), m < M,
// n < N, k < K.  a_lower: A(m, k) == 0 for k > m (skipped).  Inputs finite.
struct DgemmTc {
  MatView A, B;
  OutView C;
  int M, N, K;
  double alpha;
  bool accumulate;
  bool a_lower;
};

// Device workspace of one dgemm_tc call (bytes).
size_t dgemm_tc_workspace(int M, int N, int K);
// Enqueue on the context stream; ws holds dgemm_tc_workspace(M, N, K) bytes.
int dgemm_tc(corr_context* c, const DgemmTc& g, void* ws);

}  // namespace corr
