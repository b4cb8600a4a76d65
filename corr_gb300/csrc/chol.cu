// Blocked FP64 Cholesky factorisation of the RI metric and the triangular
// solve that applies it, for the energy-only RI pipeline.
//
// The RI-MP2 energy depends on the metric only through
//   (ia|jb) = sum_PQ (ia|P) [J^-1]_PQ (Q|jb),
// so any factor W with W^T W = J^-1 gives the same energy as the reference's
// symmetric J^-1/2 (src/POSTHF/ri.cc:50-69) whenever the reference cuts no
// eigenvalue.  With J = L L^T, W = L^-1 and B = L^-1 (P|ia) is one blocked
// forward substitution: m^2 ncols flops instead of the 2 m^2 ncols of the
// J^-1/2 product, and the factorisation costs m^3/3 instead of a full
// eigendecomposition.
//
// Whether the reference would cut an eigenvalue (lambda/lambda_max < tol) is
// decided by Sylvester's law of inertia: J - t I is positive definite exactly
// when every eigenvalue of J exceeds t.  With t = 10 tol ||J||_inf >= 10 tol
// lambda_max, a successful factorisation of J - t I certifies that no
// eigenvalue lies below tol lambda_max (the factor 10 covers the rounding of
// either factorisation, ~m eps ||J||).  Without the certificate the caller
// falls back to the eigendecomposition (jacobi.cu).
//
// Layout: row-major m x m.  Block size 64: one CTA factors the diagonal block
// in shared memory and also inverts it; the panel below is L21 = A21 L11^-T
// and the trailing update A22 -= L21 L21^T, both on gemm_fp64.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "common.cuh"
#include "dgemm_tc.h"
#include "gemm_fp64.h"
#include "kernels.h"

namespace corr {

namespace {

constexpr int NB = 64;

// A = J - shift I (m x m), Lm = 0.
__global__ void chol_init(const double* __restrict__ J, int m, double shift,
                          double* __restrict__ A, double* __restrict__ Lm) {
  const long long mm = (long long)m * m;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < mm;
       e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e / m), y = (int)(e % m);
    A[e] = J[e] - (x == y ? shift : 0.0);
    Lm[e] = 0.0;
  }
}

// One block of 256 threads: factor the nb x nb diagonal block at (k, k) of A
// (lower), write L_kk into Lm and its inverse into Linv (nb x nb, ld NB).
// A pivot that is not positive (or not finite) sets *fail.
__global__ void __launch_bounds__(256) chol_diag(const double* __restrict__ A, int m, int k,
                                                 int nb, double* __restrict__ Lm,
                                                 double* __restrict__ Linv, int* fail) {
  __shared__ double a[NB][NB + 1];
  __shared__ int bad;
  const int t = threadIdx.x;
  if (t == 0) bad = 0;
  for (int e = t; e < NB * NB; e += 256) {
    const int r = e / NB, cc = e % NB;
    a[r][cc] = (r < nb && cc < nb) ? A[(size_t)(k + r) * m + k + cc] : 0.0;
  }
  __syncthreads();
  for (int c = 0; c < nb; ++c) {
    if (t == 0) {
      const double d = a[c][c];
      if (!(d > 0.0) || !isfinite(d)) bad = 1;
      a[c][c] = (d > 0.0) ? sqrt(d) : 1.0;
    }
    __syncthreads();
    const double p = a[c][c];
    for (int r = c + 1 + t; r < nb; r += 256) a[r][c] /= p;
    __syncthreads();
    const int w = nb - c - 1;
    for (int e = t; e < w * w; e += 256) {
      const int r = c + 1 + e / w, q = c + 1 + e % w;
      if (q <= r) a[r][q] = fma(-a[r][c], a[q][c], a[r][q]);
    }
    __syncthreads();
  }
  // Linv = L^-1 row by row in shared memory: Linv[i][j] (j < i) is kept
  // transposed in the strict upper triangle a[j][i], its diagonal in dinv.
  // Row i: Linv[i][j] = -dinv[i] sum_{q=j}^{i-1} L[i][q] Linv[q][j], four
  // threads per column j (partial sums over q, combined by shuffles).
  __shared__ double dinv[NB];
  if (t < NB) dinv[t] = t < nb ? 1.0 / a[t][t] : 0.0;
  __syncthreads();
  const int j = t >> 2, part = t & 3;
  for (int i = 1; i < nb; ++i) {
    double s = 0.0;
    if (j < i)
      for (int q = j + part; q < i; q += 4) s = fma(a[i][q], q == j ? dinv[j] : a[j][q], s);
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (j < i && part == 0) a[j][i] = -dinv[i] * s;
    __syncthreads();
  }
  for (int e = t; e < NB * NB; e += 256) {
    const int r = e / NB, cc = e % NB;
    double xv = 0.0;
    if (r < nb && cc < nb && cc <= r) xv = cc == r ? dinv[r] : a[cc][r];
    Linv[e] = xv;
  }
  for (int e = t; e < nb * nb; e += 256) {
    const int r = e / nb, cc = e % nb;
    Lm[(size_t)(k + r) * m + k + cc] = (cc <= r) ? a[r][cc] : 0.0;
  }
  if (t == 0 && bad) atomicExch(fail, 1);
}

// max_r sum_c |J[r][c]| (one warp per row; non-negative doubles order as
// their bit patterns).
__global__ void norm_inf_kernel(const double* __restrict__ J, int m,
                                unsigned long long* __restrict__ out) {
  const int warps = (int)(gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (int r = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < m; r += warps) {
    double s = 0.0;
    for (int c = lane; c < m; c += 32) s += fabs(J[(size_t)r * m + c]);
    s = warp_sum(s);
    if (lane == 0) atomicMax(out, (unsigned long long)__double_as_longlong(s));
  }
}

// X[kb .. kb+nb)[kb .. kb+nb) = Linv block b, for every diagonal block (one
// block of threads per diagonal block).
__global__ void place_diag_inverses(const double* __restrict__ Linv, int m,
                                    double* __restrict__ X) {
  const int b = blockIdx.x, k = b * NB, nb = min(NB, m - k);
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int r = e / nb, cc = e % nb;
    X[(size_t)(k + r) * m + k + cc] = Linv[(size_t)b * NB * NB + r * NB + cc];
  }
}

// max_c sum_r |X[r][c]| (one thread per column, coalesced across columns).
__global__ void norm_one_kernel(const double* __restrict__ X, int m,
                                unsigned long long* __restrict__ out) {
  const int cidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (cidx >= m) return;
  double s = 0.0;
  for (int r = 0; r < m; ++r) s += fabs(X[(size_t)r * m + cidx]);
  atomicMax(out, (unsigned long long)__double_as_longlong(s));
}

}  // namespace

size_t chol_workspace_bytes(int m) {
  const int nblk = (m + NB - 1) / NB;
  return (size_t)2 * m * m * 8 + (size_t)nblk * NB * NB * 8 + 3 * 256;
}

int chol_norm_inf(corr_context* c, void* scratch, const double* J, int m, double* out) {
  unsigned long long* d = static_cast<unsigned long long*>(scratch);
  CORR_CUDA(cudaMemsetAsync(d, 0, sizeof(*d), c->stream));
  norm_inf_kernel<<<(m + 7) / 8, 256, 0, c->stream>>>(J, m, d);
  CORR_CUDA(cudaGetLastError());
  unsigned long long h = 0;
  CORR_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CORR_CUDA(cudaStreamSynchronize(c->stream));
  c->launches += 1;
  double v;
  memcpy(&v, &h, sizeof(v));
  *out = v;
  return CORR_OK;
}

// tc_ws: when non-null, the panel and trailing products run on the
// FP64-accurate digit GEMM (dgemm_tc.cu) with that workspace
// (dgemm_tc_workspace(m, m, NB) bytes); else on the FP64 GEMM.
int chol_factor_device(corr_context* c, void* ws, const double* J, int m, double shift,
                       double** Lm_out, double** Linv_out, bool* ok, void* tc_ws) {
  const int nblk = (m + NB - 1) / NB;
  Carver w{ws, 0};
  double* A = static_cast<double*>(w.take((size_t)m * m * 8));
  double* Lm = static_cast<double*>(w.take((size_t)m * m * 8));
  double* Linv = static_cast<double*>(w.take((size_t)nblk * NB * NB * 8));
  int* fail = static_cast<int*>(w.take(sizeof(int)));
  cudaStream_t s = c->stream;
  CORR_CUDA(cudaMemsetAsync(fail, 0, sizeof(int), s));
  const int ig = (int)std::min<long long>(((long long)m * m + 255) / 256, 4096);
  chol_init<<<ig, 256, 0, s>>>(J, m, shift, A, Lm);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  for (int b = 0; b < nblk; ++b) {
    const int k = b * NB, nb = std::min(NB, m - k), rem = m - k - nb;
    double* Li = Linv + (size_t)b * NB * NB;
    chol_diag<<<1, 256, 0, s>>>(A, m, k, nb, Lm, Li, fail);
    CORR_CUDA(cudaGetLastError());
    c->launches += 1;
    if (rem == 0) break;
    const double* P = Lm + (size_t)(k + nb) * m + k;
    if (tc_ws) {
      // L21 = A21 L11^-T: rows of A21 against the rows of L11^-1
      DgemmTc g;
      g.A = mat_view(A + (size_t)(k + nb) * m + k, m, 1);
      g.B = mat_view(Li, NB, 1);
      g.C = out_view(Lm + (size_t)(k + nb) * m + k, m, 1);
      g.M = rem;
      g.N = nb;
      g.K = nb;
      g.alpha = 1.0;
      g.accumulate = false;
      g.a_lower = false;
      CORR_TRY(dgemm_tc(c, g, tc_ws));
      // A22 -= L21 L21^T
      DgemmTc u = g;
      u.A = mat_view(P, m, 1);
      u.B = mat_view(P, m, 1);
      u.C = out_view(A + (size_t)(k + nb) * m + k + nb, m, 1);
      u.N = rem;
      u.alpha = -1.0;
      u.accumulate = true;
      CORR_TRY(dgemm_tc(c, u, tc_ws));
    } else {
      // L21 = A21 L11^-T
      GemmF64 g = gemm_args(A + (size_t)(k + nb) * m + k, Li, Lm + (size_t)(k + nb) * m + k, rem,
                            nb, nb, m, NB, m, 0, 1);
      CORR_TRY(gemm_f64(g, &c->dres->status, s));
      // A22 -= L21 L21^T
      GemmF64 u = gemm_args(P, P, A + (size_t)(k + nb) * m + k + nb, rem, rem, nb, m, m, m, 0, 1);
      u.alpha = -1.0;
      u.beta = 1.0;
      CORR_TRY(gemm_f64(u, &c->dres->status, s));
      c->launches += 2;
    }
  }
  int h = 0;
  CORR_CUDA(cudaMemcpyAsync(&h, fail, sizeof(int), cudaMemcpyDeviceToHost, s));
  CORR_CUDA(cudaStreamSynchronize(s));
  *ok = (h == 0);
  *Lm_out = Lm;
  *Linv_out = Linv;
  return CORR_OK;
}

int chol_solve_device(corr_context* c, const double* Lm, const double* Linv, int m, double* P,
                      long long ncols, double* out) {
  const int nblk = (m + NB - 1) / NB;
  cudaStream_t s = c->stream;
  for (int b = 0; b < nblk; ++b) {
    const int r0 = b * NB, nb = std::min(NB, m - r0);
    double* Pi = P + (size_t)r0 * ncols;
    if (r0 > 0) {
      // P_i -= L[r0:r0+nb, 0:r0] B[0:r0, :]
      GemmF64 g = gemm_args(Lm + (size_t)r0 * m, out, Pi, nb, (int)ncols, r0, m, ncols, ncols, 0,
                            0);
      g.alpha = -1.0;
      g.beta = 1.0;
      CORR_TRY(gemm_f64(g, &c->dres->status, s));
    }
    // B_i = L_ii^-1 P_i
    CORR_TRY(gemm_f64(gemm_args(Linv + (size_t)b * NB * NB, Pi, out + (size_t)r0 * ncols, nb,
                                (int)ncols, nb, NB, ncols, ncols, 0, 0),
                      &c->dres->status, s));
    c->launches += (r0 > 0) ? 2 : 1;
  }
  return CORR_OK;
}

// X = L^-1 (m x m, ld m) for the factor of chol_factor_device (Lm, and the
// inverses of its 64 x 64 diagonal blocks in Linv), by recursive blocked
// inversion on 64-aligned splits:
//   [[L11, 0], [L21, L22]]^-1 = [[X11, 0], [-X22 L21 X11, X22]].
// T: scratch of m * m doubles.  The strict upper triangle of X is zero.
int chol_inverse_device(corr_context* c, const double* Lm, const double* Linv, int m, double* X,
                        double* T, void* tc_ws) {
  const int nblk = (m + NB - 1) / NB;
  cudaStream_t s = c->stream;
  CORR_CUDA(cudaMemsetAsync(X, 0, (size_t)m * m * 8, s));
  place_diag_inverses<<<nblk, 256, 0, s>>>(Linv, m, X);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  struct Node {
    int r0, n;
  };
  // post-order over the split tree (children before their parent)
  std::vector<Node> order;
  std::vector<std::pair<Node, bool>> stack{{{0, m}, false}};
  while (!stack.empty()) {
    auto [nd, expanded] = stack.back();
    stack.pop_back();
    if (nd.n <= NB) continue;
    if (expanded) {
      order.push_back(nd);
      continue;
    }
    const int n1 = NB * (((nd.n + NB - 1) / NB + 1) / 2);
    stack.push_back({nd, true});
    stack.push_back({{nd.r0 + n1, nd.n - n1}, false});
    stack.push_back({{nd.r0, n1}, false});
  }
  for (const Node& nd : order) {
    const int n1 = NB * (((nd.n + NB - 1) / NB + 1) / 2), n2 = nd.n - n1;
    const int r0 = nd.r0, r1 = nd.r0 + n1;
    if (tc_ws && n1 >= 4 * NB) {
      // T = L21 X11: rows of L21 against the columns of X11 (read as rows over k)
      DgemmTc g;
      g.A = mat_view(Lm + (size_t)r1 * m + r0, m, 1);
      g.B = mat_view(X + (size_t)r0 * m + r0, 1, m);
      g.C = out_view(T, n1, 1);
      g.M = n2;
      g.N = n1;
      g.K = n1;
      g.alpha = 1.0;
      g.accumulate = false;
      g.a_lower = false;
      CORR_TRY(dgemm_tc(c, g, tc_ws));
      // X21 = -X22 T (X22 lower triangular)
      DgemmTc h = g;
      h.A = mat_view(X + (size_t)r1 * m + r1, m, 1);
      h.B = mat_view(T, 1, n1);
      h.C = out_view(X + (size_t)r1 * m + r0, m, 1);
      h.K = n2;
      h.alpha = -1.0;
      h.a_lower = true;
      CORR_TRY(dgemm_tc(c, h, tc_ws));
    } else {
      // T = L21 X11   (n2 x n1)
      GemmF64 g = gemm_args(Lm + (size_t)r1 * m + r0, X + (size_t)r0 * m + r0, T, n2, n1, n1, m,
                            m, n1, 0, 0);
      CORR_TRY(gemm_f64(g, &c->dres->status, s));
      // X21 = -X22 T
      GemmF64 h = gemm_args(X + (size_t)r1 * m + r1, T, X + (size_t)r1 * m + r0, n2, n1, n2, m,
                            n1, m, 0, 0);
      h.alpha = -1.0;
      CORR_TRY(gemm_f64(h, &c->dres->status, s));
      c->launches += 2;
    }
  }
  return CORR_OK;
}

// ||X||_1 ||X||_inf of an m x m matrix (scratch: 16 bytes of device memory).
int chol_norm_one_inf(corr_context* c, void* scratch, const double* X, int m, double* out) {
  unsigned long long* d = static_cast<unsigned long long*>(scratch);
  CORR_CUDA(cudaMemsetAsync(d, 0, 2 * sizeof(*d), c->stream));
  norm_one_kernel<<<(m + 255) / 256, 256, 0, c->stream>>>(X, m, d);
  norm_inf_kernel<<<(m + 7) / 8, 256, 0, c->stream>>>(X, m, d + 1);
  CORR_CUDA(cudaGetLastError());
  unsigned long long h[2] = {0, 0};
  CORR_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CORR_CUDA(cudaStreamSynchronize(c->stream));
  c->launches += 2;
  double v[2];
  memcpy(v, h, sizeof(v));
  *out = v[0] * v[1];
  return CORR_OK;
}

}  // namespace corr
