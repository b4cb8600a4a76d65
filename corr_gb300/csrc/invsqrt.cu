// J^-1/2 of a certified RI metric without an eigendecomposition: the scaled
// coupled Newton-Schulz iteration with every product on the FP64-accurate
// digit GEMM (dgemm_tc.cu).
//
// The reference (src/POSTHF/ri.cc:50-69) forms J^-1/2 = V diag(f) V^T from
// the eigenpairs of J, with f = lambda^-1/2 and f = 0 for lambda/lambda_max
// < tol.  When a Cholesky factorisation of J - t I succeeds with
// t = 10 tol ||J||_inf (>= 10 tol lambda_max, the certificate of chol.cu),
// every eigenvalue exceeds t, nothing is cut, and J^-1/2 is the unique
// symmetric positive definite inverse square root, which this iteration
// computes (Higham, "Functions of Matrices", sec. 6.7):
//   Y_0 = J / c, Z_0 = I, c >= lambda_max (c = min(||J||_inf, ||J||_F)),
//   T_k = (3 I - a_k^2 Z_k Y_k) / 2,  Y_k+1 = a_k Y_k T_k,  Z_k+1 = a_k T_k Z_k,
//   Z_k -> (J / c)^-1/2,  J^-1/2 = Z / sqrt(c).
// The eigenvalues s of (Z Y)^1/2 follow the cubic s -> p(a s), p(x) =
// x (3 - x^2) / 2, from [l_k, 1]; a_k^2 = 3 / (1 + l_k + l_k^2) makes
// p(a_k l_k) = p(a_k) (the scaling of Chen and Chow, 2014, for the sign
// iteration), so l_k+1 = p(a_k l_k) grows by ~2.6 per step instead of 1.5,
// from l_0 = (t / c)^1/2.  Then unscaled steps until max|Z Y - I| stops
// falling below 1e-14 (quadratic convergence).  Products of symmetric
// iterates are symmetric up to rounding; the result is symmetrised.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "abi_internal.h"
#include "common.cuh"
#include "dgemm_tc.h"

namespace corr {

int chol_norm_inf(corr_context* c, void* scratch, const double* J, int m, double* out);
int chol_factor_device(corr_context* c, void* ws, const double* J, int m, double shift,
                       double** Lm_out, double** Linv_out, bool* ok, void* tc_ws);
size_t chol_workspace_bytes(int m);

namespace {

// T = 1.5 I - 0.5 a2 P; err = max |a2 P - I| (bit pattern max of a non-negative double)
__global__ void ns_step_kernel(const double* __restrict__ P, int m, double a2,
                               double* __restrict__ T, unsigned long long* __restrict__ err) {
  double e = 0.0;
  const long long mm = (long long)m * m;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < mm;
       x += (long long)gridDim.x * blockDim.x) {
    const bool d = (x / m) == (x % m);
    const double q = a2 * P[x];
    e = fmax(e, fabs(q - (d ? 1.0 : 0.0)));
    T[x] = (d ? 1.5 : 0.0) - 0.5 * q;
  }
  e = fmax(e, __shfl_xor_sync(0xffffffffu, e, 16));
  e = fmax(e, __shfl_xor_sync(0xffffffffu, e, 8));
  e = fmax(e, __shfl_xor_sync(0xffffffffu, e, 4));
  e = fmax(e, __shfl_xor_sync(0xffffffffu, e, 2));
  e = fmax(e, __shfl_xor_sync(0xffffffffu, e, 1));
  if ((threadIdx.x & 31) == 0) atomicMax(err, (unsigned long long)__double_as_longlong(e));
}

// Y = J / c, Z = I
__global__ void ns_init_kernel(const double* __restrict__ J, int m, double rc,
                               double* __restrict__ Y, double* __restrict__ Z) {
  const long long mm = (long long)m * m;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < mm;
       x += (long long)gridDim.x * blockDim.x) {
    Y[x] = J[x] * rc;
    Z[x] = (x / m) == (x % m) ? 1.0 : 0.0;
  }
}

// out = (Z + Z^T) / (2 sqrt(c)); sum of squares of J for the Frobenius norm
__global__ void ns_finish_kernel(const double* __restrict__ Z, int m, double s,
                                 double* __restrict__ out) {
  const long long mm = (long long)m * m;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < mm;
       x += (long long)gridDim.x * blockDim.x) {
    const long long r = x / m, q = x % m;
    out[x] = 0.5 * s * (Z[x] + Z[q * m + r]);
  }
}

__global__ void sumsq_kernel(const double* __restrict__ J, long long n, double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
       x += (long long)gridDim.x * blockDim.x)
    s += J[x] * J[x];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

constexpr int kSqBlocks = 256;

}  // namespace

size_t ns_workspace_bytes(int m) {
  const size_t mm = (size_t)m * m * 8;
  return std::max(chol_workspace_bytes(m), 4 * mm) + dgemm_tc_workspace(m, m, m) +
         kSqBlocks * 8 + 1024;
}

// J^-1/2 into out (m x m, device) when J - 10 tol ||J||_inf I is positive
// definite; *done = false (and out untouched) otherwise or when the
// iteration does not converge.  ws: ns_workspace_bytes(m).
int ri_inv_sqrt_ns(corr_context* c, void* ws, const double* J, int m, double tol, double* out,
                   bool* done) {
  *done = false;
  cudaStream_t s = c->stream;
  const size_t mm = (size_t)m * m;
  Carver w{ws, 0};
  void* front = w.take(std::max(chol_workspace_bytes(m), 4 * mm * 8));
  void* dws = w.take(dgemm_tc_workspace(m, m, m));
  double* part = static_cast<double*>(w.take(kSqBlocks * 8));
  unsigned long long* derr = reinterpret_cast<unsigned long long*>(part);
  // norms and the certificate
  double jinf = 0.0;
  CORR_TRY(chol_norm_inf(c, part, J, m, &jinf));
  if (!(jinf > 0.0) || !std::isfinite(jinf)) return CORR_OK;
  double *Lm = nullptr, *Linv = nullptr;
  bool certified = false;
  const double t = 10.0 * tol * jinf;
  CORR_TRY(chol_factor_device(c, front, J, m, t, &Lm, &Linv, &certified, dws));
  if (!certified) return CORR_OK;
  sumsq_kernel<<<kSqBlocks, 256, 0, s>>>(J, (long long)mm, part);
  CORR_CUDA(cudaGetLastError());
  std::vector<double> hp(kSqBlocks);
  CORR_CUDA(cudaMemcpyAsync(hp.data(), part, kSqBlocks * 8, cudaMemcpyDeviceToHost, s));
  CORR_CUDA(cudaStreamSynchronize(s));
  double f2 = 0.0;
  for (double v : hp) f2 += v;
  const double cnorm = std::min(jinf, std::sqrt(f2));  // >= lambda_max
  // the iterates (over the Cholesky workspace, which is free now)
  double* Y = static_cast<double*>(front);
  double* Z = Y + mm;
  double* T = Z + mm;
  double* P = T + mm;
  const int grid = (int)std::min<long long>(((long long)mm + 255) / 256, (long long)c->sms * 8);
  ns_init_kernel<<<grid, 256, 0, s>>>(J, m, 1.0 / cnorm, Y, Z);
  CORR_CUDA(cudaGetLastError());
  c->launches += 3;
  auto gemm = [&](const double* A, const double* B, double* C, double alpha) -> int {
    DgemmTc g;
    g.A = mat_view(A, m, 1);
    g.B = mat_view(B, 1, m);  // B read as rows n over k: B[k][n]
    g.C = out_view(C, m, 1);
    g.M = m;
    g.N = m;
    g.K = m;
    g.alpha = alpha;
    g.accumulate = false;
    g.a_lower = false;
    return dgemm_tc(c, g, dws);
  };
  double l = std::sqrt(std::min(1.0, t / cnorm));  // lower bound of the s spectrum
  double prev = 1e300;
  bool conv = false;
  for (int it = 0; it < 60; ++it) {
    const bool scaled = l < 0.999;
    const double a2 = scaled ? 3.0 / (1.0 + l + l * l) : 1.0, a = std::sqrt(a2);
    CORR_TRY(gemm(Z, Y, P, 1.0));
    CORR_CUDA(cudaMemsetAsync(derr, 0, 8, s));
    ns_step_kernel<<<grid, 256, 0, s>>>(P, m, a2, T, derr);
    CORR_CUDA(cudaGetLastError());
    unsigned long long he = 0;
    CORR_CUDA(cudaMemcpyAsync(&he, derr, 8, cudaMemcpyDeviceToHost, s));
    CORR_CUDA(cudaStreamSynchronize(s));
    double err;
    std::memcpy(&err, &he, 8);
    c->launches += 1;
    if (!std::isfinite(err)) return CORR_OK;
    if (!scaled && (err < 1e-14 || (err >= 0.5 * prev && err < 1e-12))) {
      conv = true;  // converged: a further step only re-rounds
      break;
    }
    if (!scaled) prev = err;
    // Y <- a Y T, Z <- a T Z (into P, then swap)
    CORR_TRY(gemm(Y, T, P, a));
    std::swap(Y, P);
    CORR_TRY(gemm(T, Z, P, a));
    std::swap(Z, P);
    if (scaled) {
      const double x = a * l;
      l = std::min(1.0, 0.5 * x * (3.0 - x * x));
    }
  }
  if (!conv) return CORR_OK;
  ns_finish_kernel<<<grid, 256, 0, s>>>(Z, m, 1.0 / std::sqrt(cnorm), out);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  *done = true;
  return CORR_OK;
}

}  // namespace corr
