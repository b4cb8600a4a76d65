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
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "abi_internal.h"
#include "common.cuh"
#include "dgemm_tc.h"
#include "gemm_fp64.h"

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

// The whole computation for small orders (m < 256) in one cooperative launch:
// ||J||_inf and ||J||_F (c = min of the two >= lambda_max, t = 10 tol
// ||J||_inf), then the same iteration as the host loop below (scaled steps
// following the bound l from l0 = (t / c)^1/2, then unscaled steps until
// max|a^2 Z Y - I| stops falling below 1e-14), each product a grid-wide pass
// of FP64 dot products over L2-resident matrices, grid.sync() between passes;
// finally the certificate from Z itself: Z ~ (J/c)^-1/2 is symmetric, so
// lambda_min(J) = c / ||Z||_2^2 >= c / r^2 with r its largest absolute row
// sum (||Z||_2 <= (||Z||_1 ||Z||_inf)^1/2 = r); nothing is cut when that bound
// exceeds 2t.  The control flow is computed identically by every thread
// (reductions are read back from global slots after the syncs), so every
// thread reaches every grid.sync().  done[0] = 1 when converged and
// certified; out = (Z + Z^T) / (2 c^1/2).
__global__ void __launch_bounds__(256) ns_small_kernel(const double* __restrict__ J, int m,
                                                       double tol, double* Y, double* Z,
                                                       double* T, double* Y2, double* Z2,
                                                       double* __restrict__ out,
                                                       unsigned long long* slots, double* fsum,
                                                       int* done) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  const long long mm = (long long)m * m;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long nth = (long long)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  auto warp_max = [&](double v) {
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
  };
  for (long long x = tid; x < 64; x += nth) slots[x] = 0ull;
  if (tid == 0) fsum[0] = 0.0;
  grid.sync();
  // norms of J: slot 62 = max absolute row sum, fsum = sum of squares
  double rmax = 0.0, sq = 0.0;
  for (long long r = tid; r < m; r += nth) {
    double rs = 0.0;
    for (int k = 0; k < m; ++k) {
      const double v = J[r * m + k];
      rs += fabs(v);
      sq += v * v;
    }
    rmax = fmax(rmax, rs);
  }
  rmax = warp_max(rmax);
  for (int off = 16; off > 0; off >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, off);
  if (lane == 0) {
    atomicMax(&slots[62], (unsigned long long)__double_as_longlong(rmax));
    if (sq != 0.0) atomicAdd(fsum, sq);
  }
  grid.sync();
  const double jinf = __longlong_as_double((long long)slots[62]);
  const double cnorm = fmin(jinf, sqrt(fsum[0])), t = 10.0 * tol * jinf;
  if (!(cnorm > 0.0) || !isfinite(cnorm)) {
    if (tid == 0) done[0] = 0;
    return;  // uniform: every thread read the same slots
  }
  const double rc = 1.0 / cnorm;
  for (long long x = tid; x < mm; x += nth) {
    Y[x] = J[x] * rc;
    Z[x] = (x / m) == (x % m) ? 1.0 : 0.0;
  }
  grid.sync();
  double l = sqrt(fmin(1.0, t * rc)), prev = 1e300;
  bool conv = false;
  for (int it = 0; it < 60; ++it) {
    const bool scaled = l < 0.999;
    const double a2 = scaled ? 3.0 / (1.0 + l + l * l) : 1.0, a = sqrt(a2);
    double e = 0.0;
    for (long long x = tid; x < mm; x += nth) {
      const int i = (int)(x / m), j = (int)(x % m);
      double acc = 0.0;
      for (int k = 0; k < m; ++k) acc = fma(Z[(long long)i * m + k], Y[(long long)k * m + j], acc);
      const double q = a2 * acc;
      e = fmax(e, fabs(q - (i == j ? 1.0 : 0.0)));
      T[x] = (i == j ? 1.5 : 0.0) - 0.5 * q;
    }
    e = warp_max(e);
    if (lane == 0) atomicMax(&slots[it], (unsigned long long)__double_as_longlong(e));
    grid.sync();
    if (!scaled) {
      const double err = __longlong_as_double((long long)slots[it]);
      if (!isfinite(err)) break;
      if (err < 1e-14 || (err >= 0.5 * prev && err < 1e-12)) {
        conv = true;
        break;
      }
      prev = err;
    }
    // Y2 = a Y T, Z2 = a T Z
    for (long long x = tid; x < 2 * mm; x += nth) {
      const bool zpart = x >= mm;
      const long long y = zpart ? x - mm : x;
      const int i = (int)(y / m), j = (int)(y % m);
      double acc = 0.0;
      if (!zpart)
        for (int k = 0; k < m; ++k) acc = fma(Y[(long long)i * m + k], T[(long long)k * m + j], acc);
      else
        for (int k = 0; k < m; ++k) acc = fma(T[(long long)i * m + k], Z[(long long)k * m + j], acc);
      (zpart ? Z2 : Y2)[y] = a * acc;
    }
    grid.sync();
    double* tmp = Y;
    Y = Y2;
    Y2 = tmp;
    tmp = Z;
    Z = Z2;
    Z2 = tmp;
    if (scaled) {
      const double xx = a * l;
      l = fmin(1.0, 0.5 * xx * (3.0 - xx * xx));
    }
  }
  if (!conv) {
    if (tid == 0) done[0] = 0;
    return;
  }
  // certificate: slot 63 = largest absolute row sum of Z
  double zr = 0.0;
  for (long long r = tid; r < m; r += nth) {
    double rs = 0.0;
    for (int k = 0; k < m; ++k) rs += fabs(Z[r * m + k]);
    zr = fmax(zr, rs);
  }
  zr = warp_max(zr);
  if (lane == 0) atomicMax(&slots[63], (unsigned long long)__double_as_longlong(zr));
  grid.sync();
  const double rz = __longlong_as_double((long long)slots[63]);
  const bool certified = rz > 0.0 && cnorm / (rz * rz) > 2.0 * t;
  if (certified) {
    const double osc = 0.5 * sqrt(rc);
    for (long long x = tid; x < mm; x += nth) {
      const long long i = x / m, j = x % m;
      out[x] = osc * (Z[x] + Z[j * m + i]);
    }
  }
  if (tid == 0) done[0] = certified ? 1 : 0;
}

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
  if (m < 256) {
    // small orders: norms, iteration and certificate in one cooperative launch
    double* Y = static_cast<double*>(front);
    double* Z = Y + mm;
    double* T = Z + mm;
    double* Y2 = static_cast<double*>(dws);
    double* Z2 = Y2 + mm;
    double* fsum = part + 64;
    int* dflag = reinterpret_cast<int*>(part + 65);
    void* args[] = {(void*)&J,  (void*)&m,  (void*)&tol, (void*)&Y,    (void*)&Z,    (void*)&T,
                    (void*)&Y2, (void*)&Z2, (void*)&out, (void*)&derr, (void*)&fsum, (void*)&dflag};
    CORR_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(ns_small_kernel),
                                          dim3(c->sms), dim3(256), args, 0, s));
    int hd = 0;
    CORR_CUDA(cudaMemcpyAsync(&hd, dflag, sizeof(int), cudaMemcpyDeviceToHost, s));
    CORR_CUDA(cudaStreamSynchronize(s));
    c->launches += 1;
    *done = hd == 1;
    return CORR_OK;
  }
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
    c->launches += 1;
    double err = 0.0;
    if (!scaled) {  // the scaled steps follow the bound l; only the tail reads the error
      unsigned long long he = 0;
      CORR_CUDA(cudaMemcpyAsync(&he, derr, 8, cudaMemcpyDeviceToHost, s));
      CORR_CUDA(cudaStreamSynchronize(s));
      std::memcpy(&err, &he, 8);
      if (!std::isfinite(err)) return CORR_OK;
    }
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
