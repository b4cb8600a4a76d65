// RI metric J^-1/2 (src/POSTHF/ri.cc:50-69) on the GPU in FP64.
//
// The reference diagonalises J with LAPACK dsyev, zeroes every eigenvalue with
// lambda/lambda_max < 1e-10 or lambda < 0, takes lambda^-1/2 of the rest and
// assembles J^-1/2 = V diag V^T with dgemm.  Here the eigendecomposition is a
// parallel cyclic two-sided Jacobi method (Golub & Van Loan, "Matrix
// Computations", symmetric Schur decomposition and parallel Jacobi with
// round-robin ordering): every round rotates n/2 disjoint index pairs at once,
//   tau = (a_qq - a_pp) / (2 a_pq),  t = sign(tau) / (|tau| + sqrt(1 + tau^2)),
//   c = 1/sqrt(1 + t^2),  s = t c,   R = [[c, s], [-s, c]],
//   A <- R^T A R (one 2x2 block per thread, in place),  V <- V R,
// and a sweep is n-1 rounds of the circle pairing (index n-1 fixed, index r
// paired with it, (r+k) mod (n-1) with (r-k) mod (n-1)).  A pair is rotated
// only while |a_pq| > 1e-15 sqrt(|a_pp a_qq|) (the threshold rule of Demmel &
// Veselic, "Jacobi's method is more accurate than QR", 1992), and sweeps repeat
// until one sweep rotates no pair (at most 40).  The cutoff and the assembly
// V f(Lambda) V^T (gemm_fp64.cu) follow the reference.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "gemm_fp64.h"
#include "kernels.h"

namespace corr {

namespace {

__device__ __forceinline__ void round_pair(int n, int r, int k, int* p, int* q) {
  if (k == 0) {
    *p = n - 1;
    *q = r;
  } else {
    *p = (r + k) % (n - 1);
    *q = (r - k + (n - 1)) % (n - 1);
  }
}

constexpr double kRotTol = 1e-15;

__global__ void jacobi_params(const double* __restrict__ A, int n, int r, double2* __restrict__ cs,
                              int* __restrict__ rotated) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n / 2) return;
  int p, q;
  round_pair(n, r, k, &p, &q);
  const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q], apq = A[(size_t)p * n + q];
  double c = 1.0, s = 0.0;
  if (fabs(apq) > kRotTol * sqrt(fabs(app * aqq))) {
    *rotated = 1;
    const double tau = (aqq - app) / (2.0 * apq);
    const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
    c = 1.0 / sqrt(1.0 + t * t);
    s = t * c;
  }
  cs[k] = make_double2(c, s);
}

// Thread (k, l): the 2x2 block rows {p_k, q_k} x cols {p_l, q_l} of A.
// Extra threads (k == n/2 .. ) rotate the columns of V for row x.
__global__ void jacobi_apply(double* __restrict__ A, double* __restrict__ V, int n, int r,
                             const double2* __restrict__ cs) {
  const int h = n / 2;
  const long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long nA = (long long)h * h;
  if (id < nA) {
    const int k = (int)(id / h), l = (int)(id % h);
    int p, q, u, w;
    round_pair(n, r, k, &p, &q);
    round_pair(n, r, l, &u, &w);
    const double2 a = cs[k], b = cs[l];
    double* Ap = A + (size_t)p * n;
    double* Aq = A + (size_t)q * n;
    const double x00 = Ap[u], x01 = Ap[w], x10 = Aq[u], x11 = Aq[w];
    // Y = R_k^T X
    const double y00 = a.x * x00 - a.y * x10, y01 = a.x * x01 - a.y * x11;
    const double y10 = a.y * x00 + a.x * x10, y11 = a.y * x01 + a.x * x11;
    // Z = Y R_l
    Ap[u] = y00 * b.x - y01 * b.y;
    Ap[w] = y00 * b.y + y01 * b.x;
    Aq[u] = y10 * b.x - y11 * b.y;
    Aq[w] = y10 * b.y + y11 * b.x;
  } else if (id < nA + (long long)n * h) {
    const long long j = id - nA;
    const int x = (int)(j / h), l = (int)(j % h);
    int u, w;
    round_pair(n, r, l, &u, &w);
    const double2 b = cs[l];
    double* Vx = V + (size_t)x * n;
    const double vu = Vx[u], vw = Vx[w];
    Vx[u] = b.x * vu - b.y * vw;
    Vx[w] = b.y * vu + b.x * vw;
  }
}

// off = sum_{x != y} A^2, tot = sum A^2 (per block, FP64), then one block sums.
__global__ void frob_kernel(const double* __restrict__ A, int n, double* __restrict__ part) {
  double off = 0.0, tot = 0.0;
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const double a = A[e];
    tot += a * a;
    if (e / n != e % n) off += a * a;
  }
  off = warp_sum(off);
  tot = warp_sum(tot);
  __shared__ double s[2][32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    s[0][w] = off;
    s[1][w] = tot;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      a += s[0][k];
      b += s[1][k];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

// Copy the symmetric m x m matrix J into the padded n x n work matrix from one
// triangle, as dsyev reads it: upper == 1 takes the row-major upper triangle
// (LAPACKE_dsyev(LAPACK_ROW_MAJOR, 'V', 'U'), ri.cc:49), upper == 0 the
// row-major lower one (Fortran dsyev with UPLO = 'U' on a row-major array,
// ops_mat.cc:44).  V = identity.
__global__ void jacobi_init(const double* __restrict__ J, int m, int n, int upper,
                            double* __restrict__ A, double* __restrict__ V) {
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e / n), y = (int)(e % n);
    const int lo = x < y ? x : y, hi = x < y ? y : x;
    A[e] = (x < m && y < m) ? (upper ? J[(size_t)lo * m + hi] : J[(size_t)hi * m + lo]) : 0.0;
    V[e] = (x == y) ? 1.0 : 0.0;
  }
}

// W[x][k] = V[x][k] f(lambda_k) for the m real indices (row stride n).
__global__ void scale_columns(const double* __restrict__ V, const double* __restrict__ f, int m,
                              int n, double* __restrict__ W) {
  const long long mm = (long long)m * m;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < mm;
       e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e / m), k = (int)(e % m);
    W[e] = V[(size_t)x * n + k] * f[k];
  }
}

__global__ void take_diag(const double* __restrict__ A, int n, int m, double* __restrict__ d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x < m) d[x] = A[(size_t)x * n + x];
}

}  // namespace

// Cyclic sweeps on the padded n x n work matrix A (in place -> eigenvalues on
// the diagonal) accumulating the rotations into V (columns = eigenvectors),
// until a sweep rotates no pair (at most 40 sweeps).
static int jacobi_sweeps(corr_context* c, double* A, double* V, double2* cs, int* rotated,
                         int n) {
  cudaStream_t s = c->stream;
  const int h = n / 2;
  const long long napply = (long long)h * h + (long long)n * h;
  const int agrid = (int)((napply + 255) / 256);
  for (int sweeps = 0; sweeps < 40 && n >= 2; ++sweeps) {
    CORR_CUDA(cudaMemsetAsync(rotated, 0, sizeof(int), s));
    for (int r = 0; r < n - 1; ++r) {
      jacobi_params<<<(h + 127) / 128, 128, 0, s>>>(A, n, r, cs, rotated);
      jacobi_apply<<<agrid, 256, 0, s>>>(A, V, n, r, cs);
    }
    CORR_CUDA(cudaGetLastError());
    c->launches += 2LL * (n - 1);
    int hrot = 0;
    CORR_CUDA(cudaMemcpyAsync(&hrot, rotated, sizeof(int), cudaMemcpyDeviceToHost, s));
    CORR_CUDA(cudaStreamSynchronize(s));
    if (!hrot) break;
  }
  return CORR_OK;
}

// vecs[k][x] = V[x][perm[k]] (row k = eigenvector k), w[k] = lam[perm[k]]
__global__ void gather_eigvecs(const double* __restrict__ V, int n, int m,
                               const int* __restrict__ perm, double* __restrict__ vecs) {
  const long long mm = (long long)m * m;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < mm;
       e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e / m), x = (int)(e % m);
    vecs[e] = V[(size_t)x * n + perm[k]];
  }
}

// Symmetric eigendecomposition (the semantics of diag_mat, src/MATH/ops_mat.cc:21-45,
// i.e. LAPACK dsyev with JOBZ='V'): eigenvalues ascending into w, eigenvector k
// as row k of vecs (m x m).  A, w, vecs: device pointers.  Workspace: the
// caller reserved jacobi_workspace_bytes(m) + m * 4 + 256 bytes at ws.
int sym_eig_device(corr_context* c, void* ws, const double* Ain, int m, double* w, double* vecs) {
  const int n = m + (m & 1);
  Carver cw{ws, 0};
  double* A = static_cast<double*>(cw.take((size_t)n * n * 8));
  double* V = static_cast<double*>(cw.take((size_t)n * n * 8));
  (void)cw.take((size_t)n * n * 8);
  double2* cs = static_cast<double2*>(cw.take((size_t)n * 16));
  int* rotated = static_cast<int*>(cw.take((size_t)1024 * 16));
  int* dperm = static_cast<int*>(cw.take((size_t)m * 4));
  cudaStream_t s = c->stream;
  const int ig = (int)std::min<long long>(((long long)n * n + 255) / 256, 4096);
  jacobi_init<<<ig, 256, 0, s>>>(Ain, m, n, 0, A, V);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  CORR_TRY(jacobi_sweeps(c, A, V, cs, rotated, n));
  double* dlam = reinterpret_cast<double*>(cs);  // n doubles of room
  take_diag<<<(m + 255) / 256, 256, 0, s>>>(A, n, m, dlam);
  std::vector<double> lam(m), ws_sorted(m);
  std::vector<int> perm(m);
  CORR_CUDA(cudaMemcpyAsync(lam.data(), dlam, (size_t)m * 8, cudaMemcpyDeviceToHost, s));
  CORR_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < m; ++k) perm[k] = k;
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return lam[a] < lam[b]; });
  for (int k = 0; k < m; ++k) ws_sorted[k] = lam[perm[k]];
  CORR_CUDA(cudaMemcpyAsync(dperm, perm.data(), (size_t)m * 4, cudaMemcpyHostToDevice, s));
  CORR_CUDA(cudaMemcpyAsync(w, ws_sorted.data(), (size_t)m * 8, cudaMemcpyHostToDevice, s));
  const int gg = (int)std::min<long long>(((long long)m * m + 255) / 256, 4096);
  gather_eigvecs<<<gg, 256, 0, s>>>(V, n, m, dperm, vecs);
  CORR_CUDA(cudaGetLastError());
  CORR_CUDA(cudaStreamSynchronize(s));  // the host vectors above are read by the copies
  c->launches += 2;
  return CORR_OK;
}

// Eigen-decomposition + reference cutoff + assembly.  J, out: device pointers
// (m x m).  Workspace carved from c->ws (caller already reserved
// jacobi_workspace_bytes(m)).
size_t jacobi_workspace_bytes(int m) {
  const int n = m + (m & 1);
  return (size_t)3 * n * n * 8 + (size_t)n * 16 + (size_t)4096 * 16 + (size_t)4 * 256 + 64;
}

int ri_inv_sqrt_device(corr_context* c, void* ws, const double* J, int m, double tol,
                       double* out, int* ncut) {
  const int n = m + (m & 1);
  Carver w{ws, 0};
  double* A = static_cast<double*>(w.take((size_t)n * n * 8));
  double* V = static_cast<double*>(w.take((size_t)n * n * 8));
  double* W = static_cast<double*>(w.take((size_t)n * n * 8));
  double2* cs = static_cast<double2*>(w.take((size_t)n * 16));
  const int fgrid = 1024;
  double* part = static_cast<double*>(w.take((size_t)fgrid * 16));
  cudaStream_t s = c->stream;
  const int ig = (int)std::min<long long>(((long long)n * n + 255) / 256, 4096);
  jacobi_init<<<ig, 256, 0, s>>>(J, m, n, 1, A, V);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  std::vector<double> hp((size_t)fgrid * 2);
  frob_kernel<<<fgrid, 256, 0, s>>>(A, n, part);
  CORR_CUDA(cudaMemcpyAsync(hp.data(), part, hp.size() * 8, cudaMemcpyDeviceToHost, s));
  CORR_CUDA(cudaStreamSynchronize(s));
  c->launches += 1;
  double tot = 0;
  for (int k = 0; k < fgrid; ++k) tot += hp[2 * k + 1];
  if (!(tot > 0.0)) {
    set_error("RI metric is zero");
    return CORR_ERR_NOT_PD;
  }
  CORR_TRY(jacobi_sweeps(c, A, V, cs, reinterpret_cast<int*>(part), n));
  // eigenvalues -> reference cutoff (ri.cc:56-66) on the host (m values)
  double* dlam = W;  // reuse W's head as a scratch vector before W is written
  take_diag<<<(m + 255) / 256, 256, 0, s>>>(A, n, m, dlam);
  std::vector<double> lam(m), f(m);
  CORR_CUDA(cudaMemcpyAsync(lam.data(), dlam, (size_t)m * 8, cudaMemcpyDeviceToHost, s));
  CORR_CUDA(cudaStreamSynchronize(s));
  double mx = lam[0];
  for (int k = 1; k < m; ++k) mx = std::max(mx, lam[k]);
  if (!(mx > 0.0)) {
    set_error("RI metric has no positive eigenvalue");
    return CORR_ERR_NOT_PD;
  }
  int cut = 0;
  for (int k = 0; k < m; ++k) {
    if (lam[k] / mx < tol || lam[k] < 0) {
      f[k] = 0.0;
      ++cut;
    } else {
      f[k] = 1.0 / std::sqrt(lam[k]);
    }
  }
  if (ncut) *ncut = cut;
  double* df = reinterpret_cast<double*>(cs);  // n >= m doubles of room (n*16 bytes)
  CORR_CUDA(cudaMemcpyAsync(df, f.data(), (size_t)m * 8, cudaMemcpyHostToDevice, s));
  scale_columns<<<ig, 256, 0, s>>>(V, df, m, n, W);
  CORR_CUDA(cudaGetLastError());
  // J^-1/2 = W V^T restricted to the m real rows/cols (V row stride n)
  GemmF64 g = gemm_args(W, V, out, m, m, m, m, n, m, 0, 1);
  CORR_TRY(gemm_f64(g, &c->dres->status, s));
  c->launches += 3;
  return CORR_OK;
}

}  // namespace corr
