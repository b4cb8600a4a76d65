// The reference's dense FP64 helpers on the GPU (src/MATH/ops_mat.cc): a
// general row-major GEMM (mat_mat_T, mat_T_mat, transform_MOs,
// symmortho_mat and pmv are special cases) and the symmetric
// eigendecomposition with diag_mat's output convention.  Host or device
// pointers, as every entry point of the library.
#include "abi_internal.h"
#include "common.cuh"
#include "dgemm_tc.h"
#include "gemm_fp64.h"
#include "kernels.h"

namespace corr {
size_t jacobi_workspace_bytes(int m);
int sym_eig_device(corr_context* c, void* ws, const double* Ain, int m, double* w, double* vecs);

namespace {
__global__ void scale_rows_kernel(double* __restrict__ C, int m, int n, long long ldc, double b) {
  const long long mn = (long long)m * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < mn;
       e += (long long)gridDim.x * blockDim.x)
    C[(e / n) * ldc + e % n] *= b;
}
}  // namespace
}  // namespace corr

using namespace corr;

extern "C" {

int corr_dgemm(corr_context* c, int transa, int transb, int m, int n, int k, double alpha,
               const double* A, int lda, const double* B, int ldb, double beta, double* C,
               int ldc) {
  CORR_CHECK_ARG(c && A && B && C, "corr_dgemm: null argument");
  CORR_CHECK_ARG(m >= 1 && n >= 1 && k >= 1, "corr_dgemm: m, n, k must be positive");
  CORR_CHECK_ARG((transa == 0 || transa == 1) && (transb == 0 || transb == 1),
                 "corr_dgemm: transa/transb must be 0 or 1");
  // stored shapes (rows x cols, row-major): A is m x k or, transposed, k x m
  const int ar = transa ? k : m, ac = transa ? m : k;
  const int br = transb ? n : k, bc = transb ? k : n;
  CORR_CHECK_ARG(lda >= ac && ldb >= bc && ldc >= n, "corr_dgemm: leading dimension too small");
  CORR_CUDA(cudaSetDevice(c->device));
  // Host operands are packed on the device (ld = cols) with 2-D copies, so
  // only the addressed elements of the caller's arrays are read or written.
  const bool adev = is_device_ptr(A), bdev = is_device_ptr(B), cdev = is_device_ptr(C);
  const size_t na = (size_t)ar * ac, nb = (size_t)br * bc, nc = (size_t)m * n;
  Carver cv{nullptr, 0};
  if (!adev) cv.take(na * 8);
  if (!bdev) cv.take(nb * 8);
  if (!cdev) cv.take(nc * 8);
  CORR_TRY(c->ws.reserve(cv.used + 256));
  Carver w{c->ws.ptr, 0};
  double* da = adev ? const_cast<double*>(A) : static_cast<double*>(w.take(na * 8));
  double* db = bdev ? const_cast<double*>(B) : static_cast<double*>(w.take(nb * 8));
  double* dc = cdev ? C : static_cast<double*>(w.take(nc * 8));
  const long long la = adev ? lda : ac, lb = bdev ? ldb : bc, lc = cdev ? ldc : n;
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  if (!adev)
    CORR_CUDA(cudaMemcpy2DAsync(da, (size_t)ac * 8, A, (size_t)lda * 8, (size_t)ac * 8, ar,
                                cudaMemcpyHostToDevice, c->stream));
  if (!bdev)
    CORR_CUDA(cudaMemcpy2DAsync(db, (size_t)bc * 8, B, (size_t)ldb * 8, (size_t)bc * 8, br,
                                cudaMemcpyHostToDevice, c->stream));
  if (!cdev && beta != 0.0)
    CORR_CUDA(cudaMemcpy2DAsync(dc, (size_t)n * 8, C, (size_t)ldc * 8, (size_t)n * 8, m,
                                cudaMemcpyHostToDevice, c->stream));
  mark(c, 1);
  GemmF64 g = gemm_args(da, db, dc, m, n, k, la, lb, lc, transa, transb);
  g.alpha = alpha;
  g.beta = beta;
  CORR_TRY(gemm_f64(g, &c->dres->status, c->stream));
  c->launches += 1;
  mark(c, 2);
  if (!cdev)
    CORR_CUDA(cudaMemcpy2DAsync(C, (size_t)ldc * 8, dc, (size_t)n * 8, (size_t)n * 8, m,
                                cudaMemcpyDeviceToHost, c->stream));
  return finish_results(c, 0);
}

int corr_dgemm_tc(corr_context* c, int transa, int transb, int m, int n, int k, double alpha,
                  const double* A, int lda, const double* B, int ldb, double beta, double* C,
                  int ldc) {
  CORR_CHECK_ARG(c && A && B && C, "corr_dgemm_tc: null argument");
  CORR_CHECK_ARG(m >= 1 && n >= 1 && k >= 1, "corr_dgemm_tc: m, n, k must be positive");
  CORR_CHECK_ARG((transa == 0 || transa == 1) && (transb == 0 || transb == 1),
                 "corr_dgemm_tc: transa/transb must be 0 or 1");
  const int ar = transa ? k : m, ac = transa ? m : k;
  const int br = transb ? n : k, bc = transb ? k : n;
  CORR_CHECK_ARG(lda >= ac && ldb >= bc && ldc >= n, "corr_dgemm_tc: leading dimension too small");
  CORR_CUDA(cudaSetDevice(c->device));
  const bool adev = is_device_ptr(A), bdev = is_device_ptr(B), cdev = is_device_ptr(C);
  const size_t na = (size_t)ar * ac, nb = (size_t)br * bc, nc = (size_t)m * n;
  auto plan = [&](Carver& w, double** da, double** db, double** dc, void** ws) {
    *da = adev ? const_cast<double*>(A) : static_cast<double*>(w.take(na * 8));
    *db = bdev ? const_cast<double*>(B) : static_cast<double*>(w.take(nb * 8));
    *dc = cdev ? C : static_cast<double*>(w.take(nc * 8));
    *ws = w.take(dgemm_tc_workspace(m, n, k));
  };
  double *da, *db, *dc;
  void* ws;
  Carver cv{nullptr, 0};
  plan(cv, &da, &db, &dc, &ws);
  CORR_TRY(c->ws.reserve(cv.used + 256));
  Carver w{c->ws.ptr, 0};
  plan(w, &da, &db, &dc, &ws);
  const long long la = adev ? lda : ac, lb = bdev ? ldb : bc, lc = cdev ? ldc : n;
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  if (!adev)
    CORR_CUDA(cudaMemcpy2DAsync(da, (size_t)ac * 8, A, (size_t)lda * 8, (size_t)ac * 8, ar,
                                cudaMemcpyHostToDevice, c->stream));
  if (!bdev)
    CORR_CUDA(cudaMemcpy2DAsync(db, (size_t)bc * 8, B, (size_t)ldb * 8, (size_t)bc * 8, br,
                                cudaMemcpyHostToDevice, c->stream));
  if (!cdev && beta != 0.0)
    CORR_CUDA(cudaMemcpy2DAsync(dc, (size_t)n * 8, C, (size_t)ldc * 8, (size_t)n * 8, m,
                                cudaMemcpyHostToDevice, c->stream));
  mark(c, 1);
  if (beta != 0.0 && beta != 1.0) {
    scale_rows_kernel<<<std::min((int)((nc + 255) / 256), c->sms * 8), 256, 0, c->stream>>>(
        dc, m, n, lc, beta);
    CORR_CUDA(cudaGetLastError());
    c->launches += 1;
  }
  // op(A) as m rows over k; op(B)^T as n rows over k
  DgemmTc g;
  g.A = transa ? mat_view(da, 1, la) : mat_view(da, la, 1);
  g.B = transb ? mat_view(db, lb, 1) : mat_view(db, 1, lb);
  g.C = out_view(dc, lc, 1);
  g.M = m;
  g.N = n;
  g.K = k;
  g.alpha = alpha;
  g.accumulate = beta != 0.0;
  g.a_lower = false;
  CORR_TRY(dgemm_tc(c, g, ws));
  mark(c, 2);
  if (!cdev)
    CORR_CUDA(cudaMemcpy2DAsync(C, (size_t)ldc * 8, dc, (size_t)n * 8, (size_t)n * 8, m,
                                cudaMemcpyDeviceToHost, c->stream));
  return finish_results(c, 0);
}

int corr_syev(corr_context* c, int n, const double* A, double* w, double* vecs) {
  CORR_CHECK_ARG(c && A && w && vecs, "corr_syev: null argument");
  CORR_CHECK_ARG(n >= 1 && n <= 32768, "corr_syev: n must be in [1, 32768]");
  CORR_CUDA(cudaSetDevice(c->device));
  const size_t n2 = (size_t)n * n;
  const bool adev = is_device_ptr(A), wdev = is_device_ptr(w), vdev = is_device_ptr(vecs);
  auto plan = [&](Carver& cw, void** sa, double** dw, double** dv, void** ws) {
    *sa = adev ? nullptr : cw.take(n2 * 8);
    *dw = wdev ? w : static_cast<double*>(cw.take((size_t)n * 8));
    *dv = vdev ? vecs : static_cast<double*>(cw.take(n2 * 8));
    *ws = cw.take(jacobi_workspace_bytes(n) + (size_t)n * 4 + 256);
  };
  void *sa, *ws;
  double *dw, *dv;
  Carver cv{nullptr, 0};
  plan(cv, &sa, &dw, &dv, &ws);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver cw{c->ws.ptr, 0};
  plan(cw, &sa, &dw, &dv, &ws);
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* da = static_cast<const double*>(stage_in(c, A, n2 * 8, sa));
  CORR_CHECK_ARG(da, "corr_syev: host-to-device copy failed");
  mark(c, 1);
  CORR_TRY(sym_eig_device(c, ws, da, n, dw, dv));
  mark(c, 2);
  CORR_TRY(stage_out(c, w, dw, (size_t)n * 8));
  CORR_TRY(stage_out(c, vecs, dv, n2 * 8));
  return finish_results(c, 0);
}

}  // extern "C"
