// C-ABI entry points of the FP64 transforms and the canonical MP2 energy.
#include "abi_internal.h"
#include "common.cuh"
#include "dgemm_tc.h"
#include "gemm_fp64.h"
#include "kernels.h"

namespace corr {
int quarter(corr_context* c, const double* in, const double* mos, int N, int crow, int nout,
            long long M, double* out);
int launch_unpack(corr_context* c, int N, long long n, const long long* sc, const double* val,
                  const unsigned short* num, double* eri);
int launch_canonical(corr_context* c, const double* t, int full, int N, int o, int v,
                     const double* eps, double* part, int grid);
int canonical_grid(corr_context* c, long long total);

namespace {

// Stage the packed ERI list and the MO coefficients, then build (ia|jb) or the
// full MO tensor into `dst` (device).
int motrans_device(corr_context* c, Carver& w, int nroe, int N, const double* mos,
                   long long nint, const long long* sortcount, const double* intval,
                   const unsigned short* intnums, bool full, double* dst) {
  const int o = nroe / 2, v = N - o;
  const size_t n4 = (size_t)N * N * N * N;
  void* s_mos = w.take((size_t)N * N * 8);
  void* s_sc = w.take(4 * 8);
  void* s_val = w.take((size_t)(nint > 0 ? nint : 1) * 8);
  void* s_num = w.take((size_t)(nint > 0 ? nint : 1) * 8);
  double* t0 = static_cast<double*>(w.take(n4 * 8));
  double* t1 = static_cast<double*>(w.take(n4 * 8));
  const double* d_mos = static_cast<const double*>(stage_in(c, mos, (size_t)N * N * 8, s_mos));
  const long long* d_sc = static_cast<const long long*>(stage_in(c, sortcount, 32, s_sc));
  const double* d_val = nint > 0 ? static_cast<const double*>(stage_in(c, intval, nint * 8, s_val))
                                 : static_cast<const double*>(s_val);
  const unsigned short* d_num =
      nint > 0 ? static_cast<const unsigned short*>(stage_in(c, intnums, nint * 8, s_num))
               : static_cast<const unsigned short*>(s_num);
  if (!d_mos || !d_sc || !d_val || !d_num) {
    set_error("host-to-device copy failed");
    return CORR_ERR_CUDA;
  }
  CORR_TRY(launch_unpack(c, N, nint, d_sc, d_val, d_num, t0));
  const long long N3 = (long long)N * N * N;
  mark(c, 1);
  if (full) {
    CORR_TRY(quarter(c, t0, d_mos, N, 0, N, N3, t1));
    CORR_TRY(quarter(c, t1, d_mos, N, 0, N, N3, t0));
    CORR_TRY(quarter(c, t0, d_mos, N, 0, N, N3, t1));
    CORR_TRY(quarter(c, t1, d_mos, N, 0, N, N3, dst));
  } else {
    CORR_TRY(quarter(c, t0, d_mos, N, 0, o, N3, t1));                          // [bcd][i]
    CORR_TRY(quarter(c, t1, d_mos, N, o, v, (long long)N * N * o, t0));       // [cdi][a]
    CORR_TRY(quarter(c, t0, d_mos, N, 0, o, (long long)N * o * v, t1));       // [dia][j]
    CORR_TRY(quarter(c, t1, d_mos, N, o, v, (long long)o * v * o, dst));      // [iaj][b]
  }
  mark(c, 2);
  c->launches += 4;
  return CORR_OK;
}

int check_packed(int nroe, int N, long long nint, const double* mos, const long long* sc,
                 const double* val, const unsigned short* num) {
  CORR_CHECK_ARG(N >= 1 && N <= 65535, "nroao must be in [1, 65535] (uint16 indices), got %d", N);
  CORR_CHECK_ARG(nroe >= 2 && nroe % 2 == 0 && nroe / 2 < N,
                 "nroe must be even with 0 < nroe/2 < nroao (nroe=%d, nroao=%d)", nroe, N);
  CORR_CHECK_ARG(nint >= 0, "nrofint must be >= 0");
  CORR_CHECK_ARG(mos && sc && (nint == 0 || (val && num)), "null pointer argument");
  CORR_CHECK_ARG((double)N * N * N * N * 8 * 3 < 2.5e11, "nroao=%d: N^4 tensor too large", N);
  return CORR_OK;
}

}  // namespace
}  // namespace corr

using namespace corr;

extern "C" {

int corr_build_fmo(corr_context* c, int nroao, const double* mos, const double* fmat,
                   double* fmo) {
  CORR_CHECK_ARG(c && mos && fmat && fmo, "corr_build_fmo: null argument");
  CORR_CHECK_ARG(nroao >= 1, "corr_build_fmo: nroao must be positive");
  CORR_CUDA(cudaSetDevice(c->device));
  const int N = nroao;
  const size_t n2 = (size_t)N * N;
  const bool odev = is_device_ptr(fmo);
  Carver cv{nullptr, 0};
  for (int k = 0; k < 4; ++k) cv.take(n2 * 8);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_m = w.take(n2 * 8);
  void* s_f = w.take(n2 * 8);
  double* T = static_cast<double*>(w.take(n2 * 8));
  double* out = odev ? fmo : static_cast<double*>(w.take(n2 * 8));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_m = static_cast<const double*>(stage_in(c, mos, n2 * 8, s_m));
  const double* d_f = static_cast<const double*>(stage_in(c, fmat, n2 * 8, s_f));
  CORR_CHECK_ARG(d_m && d_f, "corr_build_fmo: host-to-device copy failed");
  mark(c, 1);
  // T = C F ; FMo = T C^T   (FMo[i][j] = sum C[i][mu] F[mu][nu] C[j][nu])
  CORR_TRY(gemm_f64(gemm_args(d_m, d_f, T, N, N, N, N, N, N, 0, 0), &c->dres->status, c->stream));
  CORR_TRY(gemm_f64(gemm_args(T, d_m, out, N, N, N, N, N, N, 0, 1), &c->dres->status, c->stream));
  c->launches += 2;
  mark(c, 2);
  CORR_TRY(stage_out(c, fmo, out, n2 * 8));
  return finish_results(c, 0);
}

int corr_motrans(corr_context* c, int nroe, int nroao, const double* mos, long long nrofint,
                 const long long* sortcount, const double* intval, const unsigned short* intnums,
                 double* prec) {
  CORR_CHECK_ARG(c && prec, "corr_motrans: null argument");
  CORR_TRY(check_packed(nroe, nroao, nrofint, mos, sortcount, intval, intnums));
  CORR_CUDA(cudaSetDevice(c->device));
  const int N = nroao;
  const size_t n4 = (size_t)N * N * N * N;
  const bool odev = is_device_ptr(prec);
  auto plan = [&](Carver& w, double** out) {
    w.take((size_t)N * N * 8);
    w.take(32);
    w.take((size_t)(nrofint > 0 ? nrofint : 1) * 8);
    w.take((size_t)(nrofint > 0 ? nrofint : 1) * 8);
    w.take(n4 * 8);
    w.take(n4 * 8);
    *out = odev ? prec : static_cast<double*>(w.take(n4 * 8));
  };
  double* out;
  Carver cv{nullptr, 0};
  plan(cv, &out);
  CORR_TRY(c->ws.reserve(cv.used));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  Carver w{c->ws.ptr, 0};
  // the same carving order as plan(): staging buffers first, output last
  Carver w2 = w;
  plan(w2, &out);
  CORR_TRY(motrans_device(c, w, nroe, N, mos, nrofint, sortcount, intval, intnums, true, out));
  CORR_TRY(stage_out(c, prec, out, n4 * 8));
  return finish_results(c, 0);
}

int corr_motrans_ovov(corr_context* c, int nroe, int nroao, const double* mos, long long nrofint,
                      const long long* sortcount, const double* intval,
                      const unsigned short* intnums, double* ovov) {
  CORR_CHECK_ARG(c && ovov, "corr_motrans_ovov: null argument");
  CORR_TRY(check_packed(nroe, nroao, nrofint, mos, sortcount, intval, intnums));
  CORR_CUDA(cudaSetDevice(c->device));
  const int N = nroao, o = nroe / 2, v = N - o;
  const size_t n4 = (size_t)N * N * N * N, nov = (size_t)o * v * o * v;
  const bool odev = is_device_ptr(ovov);
  Carver cv{nullptr, 0};
  cv.take((size_t)N * N * 8);
  cv.take(32);
  cv.take((size_t)(nrofint > 0 ? nrofint : 1) * 8);
  cv.take((size_t)(nrofint > 0 ? nrofint : 1) * 8);
  cv.take(n4 * 8);
  cv.take(n4 * 8);
  if (!odev) cv.take(nov * 8);
  CORR_TRY(c->ws.reserve(cv.used));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  Carver w{c->ws.ptr, 0};
  Carver wo = w;
  double* out = ovov;
  if (!odev) {
    // output staging lives after the motrans buffers
    wo.take((size_t)N * N * 8);
    wo.take(32);
    wo.take((size_t)(nrofint > 0 ? nrofint : 1) * 8);
    wo.take((size_t)(nrofint > 0 ? nrofint : 1) * 8);
    wo.take(n4 * 8);
    wo.take(n4 * 8);
    out = static_cast<double*>(wo.take(nov * 8));
  }
  CORR_TRY(motrans_device(c, w, nroe, N, mos, nrofint, sortcount, intval, intnums, false, out));
  CORR_TRY(stage_out(c, ovov, out, nov * 8));
  return finish_results(c, 0);
}

static int canonical_common(corr_context* c, const double* t, int full, int N, int o, int v,
                            const double* eps, corr_mp2_energy* out) {
  CORR_CUDA(cudaSetDevice(c->device));
  const size_t nt = full ? (size_t)N * N * N * N : (size_t)o * v * o * v;
  const bool tdev = is_device_ptr(t), edev = is_device_ptr(eps);
  const int grid = canonical_grid(c, (long long)o * o * v * v);
  Carver cv{nullptr, 0};
  if (!tdev) cv.take(nt * 8);
  if (!edev) cv.take((size_t)(o + v) * 8);
  cv.take((size_t)grid * 16);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_t = tdev ? nullptr : w.take(nt * 8);
  void* s_e = edev ? nullptr : w.take((size_t)(o + v) * 8);
  double* part = static_cast<double*>(w.take((size_t)grid * 16));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_t = static_cast<const double*>(stage_in(c, t, nt * 8, s_t));
  const double* d_e = static_cast<const double*>(stage_in(c, eps, (size_t)(o + v) * 8, s_e));
  CORR_CHECK_ARG(d_t && d_e, "host-to-device copy failed");
  mark(c, 1);
  CORR_TRY(launch_canonical(c, d_t, full, N, o, v, d_e, part, grid));
  mark(c, 2);
  CORR_TRY(finish_results(c, 4));
  out->e_ss = c->hres->e[0];
  out->e_os = c->hres->e[1];
  out->e_total = c->hres->e[2];
  out->e_scs = c->hres->e[3];
  return CORR_OK;
}

int corr_canonical_mp2(corr_context* c, int nroe, int nroao, const double* prec,
                       const double* eps, corr_mp2_energy* out) {
  CORR_CHECK_ARG(c && prec && eps && out, "corr_canonical_mp2: null argument");
  CORR_CHECK_ARG(nroao >= 1 && nroe >= 2 && nroe % 2 == 0 && nroe / 2 < nroao,
                 "corr_canonical_mp2: need even nroe with 0 < nroe/2 < nroao");
  return canonical_common(c, prec, 1, nroao, nroe / 2, nroao - nroe / 2, eps, out);
}

int corr_canonical_mp2_ovov(corr_context* c, int nocc, int nvir, const double* ovov,
                            const double* eps, corr_mp2_energy* out) {
  CORR_CHECK_ARG(c && ovov && eps && out, "corr_canonical_mp2_ovov: null argument");
  CORR_CHECK_ARG(nocc >= 1 && nvir >= 1, "corr_canonical_mp2_ovov: sizes must be positive");
  return canonical_common(c, ovov, 0, nocc + nvir, nocc, nvir, eps, out);
}

int corr_transform_ri(corr_context* c, int nroe, int nroao, int naux, const double* mos,
                      const double* bpq, double* bia) {
  CORR_CHECK_ARG(c && mos && bpq && bia, "corr_transform_ri: null argument");
  CORR_CHECK_ARG(nroao >= 1 && naux >= 1 && nroe >= 2 && nroe % 2 == 0 && nroe / 2 < nroao,
                 "corr_transform_ri: need naux >= 1 and even nroe with 0 < nroe/2 < nroao");
  CORR_CHECK_ARG(naux <= 65535, "corr_transform_ri: naux > 65535");
  CORR_CUDA(cudaSetDevice(c->device));
  const int N = nroao, o = nroe / 2, v = N - o, X = naux;
  const size_t nb = (size_t)X * N * N, nbia = (size_t)X * o * v, nbiq = (size_t)X * o * N;
  const bool mdev = is_device_ptr(mos), bdev = is_device_ptr(bpq), odev = is_device_ptr(bia);
  Carver cv{nullptr, 0};
  if (!mdev) cv.take((size_t)N * N * 8);
  if (!bdev) cv.take(nb * 8);
  cv.take(nbiq * 8);
  if (!odev) cv.take(nbia * 8);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_m = mdev ? nullptr : w.take((size_t)N * N * 8);
  void* s_b = bdev ? nullptr : w.take(nb * 8);
  double* biq = static_cast<double*>(w.take(nbiq * 8));
  double* out = odev ? bia : static_cast<double*>(w.take(nbia * 8));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_m = static_cast<const double*>(stage_in(c, mos, (size_t)N * N * 8, s_m));
  const double* d_b = static_cast<const double*>(stage_in(c, bpq, nb * 8, s_b));
  CORR_CHECK_ARG(d_m && d_b, "host-to-device copy failed");
  mark(c, 1);
  // BiQ[Q][i][nu] = sum_mu C[i][mu] BPQ[Q][mu][nu]     (batched over Q)
  GemmF64 g1 = gemm_args(d_m, d_b, biq, o, N, N, N, N, N, 0, 0);
  g1.sa = 0;
  g1.sb = (long long)N * N;
  g1.sc = (long long)o * N;
  g1.batch = X;
  CORR_TRY(gemm_f64(g1, &c->dres->status, c->stream));
  // Bia[(Q,i)][a] = sum_nu BiQ[(Q,i)][nu] C[o+a][nu]
  CORR_TRY(gemm_f64(gemm_args(biq, d_m + (size_t)o * N, out, X * o, v, N, N, N, v, 0, 1),
                    &c->dres->status, c->stream));
  c->launches += 2;
  mark(c, 2);
  CORR_TRY(stage_out(c, bia, out, nbia * 8));
  return finish_results(c, 0);
}

int corr_ri_build_bpq(corr_context* c, int naux, int nroao, const double* jm12,
                      const double* pmn, double* bpq) {
  CORR_CHECK_ARG(c && jm12 && pmn && bpq, "corr_ri_build_bpq: null argument");
  CORR_CHECK_ARG(naux >= 1 && nroao >= 1, "corr_ri_build_bpq: sizes must be positive");
  CORR_CUDA(cudaSetDevice(c->device));
  const int X = naux;
  const long long N2 = (long long)nroao * nroao;
  CORR_CHECK_ARG(N2 <= 0x7fffffffLL, "corr_ri_build_bpq: nroao^2 too large");
  const size_t np = (size_t)X * N2, nj = (size_t)X * X;
  const bool jdev = is_device_ptr(jm12), pdev = is_device_ptr(pmn), odev = is_device_ptr(bpq);
  Carver cv{nullptr, 0};
  if (!jdev) cv.take(nj * 8);
  if (!pdev) cv.take(np * 8);
  if (!odev) cv.take(np * 8);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_j = jdev ? nullptr : w.take(nj * 8);
  void* s_p = pdev ? nullptr : w.take(np * 8);
  double* out = odev ? bpq : static_cast<double*>(w.take(np * 8));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_j = static_cast<const double*>(stage_in(c, jm12, nj * 8, s_j));
  const double* d_p = static_cast<const double*>(stage_in(c, pmn, np * 8, s_p));
  CORR_CHECK_ARG(d_j && d_p, "host-to-device copy failed");
  mark(c, 1);
  CORR_TRY(gemm_f64(gemm_args(d_j, d_p, out, X, (int)N2, X, X, N2, N2, 0, 0), &c->dres->status,
                    c->stream));
  c->launches += 1;
  mark(c, 2);
  CORR_TRY(stage_out(c, bpq, out, np * 8));
  return finish_results(c, 0);
}

}  // extern "C"

namespace corr {
size_t jacobi_workspace_bytes(int m);
size_t chol_workspace_bytes(int m);
int chol_norm_inf(corr_context* c, void* scratch, const double* J, int m, double* out);
// A side stream forked from and joined back into a stream (events), and a
// scoped switch of the context's stream (restored on every exit path).
struct SideStream {
  cudaStream_t st = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int fork(cudaStream_t from) {
    CORR_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    for (cudaEvent_t& e : ev) CORR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CORR_CUDA(cudaEventRecord(ev[0], from));
    CORR_CUDA(cudaStreamWaitEvent(st, ev[0], 0));
    return CORR_OK;
  }
  int join(cudaStream_t into) {
    CORR_CUDA(cudaEventRecord(ev[1], st));
    CORR_CUDA(cudaStreamWaitEvent(into, ev[1], 0));
    return CORR_OK;
  }
  ~SideStream() {
    if (st) cudaStreamDestroy(st);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
};
struct StreamSwap {
  corr_context* c;
  cudaStream_t saved;
  StreamSwap(corr_context* ctx, cudaStream_t s) : c(ctx), saved(ctx->stream) { c->stream = s; }
  ~StreamSwap() { c->stream = saved; }
};

int chol_factor_device(corr_context* c, void* ws, const double* J, int m, double shift,
                       double** Lm_out, double** Linv_out, bool* ok, void* tc_ws);
int chol_inverse_device(corr_context* c, const double* Lm, const double* Linv, int m, double* X,
                        double* T, void* tc_ws);
int chol_norm_one_inf(corr_context* c, void* scratch, const double* X, int m, double* out);
int chol_solve_device(corr_context* c, const double* Lm, const double* Linv, int m, double* P,
                      long long ncols, double* out);
int ri_inv_sqrt_device(corr_context* c, void* ws, const double* J, int m, double tol,
                       double* out, int* ncut, bool try_ns);
}  // namespace corr

extern "C" {

int corr_ri_metric_inv_sqrt(corr_context* c, int naux, const double* J, double tol, double* jm12,
                            int* ncut) {
  CORR_CHECK_ARG(c && J && jm12, "corr_ri_metric_inv_sqrt: null argument");
  CORR_CHECK_ARG(naux >= 1 && naux <= 32768, "corr_ri_metric_inv_sqrt: naux must be in [1, 32768]");
  CORR_CHECK_ARG(tol >= 0.0, "corr_ri_metric_inv_sqrt: tol must be >= 0");
  CORR_CUDA(cudaSetDevice(c->device));
  const size_t nj = (size_t)naux * naux;
  const bool jdev = is_device_ptr(J), odev = is_device_ptr(jm12);
  Carver cv{nullptr, 0};
  if (!jdev) cv.take(nj * 8);
  if (!odev) cv.take(nj * 8);
  cv.take(jacobi_workspace_bytes(naux));
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_j = jdev ? nullptr : w.take(nj * 8);
  double* out = odev ? jm12 : static_cast<double*>(w.take(nj * 8));
  void* jws = w.take(jacobi_workspace_bytes(naux));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_j = static_cast<const double*>(stage_in(c, J, nj * 8, s_j));
  CORR_CHECK_ARG(d_j, "host-to-device copy failed");
  mark(c, 1);
  CORR_TRY(ri_inv_sqrt_device(c, jws, d_j, naux, tol, out, ncut, !c->fp64_strict));
  mark(c, 2);
  CORR_TRY(stage_out(c, jm12, out, nj * 8));
  return finish_results(c, 0);
}

int corr_calculate_ri(corr_context* c, int naux, int nroao, const double* J, const double* pmn,
                      double* bpq) {
  CORR_CHECK_ARG(c && J && pmn && bpq, "corr_calculate_ri: null argument");
  CORR_CHECK_ARG(naux >= 1 && naux <= 32768 && nroao >= 1, "corr_calculate_ri: bad sizes");
  CORR_CUDA(cudaSetDevice(c->device));
  const long long N2 = (long long)nroao * nroao;
  CORR_CHECK_ARG(N2 <= 0x7fffffffLL, "corr_calculate_ri: nroao^2 too large");
  const size_t nj = (size_t)naux * naux, np = (size_t)naux * N2;
  const bool jdev = is_device_ptr(J), pdev = is_device_ptr(pmn), odev = is_device_ptr(bpq);
  Carver cv{nullptr, 0};
  if (!jdev) cv.take(nj * 8);
  if (!pdev) cv.take(np * 8);
  if (!odev) cv.take(np * 8);
  cv.take(nj * 8);
  const size_t jwb = std::max(jacobi_workspace_bytes(naux),
                              dgemm_tc_workspace(naux, (int)N2, naux));
  cv.take(jwb);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_j = jdev ? nullptr : w.take(nj * 8);
  void* s_p = pdev ? nullptr : w.take(np * 8);
  double* out = odev ? bpq : static_cast<double*>(w.take(np * 8));
  double* jm = static_cast<double*>(w.take(nj * 8));
  void* jws = w.take(jwb);
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_j = static_cast<const double*>(stage_in(c, J, nj * 8, s_j));
  const double* d_p = static_cast<const double*>(stage_in(c, pmn, np * 8, s_p));
  CORR_CHECK_ARG(d_j && d_p, "host-to-device copy failed");
  mark(c, 1);
  // ri.cc:50-69: J^-1/2 with the 1e-10 relative eigenvalue cutoff
  CORR_TRY(ri_inv_sqrt_device(c, jws, d_j, naux, 1e-10, jm, nullptr, !c->fp64_strict));
  // ri.cc:102-103: BPQ = J^-1/2 (Q|mn), on the FP64-accurate digit GEMM
  // (rows P of J^-1/2 against the columns mn of (Q|mn) read as rows over Q),
  // or on the FP64 pipe when the context asks for strict FP64
  if (c->fp64_strict) {
    CORR_TRY(gemm_f64(gemm_args(jm, d_p, out, naux, (int)N2, naux, naux, N2, N2, 0, 0),
                      &c->dres->status, c->stream));
    c->launches += 1;
    mark(c, 2);
    CORR_TRY(stage_out(c, bpq, out, np * 8));
    return finish_results(c, 0);
  }
  DgemmTc g;
  g.A = mat_view(jm, naux, 1);
  g.B = mat_view(d_p, 1, N2);
  g.C = out_view(out, N2, 1);
  g.M = naux;
  g.N = (int)N2;
  g.K = naux;
  g.alpha = 1.0;
  g.accumulate = false;
  g.a_lower = false;
  CORR_TRY(dgemm_tc(c, g, jws));
  mark(c, 2);
  CORR_TRY(stage_out(c, bpq, out, np * 8));
  return finish_results(c, 0);
}

}  // extern "C"

extern "C" {

int corr_ri_apply_metric(corr_context* c, int naux, long long ncols, const double* jm12,
                         const double* in, double* out) {
  CORR_CHECK_ARG(c && jm12 && in && out, "corr_ri_apply_metric: null argument");
  CORR_CHECK_ARG(naux >= 1 && ncols >= 1 && ncols <= 0x7fffffffLL,
                 "corr_ri_apply_metric: bad sizes");
  CORR_CUDA(cudaSetDevice(c->device));
  const size_t nj = (size_t)naux * naux, nx = (size_t)naux * ncols;
  const bool jdev = is_device_ptr(jm12), idev = is_device_ptr(in), odev = is_device_ptr(out);
  Carver cv{nullptr, 0};
  if (!jdev) cv.take(nj * 8);
  if (!idev) cv.take(nx * 8);
  if (!odev) cv.take(nx * 8);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_j = jdev ? nullptr : w.take(nj * 8);
  void* s_i = idev ? nullptr : w.take(nx * 8);
  double* o = odev ? out : static_cast<double*>(w.take(nx * 8));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_j = static_cast<const double*>(stage_in(c, jm12, nj * 8, s_j));
  const double* d_i = static_cast<const double*>(stage_in(c, in, nx * 8, s_i));
  CORR_CHECK_ARG(d_j && d_i, "host-to-device copy failed");
  mark(c, 1);
  CORR_TRY(gemm_f64(gemm_args(d_j, d_i, o, naux, (int)ncols, naux, naux, ncols, ncols, 0, 0),
                    &c->dres->status, c->stream));
  c->launches += 1;
  mark(c, 2);
  CORR_TRY(stage_out(c, out, o, nx * 8));
  return finish_results(c, 0);
}

int corr_rimp2_energy_from_3index(corr_context* c, int nroe, int nroao, int naux,
                                  const double* mos, const double* eps, const double* J,
                                  const double* pmn, int precision, corr_mp2_energy* out,
                                  int* ncut) {
  CORR_CHECK_ARG(c && mos && eps && J && pmn && out, "corr_rimp2_energy_from_3index: null argument");
  CORR_CHECK_ARG(nroao >= 1 && naux >= 1 && naux <= 32768 && nroe >= 2 && nroe % 2 == 0 &&
                     nroe / 2 < nroao,
                 "corr_rimp2_energy_from_3index: bad sizes");
  CORR_CHECK_ARG(precision >= CORR_PREC_FP64 && precision <= CORR_PREC_SPLIT_BF16,
                 "corr_rimp2_energy_from_3index: unknown precision %d", precision);
  CORR_CUDA(cudaSetDevice(c->device));
  const int N = nroao, o = nroe / 2, v = N - o, X = naux;
  const size_t np = (size_t)X * N * N, nia = (size_t)X * o * v, nbiq = (size_t)X * o * N,
               nj = (size_t)X * X;
  const bool mdev = is_device_ptr(mos), edev = is_device_ptr(eps), jdev = is_device_ptr(J),
             pdev = is_device_ptr(pmn);
  // The precision forms run the three FP64 contractions on the tensor cores
  // (dgemm_tc.cu, FP64-accurate digit slicing); the FP64 form keeps the FP64
  // pipe throughout.
  const bool tc = precision != CORR_PREC_FP64;
  // Region 1 (persistent across the stages): staged inputs, (P|ia), B, J^-1/2.
  auto plan = [&](Carver& w, void** sm, void** se, void** sj, void** sp, double** pia,
                  double** bia, double** jm, double** biq, void** jws) {
    *sm = mdev ? nullptr : w.take((size_t)N * N * 8);
    *se = edev ? nullptr : w.take((size_t)N * 8);
    *sj = jdev ? nullptr : w.take(nj * 8);
    *sp = pdev ? nullptr : w.take(np * 8);
    *pia = static_cast<double*>(w.take(nia * 8));
    *bia = static_cast<double*>(w.take(nia * 8));
    *jm = static_cast<double*>(w.take(nj * 8));
    *biq = static_cast<double*>(w.take(nbiq * 8));
    // the eigendecomposition and the Cholesky path run one after the other
    *jws = w.take(std::max(jacobi_workspace_bytes(X), chol_workspace_bytes(X)));
  };
  void *sm, *se, *sj, *sp, *jws;
  double *pia, *bia, *jm, *biq;
  Carver cv{nullptr, 0};
  plan(cv, &sm, &se, &sj, &sp, &pia, &bia, &jm, &biq, &jws);
  // Region 2, reused: the digit planes of the tensor-core contractions (and
  // the identity that becomes L^-1), then the energy's scratch.
  const size_t ws_main =
      tc ? std::max(std::max(dgemm_tc_workspace(X * N, o, N), dgemm_tc_workspace(X * o, v, N)),
                    dgemm_tc_workspace(X, o * v, X))
         : 0;
  const size_t ws_metric = tc ? dgemm_tc_workspace(X, X, X) : 0;
  const size_t dg_bytes = tc ? ws_main + ws_metric + 2 * nj * 8 + 1024 : 0;
  CORR_TRY(c->ws.reserve(cv.used + std::max(dg_bytes, energy_scratch_bytes(c, o, v, X, precision))));
  Carver w{c->ws.ptr, 0};
  plan(w, &sm, &se, &sj, &sp, &pia, &bia, &jm, &biq, &jws);
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_m = static_cast<const double*>(stage_in(c, mos, (size_t)N * N * 8, sm));
  const double* d_e = static_cast<const double*>(stage_in(c, eps, (size_t)N * 8, se));
  const double* d_j = static_cast<const double*>(stage_in(c, J, nj * 8, sj));
  const double* d_p = static_cast<const double*>(stage_in(c, pmn, np * 8, sp));
  CORR_CHECK_ARG(d_m && d_e && d_j && d_p, "host-to-device copy failed");
  // (P|ia) = C_occ (P|mu nu) C_vir^T  (the transform_ri contractions, ri.cc:147-172)
  const double tol = 1e-10;
  double jnorm = 0.0;
  double *Lm = nullptr, *Linv = nullptr;
  bool factored = false;
  if (tc) {
    Carver r2 = w;
    void* dws = r2.take(ws_main);
    void* mws = r2.take(ws_metric);
    double* T = static_cast<double*>(r2.take(nj * 8));
    double* W = static_cast<double*>(r2.take(nj * 8));
    // The metric stage does not depend on the transform: it runs on a side
    // stream (its own digit-GEMM workspace) while the transform's products
    // run on the context stream, and is joined before B = W (P|ia).
    SideStream side;
    CORR_TRY(side.fork(c->stream));
    // (P|i nu): rows (P, nu) of (P|mu nu) (symmetric in mu nu) against the
    // occupied rows of C, written in the [P][i][nu] layout
    DgemmTc g1;
    g1.A = mat_view(d_p, N, 1);
    g1.B = mat_view(d_m, N, 1);
    g1.C = OutView{biq, (long long)o * N, 1, N, N};
    g1.M = X * N;
    g1.N = o;
    g1.K = N;
    g1.alpha = 1.0;
    g1.accumulate = false;
    g1.a_lower = false;
    CORR_TRY(dgemm_tc(c, g1, dws));
    // (P|ia): rows (P, i) against the virtual rows of C
    DgemmTc g2 = g1;
    g2.A = mat_view(biq, N, 1);
    g2.B = mat_view(d_m + (size_t)o * N, N, 1);
    g2.C = out_view(pia, v, 1);
    g2.M = X * o;
    g2.N = v;
    CORR_TRY(dgemm_tc(c, g2, dws));
    {
      StreamSwap onside(c, side.st);
      // The metric (ri.cc:50-69): one factorisation J = L L^T and W = L^-1
      // (recursive blocked inversion).  Certificate from W itself:
      // lambda_min(J) = 1 / ||L^-1||_2^2 >= 1 / (||L^-1||_1 ||L^-1||_inf);
      // when that bound does not reach twice the threshold, J - t I is
      // factored (chol.cu); without a certificate, J^-1/2 with the cutoff.
      CORR_TRY(chol_norm_inf(c, jm, d_j, X, &jnorm));
      if (jnorm > 0.0)
        CORR_TRY(chol_factor_device(c, jws, d_j, X, 0.0, &Lm, &Linv, &factored, mws));
      if (factored) {
        CORR_TRY(chol_inverse_device(c, Lm, Linv, X, W, T, mws));
        double n1inf = 0.0;
        CORR_TRY(chol_norm_one_inf(c, jm, W, X, &n1inf));
        bool certified = n1inf > 0.0 && 1.0 / n1inf > 2.0 * 10.0 * tol * jnorm;
        if (!certified)
          CORR_TRY(chol_factor_device(c, jws, d_j, X, 10.0 * tol * jnorm, &Lm, &Linv,
                                      &certified, mws));
        factored = certified;
      }
      if (factored) {
        if (ncut) *ncut = 0;
      } else {
        CORR_TRY(ri_inv_sqrt_device(c, jws, d_j, X, tol, jm, ncut, false));
        W = jm;
      }
    }
    CORR_TRY(side.join(c->stream));
    // B[Q][ia] = sum_P W[Q][P] (P|ia): rows Q of W against the columns ia of
    // (P|ia) read as rows over P
    DgemmTc g3;
    g3.A = mat_view(W, X, 1);
    g3.B = mat_view(pia, 1, (long long)o * v);
    g3.C = out_view(bia, (long long)o * v, 1);
    g3.M = X;
    g3.N = o * v;
    g3.K = X;
    g3.alpha = 1.0;
    g3.accumulate = false;
    g3.a_lower = factored;
    CORR_TRY(dgemm_tc(c, g3, dws));
  } else {
    GemmF64 g1 = gemm_args(d_m, d_p, biq, o, N, N, N, N, N, 0, 0);
    g1.sb = (long long)N * N;
    g1.sc = (long long)o * N;
    g1.batch = X;
    CORR_TRY(gemm_f64(g1, &c->dres->status, c->stream));
    CORR_TRY(gemm_f64(gemm_args(biq, d_m + (size_t)o * N, pia, X * o, v, N, N, N, v, 0, 1),
                      &c->dres->status, c->stream));
    // The metric.  The energy sees J only through J^-1 = W^T W: when the
    // reference's cutoff (ri.cc:56-66, lambda/lambda_max < 1e-10) provably
    // cuts nothing -- J - 10 tol ||J||_inf I is positive definite -- W = L^-1
    // from a Cholesky factorisation (chol.cu); otherwise W = J^-1/2 with the
    // cutoff (ri.cc:50-69), applied to the (P|ia) matrix (2 X^2 o v flops).
    CORR_TRY(chol_norm_inf(c, jm, d_j, X, &jnorm));
    bool certified = false;
    if (jnorm > 0.0) CORR_TRY(chol_factor_device(c, jws, d_j, X, 10.0 * tol * jnorm, &Lm, &Linv,
                                                 &certified, nullptr));
    if (certified)
      CORR_TRY(chol_factor_device(c, jws, d_j, X, 0.0, &Lm, &Linv, &factored, nullptr));
    if (factored) {
      CORR_TRY(chol_solve_device(c, Lm, Linv, X, pia, (long long)o * v, bia));
      if (ncut) *ncut = 0;
    } else {
      CORR_TRY(ri_inv_sqrt_device(c, jws, d_j, X, tol, jm, ncut, false));
      CORR_TRY(gemm_f64(gemm_args(jm, pia, bia, X, o * v, X, X, (long long)o * v,
                                  (long long)o * v, 0, 0),
                        &c->dres->status, c->stream));
      c->launches += 1;
    }
  }
  c->launches += 2;
  // energy on the device-resident B; its scratch is carved after region 1
  CORR_TRY(rimp2_energy_core(c, w, o, v, X, bia, d_e, precision, nullptr));
  CORR_TRY(finish_results(c, 4));
  out->e_ss = c->hres->e[0];
  out->e_os = c->hres->e[1];
  out->e_total = c->hres->e[2];
  out->e_scs = c->hres->e[3];
  return CORR_OK;
}

}  // extern "C"
