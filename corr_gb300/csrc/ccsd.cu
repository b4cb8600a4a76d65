// Spin-orbital quantities of the reference's CCSD consumer of the MO integrals
// (src/POSTHF/ccsd.cc), built on the GPU from the spatial (pq|rs) that
// corr_motrans leaves there, so the full N^4 tensor need not go back to the
// host first.
//
//   corr_ints_so   <ij||kl> over norb = 2 nroao spin orbitals (spin of
//                  orbital p: p % 2, spatial index p / 2), calc_ints_so
//                  (ccsd.cc:509-535) with get_integral (ccsd.cc:6-9):
//                  <ij||kl> = (i k | j l) [s_i = s_k][s_j = s_l]
//                           - (i l | j k) [s_i = s_l][s_j = s_k]
//   corr_cc_fock   h_pq = (C H C^T)_{p/2 q/2} [s_p = s_q] and
//                  f_pq = h_pq + sum_{j < nocc} <pj||qj>, form_fock (ccsd.cc:11-48)
//
// ints_so is written in 16 N^4 doubles: a pure gather from prec_ints
// (N^4 doubles, which stays in L2 for the sizes the reference's CCSD runs),
// bound by the HBM write of the output.
#include <algorithm>

#include "abi_internal.h"
#include "common.cuh"
#include "gemm_fp64.h"

namespace corr {

namespace {

// <ij||kl> for the spin pair l = 2L, 2L + 1 (one spatial index L): one thread
// per (i, j, k, L), one 16-byte store (M = 2N is even, so the pair is aligned).
__global__ void __launch_bounds__(256) ints_so_kernel(const double* __restrict__ prec, int N,
                                                      double* __restrict__ out) {
  const long long M = 2LL * N;
  const long long nt = M * M * M * N;
  const long long N2 = (long long)N * N, N3 = N2 * N;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt;
       t += (long long)gridDim.x * blockDim.x) {
    const int L = (int)(t % N);
    const long long ijk = t / N;
    const int k = (int)(ijk % M), j = (int)((ijk / M) % M), i = (int)(ijk / (M * M));
    double v[2];
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) {  // l = 2L + sl
      double x = 0.0;
      if ((i & 1) == (k & 1) && (j & 1) == sl)
        x = prec[(i / 2) * N3 + (k / 2) * N2 + (j / 2) * (long long)N + L];
      if ((i & 1) == sl && (j & 1) == (k & 1))
        x -= prec[(i / 2) * N3 + (long long)L * N2 + (j / 2) * (long long)N + k / 2];
      v[sl] = x;
    }
    *reinterpret_cast<double2*>(out + ijk * M + 2 * L) = make_double2(v[0], v[1]);
  }
}

// h and f over spin orbitals from the spatial hs = C H C^T
__global__ void cc_fock_kernel(const double* __restrict__ hs, const double* __restrict__ prec,
                               int N, int nocc, double* __restrict__ h, double* __restrict__ f) {
  const int M = 2 * N;
  const long long N2 = (long long)N * N, N3 = N2 * N;
  const int p = blockIdx.y, q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= M) return;
  const double hv = ((p & 1) == (q & 1)) ? hs[(p / 2) * N + q / 2] : 0.0;
  double twoe = 0.0;  // sum_{j < nocc} <pj||qj>, in the order of the reference's loop
  for (int j = 0; j < nocc; ++j) {
    double v = 0.0;
    if ((p & 1) == (q & 1)) v = prec[(p / 2) * N3 + (q / 2) * N2 + (j / 2) * (long long)N + j / 2];
    if ((p & 1) == (j & 1) && (j & 1) == (q & 1))
      v -= prec[(p / 2) * N3 + (j / 2) * N2 + (j / 2) * (long long)N + q / 2];
    twoe += v;
  }
  h[(long long)p * M + q] = hv;
  f[(long long)p * M + q] = hv + twoe;
}

}  // namespace

}  // namespace corr

using namespace corr;

extern "C" {

int corr_ints_so(corr_context* c, int nroao, const double* prec, double* ints_so) {
  CORR_CHECK_ARG(c && prec && ints_so, "corr_ints_so: null argument");
  CORR_CHECK_ARG(nroao >= 1 && nroao <= 2048, "corr_ints_so: nroao %d out of range", nroao);
  CORR_CUDA(cudaSetDevice(c->device));
  const long long N = nroao, M = 2 * N;
  const size_t n4 = (size_t)(N * N * N * N), m4 = (size_t)(M * M * M * M);
  const bool pdev = is_device_ptr(prec);
  // the kernel's 16-byte stores need an aligned output: an unaligned device
  // array is filled through the (aligned) workspace, like a host array
  const bool odev = is_device_ptr(ints_so) && ((uintptr_t)ints_so & 15) == 0;
  Carver cv{nullptr, 0};
  if (!pdev) cv.take(n4 * 8);
  if (!odev) cv.take(m4 * 8);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_p = pdev ? nullptr : w.take(n4 * 8);
  double* out = odev ? ints_so : static_cast<double*>(w.take(m4 * 8));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_p = static_cast<const double*>(stage_in(c, prec, n4 * 8, s_p));
  CORR_CHECK_ARG(d_p, "corr_ints_so: host-to-device copy failed");
  mark(c, 1);
  const long long nt = M * M * M * N;
  const int grid = (int)std::min<long long>((nt + 255) / 256, (long long)c->sms * 16);
  ints_so_kernel<<<grid, 256, 0, c->stream>>>(d_p, nroao, out);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  mark(c, 2);
  CORR_TRY(stage_out(c, ints_so, out, m4 * 8));
  return finish_results(c, 0);
}

int corr_cc_fock(corr_context* c, int nroe, int nroao, const double* mos, const double* hmat,
                 const double* prec, double* h_so, double* f_so) {
  CORR_CHECK_ARG(c && mos && hmat && prec && h_so && f_so, "corr_cc_fock: null argument");
  CORR_CHECK_ARG(nroao >= 1 && nroe >= 0 && nroe <= 2 * nroao, "corr_cc_fock: bad sizes");
  CORR_CUDA(cudaSetDevice(c->device));
  const int N = nroao, M = 2 * nroao;
  const size_t n2 = (size_t)N * N, n4 = n2 * n2, m2 = (size_t)M * M;
  const bool pdev = is_device_ptr(prec), hdev = is_device_ptr(h_so), fdev = is_device_ptr(f_so);
  auto plan = [&](Carver& w, void** s_m, void** s_h, void** s_p, double** T, double** hs,
                  double** ho, double** fo) {
    *s_m = w.take(n2 * 8);
    *s_h = w.take(n2 * 8);
    *s_p = pdev ? nullptr : w.take(n4 * 8);
    *T = static_cast<double*>(w.take(n2 * 8));
    *hs = static_cast<double*>(w.take(n2 * 8));
    *ho = hdev ? h_so : static_cast<double*>(w.take(m2 * 8));
    *fo = fdev ? f_so : static_cast<double*>(w.take(m2 * 8));
  };
  void *s_m, *s_h, *s_p;
  double *T, *hs, *ho, *fo;
  Carver cv{nullptr, 0};
  plan(cv, &s_m, &s_h, &s_p, &T, &hs, &ho, &fo);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  plan(w, &s_m, &s_h, &s_p, &T, &hs, &ho, &fo);
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_m = static_cast<const double*>(stage_in(c, mos, n2 * 8, s_m));
  const double* d_h = static_cast<const double*>(stage_in(c, hmat, n2 * 8, s_h));
  const double* d_p = static_cast<const double*>(stage_in(c, prec, n4 * 8, s_p));
  CORR_CHECK_ARG(d_m && d_h && d_p, "corr_cc_fock: host-to-device copy failed");
  mark(c, 1);
  // hs[p][q] = sum C[p][mu] H[mu][nu] C[q][nu]
  CORR_TRY(gemm_f64(gemm_args(d_m, d_h, T, N, N, N, N, N, N, 0, 0), &c->dres->status, c->stream));
  CORR_TRY(gemm_f64(gemm_args(T, d_m, hs, N, N, N, N, N, N, 0, 1), &c->dres->status, c->stream));
  dim3 grid((unsigned)((M + 127) / 128), (unsigned)M);
  cc_fock_kernel<<<grid, 128, 0, c->stream>>>(hs, d_p, N, nroe, ho, fo);
  CORR_CUDA(cudaGetLastError());
  c->launches += 3;
  mark(c, 2);
  CORR_TRY(stage_out(c, h_so, ho, m2 * 8));
  CORR_TRY(stage_out(c, f_so, fo, m2 * 8));
  return finish_results(c, 0);
}

}  // extern "C"
