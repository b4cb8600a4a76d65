// RHF on the GPU over the reference's packed ERI list (src/SCF): the Fock
// build of build_Fmat (ops_rhf.cc:549-591, the five permutation classes), the
// DIIS error and extrapolation of run_scf (scf.cc:105-143, 214-287), and the
// whole run_scf iteration (scf.cc:145-321: damped density, Fock build, DIIS,
// electronic energy, symmetric orthogonalisation and diagonalisation).
//
// Fock build: F = H + sum_ls P_ls [(mn|ls) - 1/2 (ml|ns)], the sum the five
// permutation-class loops accumulate from the unique integrals.  Here the
// packed list is unpacked once into the dense N^4 tensor on the device (the
// scatter of the MO transform), and one warp forms each F_mn as a fixed-order
// sum over (l, s) (deterministic, unlike an atomic scatter of the list).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "abi_internal.h"
#include "common.cuh"
#include "gemm_fp64.h"

namespace corr {

int launch_unpack(corr_context* c, int N, long long n, const long long* sc, const double* val,
                  const unsigned short* num, double* eri);

namespace {

__global__ void __launch_bounds__(256) fock_kernel(const double* __restrict__ eri,
                                                   const double* __restrict__ P,
                                                   const double* __restrict__ H, int N,
                                                   double* __restrict__ F) {
  const int lane = threadIdx.x & 31;
  const long long N2 = (long long)N * N;
  for (long long mn = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / 32; mn < N2;
       mn += ((long long)gridDim.x * blockDim.x) / 32) {
    const int m = (int)(mn / N), n = (int)(mn % N);
    const double* jrow = eri + mn * N2;                  // (mn|ls) over ls
    double s = 0.0;
    for (long long ls = lane; ls < N2; ls += 32) {
      const int l = (int)(ls / N), t = (int)(ls % N);
      const double k = eri[(((long long)m * N + l) * N + n) * N + t];  // (ml|ns)
      s += P[ls] * (jrow[ls] - 0.5 * k);
    }
    s = warp_sum(s);
    if (lane == 0) F[mn] = H[mn] + s;
  }
}

// P = 2 (1 - damp) sum_{i < nocc} C_i C_i^T + damp P_old   (scf.cc:41-61)
__global__ void density_kernel(const double* __restrict__ C, int N, int nocc, double damp,
                               double* __restrict__ P) {
  const long long N2 = (long long)N * N;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < N2;
       x += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(x / N), n = (int)(x % N);
    double s = 0.0;
    for (int i = 0; i < nocc; ++i) s += C[(long long)i * N + m] * C[(long long)i * N + n];
    P[x] = 2.0 * (1.0 - damp) * s + damp * P[x];
  }
}

// out[0] = sum P*(F + H) / 2 (Calc_e_el, ops_rhf.cc:593-602; F, H, P
// symmetric), out[1] = sum P*H and out[2] = sum P*F (oneE/twoE, scf.cc:83-101),
// out[3] = mean |err| (scf.cc:226-229; 0 without err).  One block, fixed order.
__global__ void scf_sums_kernel(const double* __restrict__ P, const double* __restrict__ F,
                                const double* __restrict__ H, const double* __restrict__ err,
                                long long n2, double* __restrict__ out) {
  __shared__ double red[4][256];
  double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
  for (long long x = threadIdx.x; x < n2; x += blockDim.x) {
    a += P[x] * (F[x] + H[x]);
    b += P[x] * H[x];
    c += P[x] * F[x];
    if (err) d += fabs(err[x]);
  }
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = b;
  red[2][threadIdx.x] = c;
  red[3][threadIdx.x] = d;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = 0.5 * red[0][0];
    out[1] = red[1][0];
    out[2] = red[2][0];
    out[3] = red[3][0] / (double)n2;
  }
}

// B[i][j] = err_i . err_j for the m stored error matrices (fixed-order sums)
__global__ void diis_dots_kernel(const double* const* __restrict__ E, int m, long long n2,
                                 double* __restrict__ B) {
  __shared__ double red[256];
  const int i = blockIdx.x / m, j = blockIdx.x % m;
  double s = 0.0;
  for (long long x = threadIdx.x; x < n2; x += blockDim.x) s += E[i][x] * E[j][x];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) B[i * m + j] = red[0];
}

// Least-squares solution of the bordered DIIS system (scf.cc:243-268, dgels
// with 'N'): A = [[B, -1], [-1, 0]] (d = m + 1), rhs = [0 .. 0, -1], by
// Householder QR (the method dgels uses); one thread, d <= 33.
__global__ void diis_solve_kernel(const double* __restrict__ B, int m, double* __restrict__ c) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  constexpr int DMAX = 33;
  const int d = m + 1;
  double A[DMAX][DMAX], r[DMAX];
  for (int i = 0; i < d; ++i) {
    for (int j = 0; j < d; ++j)
      A[i][j] = (i < m && j < m) ? B[i * m + j] : ((i == m && j == m) ? 0.0 : -1.0);
    r[i] = i == m ? -1.0 : 0.0;
  }
  for (int k = 0; k < d; ++k) {
    double nrm = 0.0;
    for (int i = k; i < d; ++i) nrm += A[i][k] * A[i][k];
    nrm = sqrt(nrm);
    if (nrm == 0.0) continue;
    const double alpha = A[k][k] > 0.0 ? -nrm : nrm;
    double v[DMAX];
    for (int i = 0; i < d; ++i) v[i] = i < k ? 0.0 : A[i][k];
    v[k] -= alpha;
    double vv = 0.0;
    for (int i = k; i < d; ++i) vv += v[i] * v[i];
    if (vv == 0.0) continue;
    for (int j = k; j < d; ++j) {
      double s = 0.0;
      for (int i = k; i < d; ++i) s += v[i] * A[i][j];
      s *= 2.0 / vv;
      for (int i = k; i < d; ++i) A[i][j] -= s * v[i];
    }
    double s = 0.0;
    for (int i = k; i < d; ++i) s += v[i] * r[i];
    s *= 2.0 / vv;
    for (int i = k; i < d; ++i) r[i] -= s * v[i];
  }
  for (int i = d - 1; i >= 0; --i) {  // R x = Q^T r
    double s = r[i];
    for (int j = i + 1; j < d; ++j) s -= A[i][j] * c[j];
    c[i] = A[i][i] != 0.0 ? s / A[i][i] : 0.0;
  }
}

// F = sum_j c_j F_j
__global__ void diis_combine_kernel(const double* const* __restrict__ Fh,
                                    const double* __restrict__ c, int m, long long n2,
                                    double* __restrict__ F) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n2;
       x += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s += c[j] * Fh[j][x];
    F[x] = s;
  }
}

int grid_of(corr_context* c, long long n, int per = 256) {
  return (int)std::max<long long>(1, std::min<long long>((n + per - 1) / per, (long long)c->sms * 8));
}

__global__ void sub_kernel(double* __restrict__ a, const double* __restrict__ b, long long n) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
       x += (long long)gridDim.x * blockDim.x)
    a[x] -= b[x];
}

// err = S P F - F P S (calc_diis_error, scf.cc:105-143); t1, t2 scratch
int diis_error(corr_context* c, int N, const double* F, const double* P, const double* S,
               double* t1, double* t2, double* err) {
  CORR_TRY(gemm_f64(gemm_args(P, F, t1, N, N, N, N, N, N, 0, 0), &c->dres->status, c->stream));
  CORR_TRY(gemm_f64(gemm_args(S, t1, err, N, N, N, N, N, N, 0, 0), &c->dres->status, c->stream));
  CORR_TRY(gemm_f64(gemm_args(P, S, t1, N, N, N, N, N, N, 0, 0), &c->dres->status, c->stream));
  CORR_TRY(gemm_f64(gemm_args(F, t1, t2, N, N, N, N, N, N, 0, 0), &c->dres->status, c->stream));
  const long long n2 = (long long)N * N;
  sub_kernel<<<grid_of(c, n2), 256, 0, c->stream>>>(err, t2, n2);
  CORR_CUDA(cudaGetLastError());
  c->launches += 5;
  return CORR_OK;
}

// Device buffers of one SCF run (their own allocation: the eigensolver and the
// GEMM entry points called in the loop use the context workspace).
struct ScfBuffers {
  double* base = nullptr;
  ~ScfBuffers() {
    if (base) cudaFree(base);
  }
};

}  // namespace

}  // namespace corr

using namespace corr;

extern "C" {

int corr_build_fmat(corr_context* c, int nroao, const double* pmat, const double* hmat,
                    long long nrofint, const long long* sortcount, const double* intval,
                    const unsigned short* intnums, double* fmat) {
  CORR_CHECK_ARG(c && pmat && hmat && sortcount && fmat && (nrofint == 0 || (intval && intnums)),
                 "corr_build_fmat: null argument");
  CORR_CHECK_ARG(nroao >= 1 && nroao <= 65535 && nrofint >= 0, "corr_build_fmat: bad sizes");
  CORR_CHECK_ARG((double)nroao * nroao * nroao * nroao * 8 < 1.0e11,
                 "corr_build_fmat: the N^4 tensor of nroao=%d does not fit", nroao);
  CORR_CUDA(cudaSetDevice(c->device));
  const int N = nroao;
  const size_t n2 = (size_t)N * N, n4 = n2 * n2, ni = (size_t)(nrofint > 0 ? nrofint : 1);
  const bool fdev = is_device_ptr(fmat);
  Carver cv{nullptr, 0};
  for (int k = 0; k < 2; ++k) cv.take(n2 * 8);
  cv.take(32);
  cv.take(ni * 8);
  cv.take(ni * 8);
  cv.take(n4 * 8);
  cv.take(n2 * 8);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  void* s_p = w.take(n2 * 8);
  void* s_h = w.take(n2 * 8);
  void* s_sc = w.take(32);
  void* s_v = w.take(ni * 8);
  void* s_n = w.take(ni * 8);
  double* eri = static_cast<double*>(w.take(n4 * 8));
  double* out = fdev ? fmat : static_cast<double*>(w.take(n2 * 8));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_p = static_cast<const double*>(stage_in(c, pmat, n2 * 8, s_p));
  const double* d_h = static_cast<const double*>(stage_in(c, hmat, n2 * 8, s_h));
  const long long* d_sc = static_cast<const long long*>(stage_in(c, sortcount, 32, s_sc));
  const double* d_v = nrofint ? static_cast<const double*>(stage_in(c, intval, nrofint * 8, s_v))
                              : static_cast<const double*>(s_v);
  const unsigned short* d_n =
      nrofint ? static_cast<const unsigned short*>(stage_in(c, intnums, nrofint * 8, s_n))
              : static_cast<const unsigned short*>(s_n);
  CORR_CHECK_ARG(d_p && d_h && d_sc && d_v && d_n, "corr_build_fmat: host-to-device copy failed");
  CORR_TRY(launch_unpack(c, N, nrofint, d_sc, d_v, d_n, eri));
  mark(c, 1);
  fock_kernel<<<grid_of(c, (long long)n2 * 32), 256, 0, c->stream>>>(eri, d_p, d_h, N, out);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  mark(c, 2);
  CORR_TRY(stage_out(c, fmat, out, n2 * 8));
  return finish_results(c, 0);
}

int corr_run_scf(corr_context* c, int nroe, int nroao, double ion_rep, const double* smat,
                 const double* hmat, long long nrofint, const long long* sortcount,
                 const double* intval, const unsigned short* intnums, int maxiter, double* mos,
                 double* fmat, double* moens, double* energies, int* iterations, double* pmat) {
  CORR_CHECK_ARG(c && smat && hmat && sortcount && mos && fmat && moens && energies &&
                     (nrofint == 0 || (intval && intnums)),
                 "corr_run_scf: null argument");
  CORR_CHECK_ARG(nroao >= 1 && nroao <= 2048 && nroe >= 2 && nroe % 2 == 0 && nroe / 2 <= nroao,
                 "corr_run_scf: bad sizes (nroe=%d, nroao=%d)", nroe, nroao);
  CORR_CHECK_ARG(maxiter >= 0, "corr_run_scf: maxiter must be >= 0");
  CORR_CUDA(cudaSetDevice(c->device));
  const int N = nroao, nocc = nroe / 2;
  const size_t n2 = (size_t)N * N, n4 = n2 * n2, ni = (size_t)(nrofint > 0 ? nrofint : 1);
  constexpr int kDiis = 8;           // diis_size (scf.cc:170)
  constexpr double kDiisThresh = 1e-3;
  // one allocation for the SCF state (the eigensolver and GEMM entry points
  // called below carve the context workspace); sized by a dry run of the carve
  ScfBuffers buf;
  uintptr_t base = 0;
  size_t off = 0;  // doubles
  auto take = [&](size_t n) {
    double* r = reinterpret_cast<double*>(base + off * 8);
    off += (n + 31) / 32 * 32;
    return r;
  };
  double *eri, *S, *H, *P, *F, *C, *T, *t1, *t2, *err, *w, *V, *Fo, *small, *d_val;
  double* Fh[kDiis];
  double* Eh[kDiis];
  auto carve = [&]() {
    eri = take(n4);
    S = take(n2), H = take(n2), P = take(n2), F = take(n2), C = take(n2), T = take(n2);
    t1 = take(n2), t2 = take(n2), err = take(n2), V = take(n2), Fo = take(n2), w = take(N);
    for (int k = 0; k < kDiis; ++k) {
      Fh[k] = take(n2);
      Eh[k] = take(n2);
    }
    small = take(128);  // sums [0, 4), sortcount [8, 12), pointer tables, B, c
    d_val = take(ni);
    return take(ni);    // intnums: four unsigned shorts per integral
  };
  carve();
  const size_t total = off;
  if (cudaMalloc(&buf.base, total * 8) != cudaSuccess) {
    cudaGetLastError();
    set_error("corr_run_scf: device allocation of %zu bytes failed", total * 8);
    return CORR_ERR_OOM;
  }
  base = reinterpret_cast<uintptr_t>(buf.base);
  off = 0;
  unsigned short* d_num = reinterpret_cast<unsigned short*>(carve());
  long long* d_sc = reinterpret_cast<long long*>(small + 8);
  const double** d_fh = reinterpret_cast<const double**>(small + 16);
  const double** d_eh = reinterpret_cast<const double**>(small + 16 + kDiis);
  double* d_B = small + 16 + 2 * kDiis;
  double* d_c = d_B + kDiis * kDiis;
  double* d_sums = small;
  auto h2d = [&](void* dst, const void* src, size_t bytes) -> int {
    CORR_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream));
    return CORR_OK;
  };
  CORR_TRY(h2d(S, smat, n2 * 8));
  CORR_TRY(h2d(H, hmat, n2 * 8));
  CORR_TRY(h2d(C, mos, n2 * 8));
  CORR_TRY(h2d(d_sc, sortcount, 32));
  if (nrofint) {
    CORR_TRY(h2d(d_val, intval, nrofint * 8));
    CORR_TRY(h2d(d_num, intnums, nrofint * 8));
  }
  CORR_CUDA(cudaMemsetAsync(P, 0, n2 * 8, c->stream));
  for (int k = 0; k < kDiis; ++k) {  // the history starts zeroed (scf.cc:172)
    CORR_CUDA(cudaMemsetAsync(Fh[k], 0, n2 * 8, c->stream));
    CORR_CUDA(cudaMemsetAsync(Eh[k], 0, n2 * 8, c->stream));
  }
  CORR_TRY(launch_unpack(c, N, nrofint, d_sc, d_val, d_num, eri));
  const long long nn = (long long)n2;
  // S^-1/2 = V^T diag(lambda^-1/2) V with eigenvectors as rows of V (calc_S12, ops_rhf.cc:342-386)
  CORR_TRY(corr_syev(c, N, S, w, V));
  std::vector<double> hw(N);
  CORR_CUDA(cudaMemcpy(hw.data(), w, N * 8, cudaMemcpyDeviceToHost));
  for (int k = 0; k < N; ++k) {
    CORR_CHECK_ARG(hw[k] > 0.0, "corr_run_scf: the overlap matrix is not positive definite");
    hw[k] = 1.0 / std::sqrt(hw[k]);
  }
  CORR_CUDA(cudaMemcpy(w, hw.data(), N * 8, cudaMemcpyHostToDevice));
  {
    // t1[z][y] = d_z V[z][y];  T = V^T t1
    std::vector<double> hv(n2);
    CORR_CUDA(cudaMemcpy(hv.data(), V, n2 * 8, cudaMemcpyDeviceToHost));
    for (int z = 0; z < N; ++z)
      for (int y = 0; y < N; ++y) hv[(size_t)z * N + y] *= hw[z];
    CORR_CUDA(cudaMemcpy(t1, hv.data(), n2 * 8, cudaMemcpyHostToDevice));
    CORR_TRY(corr_dgemm(c, 1, 0, N, N, N, 1.0, V, N, t1, N, 0.0, T, N));
  }
  // diag_Fmat (ops_rhf.cc:425-431): F' = T F T, eigenvectors of F' as rows, C = C' T^T
  bool diagonalised = false;
  auto diag_fmat = [&](const double* Fin) -> int {
    diagonalised = true;
    CORR_TRY(corr_dgemm(c, 0, 0, N, N, N, 1.0, T, N, Fin, N, 0.0, t1, N));
    CORR_TRY(corr_dgemm(c, 0, 0, N, N, N, 1.0, t1, N, T, N, 0.0, t2, N));
    CORR_TRY(corr_syev(c, N, t2, w, V));
    CORR_TRY(corr_dgemm(c, 0, 1, N, N, N, 1.0, V, N, T, N, 0.0, C, N));
    return CORR_OK;
  };
  // check_initial_guess (ops_rhf.cc:15-36): without orbitals, the core guess
  {
    std::vector<double> hc(n2);
    CORR_CUDA(cudaMemcpy(hc.data(), C, n2 * 8, cudaMemcpyDeviceToHost));
    double modiag = 0.0;
    for (int i = 0; i < N; ++i) modiag += hc[(size_t)i * N + i];
    if (std::fabs(modiag) < 0.1) CORR_TRY(diag_fmat(H));
  }
  std::vector<const double*> fh(Fh, Fh + kDiis), eh(Eh, Eh + kDiis);
  double damp = 0.5, Eold = 100.0, DE = 10.0, hs[4];
  bool diis = false;
  int iter = 0;
  auto sums = [&](const double* Fm, const double* e) -> int {
    scf_sums_kernel<<<1, 256, 0, c->stream>>>(P, Fm, H, e, nn, d_sums);
    CORR_CUDA(cudaGetLastError());
    CORR_CUDA(cudaMemcpyAsync(hs, d_sums, 32, cudaMemcpyDeviceToHost, c->stream));
    CORR_CUDA(cudaStreamSynchronize(c->stream));
    c->launches += 1;
    return CORR_OK;
  };
  auto density = [&](double dmp) -> int {
    density_kernel<<<grid_of(c, nn), 256, 0, c->stream>>>(C, N, nocc, dmp, P);
    CORR_CUDA(cudaGetLastError());
    return CORR_OK;
  };
  auto fock = [&]() -> int {
    fock_kernel<<<grid_of(c, nn * 32), 256, 0, c->stream>>>(eri, P, H, N, F);
    CORR_CUDA(cudaGetLastError());
    c->launches += 2;
    return CORR_OK;
  };
  CORR_TRY(density(0.0));  // build_Pmat(C, ..., 0.0) before the loop (scf.cc:197)
  while (iter < maxiter && std::fabs(DE) > 1e-8) {
    CORR_TRY(density(damp));
    CORR_TRY(fock());
    // rotate the history: the oldest slot becomes the newest (scf.cc:214-221)
    std::rotate(fh.begin(), fh.begin() + 1, fh.end());
    std::rotate(eh.begin(), eh.begin() + 1, eh.end());
    double* fnew = const_cast<double*>(fh.back());
    double* enew = const_cast<double*>(eh.back());
    CORR_CUDA(cudaMemcpyAsync(fnew, F, n2 * 8, cudaMemcpyDeviceToDevice, c->stream));
    CORR_TRY(diis_error(c, N, F, P, S, t1, t2, enew));
    CORR_TRY(sums(F, enew));
    const double error = hs[3];
    const double* Fuse = F;
    if (error < kDiisThresh && iter >= kDiis) {
      if (!diis) {
        diis = true;
        damp = 0.0;
      }
      CORR_CUDA(cudaMemcpyAsync(d_fh, fh.data(), sizeof(double*) * kDiis, cudaMemcpyHostToDevice,
                                c->stream));
      CORR_CUDA(cudaMemcpyAsync(d_eh, eh.data(), sizeof(double*) * kDiis, cudaMemcpyHostToDevice,
                                c->stream));
      diis_dots_kernel<<<kDiis * kDiis, 256, 0, c->stream>>>(d_eh, kDiis, nn, d_B);
      diis_solve_kernel<<<1, 32, 0, c->stream>>>(d_B, kDiis, d_c);
      diis_combine_kernel<<<grid_of(c, nn), 256, 0, c->stream>>>(d_fh, d_c, kDiis, nn, Fo);
      CORR_CUDA(cudaGetLastError());
      c->launches += 3;
      Fuse = Fo;
      CORR_TRY(sums(Fo, nullptr));
    }
    const double Escf = hs[0];
    DE = Escf - Eold;
    Eold = Escf;
    CORR_TRY(diag_fmat(Fuse));
    ++iter;
  }
  // final density and Fock matrix (scf.cc:289-290), the printed energies (:308-314)
  CORR_TRY(density(damp));
  CORR_TRY(fock());
  CORR_TRY(sums(F, nullptr));
  energies[0] = 0.5 * (hs[1] + hs[2]) + ion_rep;  // TOTAL E
  energies[1] = hs[1] + ion_rep;                 // ONE E
  energies[2] = 0.5 * (hs[2] - hs[1]);           // TWO E
  if (iterations) *iterations = iter;
  CORR_CUDA(cudaMemcpyAsync(mos, C, n2 * 8, cudaMemcpyDefault, c->stream));
  CORR_CUDA(cudaMemcpyAsync(fmat, F, n2 * 8, cudaMemcpyDefault, c->stream));
  if (pmat) CORR_CUDA(cudaMemcpyAsync(pmat, P, n2 * 8, cudaMemcpyDefault, c->stream));
  if (diagonalised)  // else moens keeps what the caller passed (no orbital energies exist)
    CORR_CUDA(cudaMemcpyAsync(moens, w, (size_t)N * 8, cudaMemcpyDefault, c->stream));
  CORR_CUDA(cudaStreamSynchronize(c->stream));
  return CORR_OK;
}

}  // extern "C"
