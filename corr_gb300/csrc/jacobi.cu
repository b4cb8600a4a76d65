// RI metric J^-1/2 (src/POSTHF/ri.cc:50-69) and the symmetric
// eigendecomposition of diag_mat (src/MATH/ops_mat.cc:21-45) on the GPU, FP64
// results.
//
// The reference diagonalises with LAPACK dsyev; J^-1/2 then zeroes every
// eigenvalue with lambda/lambda_max < 1e-10 or lambda < 0, takes lambda^-1/2 of
// the rest and assembles V diag V^T with dgemm.  Here the eigendecomposition is
// a parallel cyclic two-sided Jacobi method (Golub & Van Loan, "Matrix
// Computations", symmetric Schur decomposition and parallel Jacobi with
// round-robin ordering): every round rotates n/2 disjoint index pairs at once,
//   tau = (a_qq - a_pp) / (2 a_pq),  t = sign(tau) / (|tau| + sqrt(1 + tau^2)),
//   c = 1/sqrt(1 + t^2),  s = t c,   R = [[c, s], [-s, c]],
//   A <- R^T A R (one 2x2 block per thread, in place),  V <- V R,
// and a sweep is n-1 rounds of the circle pairing (index n-1 fixed, index r
// paired with it, (r+k) mod (n-1) with (r-k) mod (n-1)).  A pair is rotated
// only while |a_pq| > 1e-15 sqrt(|a_pp a_qq|) (the threshold rule of Demmel &
// Veselic, "Jacobi's method is more accurate than QR", 1992), and sweeps repeat
// until one sweep rotates no pair (at most 40).
//
// FP64 arithmetic is scarce on this GPU (about 1/60 of its FP32 rate), and a
// from-scratch Jacobi needs 15-20 sweeps.  From n = kMixedMin on, the sweeps
// run in two precisions:
//  1. A / 2^e (||A||_F in [2^(e-1), 2^e)) is rounded to FP32 and swept in FP32
//     until no pair exceeds 2^-20 sqrt(|a_pp a_qq|) nor the absolute floor
//     2^-22 / n (at most 30 sweeps); V0 is the product of those rotations.
//  2. V0 is widened to FP64 and made orthogonal to working accuracy by two
//     Newton-Schulz steps of the polar factor, Q <- Q (3 I - Q^T Q) / 2
//     (Higham, "Functions of Matrices", 8.3); ||Q^T Q - I|| goes from the
//     FP32 level (~1e-5) to ~1e-10 and then to rounding level.
//  3. A1 = Q^T A Q (FP64 GEMMs, then symmetrised) is diagonal up to the FP32
//     residual, and the FP64 sweeps above diagonalise it: A1 = V1 L V1^T in
//     typically two to four sweeps instead of fifteen or more.
//  4. V = Q V1.
// Every FP64 step is a similarity by an orthogonal matrix accurate to FP64
// rounding, so the eigenvalues and vectors carry FP64 errors, as the plain
// FP64 sweeps do; only the starting point of the FP64 sweeps comes from FP32.
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

constexpr double kRotTol = 1e-15;          // FP64 sweeps: relative threshold
constexpr float kRotTol32 = 0x1p-20f;      // FP32 sweeps: relative threshold
constexpr double kFloor32 = 0x1p-22;       // FP32 sweeps: absolute floor x n (||A||_F ~ 1)
constexpr int kMaxSweeps = 40, kMaxSweeps32 = 30;
constexpr int kStop32 = 16;                // FP32 sweeps end below 1/16 of the pairs rotated
constexpr int kMixedMin = 128;             // padded order from which the FP32 sweeps run first

template <typename T>
struct Pair2;
template <>
struct Pair2<double> {
  using type = double2;
};
template <>
struct Pair2<float> {
  using type = float2;
};

// (c, s) of the round-r rotation of pair k; (1, 0) exactly when the pair is
// not rotated.  *rotated counts the rotated pairs (one atomic per warp).
template <typename T>
__global__ void jacobi_params(const T* __restrict__ A, int n, int r, T tol, T floor_abs,
                              typename Pair2<T>::type* __restrict__ cs, int* __restrict__ rotated) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  bool rot = false;
  if (k < n / 2) {
    int p, q;
    round_pair(n, r, k, &p, &q);
    const T app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q], apq = A[(size_t)p * n + q];
    T c = 1, s = 0;
    const T mag = fabs(apq);
    if (mag > tol * sqrt(fabs(app * aqq)) && mag > floor_abs) {
      rot = true;
      const T tau = (aqq - app) / (T(2) * apq);
      const T t = (tau >= T(0) ? T(1) : T(-1)) / (fabs(tau) + sqrt(T(1) + tau * tau));
      c = T(1) / sqrt(T(1) + t * t);
      s = t * c;
    }
    cs[k].x = c;
    cs[k].y = s;
  }
  const unsigned m = __ballot_sync(0xffffffffu, rot);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(rotated, __popc(m));
}

// Pair k+1 of a round from pair k.
__device__ __forceinline__ void next_pair(int n, int r, int k, int* p, int* q) {
  if (k == 0) {
    round_pair(n, r, 1, p, q);
  } else {
    *p = (*p + 1 == n - 1) ? 0 : *p + 1;
    *q = (*q == 0) ? n - 2 : *q - 1;
  }
}

constexpr int kRowsA = 4;  // row pairs k per thread of the A update
constexpr int kRowsV = 4;  // rows x per thread of the V update

// Thread (kb, l) of the A update: the 2x2 blocks rows {p_k, q_k} x cols
// {p_l, q_l} for the kRowsA row pairs k = kb kRowsA .. ; thread (xb, l) of the
// V update: columns {p_l, q_l} of kRowsV rows.  Every load of a thread is
// issued before its first store, so each thread has 4 kRowsA (2 kRowsV)
// independent loads in flight.  A block whose two rotations are both the
// identity is left as it is (the product would reproduce it exactly).
// n <= 32768, so every index fits 32 bits.
template <typename T>
__global__ void jacobi_apply(T* __restrict__ A, T* __restrict__ V, int n, int r,
                             const typename Pair2<T>::type* __restrict__ cs) {
  using P2 = typename Pair2<T>::type;
  const unsigned h = (unsigned)n / 2;
  const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned nA = (h + kRowsA - 1) / kRowsA * h;
  const unsigned nV = ((unsigned)n + kRowsV - 1) / kRowsV * h;
  if (id < nA) {
    const int kb = (int)(id / h), l = (int)(id % h);
    const P2 b = cs[l];
    int u, w;
    round_pair(n, r, l, &u, &w);
    const int k0 = kb * kRowsA;
    P2 a[kRowsA];
    int p[kRowsA], q[kRowsA];
    bool on[kRowsA];
#pragma unroll
    for (int i = 0; i < kRowsA; ++i) {
      const int k = k0 + i;
      if (i == 0)
        round_pair(n, r, k0, &p[0], &q[0]);
      else {
        p[i] = p[i - 1];
        q[i] = q[i - 1];
        if (k < (int)h) next_pair(n, r, k - 1, &p[i], &q[i]);
      }
      on[i] = k < (int)h;
      a[i] = on[i] ? cs[k] : b;
      on[i] = on[i] && !(a[i].y == T(0) && b.y == T(0));
    }
    T x[kRowsA][4];
#pragma unroll
    for (int i = 0; i < kRowsA; ++i) {
      if (on[i]) {
        const T* Ap = A + (size_t)p[i] * n;
        const T* Aq = A + (size_t)q[i] * n;
        x[i][0] = Ap[u];
        x[i][1] = Ap[w];
        x[i][2] = Aq[u];
        x[i][3] = Aq[w];
      }
    }
    // Rotations by angles below ~sqrt(eps) have c == 1 exactly (all of them
    // once the sweeps are near convergence): x' = x - s y, y' = y + s x, one
    // FMA per element, taken when the whole warp qualifies.
    bool unit = b.x == T(1);
#pragma unroll
    for (int i = 0; i < kRowsA; ++i) unit = unit && (!on[i] || a[i].x == T(1));
    if (__all_sync(__activemask(), unit)) {
#pragma unroll
      for (int i = 0; i < kRowsA; ++i) {
        if (on[i]) {
          const T y00 = fma(-a[i].y, x[i][2], x[i][0]), y01 = fma(-a[i].y, x[i][3], x[i][1]);
          const T y10 = fma(a[i].y, x[i][0], x[i][2]), y11 = fma(a[i].y, x[i][1], x[i][3]);
          T* Ap = A + (size_t)p[i] * n;
          T* Aq = A + (size_t)q[i] * n;
          Ap[u] = fma(-b.y, y01, y00);
          Ap[w] = fma(b.y, y00, y01);
          Aq[u] = fma(-b.y, y11, y10);
          Aq[w] = fma(b.y, y10, y11);
        }
      }
      return;
    }
#pragma unroll
    for (int i = 0; i < kRowsA; ++i) {
      if (on[i]) {
        // Y = R_k^T X, then Z = Y R_l
        const T y00 = a[i].x * x[i][0] - a[i].y * x[i][2];
        const T y01 = a[i].x * x[i][1] - a[i].y * x[i][3];
        const T y10 = a[i].y * x[i][0] + a[i].x * x[i][2];
        const T y11 = a[i].y * x[i][1] + a[i].x * x[i][3];
        T* Ap = A + (size_t)p[i] * n;
        T* Aq = A + (size_t)q[i] * n;
        Ap[u] = y00 * b.x - y01 * b.y;
        Ap[w] = y00 * b.y + y01 * b.x;
        Aq[u] = y10 * b.x - y11 * b.y;
        Aq[w] = y10 * b.y + y11 * b.x;
      }
    }
  } else if (id < nA + nV) {
    const unsigned j = id - nA;
    const int xb = (int)(j / h), l = (int)(j % h);
    const P2 b = cs[l];
    if (b.y == T(0)) return;
    int u, w;
    round_pair(n, r, l, &u, &w);
    T vu[kRowsV], vw[kRowsV];
#pragma unroll
    for (int i = 0; i < kRowsV; ++i) {
      const int x = xb * kRowsV + i;
      if (x < n) {
        vu[i] = V[(size_t)x * n + u];
        vw[i] = V[(size_t)x * n + w];
      }
    }
    if (__all_sync(__activemask(), b.x == T(1))) {
#pragma unroll
      for (int i = 0; i < kRowsV; ++i) {
        const int x = xb * kRowsV + i;
        if (x < n) {
          V[(size_t)x * n + u] = fma(-b.y, vw[i], vu[i]);
          V[(size_t)x * n + w] = fma(b.y, vu[i], vw[i]);
        }
      }
      return;
    }
#pragma unroll
    for (int i = 0; i < kRowsV; ++i) {
      const int x = xb * kRowsV + i;
      if (x < n) {
        V[(size_t)x * n + u] = b.x * vu[i] - b.y * vw[i];
        V[(size_t)x * n + w] = b.y * vu[i] + b.x * vw[i];
      }
    }
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
// ops_mat.cc:44).
__global__ void jacobi_init(const double* __restrict__ J, int m, int n, int upper,
                            double* __restrict__ A) {
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e / n), y = (int)(e % n);
    const int lo = x < y ? x : y, hi = x < y ? y : x;
    A[e] = (x < m && y < m) ? (upper ? J[(size_t)lo * m + hi] : J[(size_t)hi * m + lo]) : 0.0;
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

// Af = A * scale rounded to FP32, Vf = identity (n x n).
__global__ void narrow_scaled(const double* __restrict__ A, int n, double scale,
                              float* __restrict__ Af, float* __restrict__ Vf) {
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    Af[e] = (float)(A[e] * scale);
    Vf[e] = (e / n == e % n) ? 1.0f : 0.0f;
  }
}

__global__ void widen(const float* __restrict__ src, long long count, double* __restrict__ dst) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count;
       e += (long long)gridDim.x * blockDim.x)
    dst[e] = (double)src[e];
}

// A <- (A + A^T) / 2 (the thread of entry (x, y), x < y, writes both), V = I.
__global__ void symmetrize_and_identity(double* __restrict__ A, double* __restrict__ V, int n) {
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e / n), y = (int)(e % n);
    if (x < y) {
      const double avg = 0.5 * (A[e] + A[(size_t)y * n + x]);
      A[e] = avg;
      A[(size_t)y * n + x] = avg;
    }
    V[e] = (x == y) ? 1.0 : 0.0;
  }
}

}  // namespace

// One sweep -- the flag reset and the n-1 rounds of two launches -- captured
// as a CUDA graph on a private stream: a round is a few microseconds of work,
// and launched one by one from the host the rounds would wait on the launches.
template <typename T>
static int capture_sweep(T* A, T* V, typename Pair2<T>::type* cs, int* rotated, int n, T tol,
                         T floor_abs, cudaGraphExec_t* exec) {
  const int h = n / 2;
  const long long napply = (long long)(h + kRowsA - 1) / kRowsA * h +
                           (long long)(n + kRowsV - 1) / kRowsV * h;
  const int agrid = (int)((napply + 255) / 256);
  cudaStream_t cap = nullptr;
  CORR_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  cudaError_t err = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (err == cudaSuccess) {
    cudaMemsetAsync(rotated, 0, sizeof(int), cap);
    for (int r = 0; r < n - 1; ++r) {
      jacobi_params<T><<<(h + 127) / 128, 128, 0, cap>>>(A, n, r, tol, floor_abs, cs, rotated);
      jacobi_apply<T><<<agrid, 256, 0, cap>>>(A, V, n, r, cs);
    }
    err = cudaStreamEndCapture(cap, &graph);
  }
  (void)cudaGetLastError();
  if (err == cudaSuccess) err = cudaGraphInstantiate(exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(cap);
  if (err != cudaSuccess) {
    set_error("Jacobi sweep graph: %s", cudaGetErrorString(err));
    return CORR_ERR_CUDA;
  }
  return CORR_OK;
}

// Cyclic sweeps on the padded n x n work matrix A (in place -> eigenvalues on
// the diagonal) accumulating the rotations into V (columns = eigenvectors),
// until a sweep rotates fewer than stop_below pairs or max_sweeps sweeps ran.
template <typename T>
static int jacobi_sweeps(corr_context* c, T* A, T* V, typename Pair2<T>::type* cs, int* rotated,
                         int n, T tol, T floor_abs, int max_sweeps, long long stop_below = 1) {
  if (n < 2) return CORR_OK;
  cudaStream_t s = c->stream;
  cudaGraphExec_t exec = nullptr;
  CORR_TRY(capture_sweep<T>(A, V, cs, rotated, n, tol, floor_abs, &exec));
  int status = CORR_OK;
  for (int sweeps = 0; sweeps < max_sweeps; ++sweeps) {
    int hrot = 0;
    cudaError_t err = cudaGraphLaunch(exec, s);
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(&hrot, rotated, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) {
      set_error("Jacobi sweep: %s", cudaGetErrorString(err));
      status = CORR_ERR_CUDA;
      break;
    }
    c->launches += 2LL * (n - 1);
    if (hrot < stop_below) break;
  }
  cudaGraphExecDestroy(exec);
  return status;
}

// The four n x n FP64 buffers and the small scratch of one eigendecomposition.
struct EigWork {
  double* buf[4];
  double2* cs;    // n pairs (also n FP32 pairs, and n doubles of host-bound scratch)
  double* part;   // 2 * kFrobBlocks doubles; its head doubles as the sweep flag
};
constexpr int kFrobBlocks = 1024;

static EigWork carve_eig(Carver& w, int n) {
  EigWork e;
  for (int b = 0; b < 4; ++b) e.buf[b] = static_cast<double*>(w.take((size_t)n * n * 8));
  e.cs = static_cast<double2*>(w.take((size_t)n * 16));
  e.part = static_cast<double*>(w.take((size_t)kFrobBlocks * 16));
  return e;
}

static int frob_norm2(corr_context* c, const double* A, int n, double* part, double* tot) {
  cudaStream_t s = c->stream;
  std::vector<double> hp((size_t)kFrobBlocks * 2);
  frob_kernel<<<kFrobBlocks, 256, 0, s>>>(A, n, part);
  CORR_CUDA(cudaGetLastError());
  CORR_CUDA(cudaMemcpyAsync(hp.data(), part, hp.size() * 8, cudaMemcpyDeviceToHost, s));
  CORR_CUDA(cudaStreamSynchronize(s));
  c->launches += 1;
  double t = 0;
  for (int k = 0; k < kFrobBlocks; ++k) t += hp[2 * k + 1];
  *tot = t;
  return CORR_OK;
}

static int gemm_nn(corr_context* c, const double* A, const double* B, double* C, int n, int ta,
                   double alpha, double beta) {
  GemmF64 g = gemm_args(A, B, C, n, n, n, n, n, n, ta, 0);
  g.alpha = alpha;
  g.beta = beta;
  CORR_TRY(gemm_f64(g, &c->dres->status, c->stream));
  c->launches += 1;
  return CORR_OK;
}

// Eigendecomposition of the symmetric padded n x n matrix in e.buf[0] (V not
// yet set).  On return *Aout holds the eigenvalues on its diagonal, *Vout the
// eigenvectors as columns, and *spare is an n x n buffer free for the caller.
// ||A||_F^2 = tot > 0.
static int eig_work(corr_context* c, const EigWork& e, int n, double tot, double** Aout,
                    double** Vout, double** spare) {
  cudaStream_t s = c->stream;
  const long long nn = (long long)n * n;
  const int ig = (int)std::min<long long>((nn + 255) / 256, 4096);
  int* rotated = reinterpret_cast<int*>(e.part);
  if (n < kMixedMin || !(tot > 0.0) || !std::isfinite(tot)) {
    symmetrize_and_identity<<<ig, 256, 0, s>>>(e.buf[0], e.buf[1], n);
    CORR_CUDA(cudaGetLastError());
    c->launches += 1;
    CORR_TRY(jacobi_sweeps<double>(c, e.buf[0], e.buf[1], e.cs, rotated, n, kRotTol, 0.0,
                                   kMaxSweeps));
    *Aout = e.buf[0];
    *Vout = e.buf[1];
    *spare = e.buf[2];
    return CORR_OK;
  }
  // 1. FP32 sweeps on A / 2^e in buf[3] (Af, Vf: n^2 floats each)
  int ex = 0;
  std::frexp(std::sqrt(tot), &ex);
  float* Af = reinterpret_cast<float*>(e.buf[3]);
  float* Vf = Af + nn;
  narrow_scaled<<<ig, 256, 0, s>>>(e.buf[0], n, std::ldexp(1.0, -ex), Af, Vf);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  CORR_TRY(jacobi_sweeps<float>(c, Af, Vf, reinterpret_cast<float2*>(e.cs), rotated, n,
                                kRotTol32, (float)(kFloor32 / n), kMaxSweeps32,
                                (long long)(n / 2) * (n - 1) / kStop32 + 1));
  // 2. Q = Vf in FP64, two Newton-Schulz steps Q <- 1.5 Q - 0.5 Q (Q^T Q)
  double* Q = e.buf[1];
  double* Qn = e.buf[3];
  widen<<<ig, 256, 0, s>>>(Vf, nn, Q);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  for (int it = 0; it < 2; ++it) {
    CORR_TRY(gemm_nn(c, Q, Q, e.buf[2], n, 1, 1.0, 0.0));
    CORR_CUDA(cudaMemcpyAsync(Qn, Q, (size_t)nn * 8, cudaMemcpyDeviceToDevice, s));
    CORR_TRY(gemm_nn(c, Q, e.buf[2], Qn, n, 0, -0.5, 1.5));
    std::swap(Q, Qn);
  }
  // Q is back in buf[1]; 3. A1 = Q^T (A Q) into buf[3], symmetrised; V1 = I in buf[0]
  CORR_TRY(gemm_nn(c, e.buf[0], Q, e.buf[2], n, 0, 1.0, 0.0));
  CORR_TRY(gemm_nn(c, Q, e.buf[2], e.buf[3], n, 1, 1.0, 0.0));
  symmetrize_and_identity<<<ig, 256, 0, s>>>(e.buf[3], e.buf[0], n);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  CORR_TRY(jacobi_sweeps<double>(c, e.buf[3], e.buf[0], e.cs, rotated, n, kRotTol, 0.0,
                                 kMaxSweeps));
  // 4. V = Q V1 into buf[2]
  CORR_TRY(gemm_nn(c, Q, e.buf[0], e.buf[2], n, 0, 1.0, 0.0));
  *Aout = e.buf[3];
  *Vout = e.buf[2];
  *spare = e.buf[0];
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
  const EigWork e = carve_eig(cw, n);
  int* dperm = static_cast<int*>(cw.take((size_t)m * 4));
  cudaStream_t s = c->stream;
  const int ig = (int)std::min<long long>(((long long)n * n + 255) / 256, 4096);
  jacobi_init<<<ig, 256, 0, s>>>(Ain, m, n, 0, e.buf[0]);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  double tot = 0.0, *A = nullptr, *V = nullptr, *spare = nullptr;
  CORR_TRY(frob_norm2(c, e.buf[0], n, e.part, &tot));
  CORR_TRY(eig_work(c, e, n, tot, &A, &V, &spare));
  double* dlam = reinterpret_cast<double*>(e.cs);  // n doubles of room
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
  return (size_t)4 * n * n * 8 + (size_t)n * 16 + (size_t)kFrobBlocks * 16 + (size_t)8 * 256;
}

int ri_inv_sqrt_device(corr_context* c, void* ws, const double* J, int m, double tol,
                       double* out, int* ncut) {
  const int n = m + (m & 1);
  Carver cw{ws, 0};
  const EigWork e = carve_eig(cw, n);
  cudaStream_t s = c->stream;
  const int ig = (int)std::min<long long>(((long long)n * n + 255) / 256, 4096);
  jacobi_init<<<ig, 256, 0, s>>>(J, m, n, 1, e.buf[0]);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  double tot = 0.0, *A = nullptr, *V = nullptr, *W = nullptr;
  CORR_TRY(frob_norm2(c, e.buf[0], n, e.part, &tot));
  if (!(tot > 0.0)) {
    set_error("RI metric is zero");
    return CORR_ERR_NOT_PD;
  }
  CORR_TRY(eig_work(c, e, n, tot, &A, &V, &W));
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
  double* df = reinterpret_cast<double*>(e.cs);  // n >= m doubles of room (n*16 bytes)
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
