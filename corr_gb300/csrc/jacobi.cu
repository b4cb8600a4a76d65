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
//  1. A / 2^e (||A||_F in [2^(e-1), 2^e)) is rounded to FP32, zero-padded to
//     a multiple of 64 and swept by the FP32 block Jacobi method below (pairs
//     rotated while above 2^-20 sqrt(|a_pp a_qq|) and the absolute floor
//     2^-22 / n) until a sweep applies fewer than 1/32 of its inner rotations
//     (at most 30 sweeps); V0 is the product of those rotations.
//  2. V0 is widened to FP64 and made orthogonal to working accuracy by two
//     Newton-Schulz steps of the polar factor, Q <- Q (3 I - Q^T Q) / 2
//     (Higham, "Functions of Matrices", 8.3); ||Q^T Q - I|| goes from the
//     FP32 level (~1e-5) to ~1e-10 and then to rounding level.
//  3. A1 = Q^T A Q (FP64 GEMMs, then symmetrised) is diagonal up to the FP32
//     residual, and the FP64 sweeps above diagonalise it: A1 = V1 L V1^T in
//     about six sweeps (two of them full) instead of fifteen or more.
//  4. V = Q V1.
// Every FP64 step is a similarity by an orthogonal matrix accurate to FP64
// rounding, so the eigenvalues and vectors carry FP64 errors, as the plain
// FP64 sweeps do; only the starting point of the FP64 sweeps comes from FP32.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
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

// Element (x, y) of the symmetric work matrix: the FP64 sweeps keep and
// update its upper triangle only.
__device__ __forceinline__ size_t sym_at(int x, int y, int n) {
  return x < y ? (size_t)x * n + y : (size_t)y * n + x;
}

constexpr double kRotTol = 1e-15;          // FP64 sweeps: relative threshold
constexpr float kRotTol32 = 0x1p-20f;      // FP32 sweeps: relative threshold
constexpr double kFloor32 = 0x1p-22;       // FP32 sweeps: absolute floor x n (||A||_F ~ 1)
constexpr int kMaxSweeps = 40, kMaxSweeps32 = 30;
constexpr int kStop32 = 32;                // FP32 sweeps end below 1/32 of the inner rotations
constexpr int kMixedMin = 64;              // padded order from which the FP32 sweeps run first

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
    const T app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q], apq = A[sym_at(p, q, n)];
    T c = 1, s = 0;
    const T mag = fabs(apq);
    // |a_pq| > tol sqrt|a_pp a_qq| in squared form (no square root for the pairs
    // that stay: FP64 arithmetic is a long dependent chain here)
    if (mag * mag > (tol * tol) * fabs(app * aqq) && mag > floor_abs) {
      rot = true;
      const T tau = (aqq - app) / (T(2) * apq);
      const T at = fabs(tau);
      if (at > T(134217728)) {
        // |tau| > 2^27: t = sign / (2 |tau|) to within rounding, t^2 < 2^-56, so
        // (c, s) = (1, t) is orthogonal to working precision
        s = (tau >= T(0) ? T(0.5) : T(-0.5)) / at;
      } else {
        const T t = (tau >= T(0) ? T(1) : T(-1)) / (at + sqrt(T(1) + tau * tau));
        c = T(1) / sqrt(T(1) + t * t);
        s = t * c;
      }
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
// {p_l, q_l} for the row pairs k = kb kRowsA .. with k <= l -- A is symmetric,
// block (l, k) is the transpose of block (k, l), and every element is kept
// once, in the upper triangle (sym_at); the diagonal block k == l stores its
// off-diagonal element twice, the same value from the same thread.  Thread
// (xb, l) of the V update: columns {p_l, q_l} of kRowsV rows.  Every load of a thread is
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
      on[i] = k < (int)h && k <= l;
      a[i] = on[i] ? cs[k] : b;
      on[i] = on[i] && !(a[i].y == T(0) && b.y == T(0));
    }
    T x[kRowsA][4];
#pragma unroll
    for (int i = 0; i < kRowsA; ++i) {
      if (on[i]) {
        x[i][0] = A[sym_at(p[i], u, n)];
        x[i][1] = A[sym_at(p[i], w, n)];
        x[i][2] = A[sym_at(q[i], u, n)];
        x[i][3] = A[sym_at(q[i], w, n)];
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
          A[sym_at(p[i], u, n)] = fma(-b.y, y01, y00);
          A[sym_at(p[i], w, n)] = fma(b.y, y00, y01);
          A[sym_at(q[i], u, n)] = fma(-b.y, y11, y10);
          A[sym_at(q[i], w, n)] = fma(b.y, y10, y11);
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
        A[sym_at(p[i], u, n)] = y00 * b.x - y01 * b.y;
        A[sym_at(p[i], w, n)] = y00 * b.y + y01 * b.x;
        A[sym_at(q[i], u, n)] = y10 * b.x - y11 * b.y;
        A[sym_at(q[i], w, n)] = y10 * b.y + y11 * b.x;
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

// ---------------------------------------------------------------------------
// FP32 stage as a two-sided block Jacobi method (Golub & Van Loan, block
// Jacobi with the same round-robin ordering, on blocks of kBlk indices): the
// padded order np is a multiple of 2 kBlk, the m = np / kBlk index blocks are
// paired as the scalar indices are, and a round
//   1. diagonalises, for each block pair (I, J), the 2kBlk x 2kBlk matrix
//      A[I+J, I+J] approximately by one cyclic Jacobi sweep in shared memory
//      (same rotation formula and threshold as above), giving U_IJ;
//   2. applies all U at once: A[I+J, K+L] <- U_IJ^T A[I+J, K+L] U_KL and
//      V[:, K+L] <- V[:, K+L] U_KL, as 64 x 64 tile products.
// A sweep is m-1 rounds instead of n-1, and the work of a round is a dense
// product rather than n/2 dependent 2x2 rotations, so the FP32 stage is no
// longer bound by the latency of 1500 rounds per sweep.
// ---------------------------------------------------------------------------
constexpr int kBlk = 32, kBlk2 = 64, kSLd = 65;

__device__ __forceinline__ int block_row(int I, int J, int x) {
  return x < kBlk ? I * kBlk + x : J * kBlk + (x - kBlk);
}

// CTA t (1024 threads): block pair t of round r.  U_t (64 x 64, row-major)
// -> Ug + t 4096; *rotated += the rotations applied.  Thread x owns the 2x2
// block (x / 32, x % 32) of S and the pairs x % 32 of rows x / 32 and
// x / 32 + 32 of U, so an inner round is one dependent step per thread.  The
// FP32 stage only has to come close: its rotations are formed with fast
// division and reciprocal square root, and the FP64 steps after it restore
// orthogonality.
constexpr int kInnerThreads = 1024;

__global__ void __launch_bounds__(kInnerThreads) block_inner(const float* __restrict__ Af, int np,
                                                             int r, float tol, float floor_abs,
                                                             float* __restrict__ Ug,
                                                             int* __restrict__ rotated) {
  __shared__ float S[kBlk2 * kSLd];
  __shared__ float U[kBlk2 * kSLd];
  __shared__ float2 cs[kBlk];
  __shared__ unsigned char pt[kBlk2 - 1][kBlk][2];  // pair table of the 63 inner rounds
  const int m = np / kBlk;
  const int tid = threadIdx.x;
  int I, J;
  round_pair(m, r, blockIdx.x, &I, &J);
  for (int e = tid; e < kBlk2 * kBlk2; e += kInnerThreads) {
    const int x = e / kBlk2, y = e % kBlk2;
    S[x * kSLd + y] = Af[(size_t)block_row(I, J, x) * np + block_row(I, J, y)];
    U[x * kSLd + y] = (x == y) ? 1.0f : 0.0f;
  }
  for (int e = tid; e < (kBlk2 - 1) * kBlk; e += kInnerThreads) {
    int p, q;
    round_pair(kBlk2, e / kBlk, e % kBlk, &p, &q);
    pt[e / kBlk][e % kBlk][0] = (unsigned char)p;
    pt[e / kBlk][e % kBlk][1] = (unsigned char)q;
  }
  __syncthreads();
  const float tol2 = tol * tol, floor2 = floor_abs * floor_abs;
  const int k = tid / kBlk, l = tid % kBlk;  // S block (k, l); U rows k, k + 32, pair l
  int rot = 0;
  for (int rr = 0; rr < kBlk2 - 1; ++rr) {
    if (tid < kBlk) {
      const int p = pt[rr][tid][0], q = pt[rr][tid][1];
      const float app = S[p * kSLd + p], aqq = S[q * kSLd + q], apq = S[p * kSLd + q];
      float c = 1.0f, sn = 0.0f;
      const float a2 = apq * apq;
      if (a2 > tol2 * fabsf(app * aqq) && a2 > floor2) {
        ++rot;
        const float tau = __fdividef(aqq - app, 2.0f * apq);
        const float t = __fdividef(copysignf(1.0f, tau), fabsf(tau) + sqrtf(1.0f + tau * tau));
        c = rsqrtf(1.0f + t * t);
        sn = t * c;
        // one Newton step on c^2 + s^2 = 1: the approximate reciprocal square
        // root is biased, and its error would compound over the ~10^4
        // rotations that reach every index
        const float f = 1.5f - 0.5f * (c * c + sn * sn);
        c *= f;
        sn *= f;
      }
      cs[tid] = make_float2(c, sn);
    }
    __syncthreads();
    const float2 a = cs[k], b = cs[l];
    const int p = pt[rr][k][0], q = pt[rr][k][1], u = pt[rr][l][0], w = pt[rr][l][1];
    float* Sp = S + p * kSLd;
    float* Sq = S + q * kSLd;
    float* U0 = U + k * kSLd;
    float* U1 = U + (k + kBlk) * kSLd;
    const bool doS = !(a.y == 0.0f && b.y == 0.0f), doU = b.y != 0.0f;
    float x00 = 0, x01 = 0, x10 = 0, x11 = 0, v0u = 0, v0w = 0, v1u = 0, v1w = 0;
    if (doS) {
      x00 = Sp[u];
      x01 = Sp[w];
      x10 = Sq[u];
      x11 = Sq[w];
    }
    if (doU) {
      v0u = U0[u];
      v0w = U0[w];
      v1u = U1[u];
      v1w = U1[w];
    }
    if (doS) {
      const float y00 = a.x * x00 - a.y * x10, y01 = a.x * x01 - a.y * x11;
      const float y10 = a.y * x00 + a.x * x10, y11 = a.y * x01 + a.x * x11;
      Sp[u] = y00 * b.x - y01 * b.y;
      Sp[w] = y00 * b.y + y01 * b.x;
      Sq[u] = y10 * b.x - y11 * b.y;
      Sq[w] = y10 * b.y + y11 * b.x;
    }
    if (doU) {
      U0[u] = b.x * v0u - b.y * v0w;
      U0[w] = b.y * v0u + b.x * v0w;
      U1[u] = b.x * v1u - b.y * v1w;
      U1[w] = b.y * v1u + b.x * v1w;
    }
    __syncthreads();
  }
  float* Ut = Ug + (size_t)blockIdx.x * kBlk2 * kBlk2;
  for (int e = tid; e < kBlk2 * kBlk2; e += kInnerThreads)
    Ut[e] = U[(e / kBlk2) * kSLd + e % kBlk2];
  if (tid < 32) {
    for (int o = 16; o > 0; o >>= 1) rot += __shfl_xor_sync(0xffffffffu, rot, o);
    if (tid == 0 && rot) atomicAdd(rotated, rot);
  }
}

// acc[i][j] += sum_k L[k][ri + i] R[k][rj + j]  (L transposed)  or
// acc[i][j] += sum_k L[ri + i][k] R[k][rj + j]  (L as is), 64 x 64 operands.
template <bool LT>
__device__ __forceinline__ void tile_mm(const float* __restrict__ L, const float* __restrict__ R,
                                        int ri, int rj, float (&acc)[4][4]) {
#pragma unroll 8
  for (int k = 0; k < kBlk2; ++k) {
    float l4[4];
    if (LT) {
      const float4 v = *reinterpret_cast<const float4*>(L + k * kBlk2 + ri);
      l4[0] = v.x; l4[1] = v.y; l4[2] = v.z; l4[3] = v.w;
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) l4[i] = L[(ri + i) * kBlk2 + k];
    }
    const float4 r4 = *reinterpret_cast<const float4*>(R + k * kBlk2 + rj);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      acc[i][0] = fmaf(l4[i], r4.x, acc[i][0]);
      acc[i][1] = fmaf(l4[i], r4.y, acc[i][1]);
      acc[i][2] = fmaf(l4[i], r4.z, acc[i][2]);
      acc[i][3] = fmaf(l4[i], r4.w, acc[i][3]);
    }
  }
}

// CTAs [0, (m/2)^2): tile (s, t) of A <- U_s^T A[I_s+J_s, I_t+J_t] U_t;
// CTAs [(m/2)^2, (m/2)^2 + (np/64)(m/2)): rows 64 rb .. of V[:, I_t+J_t] <- . U_t.
// Each tile is owned by one CTA, so the update is in place.
__global__ void __launch_bounds__(256) block_apply(float* __restrict__ Af, float* __restrict__ Vf,
                                                   int np, int r,
                                                   const float* __restrict__ Ug) {
  __shared__ __align__(16) float X[kBlk2 * kBlk2];
  __shared__ __align__(16) float Ls[kBlk2 * kBlk2];
  __shared__ __align__(16) float Rs[kBlk2 * kBlk2];
  const int m = np / kBlk, h = m / 2;
  const int cta = blockIdx.x;
  const bool onA = cta < h * h;
  int s, t, rb = 0;
  if (onA) {
    s = cta / h;
    t = cta % h;
  } else {
    const int j = cta - h * h;
    rb = j / h;
    t = j % h;
    s = 0;
  }
  int It, Jt, Is = 0, Js = 0;
  round_pair(m, r, t, &It, &Jt);
  if (onA) round_pair(m, r, s, &Is, &Js);
  float* M = onA ? Af : Vf;
  const int ri = (threadIdx.x >> 4) * 4, rj = (threadIdx.x & 15) * 4;
  // load the 64 x 64 tile (rows: I_s+J_s or 64 rb .., cols: I_t+J_t) and U_t (and U_s)
  for (int e = threadIdx.x; e < kBlk2 * kBlk2 / 4; e += blockDim.x) {
    const int x = e / (kBlk2 / 4), y4 = (e % (kBlk2 / 4)) * 4;
    const int gx = onA ? block_row(Is, Js, x) : rb * kBlk2 + x;
    const int gy = block_row(It, Jt, y4);
    *reinterpret_cast<float4*>(X + x * kBlk2 + y4) =
        *reinterpret_cast<const float4*>(M + (size_t)gx * np + gy);
    *reinterpret_cast<float4*>(Rs + x * kBlk2 + y4) =
        *reinterpret_cast<const float4*>(Ug + (size_t)t * kBlk2 * kBlk2 + x * kBlk2 + y4);
    if (onA)
      *reinterpret_cast<float4*>(Ls + x * kBlk2 + y4) =
          *reinterpret_cast<const float4*>(Ug + (size_t)s * kBlk2 * kBlk2 + x * kBlk2 + y4);
  }
  __syncthreads();
  float acc[4][4] = {};
  if (onA) {
    tile_mm<true>(Ls, X, ri, rj, acc);  // Y = U_s^T X
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i)
      *reinterpret_cast<float4*>(X + (ri + i) * kBlk2 + rj) =
          make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
  }
  tile_mm<false>(X, Rs, ri, rj, acc);  // Z = Y U_t (or X U_t)
  for (int i = 0; i < 4; ++i) {
    const int gx = onA ? block_row(Is, Js, ri + i) : rb * kBlk2 + ri + i;
    const int gy = block_row(It, Jt, rj);
    *reinterpret_cast<float4*>(M + (size_t)gx * np + gy) =
        make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
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

// Af = A * scale rounded to FP32 and zero-padded to np x np, Vf = identity.
__global__ void narrow_scaled(const double* __restrict__ A, int n, int np, double scale,
                              float* __restrict__ Af, float* __restrict__ Vf) {
  const long long nn = (long long)np * np;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e / np), y = (int)(e % np);
    Af[e] = (x < n && y < n) ? (float)(A[(size_t)x * n + y] * scale) : 0.0f;
    Vf[e] = (x == y) ? 1.0f : 0.0f;
  }
}

// Q (n x n) = the leading n x n block of Vf (np x np), widened to FP64.
__global__ void widen(const float* __restrict__ Vf, int np, int n, double* __restrict__ Q) {
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x)
    Q[e] = (double)Vf[(size_t)(e / n) * np + e % n];
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

// A sweep -- the counter reset and its rounds -- is captured as a CUDA graph
// on a private stream and replayed once per sweep: a round is a few
// microseconds of work, and launched one by one from the host the rounds
// would wait on the launches.
template <typename F>
static int capture_graph(F&& enqueue, cudaGraphExec_t* exec) {
  cudaStream_t cap = nullptr;
  CORR_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  cudaError_t err = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (err == cudaSuccess) {
    enqueue(cap);
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

// The context's instantiated sweep graph for (kind, n, buffers), captured by
// `enqueue` on a miss (the oldest of kSweepGraphs entries is replaced).
template <typename F>
static int sweep_graph(corr_context* c, int kind, int n, const void* const (&ptr)[5], F&& enqueue,
                       cudaGraphExec_t* exec) {
  for (auto& g : c->sweep_graph) {
    bool same = g.exec && g.kind == kind && g.n == n;
    for (int k = 0; same && k < 5; ++k) same = g.ptr[k] == ptr[k];
    if (same) {
      *exec = g.exec;
      return CORR_OK;
    }
  }
  CORR_TRY(capture_graph(enqueue, exec));
  auto& g = c->sweep_graph[c->sweep_graph_next];
  c->sweep_graph_next = (c->sweep_graph_next + 1) % corr_context::kSweepGraphs;
  if (g.exec) cudaGraphExecDestroy(g.exec);  // its last launch was synchronised
  g.kind = kind;
  g.n = n;
  for (int k = 0; k < 5; ++k) g.ptr[k] = ptr[k];
  g.exec = *exec;
  return CORR_OK;
}

// Replays the sweep graph until a sweep rotates fewer than stop_below pairs
// (the count the sweep leaves in *rotated) or max_sweeps sweeps ran.
static int run_sweeps(corr_context* c, cudaGraphExec_t exec, const int* rotated, int max_sweeps,
                      long long stop_below, long long launches_per_sweep) {
  cudaStream_t s = c->stream;
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
    c->launches += launches_per_sweep;
    if (hrot < stop_below) break;
  }
  return status;
}

// Cyclic sweeps on the padded n x n work matrix A (in place -> eigenvalues on
// the diagonal) accumulating the rotations into V (columns = eigenvectors),
// until a sweep rotates no pair or max_sweeps sweeps ran.
template <typename T>
static int jacobi_sweeps(corr_context* c, T* A, T* V, typename Pair2<T>::type* cs, int* rotated,
                         int n, T tol, T floor_abs, int max_sweeps) {
  if (n < 2) return CORR_OK;
  const int h = n / 2;
  const long long napply = (long long)(h + kRowsA - 1) / kRowsA * h +
                           (long long)(n + kRowsV - 1) / kRowsV * h;
  const int agrid = (int)((napply + 255) / 256);
  cudaGraphExec_t exec = nullptr;
  static_assert(sizeof(T) == 8, "the FP64 sweep graphs are cached as kind 0");
  const void* const key[5] = {A, V, cs, rotated, nullptr};
  CORR_TRY(sweep_graph(
      c, 0, n, key,
      [&](cudaStream_t cap) {
        cudaMemsetAsync(rotated, 0, sizeof(int), cap);
        for (int r = 0; r < n - 1; ++r) {
          jacobi_params<T><<<(h + 127) / 128, 128, 0, cap>>>(A, n, r, tol, floor_abs, cs, rotated);
          jacobi_apply<T><<<agrid, 256, 0, cap>>>(A, V, n, r, cs);
        }
      },
      &exec));
  return run_sweeps(c, exec, rotated, max_sweeps, 1, 2LL * (n - 1));
}

// FP32 block sweeps on the np x np matrices Af, Vf (np a multiple of 64),
// ending when a sweep applies fewer than 1/kStop32 of its inner rotations.
static int block_sweeps(corr_context* c, float* Af, float* Vf, float* Ug, int* rotated, int np,
                        float tol, float floor_abs) {
  const int m = np / kBlk, h = m / 2;
  const int agrid = h * h + (np / kBlk2) * h;
  cudaGraphExec_t exec = nullptr;
  // the graph bakes in the absolute floor (2^-22 / n: orders sharing np differ in it)
  uint32_t floor_bits = 0;
  std::memcpy(&floor_bits, &floor_abs, sizeof floor_bits);
  const void* const key[5] = {Af, Vf, Ug, rotated,
                              reinterpret_cast<const void*>((uintptr_t)floor_bits + 1)};
  CORR_TRY(sweep_graph(
      c, 1, np, key,
      [&](cudaStream_t cap) {
        cudaMemsetAsync(rotated, 0, sizeof(int), cap);
        for (int r = 0; r < m - 1; ++r) {
          block_inner<<<h, kInnerThreads, 0, cap>>>(Af, np, r, tol, floor_abs, Ug, rotated);
          block_apply<<<agrid, 256, 0, cap>>>(Af, Vf, np, r, Ug);
        }
      },
      &exec));
  const long long visits = (long long)(m - 1) * h * (kBlk2 - 1) * kBlk;
  return run_sweeps(c, exec, rotated, kMaxSweeps32, visits / kStop32 + 1, 2LL * (m - 1));
}

// The four n x n FP64 buffers, the FP32 block-sweep matrices and the small
// scratch of one eigendecomposition.
struct EigWork {
  double* buf[4];
  float* f32;     // Af, Vf (np x np each) and the U of one round (np/64 x 64 x 64)
  double2* cs;    // n pairs (also n doubles of host-bound scratch)
  double* part;   // 2 * kFrobBlocks doubles; its head doubles as the sweep counter
};
constexpr int kFrobBlocks = 1024;

static int padded64(int n) { return (n + kBlk2 - 1) / kBlk2 * kBlk2; }

static size_t f32_floats(int n) {
  const size_t np = (size_t)padded64(n);
  return 2 * np * np + np * kBlk2;
}

static EigWork carve_eig(Carver& w, int n) {
  EigWork e;
  for (int b = 0; b < 4; ++b) e.buf[b] = static_cast<double*>(w.take((size_t)n * n * 8));
  e.f32 = n >= kMixedMin ? static_cast<float*>(w.take(f32_floats(n) * 4)) : nullptr;
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
  // 1. FP32 block sweeps on A / 2^e, zero-padded to np (a multiple of 64)
  int ex = 0;
  std::frexp(std::sqrt(tot), &ex);
  const int np = padded64(n);
  const long long npp = (long long)np * np;
  float* Af = e.f32;
  float* Vf = Af + npp;
  float* Ug = Vf + npp;
  const int pg = (int)std::min<long long>((npp + 255) / 256, 4096);
  narrow_scaled<<<pg, 256, 0, s>>>(e.buf[0], n, np, std::ldexp(1.0, -ex), Af, Vf);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  CORR_TRY(block_sweeps(c, Af, Vf, Ug, rotated, np, kRotTol32, (float)(kFloor32 / n)));
  // 2. Q = Vf[:n, :n] in FP64, two Newton-Schulz steps Q <- 1.5 Q - 0.5 Q (Q^T Q)
  double* Q = e.buf[1];
  double* Qn = e.buf[3];
  widen<<<ig, 256, 0, s>>>(Vf, np, n, Q);
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
size_t ns_workspace_bytes(int m);
int ri_inv_sqrt_ns(corr_context* c, void* ws, const double* J, int m, double tol, double* out,
                   bool* done);

size_t jacobi_workspace_bytes(int m) {
  const int n = m + (m & 1);
  return std::max((size_t)4 * n * n * 8 + (n >= kMixedMin ? f32_floats(n) * 4 : 0) +
                      (size_t)n * 16 + (size_t)kFrobBlocks * 16 + (size_t)8 * 256,
                  ns_workspace_bytes(m));
}

// J^-1/2 with the reference's cutoff.  try_ns: first the certificate and, if
// nothing can be cut, the Newton-Schulz iteration (invsqrt.cu); otherwise
// (or if it does not converge) the eigendecomposition below.
int ri_inv_sqrt_device(corr_context* c, void* ws, const double* J, int m, double tol,
                       double* out, int* ncut, bool try_ns) {
  if (try_ns && m >= kMixedMin) {
    bool done = false;
    CORR_TRY(ri_inv_sqrt_ns(c, ws, J, m, tol, out, &done));
    if (done) {
      if (ncut) *ncut = 0;
      return CORR_OK;
    }
  }
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
