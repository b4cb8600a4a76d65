// Pre-pass of the RI-MP2 precision form and the final energy reduction.
//
// The tensor cores' FP32 accumulator truncates every partial sum toward zero,
// which biases |(ia|jb)| low by ~1e-5 relative for naux ~ 1e3 when 16-bit
// hi/lo products are simply accumulated.  The precision form therefore makes
// every tensor-core partial sum an exact integer below 2^24:
//
//   B^Q_r = 2^(e_r) (s0 + s1/L + s2/L^2),   r = (i,a),  L = 2^(p+1),
//   s_k = integers in [-2^p, 2^p] (exact in FP16 and BF16), p = 6..8 chosen from naux,
//   e_r = ilogb(max_Q |B^Q_r|) - (p-1)  (one power-of-two scale per row).
//
// The energy kernel forms  acc_m = sum_{k+l=m} sum_Q s_k(ia) s_l(jb)  for
// m = 0, 1, 2 in separate TMEM accumulators; acc_0 and acc_1 stay exact
// (|acc| <= 2 K 2^(2p) <= 2^24), acc_2 enters at L^-2.  Representation error is
// ~2^-21 of the row maximum, round-to-nearest and unbiased.
//
// The diagonal elements (ia|ia) = sum_Q (B^Q_ia)^2 are all-positive sums that
// dominate the bias of any truncated scheme; they are formed here to FP64
// accuracy and substituted by the energy kernel.
//
// Scheme 1 (FP16 slices): two digits per element,
//
//   B^Q_r = 2^(e_r) (s0 + s1/L),   s0 = round(x), s1 = round(L (x - s0)),
//   x = B^Q_r 2^(-e_r),
//
// and four products per pair of rows into three accumulators,
//
//   acc_0 = s0.s0',  acc_1 = s0.s1' + s1.s0',  acc_2 = s1.s1',
//   x.x' = acc_0 + acc_1/L + acc_2/L^2   (exact for the two-digit values).
//
// Dropping the s1.s1' product (plain two-term hi/lo splitting) loses every
// product of two sub-digit elements and biases molecular energies, so it is
// kept.  (Karatsuba's identity would need three products, but a third plane
// s0 + s1 per operand: more operand bytes per product, and measured slower.)
// Each accumulator is a tensor-core sum of
// integer products, exact in FP32 when every partial sum stays within 2^24;
// by Cauchy-Schwarz that holds when ||s0||, ||s1|| <= 2^11.5 for every row
// (acc_1 <= 2 2^11.5 2^11.5), which the pre-pass enforces:
//   e_r: ||x|| <= 2^11.5 - sqrt(naux)/2 - 1 and max|x| <= 2^11 - 2^9 - 1
//        (so ||s0|| <= 2^11.5 - 1 and |s0| <= 2^11: exact in FP16);
//   L = 2^k, the largest k <= 10 such that for every row
//     L ||r|| + (1/2 + 2^-10) sqrt(naux) <= 2^11.5     (bounds ||s1||),
//   with r = x - s0 and c = ||r||^2 taken in a second pass over the row (FP32,
//   with a 2^-10 margin); |s1| <= L/2 <= 2^9.
// Digits come from the 20-bit fixed-point value X20 = round(x 2^20) (32-bit
// integer arithmetic on the IEEE fields): s0 = round(X20 / 2^20), r = X20 2^-20
// - s0, s1 = round(L r).  The diagonal sum_Q B^2 is the exact integer sum of
// floor(X20^2 / 2^10) (relative error ~1e-10).  Per element the pre-pass uses
// no FP64 instruction: GB300's FP64 pipe is ~2 operations per clock per SM.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <atomic>
#include <cmath>

#include "common.cuh"
#include "kernels.h"

namespace corr {

namespace {

// |x| as an ordered integer (IEEE bit pattern without the sign).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// smallest e with y 2^-e <= 1 (y > 0)
__device__ __forceinline__ int ceil_log2(double y) {
  int k;
  const double f = frexp(y, &k);  // y = f 2^k, f in [0.5, 1)
  return f == 0.5 ? k - 1 : k;
}

constexpr int kMaxLevelExp = 10;

// Per-call constants of the scheme-1 row statistics, from naux on the host.
// The reciprocals are inflated by 2^-40 relative (far above the few roundings
// of their computation), so every bound they enter stays conservative.
struct StatConsts {
  double sest_factor;  // 1 + 2^-16 + (naux + 32) 2^-23: the FP32 estimate's error margin
  double inv_t0sq;     // 1 / t0^2,  t0 = 2^11.5 - sqrt(naux)/2 - 1
  double inv_xmax;     // 1 / (2^11 - 2^9 - 1)
  double inv_tsq;      // 1 / T^2,   T = 2^11.5 - (1/2 + 2^-10) sqrt(naux)
};

StatConsts stat_consts(int naux) {
  const double up = 1.0 + 0x1p-40;
  const double sq = std::sqrt((double)naux);
  const double t0 = 2896.309375740099 - 0.5 * sq - 1.0;
  const double T = 2896.309375740099 - (0.5 + 0x1p-10) * sq;
  StatConsts k;
  k.sest_factor = 1.0 + 0x1p-16 + (double)(naux + 32) * 0x1p-23;
  k.inv_t0sq = up / (t0 * t0);
  k.inv_xmax = up / (2048.0 - 512.0 - 1.0);
  k.inv_tsq = up / (T * T);
  return k;
}

// round(b * 2^c) to nearest (ties away from zero) by 32-bit integer
// arithmetic on the IEEE-754 fields; exact whenever |b 2^c| < 2^31 (callers
// guarantee |b 2^c| < 2^31 - 1).  Zero and subnormal b map to 0 (their
// contribution lies far below the row scale).  With m the 53-bit significand,
// b 2^c = m 2^-(sh) and round = ((m >> (sh - 1)) + 1) >> 1, where
// m >> (sh - 1) < 2^32 because sh - 1 >= 21.
__device__ __forceinline__ int round_scaled32(double b, int c) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(b);
  const unsigned hi = (unsigned)(bits >> 32), lo = (unsigned)bits;
  const int E = (int)((hi >> 20) & 0x7ffu);
  const unsigned m21 = __funnelshift_l(lo, (hi & 0xfffffu) | 0x100000u, 11);  // m >> 21
  const unsigned sh = (unsigned)(1074 - E - c - 21);  // (sh - 1) - 21; "negative" = huge
  const unsigned t = sh < 32u ? (m21 >> sh) : 0u;
  const int X = (int)((t + 1u) >> 1);
  return E == 0 ? 0 : ((int)hi < 0 ? -X : X);
}

// Small integer (|v| < 2^22) to FP32 on the integer and FP32 pipes.
__device__ __forceinline__ float small_int_to_float(int v) {
  return __int_as_float(0x4b400000 + v) - 12582912.0f;
}

// Scheme-1 digits of one element from its 20-bit fixed-point value
// X20 = round(x 2^20) (|x| < 2^11): s0 = round(x) (ties up),
// r20 = X20 - s0 2^20, s1 = round(r20 2^(k - 20)) (ties up), k <= 10.
__device__ __forceinline__ void digits2(int X20, int k, int* s0, int* s1) {
  const int h = (X20 + (1 << 19)) >> 20;
  const int r20 = X20 - (h << 20);
  *s0 = h;
  *s1 = (r20 + (1 << (19 - k))) >> (20 - k);
}

// Pass-1 contribution of one element: the high word of |x| (the maximum of
// these bounds max |x| from above) and |x| truncated to FP32 from that word
// (20 significand bits: low by less than 2^-20 relative; 0 below 2^-126,
// FLT_MAX above).
__device__ __forceinline__ void pass1_elem(double x, unsigned* mhi, float* sf) {
  const unsigned h = (unsigned)((unsigned long long)__double_as_longlong(x) >> 32) & 0x7fffffffu;
  *mhi = h > *mhi ? h : *mhi;
  int t = (int)h - (896 << 20);
  t = t < 0 ? 0 : (t > 0x0fefffff ? 0x0fefffff : t);
  const float f = __int_as_float(t << 3);
  *sf = fmaf(f, f, *sf);
}

// Pass-2 statistics of a row at scale e (scheme 1): c = sum r20^2 (FP32)
// and the diagonal as the exact integer sum of floor(X20^2 / 2^10) (< 2^53 for
// any row the scale admits: ||x|| <= 2^11.5).
struct RowStats2 {
  float c = 0.f;
  unsigned long long d = 0;
};

__device__ __forceinline__ int pass2_elem_x(double x, int e, RowStats2& st) {
  const int X = round_scaled32(x, 20 - e);
  const int s0 = (X + (1 << 19)) >> 20;
  const float fr = small_int_to_float(X - (s0 << 20));
  st.c = fmaf(fr, fr, st.c);
  st.d += (unsigned long long)((long long)X * X) >> 10;
  return X;
}

__device__ __forceinline__ void pass2_elem(double x, int e, RowStats2& st) {
  (void)pass2_elem_x(x, e, st);
}

// ceil_log2 of y >= 0 from its IEEE fields (integer instructions only; the
// FP64 pipe is ~1/64 rate here): y = 1.m 2^(E - 1023) <= 2^c for the smallest
// c = E - 1023 (m == 0) or E - 1022; 0 for y == 0, as ceil_log2.
__device__ __forceinline__ int ceil_log2_bits(double y) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(y);
  const int E = (int)(u >> 52) & 0x7ff;
  if (E == 0) return u == 0 ? 0 : ceil_log2(y);  // subnormal: the general path
  return (u & 0xfffffffffffffull) == 0 ? E - 1023 : E - 1022;
}

// x 2^p for an integer-valued x >= 0 (exact by a power-of-two product when
// 2^p is a normal double, else through ldexp).
__device__ __forceinline__ double times_pow2(double x, int p) {
  if (p < -1022 || p > 1023) return ldexp(x, p);
  return x * __longlong_as_double((long long)(1023 + p) << 52);
}

// Row scale e_r of scheme 1 from the pass-1 results: ||x|| <= 2^11.5 -
// sqrt(naux)/2 - 1 (from the FP32 estimate with its error margin) and
// max|x| <= 2^11 - 2^9 - 1 (from the upper bound mhi + 1).  INT_MIN/4 for a
// row without normal elements.  The bounds are compared squared against
// reciprocals precomputed on the host and rounded up (StatConsts), so e_r is
// never below the smallest admissible scale; two FP64 products per row.
__device__ __forceinline__ int row_scale2(unsigned mhi, float sfl, const StatConsts& kc) {
  if ((mhi >> 20) == 0) return INT_MIN / 4;
  const double sest = (double)sfl * kc.sest_factor;
  const double mx = __longlong_as_double((long long)((unsigned long long)(mhi + 1u) << 32));
  const int c2 = ceil_log2_bits(sest * kc.inv_t0sq);  // sest / t0^2 <= 2^c2
  const int en = (c2 + 1) >> 1;                       // sqrt(sest) / t0 <= 2^en
  const int ec = ceil_log2_bits(mx * kc.inv_xmax);    // max|x| / (2^11 - 2^9 - 1) <= 2^ec
  return en > ec ? en : ec;
}

// Largest level exponent k (L = 2^k, 0 <= k <= 10) that keeps ||s1|| <= 2^11.5
// for a row with pass-2 statistics st, i.e. 2^k sqrt(C) + slack <= 2^11.5 with
// slack = (1/2 + 2^-10) sqrt(naux), or 4^k C <= T^2 with T = 2^11.5 - slack
// (0 when none does); also writes the row's diagonal sum_Q B^2.  The FP32 sum
// c is low by at most ~2^-19 relative: margin 2^-10.
__device__ __forceinline__ int row_level2(const RowStats2& st, int e, const StatConsts& kc,
                                          double* diag) {
  *diag = times_pow2((double)st.d, 2 * e - 30);
  if (st.c == 0.0f) return kMaxLevelExp;
  const double C = (double)st.c * (0x1p-40 * (1.0 + 0x1p-10));
  const int c = ceil_log2_bits(C * kc.inv_tsq);  // C / T^2 <= 2^c
  const int k = (-c) >> 1;                       // the largest k with 2k <= -c
  return k < 0 ? 0 : (k > kMaxLevelExp ? kMaxLevelExp : k);
}

// Row statistics are taken by blocks of 32 rows x QG Q-groups: for a fixed
// Q the 32 threads of a warp read 32 consecutive rows (coalesced), and every
// thread keeps kUnroll independent loads in flight.
constexpr int QG = 32;
constexpr int kUnroll = 4;

// Pass 1 over one row slice: max |B| (as IEEE bits) and sum B^2 (FP64).
__device__ __forceinline__ void row_pass1(const double* __restrict__ b, int naux, long long R,
                                          long long r, int ty, unsigned long long* mo,
                                          double* so) {
  unsigned long long m[kUnroll] = {};
  double s[kUnroll] = {};
  int q = ty;
  for (; q + (kUnroll - 1) * QG < naux; q += kUnroll * QG) {
    double x[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) x[u] = b[(long long)(q + u * QG) * R + r];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const unsigned long long ax = abs_bits(x[u]);
      m[u] = ax > m[u] ? ax : m[u];
      s[u] = fma(x[u], x[u], s[u]);
    }
  }
  for (; q < naux; q += QG) {
    const double x = b[(long long)q * R + r];
    const unsigned long long ax = abs_bits(x);
    m[0] = ax > m[0] ? ax : m[0];
    s[0] = fma(x, x, s[0]);
  }
  unsigned long long mm = m[0];
  double ss = s[0];
#pragma unroll
  for (int u = 1; u < kUnroll; ++u) {
    mm = m[u] > mm ? m[u] : mm;
    ss += s[u];
  }
  *mo = mm;
  *so = ss;
}

// Pass 1 of scheme 1 over one row slice (strided by QG in Q).
__device__ __forceinline__ void row_pass1_est(const double* __restrict__ b, int naux, long long R,
                                              long long r, int ty, unsigned* mo, float* so) {
  unsigned m[kUnroll] = {};
  float s[kUnroll] = {};
  int q = ty;
  for (; q + (kUnroll - 1) * QG < naux; q += kUnroll * QG) {
    double x[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) x[u] = b[(long long)(q + u * QG) * R + r];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) pass1_elem(x[u], &m[u], &s[u]);
  }
  for (; q < naux; q += QG) pass1_elem(b[(long long)q * R + r], &m[0], &s[0]);
  unsigned mm = m[0];
  float ss = s[0];
#pragma unroll
  for (int u = 1; u < kUnroll; ++u) {
    mm = m[u] > mm ? m[u] : mm;
    ss += s[u];
  }
  *mo = mm;
  *so = ss;
}

// Scheme 1 row statistics, two passes over global memory (the form for naux
// too large to stage a block's rows in shared memory): per row r, e_r from the
// first pass (row_scale2), then the pass-2 statistics (pass2_elem), the level
// exponent k_r (min-reduced into kglob) and the diagonal.  Block = 32 rows x QG
// Q-groups; partial results summed over the Q-groups in order.
__global__ void __launch_bounds__(32 * QG) rowstat2_kernel(const double* __restrict__ b,
                                                           int naux, long long R,
                                                           long long rbeg, long long rend,
                                                           int* __restrict__ erow,
                                                           double* __restrict__ diag, int* eref,
                                                           int* kglob, StatConsts kc) {
  __shared__ unsigned smax[QG][32];
  __shared__ float ssum[QG][32];
  __shared__ unsigned long long sd[QG][32];
  __shared__ int se[32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long r = rbeg + (long long)blockIdx.x * 32 + tx;
  unsigned m = 0;
  float sf = 0.f;
  if (r < rend) row_pass1_est(b, naux, R, r, ty, &m, &sf);
  smax[ty][tx] = m;
  ssum[ty][tx] = sf;
  __syncthreads();
  if (ty == 0) {
    int e = INT_MIN / 4;
    if (r < rend) {
      float sfl = sf;
      for (int k = 1; k < QG; ++k) {
        m = smax[k][tx] > m ? smax[k][tx] : m;
        sfl += ssum[k][tx];
      }
      e = row_scale2(m, sfl, kc);
      if (e > INT_MIN / 8) atomicMax(eref, e);
      erow[r] = e;
      if (e <= INT_MIN / 8) diag[r] = 0.0;
    }
    se[tx] = e;
  }
  __syncthreads();
  const int e = se[tx];
  const bool live = r < rend && e > INT_MIN / 8;
  RowStats2 st;
  if (live) {
#pragma unroll 4
    for (int q = ty; q < naux; q += QG) pass2_elem(b[(long long)q * R + r], e, st);
  }
  ssum[ty][tx] = st.c;
  sd[ty][tx] = st.d;
  __syncthreads();
  if (ty == 0 && live) {
    for (int k = 1; k < QG; ++k) {
      st.c += ssum[k][tx];
      st.d += sd[k][tx];
    }
    double dg;
    const int k = row_level2(st, e, kc, &dg);
    diag[r] = dg;
    atomicMin(kglob, k);
  }
}

// 8-byte asynchronous global -> shared copy (zero-filled when !valid).
__device__ __forceinline__ void cp_async8(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 8 : 0)
               : "memory");
}

// 4-byte asynchronous global -> shared copy (zero-filled when !valid).
__device__ __forceinline__ void cp_async4(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 4 : 0)
               : "memory");
}

// 16-byte asynchronous global -> shared copy of `bytes` (0, 8 or 16) source
// bytes, zero-filling the rest; both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" "cp.async.wait_group 0;\n" ::: "memory");
}

// Scheme 1 row statistics with each block's rows staged in shared memory:
// the same e_r, k_r and diagonal as rowstat2_kernel (the same per-element
// helpers), but B is read from HBM once (8-byte asynchronous copies, every
// element of the block in flight at once) and both passes run from shared
// memory.  Block = 512 threads on RB consecutive rows x all naux Q; shared
// image s[q * RB + row] = B^q_(r0 + row), thread t handles elements t + 512 k
// (row t % RB).  Sums over the threads of a row: lanes by shuffles in a fixed
// tree, then the 16 warps in order (deterministic).
constexpr int kStatThreads = 512;

template <int RB>
__global__ void __launch_bounds__(kStatThreads) rowstat2_smem_kernel(
    const double* __restrict__ b, int naux, long long R, long long rbeg, long long rend,
    int* __restrict__ erow,
    double* __restrict__ diag, int* eref, int* kglob, StatConsts kc, int* __restrict__ x20) {
  constexpr int NW = kStatThreads / 32;
  extern __shared__ __align__(16) double stage[];
  __shared__ unsigned long long w_d[NW][RB];
  __shared__ unsigned w_u[NW][RB];
  __shared__ float w_f[NW][RB];
  __shared__ int se[RB];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5, row = t & (RB - 1);
  const long long r0 = rbeg + (long long)blockIdx.x * RB;
  const int n = naux * RB;
  if ((R & 1) == 0 && (rbeg & 1) == 0 && ((uintptr_t)b & 15) == 0) {
    // rows in pairs: 16-byte copies (every row pair's address is 16-byte aligned)
    for (int k2 = t; 2 * k2 < n; k2 += kStatThreads) {
      const int k = 2 * k2, q = k / RB, rr = k & (RB - 1);
      const long long left = rend - (r0 + rr);  // rows left from this pair on
      const int bytes = left >= 2 ? 16 : (left == 1 ? 8 : 0);
      cp_async16(stage + k, bytes ? b + (long long)q * R + r0 + rr : b, bytes);
    }
  } else {
    for (int k = t; k < n; k += kStatThreads) {
      const int q = k / RB, rr = k & (RB - 1);
      const bool valid = r0 + rr < rend;
      cp_async8(stage + k, valid ? b + (long long)q * R + r0 + rr : b, valid);
    }
  }
  cp_async_wait_all();
  __syncthreads();

  // pass 1
  unsigned m = 0;
  float sf = 0.f;
  for (int k = t; k < n; k += kStatThreads) pass1_elem(stage[k], &m, &sf);
#pragma unroll
  for (int o = RB; o < 32; o <<= 1) {
    const unsigned mo = __shfl_xor_sync(0xffffffffu, m, o);
    m = mo > m ? mo : m;
    sf += __shfl_xor_sync(0xffffffffu, sf, o);
  }
  if (lane < RB) {
    w_u[warp][lane] = m;
    w_f[warp][lane] = sf;
  }
  __syncthreads();
  if (t < RB) {
    const long long r = r0 + t;
    m = 0;
    float sfl = 0.f;
    for (int w = 0; w < NW; ++w) {
      m = w_u[w][t] > m ? w_u[w][t] : m;
      sfl += w_f[w][t];
    }
    int e = INT_MIN / 4;
    if (r < rend) {
      e = row_scale2(m, sfl, kc);
      if (e > INT_MIN / 8) atomicMax(eref, e);
      erow[r] = e;
      if (e <= INT_MIN / 8) diag[r] = 0.0;
    }
    se[t] = e;
  }
  __syncthreads();

  // pass 2 at the row's scale; with x20, every row of the range also leaves
  // its fixed-point values X20 (0 for a row without normal elements) for the
  // slice, which then reads 4 bytes per element instead of 8
  const int e = se[row];
  const bool inrange = r0 + row < rend;
  const bool live = inrange && e > INT_MIN / 8;
  RowStats2 st;
  if (x20) {
    if (inrange) {
      // element k = t + 512 j is (q, row) = (k / RB, k % RB): q advances by 512 / RB per step
      int* xp = x20 + (long long)(t / RB) * R + r0 + row;
      const long long step = (long long)(kStatThreads / RB) * R;
      for (int k = t; k < n; k += kStatThreads, xp += step) {
        int X = 0;
        if (live) X = pass2_elem_x(stage[k], e, st);
        *xp = X;
      }
    }
  } else if (live) {
    for (int k = t; k < n; k += kStatThreads) pass2_elem(stage[k], e, st);
  }
#pragma unroll
  for (int o = RB; o < 32; o <<= 1) {
    st.c += __shfl_xor_sync(0xffffffffu, st.c, o);
    st.d += __shfl_xor_sync(0xffffffffu, st.d, o);
  }
  if (lane < RB) {  // (the row threads' reads of w_f precede the barrier above)
    w_f[warp][lane] = st.c;
    w_d[warp][lane] = st.d;
  }
  __syncthreads();
  if (t < RB && r0 + t < rend && se[t] > INT_MIN / 8) {
    RowStats2 tot;
    for (int w = 0; w < NW; ++w) {
      tot.c += w_f[w][t];
      tot.d += w_d[w][t];
    }
    double dg;
    const int k = row_level2(tot, se[t], kc, &dg);
    diag[r0 + t] = dg;
    atomicMin(kglob, k);
  }
}

// Row statistics over Q for each r (scheme 0): e_r, the FP64 diagonal
// sum_Q B^2, and the global maximum exponent (atomicMax).  The maximum is
// taken on the integer bit patterns (no FP64 compare); the diagonal needs one
// FP64 FMA per element.
__global__ void __launch_bounds__(32 * QG) rowstat_kernel(const double* __restrict__ b, int naux,
                                                          long long R, long long rbeg,
                                                          long long rend, int p,
                                                          int* __restrict__ erow,
                                                          double* __restrict__ diag, int* eref) {
  __shared__ unsigned long long smax[QG][32];
  __shared__ double ssum[QG][32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long r = rbeg + (long long)blockIdx.x * 32 + tx;
  unsigned long long m = 0;
  double s = 0.0;
  if (r < rend) row_pass1(b, naux, R, r, ty, &m, &s);
  smax[ty][tx] = m;
  ssum[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && r < rend) {
    for (int k = 1; k < QG; ++k) {
      m = smax[k][tx] > m ? smax[k][tx] : m;
      s += ssum[k][tx];
    }
    const int E = (int)(m >> 52);  // biased exponent of the row maximum
    const bool live = m != 0 && E != 0;
    const int e = live ? (E - 1023) - (p - 1) : INT_MIN / 4;
    erow[r] = e;
    diag[r] = s;
    if (live) atomicMax(eref, e);
  }
}

// Two small integers (exact in the format) as a packed FP16 (FMT 0) or BF16
// (FMT 1) pair, low half = v0.
template <int FMT>
__device__ __forceinline__ uint32_t pack16(int v0, int v1) {
  const float f0 = small_int_to_float(v0), f1 = small_int_to_float(v1);
  if (FMT == 0) {
    const __half2 h = __floats2half2_rn(f0, f1);
    return *reinterpret_cast<const uint32_t*>(&h);
  }
  const __nv_bfloat162 h = __floats2bfloat162_rn(f0, f1);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// B[Q][r] -> digit planes in the tiled layout of the energy kernels
// (kernels.h, slice_tile_offset): one 16 KB tile per (i, 64-Q block, plane,
// 128-row virtual tile), each stored exactly as the 128-byte-swizzled shared
// memory image the tensor-core descriptors read, so the kernels fetch a
// tile with one linear bulk copy.  Rows a >= nvir of the last tile and
// Q >= naux are zero.
//
// Block = 256 threads on a 64 (padded row) x 64 (Q) tile: 8-byte asynchronous
// copies coalesced along r (all 16 of a thread in flight at once), then each
// thread converts 16 consecutive Q of its row to the fixed-point integer of
// the row scale (round_scaled32) and to digits (a warp: 32 consecutive rows,
// conflict-free shared reads) and stores one 32-byte sector per plane.  Scheme 0 (levels):
// X = round(B 2^(2(p+1) - e_r)), s0 = round(X/L^2), s1 = round((X - s0 L^2)/L),
// s2 = remainder; scheme 1: X20 = round(B 2^(20 - e_r)) and digits2, planes
// s0, s1.  X20IN (scheme 1): the tile holds the X20 values the row statistics
// stored (4-byte copies of SliceWork::x20) instead of B, and no conversion runs.
template <int SCHEME, int FMT, bool X20IN>
__global__ void __launch_bounds__(256) slice_kernel(const double* __restrict__ b,
                                                    const int* __restrict__ x20, int naux,
                                                    int nocc, int nvir, int Qp, int p,
                                                    const int* __restrict__ erow,
                                                    const int* __restrict__ eref,
                                                    uint16_t* __restrict__ S,
                                                    const double* __restrict__ diag,
                                                    float* __restrict__ sc,
                                                    float2* __restrict__ dg, double* scale_out) {
  const int* kglob = eref + 1;
  __shared__ __align__(16) double tile[64][65];
  int(*tilei)[65] = reinterpret_cast<int(*)[65]>(&tile[0][0]);  // X20IN: X20 values
  const int t = threadIdx.x;
  const int ntiles = (nvir + 127) / 128, vp = ntiles * 128;
  const long long R = (long long)nocc * nvir, Rp = (long long)nocc * vp;
  // Blocks walk the rows from the last to the first, all Q of a row tile
  // together: the row-statistics pass just streamed B in ascending row order,
  // so the L2 still holds its last rows, and they are read first here.
  const long long lin = (long long)blockIdx.y * gridDim.x + blockIdx.x;
  const long long r0 = (long long)(gridDim.x - 1 - lin / gridDim.y) * 64;
  const int q0 = (int)(lin % gridDim.y) * 64;
  // thread's row (the same in both phases): padded row r0 + (t % 64)
  const int rl = t & 63;
  const long long rp = r0 + rl;
  const int i = (int)(rp / vp), a = (int)(rp % vp);
  const bool real = rp < Rp && a < nvir;
  const long long r = (long long)i * nvir + a;
#pragma unroll
  for (int k = t >> 6; k < 64; k += 4) {  // 16 asynchronous copies, all in flight
    const int q = q0 + k;
    const bool valid = real && q < naux;
    if (X20IN)
      cp_async4(&tilei[k][rl], valid ? x20 + (long long)q * R + r : x20, valid);
    else
      cp_async8(&tile[k][rl], valid ? b + (long long)q * R + r : b, valid);
  }
  cp_async_wait_all();
  __syncthreads();
  const int qc = (t >> 6) * 16;
  if (rp >= Rp || q0 + qc >= Qp) return;
  const int e = real ? erow[r] : INT_MIN / 4;
  const bool live = e > INT_MIN / 8;
  const int cs = (SCHEME == kSchemeDigits2 ? 20 : 2 * (p + 1)) - e;
  if (q0 == 0 && qc == 0) {
    // per-row FP32 factors for the energy kernel (the Q-block-0 tiles cover
    // every row once): sc_r = 2^(e_r - e_ref), dg_r = diag_r 2^(-2 e_ref), and
    // the global factors 2^(4 e_ref) and 1/L
    int er = *eref;
    if (er < -4000) er = 0;  // every row zero
    if (real) {
      sc[r] = live ? (float)ldexp(1.0, e - er) : 0.0f;
      const double d = ldexp(diag[r], -2 * er);
      const float dh = (float)d;
      dg[r] = make_float2(dh, (float)(d - (double)dh));
    }
    if (lin == 0 && t == 0) {
      scale_out[0] = ldexp(1.0, 4 * er);
      scale_out[1] = ldexp(1.0, -(SCHEME == kSchemeDigits2 ? eref[1] : p + 1));
    }
  }
  const int q = q0 + qc;
  constexpr int NPL = planes_for_scheme(SCHEME);
  const int nkb = Qp / kSliceQ, kb = q / kSliceQ, c0 = (q % kSliceQ) / 8;
  const size_t plane = kSliceTileElems;  // the planes of a tile are adjacent
  const size_t base = slice_tile_offset(0, i, kb, a / 128, nkb, ntiles, NPL);
  const int row = a % 128;
  int k = 0;
  if (SCHEME == kSchemeDigits2) {
    k = *kglob;  // no live row at all: every X is 0, any level works
    k = k < 0 ? 0 : (k > kMaxLevelExp ? kMaxLevelExp : k);
  }
  const int lb = p + 1;  // scheme 0: bits per level
#pragma unroll
  for (int h = 0; h < 2; ++h) {  // two 16-byte chunks (8 Q each) per plane
    uint32_t w0[4], w1[4], w2[4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      int d0[2], d1[2], d2[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int X = !live ? 0
                      : (X20IN ? tilei[qc + 8 * h + j + u][rl]
                               : round_scaled32(tile[qc + 8 * h + j + u][rl], cs));
        if (SCHEME == kSchemeDigits2) {
          digits2(X, k, &d0[u], &d1[u]);
          d2[u] = 0;
        } else {
          d0[u] = (X + (1 << (2 * lb - 1))) >> (2 * lb);
          const int rem = X - (d0[u] << (2 * lb));
          d1[u] = (rem + (1 << (lb - 1))) >> lb;
          d2[u] = rem - (d1[u] << lb);
        }
      }
      w0[j / 2] = pack16<FMT>(d0[0], d0[1]);
      w1[j / 2] = pack16<FMT>(d1[0], d1[1]);
      w2[j / 2] = pack16<FMT>(d2[0], d2[1]);
    }
    const size_t at = base + slice_chunk_offset(row, c0 + h);
    *reinterpret_cast<uint4*>(S + at) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
    *reinterpret_cast<uint4*>(S + plane + at) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
    if (NPL == 3)
      *reinterpret_cast<uint4*>(S + 2 * plane + at) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
  }
}

__global__ void energy_reduce_kernel(const double* __restrict__ part, int n,
                                     const double* __restrict__ scale, double* out) {
  __shared__ double s_os[256], s_ss[256];
  double os = 0.0, ss = 0.0, cos_ = 0.0, css = 0.0;
  for (int k = threadIdx.x; k < n; k += 256) {  // compensated, fixed order
    double y = part[2 * k] - cos_;
    double t = os + y;
    cos_ = (t - os) - y;
    os = t;
    y = part[2 * k + 1] - css;
    t = ss + y;
    css = (t - ss) - y;
    ss = t;
  }
  s_os[threadIdx.x] = os;
  s_ss[threadIdx.x] = ss;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s_os[threadIdx.x] += s_os[threadIdx.x + w];
      s_ss[threadIdx.x] += s_ss[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double sc = scale ? scale[0] : 1.0;
    double eos = s_os[0] * sc, ess = s_ss[0] * sc;
    out[0] = ess;
    out[1] = eos;
    out[2] = ess + eos;
    out[3] = ess / 3.0 + eos * 6.0 / 5.0;
  }
}

}  // namespace

int slice_bits_for(int Qp) {
  // Largest p with 2 * Qp * 2^(2p) <= 2^24, so acc_0 and acc_1 stay exact
  // integers for any data; at most 8, so every digit in [-2^p, 2^p] is an
  // exact BF16 (and FP16) value.  naux <= 2048 gives p >= 6 (21+ bits).
  int p = 8;
  while (p > 1 && (double)2 * Qp * (double)(1ll << (2 * p)) > 16777216.0) --p;
  return p;
}

// Dynamic shared memory of the staged row-statistics kernel: at most this
// many bytes per block (naux <= 1600 for 8 rows per block, 3200 for 4).
constexpr size_t kStatSmemMax = 100 * 1024;

// Raise the kernel's dynamic shared memory limit once per device (safe under
// stream capture: not a stream operation).
template <int RB>
static cudaError_t set_stat_smem() {
  static std::atomic<unsigned long long> done{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load() & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(rowstat2_smem_kernel<RB>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStatSmemMax);
  if (e == cudaSuccess) done.fetch_or(bit);
  return e;
}

// One bit coarser two-digit grid (L/2) for the error estimate of the
// precision form: k = max(k - 1, 0).
__global__ void coarsen_level_kernel(int* kglob) {
  const int k = *kglob;
  if (k > 0 && k <= kMaxLevelExp) *kglob = k - 1;
}

cudaError_t coarsen_level(SliceWork w, cudaStream_t s) {
  coarsen_level_kernel<<<1, 1, 0, s>>>(w.eref + 1);
  return cudaGetLastError();
}

cudaError_t reset_row_stats(SliceWork w, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(w.eref, 0x80, sizeof(int), s);  // very negative start
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(w.eref + 1, 0x7f, sizeof(int), s);  // level exponent: min-reduced
}

cudaError_t launch_row_stats(const double* b, int naux, int nocc, int nvir, int scheme, int p,
                             SliceWork w, long long rbeg, long long rend, cudaStream_t s) {
  const long long R = (long long)nocc * nvir, n = rend - rbeg;
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  if (scheme == kSchemeDigits2) {
    // rows staged in shared memory: 8 rows per block (two blocks per SM) up to
    // naux = 1600, 4 rows per block up to 3200, else the two-pass global form
    const size_t img8 = (size_t)naux * 8 * 8, img4 = (size_t)naux * 4 * 8;
    if (img8 <= kStatSmemMax) {
      e = set_stat_smem<8>();
      if (e != cudaSuccess) return e;
      rowstat2_smem_kernel<8><<<(unsigned)((n + 7) / 8), kStatThreads, img8, s>>>(
          b, naux, R, rbeg, rend, w.erow, w.diag, w.eref, w.eref + 1, stat_consts(naux), w.x20);
    } else if (img4 <= kStatSmemMax) {
      e = set_stat_smem<4>();
      if (e != cudaSuccess) return e;
      rowstat2_smem_kernel<4><<<(unsigned)((n + 3) / 4), kStatThreads, img4, s>>>(
          b, naux, R, rbeg, rend, w.erow, w.diag, w.eref, w.eref + 1, stat_consts(naux), w.x20);
    } else {
      rowstat2_kernel<<<(unsigned)((n + 31) / 32), dim3(32, QG), 0, s>>>(
          b, naux, R, rbeg, rend, w.erow, w.diag, w.eref, w.eref + 1, stat_consts(naux));
    }
  } else {
    rowstat_kernel<<<(unsigned)((n + 31) / 32), dim3(32, QG), 0, s>>>(b, naux, R, rbeg, rend, p,
                                                                     w.erow, w.diag, w.eref);
  }
  return cudaGetLastError();
}

bool row_stats_stage_x20(int naux) { return (size_t)naux * 4 * 8 <= kStatSmemMax; }

cudaError_t launch_slice_planes(const double* b, int naux, int nocc, int nvir, int Qp,
                                int scheme, int fmt, int p, SliceWork w, cudaStream_t s) {
  const long long Rp = (long long)nocc * ((nvir + 127) / 128) * 128;
  dim3 grid((unsigned)((Rp + 63) / 64), (unsigned)((Qp + 63) / 64));
  if (scheme == kSchemeDigits2 && w.x20 && row_stats_stage_x20(naux))
    slice_kernel<kSchemeDigits2, 0, true><<<grid, 256, 0, s>>>(
        b, w.x20, naux, nocc, nvir, Qp, p, w.erow, w.eref, w.S, w.diag, w.sc, w.dg, w.scale);
  else if (scheme == kSchemeDigits2)
    slice_kernel<kSchemeDigits2, 0, false><<<grid, 256, 0, s>>>(
        b, nullptr, naux, nocc, nvir, Qp, p, w.erow, w.eref, w.S, w.diag, w.sc, w.dg, w.scale);
  else if (fmt == 0)
    slice_kernel<kSchemeDigits3, 0, false><<<grid, 256, 0, s>>>(
        b, nullptr, naux, nocc, nvir, Qp, p, w.erow, w.eref, w.S, w.diag, w.sc, w.dg, w.scale);
  else
    slice_kernel<kSchemeDigits3, 1, false><<<grid, 256, 0, s>>>(
        b, nullptr, naux, nocc, nvir, Qp, p, w.erow, w.eref, w.S, w.diag, w.sc, w.dg, w.scale);
  return cudaGetLastError();
}

cudaError_t launch_slices(const double* b, int naux, int nocc, int nvir, int Qp, int scheme,
                          int fmt, int p, SliceWork w, cudaStream_t s) {
  cudaError_t e = reset_row_stats(w, s);
  if (e == cudaSuccess)
    e = launch_row_stats(b, naux, nocc, nvir, scheme, p, w, 0, (long long)nocc * nvir, s);
  if (e == cudaSuccess) e = launch_slice_planes(b, naux, nocc, nvir, Qp, scheme, fmt, p, w, s);
  return e;
}

// Fixed-order reduction of n {os, ss} pairs in one launch: block b sums the
// contiguous chunk [b chunk, (b+1) chunk) (compensated per thread, then a
// shared-memory tree) into scratch[2b], scratch[2b+1]; the last block to finish
// (each block takes a ticket after a fenced write of its sums; no block waits
// for another) forms the energy from the chunk sums in chunk order, exactly as
// energy_reduce_kernel does from per-CTA partials.  *ticket is 0 on entry.
__global__ void reduce_chunks_last_kernel(const double* __restrict__ part, int n, int chunk,
                                          double* scratch, unsigned* ticket,
                                          const double* __restrict__ scale, double* out) {
  __shared__ double s_os[256], s_ss[256];
  __shared__ bool last;
  const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  double os = 0.0, ss = 0.0, cos_ = 0.0, css = 0.0;
  for (int k = lo + threadIdx.x; k < hi; k += 256) {
    double y = part[2 * k] - cos_;
    double t = os + y;
    cos_ = (t - os) - y;
    os = t;
    y = part[2 * k + 1] - css;
    t = ss + y;
    css = (t - ss) - y;
    ss = t;
  }
  s_os[threadIdx.x] = os;
  s_ss[threadIdx.x] = ss;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s_os[threadIdx.x] += s_os[threadIdx.x + w];
      s_ss[threadIdx.x] += s_ss[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    scratch[2 * blockIdx.x] = s_os[0];
    scratch[2 * blockIdx.x + 1] = s_ss[0];
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int nb = (int)gridDim.x;
  os = ss = cos_ = css = 0.0;
  for (int k = threadIdx.x; k < nb; k += 256) {  // compensated, fixed order
    double y = __ldcg(&scratch[2 * k]) - cos_;
    double t = os + y;
    cos_ = (t - os) - y;
    os = t;
    y = __ldcg(&scratch[2 * k + 1]) - css;
    t = ss + y;
    css = (t - ss) - y;
    ss = t;
  }
  s_os[threadIdx.x] = os;
  s_ss[threadIdx.x] = ss;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s_os[threadIdx.x] += s_os[threadIdx.x + w];
      s_ss[threadIdx.x] += s_ss[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double sc = scale ? scale[0] : 1.0;
    const double eos = s_os[0] * sc, ess = s_ss[0] * sc;
    out[0] = ess;
    out[1] = eos;
    out[2] = ess + eos;
    out[3] = ess / 3.0 + eos * 6.0 / 5.0;
  }
}

int launch_unit_reduce(const double* partials, int n, const double* scale, double* out,
                       double* scratch, unsigned* ticket, cudaStream_t s) {
  if (n <= 2048) {
    energy_reduce_kernel<<<1, 256, 0, s>>>(partials, n, scale, out);
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
  }
  const int nb = kReduceBlocks, chunk = (n + nb - 1) / nb;
  reduce_chunks_last_kernel<<<nb, 256, 0, s>>>(partials, n, chunk, scratch, ticket, scale, out);
  return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

cudaError_t launch_energy_reduce(const double* partials, int n, const double* scale, double* out,
                                 cudaStream_t s) {
  energy_reduce_kernel<<<1, 256, 0, s>>>(partials, n, scale, out);
  return cudaGetLastError();
}

}  // namespace corr
