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
// dominate the bias of any truncated scheme; they are formed here in FP64 and
// substituted by the energy kernel.
//
// Scheme 1 (FP16 slices, Karatsuba): two digits per element,
//
//   B^Q_r = 2^(e_r) (s0 + s1/L),   s0 = round(x), s1 = round(L (x - s0)),
//   x = B^Q_r 2^(-e_r),  u = s0 + s1,
//
// and three products per pair of rows (Karatsuba's identity for the cross term),
//
//   P0 = s0.s0',  Pm = u.u',  P2 = s1.s1',
//   x.x' = P0 + (Pm - P0 - P2)/L + P2/L^2   (exact for the two-digit values).
//
// Dropping the s1.s1' product (plain two-term hi/lo splitting) loses every
// product of two sub-digit elements and biases molecular energies; the
// Karatsuba form keeps it at the cost of three products, not four.  Each of
// P0, Pm, P2 is a tensor-core sum of integer products, exact in FP32 when
// every partial sum stays below 2^24; by Cauchy-Schwarz that holds when
// ||s0||, ||u||, ||s1|| <= 2^12 for every row, which the pre-pass enforces:
//   e_r: ||x|| <= 2^11.5 - sqrt(naux)/2 - 1 and max|x| <= 2^11 - 2^9 - 1;
//   L = 2^k, the largest k <= 10 such that for every row
//     ||s0 + L r|| + (1/2 + 2^-10) sqrt(naux) <= 2^12   (bounds ||u||),
//     L ||r|| + (1/2 + 2^-10) sqrt(naux) <= 2^12        (bounds ||s1||),
//     max|s0| + L/2 <= 2^11                            (u exact in FP16),
//   with r = x - s0 and the row sums a = ||s0||^2, b = s0.r, c = ||r||^2 taken
//   in a second pass over the row (a exact, b and c with a 2^-10 margin).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"
#include "kernels.h"

namespace corr {

namespace {

// |x| as an ordered integer (IEEE bit pattern without the sign).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// round(b * 2^k) to nearest (ties away from zero) by integer arithmetic on the
// IEEE-754 fields; exact for every |result| < 2^31.  Zero and subnormal b map
// to 0 (their contribution lies far below the row scale).
__device__ __forceinline__ int round_scaled(double b, int k) {
  const long long bits = __double_as_longlong(b);
  const int E = (int)((bits >> 52) & 0x7ff);
  if (E == 0) return 0;
  const long long m = (bits & 0xfffffffffffffll) | (1ll << 52);
  const int sh = 1075 - E - k;  // value = m * 2^-sh
  long long X;
  if (sh <= 0) X = m << (-sh > 10 ? 10 : -sh);  // not reached for |b| <= row max
  else if (sh > 62) X = 0;
  else X = (m + (1ll << (sh - 1))) >> sh;
  return bits < 0 ? -(int)X : (int)X;
}

// round(b * 2^k) as a 64-bit integer (same rounding as round_scaled); exact
// for |result| < 2^62.
__device__ __forceinline__ long long round_scaled64(double b, int k) {
  const long long bits = __double_as_longlong(b);
  const int E = (int)((bits >> 52) & 0x7ff);
  if (E == 0) return 0;
  const long long m = (bits & 0xfffffffffffffll) | (1ll << 52);
  const int sh = 1075 - E - k;
  long long X;
  if (sh <= 0) X = m << (-sh > 9 ? 9 : -sh);  // not reached for |x| < 2^11
  else if (sh > 62) X = 0;
  else X = (m + (1ll << (sh - 1))) >> sh;
  return bits < 0 ? -X : X;
}

// Scheme-1 digits of one element from its 24-bit fixed-point value
// X24 = round(x 2^24): s0 = round(x) (ties up), r24 = X24 - s0 2^24.
__device__ __forceinline__ void kara_digits(long long X24, int k, int* s0, int* s1) {
  const long long h = (X24 + (1ll << 23)) >> 24;
  const int r24 = (int)(X24 - (h << 24));
  *s0 = (int)h;
  *s1 = (r24 + (1 << (23 - k))) >> (24 - k);
}

// smallest e with y 2^-e <= 1 (y > 0)
__device__ __forceinline__ int ceil_log2(double y) {
  int k;
  const double f = frexp(y, &k);  // y = f 2^k, f in [0.5, 1)
  return f == 0.5 ? k - 1 : k;
}

constexpr int kKaraMaxK = 10;

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

// |x| truncated to FP32 from its IEEE fields (integer operations only; GB300's
// FP64 pipe is the slow one): relative error below 2^-23, always low; 0 for
// |x| < 2^-126 and 2^127 for |x| >= 2^128.
__device__ __forceinline__ float abs_to_float_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  const int E = (int)(b >> 52) - 1023;
  if (E < -126) return 0.0f;
  if (E > 127) return 1.7014118346046923e38f;
  return __uint_as_float((unsigned)((E + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

// Pass 1 of scheme 1 over one row slice: max |B| (IEEE bits) and an FP32
// estimate of sum B^2 (only used to pick the row scale, with a margin).
__device__ __forceinline__ void row_pass1_est(const double* __restrict__ b, int naux, long long R,
                                              long long r, int ty, unsigned long long* mo,
                                              float* so) {
  unsigned long long m[kUnroll] = {};
  float s[kUnroll] = {};
  int q = ty;
  for (; q + (kUnroll - 1) * QG < naux; q += kUnroll * QG) {
    double x[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) x[u] = b[(long long)(q + u * QG) * R + r];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const unsigned long long ax = abs_bits(x[u]);
      m[u] = ax > m[u] ? ax : m[u];
      const float f = abs_to_float_trunc(x[u]);
      s[u] = fmaf(f, f, s[u]);
    }
  }
  for (; q < naux; q += QG) {
    const double x = b[(long long)q * R + r];
    const unsigned long long ax = abs_bits(x);
    m[0] = ax > m[0] ? ax : m[0];
    const float f = abs_to_float_trunc(x);
    s[0] = fmaf(f, f, s[0]);
  }
  unsigned long long mm = m[0];
  float ss = s[0];
#pragma unroll
  for (int u = 1; u < kUnroll; ++u) {
    mm = m[u] > mm ? m[u] : mm;
    ss += s[u];
  }
  *mo = mm;
  *so = ss;
}

// Scheme 1: per row r, e_r from the row maximum and an FP32 norm estimate
// (first pass), then, in a second pass (a re-read that the L2 serves: a
// block's rows were read just before), the digit statistics, the largest
// admissible level exponent k_r (min-reduced into kglob) and the diagonal
// sum_Q B^2 from the exact 128-bit integer sum of the fixed-point squares
// X24^2 (|x - X24 2^-24| <= 2^-25 with ||x|| ~ 2^11.5: relative error below
// 1e-9).  Block = 32 rows x QG Q-groups.
__global__ void __launch_bounds__(32 * QG) rowstat_kara_kernel(const double* __restrict__ b,
                                                               int naux, long long R,
                                                               int* __restrict__ erow,
                                                               double* __restrict__ diag,
                                                               int* eref, int* kglob) {
  __shared__ unsigned long long smax[QG][32];
  __shared__ float ssum[QG][32];
  __shared__ float sb[QG][32], scc[QG][32];
  __shared__ int sa[QG][32], sm0[QG][32];
  __shared__ unsigned long long sdl[QG][32], sdh[QG][32];
  __shared__ int se[32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long r = (long long)blockIdx.x * 32 + tx;
  unsigned long long m = 0;
  float sf = 0.f;
  if (r < R) row_pass1_est(b, naux, R, r, ty, &m, &sf);
  smax[ty][tx] = m;
  ssum[ty][tx] = sf;
  __syncthreads();
  const double hs = 0.5 * sqrt((double)naux);
  if (ty == 0) {
    int e = INT_MIN / 4;
    if (r < R) {
      float sfl = sf;
      for (int k = 1; k < QG; ++k) {
        m = smax[k][tx] > m ? smax[k][tx] : m;
        sfl += ssum[k][tx];
      }
      // the FP32 estimate is low by at most ~2^-22 + (naux + 32) 2^-24 relative
      const double s = (double)sfl * (1.0 + 0x1p-16 + (double)(naux + 32) * 0x1p-23);
      const bool live = m != 0 && (m >> 52) != 0;
      if (live) {
        const double mx = __longlong_as_double((long long)m);
        const double t0 = 2896.309375740099 - hs - 1.0;  // 2^11.5 - sqrt(naux)/2 - 1
        const int en = ceil_log2(sqrt(s) / t0);
        const int ec = ceil_log2(mx / (2048.0 - 512.0 - 1.0));
        e = en > ec ? en : ec;
        atomicMax(eref, e);
      }
      erow[r] = e;
      if (!live) diag[r] = 0.0;
    }
    se[tx] = e;
  }
  __syncthreads();
  const int e = se[tx];
  const bool live = r < R && e > INT_MIN / 8;
  int a = 0, m0 = 0;
  float bb = 0.f, cc = 0.f;
  unsigned __int128 dsq = 0;  // exact sum of X24^2 (< 2^72 each)
  if (live) {
#pragma unroll 4
    for (int q = ty; q < naux; q += QG) {
      const long long X24 = round_scaled64(b[(long long)q * R + r], 24 - e);
      const long long h = (X24 + (1ll << 23)) >> 24;
      const float rf = (float)(int)(X24 - (h << 24));
      const int s0 = (int)h;
      const unsigned long long ax = (unsigned long long)(X24 < 0 ? -X24 : X24);
      dsq += (unsigned __int128)ax * ax;
      a += s0 * s0;
      m0 = max(m0, abs(s0));
      bb = fmaf((float)s0, rf, bb);
      cc = fmaf(rf, rf, cc);
    }
  }
  sa[ty][tx] = a;
  sm0[ty][tx] = m0;
  sb[ty][tx] = bb;
  scc[ty][tx] = cc;
  sdl[ty][tx] = (unsigned long long)dsq;
  sdh[ty][tx] = (unsigned long long)(dsq >> 64);
  __syncthreads();
  if (ty == 0 && live) {
    // FP32 sums of the FP32 partials: their error (< 2^-19 relative) sits
    // far inside the 2^-10 margins of the bounds below
    float bsf = 0.f, csf = 0.f;
    unsigned __int128 dt = 0;
    for (int k = 0; k < QG; ++k) {
      if (k) {
        a += sa[k][tx];
        m0 = max(m0, sm0[k][tx]);
      }
      bsf += sb[k][tx];
      csf += scc[k][tx];
      dt += ((unsigned __int128)sdh[k][tx] << 64) | sdl[k][tx];
    }
    const double bsum = (double)bsf, csum = (double)csf;
    // diag = sum X24^2 2^(2e - 48)
    const double dhi = (double)(unsigned long long)(dt >> 64), dlo = (double)(unsigned long long)dt;
    diag[r] = ldexp(fma(dhi, 0x1p64, dlo), 2 * e - 48);
    const double A = (double)a, Bx = bsum * 0x1p-24, C = csum * 0x1p-48;
    const double marg = 1.0 + 0x1p-10;
    const double slack = (0.5 + 0x1p-10) * sqrt((double)naux);
    const double bpos = Bx + 0x1p-10 * sqrt(A * C * marg);  // upper bound on s0.r
    int k = kKaraMaxK;
    for (; k > 0; --k) {
      const double L = (double)(1 << k);
      const double nu2 = A + 2.0 * L * bpos + L * L * C * marg;
      const bool ok = sqrt(nu2 > 0.0 ? nu2 : 0.0) + slack <= 4096.0 &&
                      L * sqrt(C * marg) + slack <= 4096.0 && m0 + (1 << (k - 1)) <= 2048;
      if (ok) break;
    }
    atomicMin(kglob, k);
  }
}

// Row statistics over Q for each r (scheme 0): e_r, the FP64 diagonal
// sum_Q B^2, and the global maximum exponent (atomicMax).  The maximum is
// taken on the integer bit patterns (no FP64 compare); the diagonal needs one
// FP64 FMA per element.
__global__ void __launch_bounds__(32 * QG) rowstat_kernel(const double* __restrict__ b, int naux,
                                                          long long R, int p,
                                                          int* __restrict__ erow,
                                                          double* __restrict__ diag, int* eref) {
  __shared__ unsigned long long smax[QG][32];
  __shared__ double ssum[QG][32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long r = (long long)blockIdx.x * 32 + tx;
  unsigned long long m = 0;
  double s = 0.0;
  if (r < R) row_pass1(b, naux, R, r, ty, &m, &s);
  smax[ty][tx] = m;
  ssum[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && r < R) {
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

template <int FMT>
__device__ __forceinline__ uint16_t to16i(int v) {
  if (FMT == 0) return __half_as_ushort(__int2half_rn(v));
  return __bfloat16_as_ushort(__int2bfloat16_rn(v));
}

// B[Q][r] -> digit planes in the tiled layout of the energy kernels
// (kernels.h, slice_tile_offset): one 8 KB tile per (i, 32-Q block, plane,
// 128-row virtual tile), each stored exactly as the 64-byte-swizzled shared
// memory image the tensor-core descriptors read, so the kernels fetch a
// tile with one linear bulk copy.  Rows a >= nvir of the last tile and
// Q >= naux are zero.
//
// Block = 256 threads on a 64 (padded row) x 64 (Q) tile: reads coalesced
// along r, then each thread converts 16 consecutive Q of one row and stores
// two 16-byte chunks per plane.  Digits by integer arithmetic on the IEEE
// fields: scheme 0 (levels) X = round(B 2^(2(p+1) - e_r)), s0 = round(X/L^2),
// s1 = round((X - s0 L^2)/L), s2 = remainder; scheme 1 (Karatsuba) as
// kara_digits, planes s0, s0 + s1, s1.
template <int SCHEME, int FMT>
__global__ void __launch_bounds__(256) slice_kernel(const double* __restrict__ b, int naux,
                                                    int nocc, int nvir, int Qp, int p,
                                                    const int* __restrict__ erow,
                                                    const int* __restrict__ kglob,
                                                    uint16_t* __restrict__ S) {
  __shared__ double tile[64][65];
  const int t = threadIdx.x;
  const int ntiles = (nvir + 127) / 128, vp = ntiles * 128;
  const long long R = (long long)nocc * nvir, Rp = (long long)nocc * vp;
  const long long r0 = (long long)blockIdx.x * 64;
  const int q0 = blockIdx.y * 64;
  {
    const int c = t & 63;
    const long long rp = r0 + c;
    const int i = (int)(rp / vp), a = (int)(rp % vp);
    const bool real = rp < Rp && a < nvir;
    const long long r = (long long)i * nvir + a;
#pragma unroll 4
    for (int k = t >> 6; k < 64; k += 4) {
      const int q = q0 + k;
      tile[k][c] = (q < naux && real) ? b[(long long)q * R + r] : 0.0;
    }
  }
  __syncthreads();
  const int rl = t >> 2, qc = (t & 3) * 16;
  const long long rp = r0 + rl;
  if (rp >= Rp || q0 + qc >= Qp) return;
  const int i = (int)(rp / vp), a = (int)(rp % vp);
  const int e = a < nvir ? erow[(long long)i * nvir + a] : INT_MIN / 4;
  const bool live = e > INT_MIN / 8;
  __align__(16) uint16_t h0[16];
  __align__(16) uint16_t h1[16];
  __align__(16) uint16_t h2[16];
  if (SCHEME == kSchemeKara) {
    const int k = live ? *kglob : 0;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      int s0 = 0, s1 = 0;
      if (live) kara_digits(round_scaled64(tile[qc + j][rl], 24 - e), k, &s0, &s1);
      h0[j] = to16i<FMT>(s0);
      h1[j] = to16i<FMT>(s0 + s1);
      h2[j] = to16i<FMT>(s1);
    }
  } else {
    const int lb = p + 1;       // bits per level
    const int k2 = 2 * lb - e;  // X = B 2^k2
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int X = live ? round_scaled(tile[qc + j][rl], k2) : 0;
      const int s0 = (X + (1 << (2 * lb - 1))) >> (2 * lb);
      const int rem = X - (s0 << (2 * lb));
      const int s1 = (rem + (1 << (lb - 1))) >> lb;
      const int s2 = rem - (s1 << lb);
      h0[j] = to16i<FMT>(s0);
      h1[j] = to16i<FMT>(s1);
      h2[j] = to16i<FMT>(s2);
    }
  }
  const int q = q0 + qc;
  const int nkb = Qp / 32, kb = q / 32, c0 = (q % 32) / 8;
  const size_t plane = 4096;  // the three planes of a tile are adjacent
  const size_t base = slice_tile_offset(0, i, kb, a / 128, nocc, nkb, ntiles);
  const int row = a % 128;
  const size_t at0 = base + slice_chunk_offset(row, c0);
  const size_t at1 = base + slice_chunk_offset(row, c0 + 1);
  const uint4* v0 = reinterpret_cast<const uint4*>(h0);
  const uint4* v1 = reinterpret_cast<const uint4*>(h1);
  const uint4* v2 = reinterpret_cast<const uint4*>(h2);
  *reinterpret_cast<uint4*>(S + at0) = v0[0];
  *reinterpret_cast<uint4*>(S + at1) = v0[1];
  *reinterpret_cast<uint4*>(S + plane + at0) = v1[0];
  *reinterpret_cast<uint4*>(S + plane + at1) = v1[1];
  *reinterpret_cast<uint4*>(S + 2 * plane + at0) = v2[0];
  *reinterpret_cast<uint4*>(S + 2 * plane + at1) = v2[1];
}

// Per-row FP32 factors for the energy kernel: sc_r = 2^(e_r - e_ref) and the
// diagonal sum in the same units, dg_r = diag_r 2^(-2 e_ref).  Also writes
// the global energy factor 2^(4 e_ref) into scale_out[0] and the level
// factor 1/L into scale_out[1] (scheme 1: L = 2^eref[1]; scheme 0: L = 2^(p+1)).
__global__ void rowfactor_kernel(const int* __restrict__ erow, const double* __restrict__ diag,
                                 long long R, const int* eref, int level_log2,
                                 float* __restrict__ sc, float* __restrict__ dg,
                                 double* scale_out) {
  int er = *eref;
  if (er < -4000) er = 0;  // every row zero
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < R;
       r += (long long)gridDim.x * blockDim.x) {
    int e = erow[r];
    sc[r] = (e > INT_MIN / 8) ? (float)ldexp(1.0, e - er) : 0.0f;
    dg[r] = (float)ldexp(diag[r], -2 * er);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scale_out[0] = ldexp(1.0, 4 * er);
    scale_out[1] = ldexp(1.0, -(level_log2 >= 0 ? level_log2 : eref[1]));
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

cudaError_t launch_slices(const double* b, int naux, int nocc, int nvir, int Qp, int scheme,
                          int fmt, int p, SliceWork w, cudaStream_t s) {
  const long long R = (long long)nocc * nvir;
  cudaError_t e = cudaMemsetAsync(w.eref, 0x80, sizeof(int), s);  // very negative start
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(w.eref + 1, 0x7f, sizeof(int), s);  // level exponent: min-reduced
  if (e != cudaSuccess) return e;
  const long long Rp = (long long)nocc * ((nvir + 127) / 128) * 128;
  dim3 grid((unsigned)((Rp + 63) / 64), (unsigned)((Qp + 63) / 64));
  if (scheme == kSchemeKara) {
    rowstat_kara_kernel<<<(unsigned)((R + 31) / 32), dim3(32, QG), 0, s>>>(b, naux, R, w.erow,
                                                                          w.diag, w.eref,
                                                                          w.eref + 1);
    slice_kernel<kSchemeKara, 0><<<grid, 256, 0, s>>>(b, naux, nocc, nvir, Qp, p, w.erow,
                                                      w.eref + 1, w.S);
  } else {
    rowstat_kernel<<<(unsigned)((R + 31) / 32), dim3(32, QG), 0, s>>>(b, naux, R, p, w.erow,
                                                                     w.diag, w.eref);
    if (fmt == 0)
      slice_kernel<kSchemeDigits3, 0><<<grid, 256, 0, s>>>(b, naux, nocc, nvir, Qp, p, w.erow,
                                                           w.eref + 1, w.S);
    else
      slice_kernel<kSchemeDigits3, 1><<<grid, 256, 0, s>>>(b, naux, nocc, nvir, Qp, p, w.erow,
                                                           w.eref + 1, w.S);
  }
  rowfactor_kernel<<<(unsigned)((R + 255) / 256 < 1024 ? (R + 255) / 256 : 1024), 256, 0, s>>>(
      w.erow, w.diag, R, w.eref, scheme == kSchemeKara ? -1 : p + 1, w.sc, w.dg, w.scale);
  return cudaGetLastError();
}

cudaError_t launch_energy_reduce(const double* partials, int n, const double* scale, double* out,
                                 cudaStream_t s) {
  energy_reduce_kernel<<<1, 256, 0, s>>>(partials, n, scale, out);
  return cudaGetLastError();
}

}  // namespace corr
