// FP64-accurate GEMM on the 5th-generation tensor cores by exact digit
// slicing (the error-free splitting of Ozaki, Ogita, Oishi and Rump, 2012,
// with integer digits), for the FP64 contractions of the RI pipeline: the
// two transform_ri products (src/POSTHF/ri.cc:147-172) and the metric
// application B = L^-1 (P|ia) (the calculate_ri product, ri.cc:102-103).
//
// Slicing.  Row r of an operand is scaled by 2^-e_r (e_r: the binary exponent
// of its largest element, so every scaled value lies in (-1, 1)) and written
// as eight balanced base-128 digits,
//   x / 2^e_r = sum_{s=0..7} d_s 2^(-7 (s+1)) + rho,  |d_0| <= 128,
//   |d_s| <= 64 (s >= 1),  |rho| <= 2^-57,
// computed with integer operations on the FP64 bit pattern (no FP64
// arithmetic: GB300 runs FP64 at 1/64 of the FP32 rate).  Digits are small
// integers, exact in BF16.
//
// Products.  C(m, n) = 2^(e_m + f_n) sum_L 2^(-7 (L+2)) acc_L(m, n) with the
// level sums acc_L = sum_{s+t=L} sum_k d_s(A)[m][k] d_t(B)[n][k], L = 0..7
// (36 digit products; the levels L >= 8 fall below 2^-56 of the row and
// column scales).  With K <= 512 per pass every level L <= 5 stays below 2^24
// in magnitude -- (L+1) products of at most 128 * 64 per k, or 128^2 for
// L = 0 -- so its FP32 accumulation in TMEM is exact; levels 6 and 7 carry
// weights 2^-56 and 2^-63 and their FP32 rounding is far below FP64 rounding.
// Longer K runs in passes of 512 that accumulate into C.
//
// Tensor-core layout.  Output tile 128 x 64.  The eight digit planes of the
// column operand are stacked along N in shared memory (plane t = rows
// 64 t .. 64 t + 63), so one MMA per row digit s covers every column digit
// t <= 7 - s at once: D columns [64 s, 512) receive A_s B_t into level block
// s + t.  TMEM holds the eight level blocks (512 columns); an MMA wider than
// 256 columns is issued as two, reusing A through the collector buffer.
//
// Recombination (epilogue, per element): the exact levels 0..5 are combined
// in a 64-bit integer, levels 6..7 in FP32 and rounded in at 2^-3 of a level-5
// unit; the single rounding to FP64 is that of the integer conversion, and
// the scale 2^(e_m + f_n) is applied to the exponent field.
//
// CTA = 6 warps, persistent, one CTA per SM, output tiles assigned round
// robin: warp 0 bulk-copies the digit planes (two stages of 96 KB: 8 row
// planes of 128 x 32 and 8 column planes of 64 x 32, each a 64-byte-swizzled
// shared-memory image), warp 1 owns TMEM and issues the MMAs, warps 2..5
// read TMEM and write C.  Every wait is bounded.
#include <algorithm>

#include "common.cuh"
#include "dgemm_tc.h"
#include "tc_common.cuh"

namespace corr {

namespace {

constexpr int DS = 8;                     // digit planes per operand
constexpr int TM = 128;                   // output tile rows
constexpr int TN = 64;                    // output tile columns
constexpr int DKB = 32;                   // K per stage: 64-byte tile rows
constexpr int KPASS = 512;                // K per pass (exact levels 0..5)
constexpr int A_PLANE = TM * DKB * 2;     // 8 KB
constexpr int B_PLANE = TN * DKB * 2;     // 4 KB
constexpr int A_BYTES = DS * A_PLANE;     // 64 KB
constexpr int STAGE = A_BYTES + DS * B_PLANE;  // 96 KB
constexpr int NSTAGE = 2;
constexpr int NTHREADS = 192;
constexpr uint32_t SW64 = 4;              // descriptor layout type: 64-byte swizzle
constexpr uint32_t TMEM_COLS = 512;

// Element offset of (row rr, k kk) inside one TR x 32 plane image: 16-byte
// chunk c of row rr sits at chunk c ^ ((rr >> 1) & 3).
__host__ __device__ inline int plane_offset(int rr, int kk) {
  return rr * DKB + ((((kk >> 3) ^ (rr >> 1)) & 3) << 3) + (kk & 7);
}

__device__ __forceinline__ long long view_row(const MatView& v, long long r) {
  return (r / v.rdiv) * v.rs_hi + (r % v.rdiv) * v.rs_lo;
}

// ---------------------------------------------------------------- slicing
// e[r] = (largest biased exponent of row r over k0 <= k < k0 + kn) - 1022,
// so |x| < 2^e[r]; rows without a normal value get 0 (all digits zero).
template <bool WARP_ROW>
__global__ void __launch_bounds__(256) row_exponent_kernel(MatView v, int rows, int rows_pad,
                                                           int k0, int kn, int* __restrict__ e) {
  if (WARP_ROW) {  // one warp per row, k contiguous
    const int lane = threadIdx.x & 31;
    for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < rows_pad;
         r += ((long long)gridDim.x * blockDim.x) >> 5) {
      int em = 0;
      if (r < rows) {
        const double* p = v.p + view_row(v, r) + (long long)k0 * v.ks;
        for (int k = lane; k < kn; k += 32)
          em = max(em, (int)((__double_as_longlong(p[(long long)k * v.ks]) >> 52) & 0x7FF));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o));
      if (lane == 0) e[r] = em > 0 ? em - 1022 : 0;
    }
  } else {  // one thread per row (coalesced when consecutive rows are adjacent)
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows_pad;
         r += (long long)gridDim.x * blockDim.x) {
      int em = 0;
      if (r < rows) {
        const double* p = v.p + view_row(v, r) + (long long)k0 * v.ks;
        for (int k = 0; k < kn; ++k)
          em = max(em, (int)((__double_as_longlong(p[(long long)k * v.ks]) >> 52) & 0x7FF));
      }
      e[r] = em > 0 ? em - 1022 : 0;
    }
  }
}

// The eight BF16 digit bit patterns of x / 2^er, most significant first.
__device__ __forceinline__ void digits_of(double x, int er, uint32_t (&d)[DS]) {
  const long long bits = __double_as_longlong(x);
  const int E = (int)((bits >> 52) & 0x7FF);
  const uint32_t sgn = bits < 0 ? 0x8000u : 0u;
  unsigned long long H = 0;  // round(|x| 2^(56 - er)) <= 2^56
  if (E > 0) {
    const unsigned long long m = ((unsigned long long)bits & ((1ull << 52) - 1)) | (1ull << 52);
    const int t = E - 1019 - er;  // <= 3
    if (t >= 0) H = m << t;
    else if (t > -54) H = (m + (1ull << (-t - 1))) >> (-t);
  }
  // balanced digits: add 64 at each of the seven low base-128 positions
  constexpr unsigned long long BIAS = 0x40ull | (0x40ull << 7) | (0x40ull << 14) |
                                      (0x40ull << 21) | (0x40ull << 28) | (0x40ull << 35) |
                                      (0x40ull << 42);
  const unsigned long long Hb = H + BIAS;
#pragma unroll
  for (int p = 0; p < 7; ++p) {
    const uint32_t u = (uint32_t)(Hb >> (7 * p)) & 127u;
    const float f = __int_as_float(0x4B000000 | (int)u) - 8388672.0f;  // u - 64, exact
    d[DS - 1 - p] = (__float_as_uint(f) >> 16) ^ sgn;
  }
  const uint32_t top = (uint32_t)(Hb >> 49);  // 0 .. 128
  const float f = __int_as_float(0x4B000000 | (int)top) - 8388608.0f;
  d[0] = (__float_as_uint(f) >> 16) ^ sgn;
}

// Digit planes of rows [0, rows_pad) over k0 <= k < k0 + kn (zero beyond rows
// and kn), tile images [rt][kb][s] of TR x 32.  One thread per (row, 8 k).
// ROW_FAST: consecutive threads take consecutive rows (for views whose rows
// are adjacent in memory); else consecutive k chunks of one row.
template <int TR, bool ROW_FAST>
__global__ void __launch_bounds__(256) slice_digits_kernel(MatView v, int rows, int rows_pad,
                                                           int k0, int kn, int nkb,
                                                           const int* __restrict__ e,
                                                           uint16_t* __restrict__ out) {
  const int nch = nkb * (DKB / 8);
  const long long total = (long long)rows_pad * nch;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long r;
    int kc;
    if (ROW_FAST) {
      r = t % rows_pad;
      kc = (int)(t / rows_pad);
    } else {
      r = t / nch;
      kc = (int)(t % nch);
    }
    uint32_t dg[8][DS];
    const int er = e[r];
    const double* p = r < rows ? v.p + view_row(v, r) + (long long)k0 * v.ks : nullptr;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = kc * 8 + j;
      const double x = (p && k < kn) ? p[(long long)k * v.ks] : 0.0;
      digits_of(x, er, dg[j]);
    }
    const int rt = (int)(r / TR), rr = (int)(r % TR), kb = kc >> 2;
    uint16_t* tile = out + ((size_t)rt * nkb + kb) * DS * (TR * DKB);
    const int off = plane_offset(rr, (kc & 3) * 8);
#pragma unroll
    for (int s = 0; s < DS; ++s) {
      uint4 w;
      w.x = dg[0][s] | (dg[1][s] << 16);
      w.y = dg[2][s] | (dg[3][s] << 16);
      w.z = dg[4][s] | (dg[5][s] << 16);
      w.w = dg[6][s] | (dg[7][s] << 16);
      *reinterpret_cast<uint4*>(tile + (size_t)s * (TR * DKB) + off) = w;
    }
  }
}

// ---------------------------------------------------------------- product
struct DgArgs {
  const uint16_t* Ad;  // row-operand digit tiles [mt][kb][s] (128 x 32)
  const uint16_t* Bd;  // column-operand digit tiles [nt][kb][s] (64 x 32)
  const int* ea;       // row exponents (padded)
  const int* eb;       // column exponents (padded)
  OutView C;
  double alpha;
  int M, N, nkb, mtn, ntn;
  int col_major_order;  // units nt-major (shared column tile adjacent)
  int a_lower, k0, accumulate;
  long long total;
};

struct DgCtl {
  uint64_t full[NSTAGE];
  uint64_t empty[NSTAGE];
  uint64_t afull;
  uint64_t aempty;
  uint64_t fin;
  uint32_t tmem;
  int abort;
};

__device__ __forceinline__ void unit_tile(const DgArgs& a, long long u, int* mt, int* nt) {
  if (a.col_major_order) {
    *nt = (int)(u / a.mtn);
    *mt = (int)(u % a.mtn);
  } else {
    *mt = (int)(u / a.ntn);
    *nt = (int)(u % a.ntn);
  }
}

// K blocks of this pass that tile row mt needs (lower-triangular A: k <= m).
__device__ __forceinline__ int unit_kblocks(const DgArgs& a, int mt) {
  if (!a.a_lower) return a.nkb;
  const int kend = (mt + 1) * TM - a.k0;  // local k < kend can be nonzero
  return kend <= 0 ? 0 : min(a.nkb, (kend + DKB - 1) / DKB);
}

// FP64 value of one output element from its eight level sums (lv[L]).
__device__ __forceinline__ double combine_levels(const float* lv, int sh) {
  long long hi = __float2int_rn(lv[0]);
#pragma unroll
  for (int L = 1; L < 6; ++L) hi = hi * 128 + __float2int_rn(lv[L]);  // |hi| < 2^59.1
  const float tail = fmaf(lv[7], 0.0078125f, lv[6]) * 0.0078125f;     // level-5 units
  const long long V = hi * 8 + __float2ll_rn(tail * 8.0f);
  double r = (double)V;  // the one rounding
  if (V != 0) {
    const long long b = __double_as_longlong(r);
    const int ex = (int)((b >> 52) & 0x7FF) + sh;
    r = (ex > 0 && ex < 2047) ? __longlong_as_double(b + ((long long)sh << 52)) : ldexp(r, sh);
  }
  return r;
}

__global__ void __launch_bounds__(NTHREADS, 1) dgemm_tc_kernel(DgArgs a, int* status) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  DgCtl* ctl = reinterpret_cast<DgCtl*>(tiles + NSTAGE * STAGE);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(&ctl->full[s], 1);
      mbar_init(&ctl->empty[s], 1);
    }
    mbar_init(&ctl->afull, 1);
    mbar_init(&ctl->aempty, 4);
    mbar_init(&ctl->fin, 1);
    ctl->abort = 0;
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&ctl->tmem, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = ctl->tmem;
  volatile int* abort = &ctl->abort;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    int st = 0;
    uint32_t ph = 0;
    uint32_t last_ph[NSTAGE];
    bool has[NSTAGE];
    for (int s = 0; s < NSTAGE; ++s) has[s] = false;
    bool ok = true;
    for (long long u = blockIdx.x; u < a.total && ok; u += gridDim.x) {
      int mt, nt;
      unit_tile(a, u, &mt, &nt);
      const int nkb = unit_kblocks(a, mt);
      for (int kb = 0; kb < nkb; ++kb) {
        bool got = true;
        if (lane == 0) got = mbar_wait(&ctl->empty[st], ph ^ 1, abort, status);
        if (!__shfl_sync(0xffffffffu, got ? 1 : 0, 0)) {
          ok = false;
          break;
        }
        uint64_t* bar = &ctl->full[st];
        if (lane == 0) mbar_expect_tx(bar, STAGE);
        __syncwarp();
        uint8_t* sb = tiles + (size_t)st * STAGE;
        if (lane < DS)
          bulk_load(sb + lane * A_PLANE,
                    a.Ad + (((size_t)mt * a.nkb + kb) * DS + lane) * (TM * DKB), A_PLANE, bar);
        else if (lane < 2 * DS)
          bulk_load(sb + A_BYTES + (lane - DS) * B_PLANE,
                    a.Bd + (((size_t)nt * a.nkb + kb) * DS + (lane - DS)) * (TN * DKB), B_PLANE,
                    bar);
        has[st] = true;
        last_ph[st] = ph;
        if (++st == NSTAGE) {
          st = 0;
          ph ^= 1;
        }
      }
    }
    if (lane == 0) {  // never leave with a copy still landing in shared memory
      int never = 0;
      for (int s = 0; s < NSTAGE; ++s)
        if (has[s]) mbar_wait(&ctl->full[s], last_ph[s], &never, status);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int st = 0;
      uint32_t ph = 0, nuse = 0;
      bool ok = true;
      uint32_t idn[5];  // instruction descriptors for N = 64 k, k = 1..4
      for (int k = 1; k <= 4; ++k) idn[k] = idesc_f16(1u, TM, 64u * k);
      const uint64_t dbase = smem_desc(smem_u32(tiles), 16, 512, SW64);
      for (long long u = blockIdx.x; u < a.total && ok; u += gridDim.x) {
        int mt, nt;
        unit_tile(a, u, &mt, &nt);
        const int nkb = unit_kblocks(a, mt);
        if (nkb == 0) continue;
        if (!mbar_wait(&ctl->aempty, (nuse & 1) ^ 1, abort, status)) break;
        tc_fence_after();
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&ctl->full[st], ph, abort, status)) {
            ok = false;
            break;
          }
          const uint64_t ds = dbase + (uint64_t)(((uint32_t)st * STAGE) >> 4);
#pragma unroll
          for (int kk = 0; kk < DKB / 16; ++kk) {
            const uint64_t bq = ds + (uint64_t)((A_BYTES + kk * 32) >> 4);
#pragma unroll
            for (int s = 0; s < DS; ++s) {
              const uint64_t ar = ds + (uint64_t)((s * A_PLANE + kk * 32) >> 4);
              const uint32_t acc = (kb | kk | s) ? 1u : 0u;
              const uint32_t d = tmem + 64u * s;
              const int nblk = DS - s;  // column planes 0 .. 7 - s
              if (nblk > 4) {
                tc_mma_f16_ca<0>(d, ar, bq, idn[4], acc);
                tc_mma_f16_ca<2>(d + 256u, ar, bq + (uint64_t)((4 * B_PLANE) >> 4),
                                 idn[nblk - 4], acc);
              } else {
                tc_mma_f16(d, ar, bq, idn[nblk], acc);
              }
            }
          }
          tc_commit(&ctl->empty[st]);
          if (++st == NSTAGE) {
            st = 0;
            ph ^= 1;
          }
        }
        if (ok) tc_commit(&ctl->afull);
        ++nuse;
      }
      tc_commit(&ctl->fin);
      int never = 0;
      mbar_wait(&ctl->fin, 0, &never, status);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;  // TMEM lane quarter of this warp
    const int arow = 32 * q + lane;
    const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16);
    uint32_t nuse = 0;
    for (long long u = blockIdx.x; u < a.total; u += gridDim.x) {
      int mt, nt;
      unit_tile(a, u, &mt, &nt);
      if (unit_kblocks(a, mt) == 0) continue;
      const bool got = mbar_wait(&ctl->afull, nuse & 1, abort, status);
      if (!__all_sync(0xffffffffu, got)) break;
      tc_fence_after();
      const long long m = (long long)mt * TM + arow;
      const bool mlive = m < a.M;
      const int em = a.ea[m];
      double* crow = mlive ? a.C.p + (m / a.C.rdiv) * a.C.rs_hi + (m % a.C.rdiv) * a.C.rs_lo
                           : nullptr;
#pragma unroll 1
      for (int c = 0; c < TN / 16; ++c) {
        float lv[DS][16];
#pragma unroll
        for (int L = 0; L < DS; ++L) tmem_ld16(tq + 64u * L + 16u * c, lv[L]);
        tc_wait_ld();
#pragma unroll
        for (int L = 0; L < DS; ++L) ld_ready<16>(lv[L]);
        if (c == TN / 16 - 1) {  // every TMEM read of this unit is done
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ctl->aempty);
        }
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const int n = nt * TN + 16 * c + e;
          float l8[DS];
#pragma unroll
          for (int L = 0; L < DS; ++L) l8[L] = lv[L][e];
          if (mlive && n < a.N) {
            double r = combine_levels(l8, em + a.eb[n] - 52);
            if (a.alpha != 1.0) r *= a.alpha;
            double* dst = crow + (long long)n * a.C.cs;
            *dst = a.accumulate ? *dst + r : r;
          }
        }
      }
      ++nuse;
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

constexpr size_t kDgSmem = (size_t)NSTAGE * STAGE + sizeof(DgCtl) + 1024;
static_assert(kDgSmem <= 227 * 1024, "shared memory");

int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

template <int TR>
int slice_operand(corr_context* c, const MatView& v, int rows, int rows_pad, int k0, int kn,
                  int nkb, int* e, uint16_t* out) {
  const bool krow = v.ks == 1;  // k contiguous: warp per row, k-fast chunks
  const int cap = c->sms * 16;
  if (krow)
    row_exponent_kernel<true><<<std::min(ceil_div((long long)rows_pad * 32, 256), cap), 256, 0,
                                 c->stream>>>(v, rows, rows_pad, k0, kn, e);
  else
    row_exponent_kernel<false><<<std::min(ceil_div(rows_pad, 256), cap), 256, 0, c->stream>>>(
        v, rows, rows_pad, k0, kn, e);
  CORR_CUDA(cudaGetLastError());
  const long long work = (long long)rows_pad * nkb * (DKB / 8);
  const int grid = std::min(ceil_div(work, 256), cap);
  if (krow)
    slice_digits_kernel<TR, false><<<grid, 256, 0, c->stream>>>(v, rows, rows_pad, k0, kn, nkb,
                                                                  e, out);
  else
    slice_digits_kernel<TR, true><<<grid, 256, 0, c->stream>>>(v, rows, rows_pad, k0, kn, nkb, e,
                                                                 out);
  CORR_CUDA(cudaGetLastError());
  c->launches += 2;
  return CORR_OK;
}

}  // namespace

size_t dgemm_tc_workspace(int M, int N, int K) {
  const size_t mp = (size_t)ceil_div(M, TM) * TM, np = (size_t)ceil_div(N, TN) * TN;
  const size_t kp = (size_t)ceil_div(std::min(K, KPASS), DKB) * DKB;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  return al(mp * kp * DS * 2) + al(np * kp * DS * 2) + al(mp * 4) + al(np * 4);
}

int dgemm_tc(corr_context* c, const DgemmTc& g, void* ws) {
  if (g.M <= 0 || g.N <= 0) return CORR_OK;
  const int mtn = ceil_div(g.M, TM), ntn = ceil_div(g.N, TN);
  const int mp = mtn * TM, np = ntn * TN;
  const size_t kp = (size_t)ceil_div(std::min(std::max(g.K, 1), KPASS), DKB) * DKB;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  uint8_t* w = static_cast<uint8_t*>(ws);
  uint16_t* Ad = reinterpret_cast<uint16_t*>(w);
  w += al((size_t)mp * kp * DS * 2);
  uint16_t* Bd = reinterpret_cast<uint16_t*>(w);
  w += al((size_t)np * kp * DS * 2);
  int* ea = reinterpret_cast<int*>(w);
  w += al((size_t)mp * 4);
  int* eb = reinterpret_cast<int*>(w);
  static bool attr[64] = {};
  if (c->device < 0 || c->device >= 64 || !attr[c->device]) {
    CORR_CUDA(cudaFuncSetAttribute(dgemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kDgSmem));
    if (c->device >= 0 && c->device < 64) attr[c->device] = true;
  }
  const int passes = std::max(1, ceil_div(g.K, KPASS));
  for (int p = 0; p < passes; ++p) {
    const int k0 = p * KPASS, kn = std::min(KPASS, g.K - k0);
    const int nkb = ceil_div(std::max(kn, 1), DKB);
    if (kn > 0) {
      CORR_TRY(slice_operand<TM>(c, g.A, g.M, mp, k0, kn, nkb, ea, Ad));
      CORR_TRY(slice_operand<TN>(c, g.B, g.N, np, k0, kn, nkb, eb, Bd));
    } else {  // K == 0: zero digits give C = 0 (or C unchanged when accumulating)
      CORR_CUDA(cudaMemsetAsync(Ad, 0, (size_t)mp * kp * DS * 2, c->stream));
      CORR_CUDA(cudaMemsetAsync(Bd, 0, (size_t)np * kp * DS * 2, c->stream));
      CORR_CUDA(cudaMemsetAsync(ea, 0, (size_t)mp * 4, c->stream));
      CORR_CUDA(cudaMemsetAsync(eb, 0, (size_t)np * 4, c->stream));
    }
    DgArgs a;
    a.Ad = Ad;
    a.Bd = Bd;
    a.ea = ea;
    a.eb = eb;
    a.C = g.C;
    a.alpha = g.alpha;
    a.M = g.M;
    a.N = g.N;
    a.nkb = nkb;
    a.mtn = mtn;
    a.ntn = ntn;
    // keep the larger operand's tile shared by adjacent units (L2 reuse)
    a.col_major_order = (long long)np > (long long)mp ? 1 : 0;
    a.a_lower = g.a_lower ? 1 : 0;
    a.k0 = k0;
    a.accumulate = (g.accumulate || p > 0) ? 1 : 0;
    a.total = (long long)mtn * ntn;
    const int grid = (int)std::min<long long>(a.total, c->sms);
    dgemm_tc_kernel<<<grid, NTHREADS, kDgSmem, c->stream>>>(a, &c->dres->status);
    CORR_CUDA(cudaGetLastError());
    c->launches += 1;
  }
  return CORR_OK;
}

}  // namespace corr
