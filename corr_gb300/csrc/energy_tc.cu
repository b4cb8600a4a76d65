// Split-precision fused RI-MP2 energy on the 5th-generation tensor cores.
//
// Input: the pre-pass output hi/lo[i][a][Qp] (16-bit, K-major, see split.cu).
// Work unit = (occupied pair i<=j, virtual tile pair A<=B), tiles of 128.
// Per unit two 128x128 FP32 accumulators live in TMEM:
//   D1 = hi_iA.hi_jB^T + hi_iA.lo_jB^T + lo_iA.hi_jB^T  ~ g^2 (ia|jb)
//   D2 = hi_jA.hi_iB^T + hi_jA.lo_iB^T + lo_jA.hi_iB^T  ~ g^2 (ib|ja)
// and the epilogue folds them into E_OS/E_SS exactly as the FP64 kernel does
// (energy_fp64.cu has the derivation), so no (ia|jb) value reaches HBM.
//
// CTA = 6 warps, persistent, one CTA per SM:
//   warp 0     TMA producer (one thread): 8 tiles of 128x32 per stage, 3 stages
//   warp 1     TMEM owner + MMA issuer (one thread), tcgen05.mma kind::f16
//   warps 2-5  epilogue: tcgen05.ld of their 32-lane quarter, FP32 per-element
//              math (IEEE reciprocal of the denominator), FP64 per-unit sums
// TMEM holds two accumulator pairs (2 x 256 columns) so the epilogue of one
// unit overlaps the MMAs of the next.
#include "common.cuh"
#include "kernels.h"

namespace corr {

namespace {

constexpr int TILE = kTcTile;                 // 128
constexpr int KB = 32;                        // 16-bit Q elements per stage row (64 B)
constexpr int STAGES = 3;
constexpr int NTILES = 8;                     // tiles per stage
constexpr int TILE_BYTES = TILE * KB * 2;     // 8 KB
constexpr int STAGE_BYTES = NTILES * TILE_BYTES;
constexpr int NTHREADS = 192;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t SW64 = 4;                  // descriptor layout type: 64B swizzle

struct Ctl {
  uint64_t full[STAGES];
  uint64_t empty[STAGES];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint64_t fin;
  uint32_t tmem;
  int abort;
  float db[2][TILE];
  double red[2][4];
};

constexpr size_t kSmemBytes = (size_t)STAGES * STAGE_BYTES + sizeof(Ctl) + 1024;

__device__ __forceinline__ void unit_decode(long long u, const EnergyShape& sh, int* i, int* j,
                                            int* A, int* B) {
  int p = (int)(u / sh.ntpairs), tp = (int)(u % sh.ntpairs);
  pair_decode(p, sh.nocc, i, j);
  tpair_decode(tp, sh.ntiles, A, B);
}

__global__ void __launch_bounds__(NTHREADS, 1)
    energy_tc_kernel(const __grid_constant__ CUtensorMap tm_hi,
                     const __grid_constant__ CUtensorMap tm_lo, const double* __restrict__ eps,
                     EnergyShape sh, int nkb, uint32_t idesc, double* __restrict__ partials,
                     int* status) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  Ctl* ctl = reinterpret_cast<Ctl*>(tiles + (size_t)STAGES * STAGE_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o = sh.nocc, v = sh.nvir;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&ctl->full[s], 1);
      mbar_init(&ctl->empty[s], 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&ctl->tfull[s], 1);
      mbar_init(&ctl->tempty[s], 4);
    }
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
    if (lane == 0) {
      prefetch_tmap(&tm_hi);
      prefetch_tmap(&tm_lo);
      int st = 0;
      uint32_t ph = 0;
      uint32_t last_ph[STAGES];
      bool has[STAGES];
      for (int s = 0; s < STAGES; ++s) has[s] = false;
      bool ok = true;
      for (long long u = blockIdx.x; u < sh.nunits && ok; u += gridDim.x) {
        int i, j, A, B;
        unit_decode(u, sh, &i, &j, &A, &B);
        const int A0 = A * TILE, B0 = B * TILE;
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&ctl->empty[st], ph ^ 1, abort, status)) {
            ok = false;
            break;
          }
          uint64_t* bar = &ctl->full[st];
          mbar_expect_tx(bar, STAGE_BYTES);
          uint8_t* sb = tiles + (size_t)st * STAGE_BYTES;
          const int k0 = kb * KB;
          tma_load_3d(sb + 0 * TILE_BYTES, &tm_hi, bar, k0, A0, i);
          tma_load_3d(sb + 1 * TILE_BYTES, &tm_hi, bar, k0, B0, j);
          tma_load_3d(sb + 2 * TILE_BYTES, &tm_hi, bar, k0, A0, j);
          tma_load_3d(sb + 3 * TILE_BYTES, &tm_hi, bar, k0, B0, i);
          tma_load_3d(sb + 4 * TILE_BYTES, &tm_lo, bar, k0, A0, i);
          tma_load_3d(sb + 5 * TILE_BYTES, &tm_lo, bar, k0, B0, j);
          tma_load_3d(sb + 6 * TILE_BYTES, &tm_lo, bar, k0, A0, j);
          tma_load_3d(sb + 7 * TILE_BYTES, &tm_lo, bar, k0, B0, i);
          has[st] = true;
          last_ph[st] = ph;
          if (++st == STAGES) {
            st = 0;
            ph ^= 1;
          }
        }
      }
      // Never leave with a bulk copy still landing in shared memory.
      int never = 0;
      for (int s = 0; s < STAGES; ++s)
        if (has[s]) mbar_wait(&ctl->full[s], last_ph[s], &never, status);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int st = 0;
      uint32_t ph = 0;
      long long t = 0;
      bool ok = true;
      for (long long u = blockIdx.x; u < sh.nunits && ok; u += gridDim.x, ++t) {
        const int s = (int)(t & 1);
        const uint32_t use = (uint32_t)(t >> 1);
        if (!mbar_wait(&ctl->tempty[s], (use & 1) ^ 1, abort, status)) break;
        tc_fence_after();
        const uint32_t d1 = tmem + (uint32_t)s * 256u, d2 = d1 + 128u;
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&ctl->full[st], ph, abort, status)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sb = smem_u32(tiles + (size_t)st * STAGE_BYTES);
#pragma unroll
          for (int kk = 0; kk < KB / 16; ++kk) {
            const uint32_t off = (uint32_t)kk * 32u;  // 16 elements x 2 B
            uint64_t dsc[NTILES];
#pragma unroll
            for (int n = 0; n < NTILES; ++n)
              dsc[n] = smem_desc(sb + (uint32_t)n * TILE_BYTES + off, 16, 512, SW64);
            const uint32_t acc = (kb | kk) ? 1u : 0u;
            tc_mma_f16(d1, dsc[0], dsc[1], idesc, acc);
            tc_mma_f16(d1, dsc[0], dsc[5], idesc, 1u);
            tc_mma_f16(d1, dsc[4], dsc[1], idesc, 1u);
            tc_mma_f16(d2, dsc[2], dsc[3], idesc, acc);
            tc_mma_f16(d2, dsc[2], dsc[7], idesc, 1u);
            tc_mma_f16(d2, dsc[6], dsc[3], idesc, 1u);
          }
          tc_commit(&ctl->empty[st]);  // stage reusable once these MMAs finish
          if (++st == STAGES) {
            st = 0;
            ph ^= 1;
          }
        }
        if (ok) tc_commit(&ctl->tfull[s]);
      }
      // wait until every MMA this thread issued has retired
      tc_commit(&ctl->fin);
      int never = 0;
      mbar_wait(&ctl->fin, 0, &never, status);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;               // TMEM lane quarter of this warp
    const int et = threadIdx.x - 64;      // 0..127
    const int arow = 32 * q + lane;       // accumulator row = TMEM lane
    double tot_os = 0.0, tot_ss = 0.0;
    bool dead = false;
    long long t = 0;
    for (long long u = blockIdx.x; u < sh.nunits; u += gridDim.x, ++t) {
      const int s = (int)(t & 1);
      const uint32_t use = (uint32_t)(t >> 1);
      int i, j, A, B;
      unit_decode(u, sh, &i, &j, &A, &B);
      const int A0 = A * TILE, B0 = B * TILE;
      {
        const int b = B0 + et;
        ctl->db[s][et] = b < v ? (float)(eps[o + b] - eps[j]) : __int_as_float(0x7f800000);
      }
      named_bar(1, 128);
      if (!dead) {
        const int a = A0 + arow;
        const float da = a < v ? (float)(eps[o + a] - eps[i]) : __int_as_float(0x7f800000);
        // warp-uniform outcome: tcgen05.ld below is .sync.aligned
        const bool got = __all_sync(0xffffffffu, mbar_wait(&ctl->tfull[s], use & 1, abort, status));
        if (!got) {
          dead = true;
        } else {
          tc_fence_after();
          const uint32_t tb = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)s * 256u;
          double uos = 0.0, uss = 0.0;
#pragma unroll 1
          for (int c = 0; c < TILE; c += 32) {
            float m1[32], m2[32];
            tmem_ld32(tb + (uint32_t)c, m1);
            tmem_ld32(tb + 128u + (uint32_t)c, m2);
            tc_wait_ld();
            float fos = 0.f, fss = 0.f;
#pragma unroll
            for (int k = 0; k < 32; ++k) {
              const float r = __frcp_rn(da + ctl->db[s][c + k]);
              const float x = m1[k], y = m2[k];
              fos = fmaf(fmaf(x, x, y * y), r, fos);
              const float df = x - y;
              fss = fmaf(df * df, r, fss);
            }
            uos += (double)fos;
            uss += (double)fss;
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ctl->tempty[s]);
          const double fw = (A < B ? 2.0 : 1.0) * (i < j ? 1.0 : 0.5);
          tot_os -= fw * uos;
          tot_ss -= fw * uss;
        }
      }
    }
    tot_os = warp_sum(tot_os);
    tot_ss = warp_sum(tot_ss);
    if (lane == 0) {
      ctl->red[0][warp - 2] = tot_os;
      ctl->red[1][warp - 2] = tot_ss;
    }
    named_bar(1, 128);
    if (et == 0) {
      partials[2 * blockIdx.x] = (ctl->red[0][0] + ctl->red[0][1]) + (ctl->red[0][2] + ctl->red[0][3]);
      partials[2 * blockIdx.x + 1] =
          (ctl->red[1][0] + ctl->red[1][1]) + (ctl->red[1][2] + ctl->red[1][3]);
    }
  }

  __syncwarp();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, TMEM_COLS);
}

}  // namespace

cudaError_t launch_energy_tc(const CUtensorMap& tmap_hi, const CUtensorMap& tmap_lo,
                             const double* eps, const EnergyShape& sh, int Qp, int fmt,
                             double* partials, int grid, int* status, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(energy_tc_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSmemBytes);
  if (e != cudaSuccess) return e;
  const uint32_t idesc = idesc_f16((uint32_t)fmt, TILE, TILE);
  energy_tc_kernel<<<grid, NTHREADS, kSmemBytes, s>>>(tmap_hi, tmap_lo, eps, sh, Qp / KB, idesc,
                                                      partials, status);
  return cudaGetLastError();
}

}  // namespace corr
