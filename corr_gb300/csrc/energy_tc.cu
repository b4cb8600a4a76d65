// Precision-form fused RI-MP2 energy on the 5th-generation tensor cores.
//
// Input: the three 16-bit integer planes of B (split.cu) in the tiled
// layout of kernels.h: every 128 x 32 operand tile is one contiguous,
// pre-swizzled 8 KB block fetched with a linear bulk copy (whole 128-byte
// lines from L2).
// Work unit = (occupied pair i<=j, virtual tile pair A<=B), tiles of 128.
//
// Phase 1 forms D1[a][b] = (ia|jb) for a in A, b in B; phase 2 forms
// D2[a][b] = (ib|ja).  Each phase accumulates three exact integer sums in
// TMEM (split.cu), by scheme:
//   0: acc_m = sum_{k+l=m} s_k(row) . s_l(col)^T   (m = 0..2, six MMAs per K=16)
//   1: P0 = s0.s0', Pm = u.u', P2 = s1.s1'        (three MMAs per K=16)
// and the epilogue forms d = sc_row sc_col (value of the digits) in FP32 with
// round-to-nearest (tc_common.cuh).
// D1 is parked in TMEM columns 384-511 while D2 accumulates in 0-383.  For
// i == j, D2 == D1 and phase 2 is skipped; for A == B, D2 = D1^T is obtained
// by a 32x32-block exchange through shared memory instead of a second pass.  On the (i==j, A==B) diagonal the
// element (ia|ia) is replaced by its FP64 value.  The energy epilogue is the
// one of energy_fp64.cu:
//   E_OS -= f w (D1^2 + D2^2)/D,  E_SS -= f w (D1 - D2)^2/D,
// with 1/D as an IEEE-rounded FP32 reciprocal and FP64 sums per unit.
//
// CTA = 6 warps, persistent, one CTA per SM:
//   warp 0     bulk-copy producer (one thread), 6 tiles of 128x32 per stage, 4 stages
//   warp 1     TMEM owner + MMA issuer (one thread), tcgen05.mma kind::f16
//   warps 2-5  epilogue, one TMEM lane quarter each
// Every wait is bounded (common.cuh); on a timeout the CTA winds down and the
// host sees CORR_ERR_DEVICE_TIMEOUT.
#include "common.cuh"
#include "kernels.h"
#include "tc_common.cuh"

namespace corr {

namespace {

constexpr int TILE = kTcTile;                 // 128
constexpr int KB = 32;                        // 16-bit Q elements per stage row (64 B)
constexpr int STAGES = 4;
constexpr int NTILES = 6;                     // 3 slices x (row operand, col operand)
constexpr int TILE_BYTES = TILE * KB * 2;     // 8 KB
constexpr int STAGE_BYTES = NTILES * TILE_BYTES;
constexpr int NTHREADS = 192;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t COL_STASH = 384;           // parked D1
constexpr uint32_t SW64 = 4;                  // descriptor layout type: 64B swizzle

struct Ctl {
  uint64_t full[STAGES];
  uint64_t empty[STAGES];
  uint64_t afull;
  uint64_t aempty;
  uint64_t fin;
  uint32_t tmem;
  int abort;
  float db[TILE];
  float scb[TILE];
  double red[2][4];
  float tbuf[4][32][33];  // D1 -> D1^T exchange on diagonal tile pairs
  int wok[2][4];          // per-warp wait outcome, combined into one decision
};

constexpr size_t kSmemBytes = (size_t)STAGES * STAGE_BYTES + sizeof(Ctl) + 1024;

__device__ __forceinline__ void unit_decode(long long u, const EnergyShape& sh, int* i, int* j,
                                            int* A, int* B) {
  int p = (int)(u / sh.ntpairs), tp = (int)(u % sh.ntpairs);
  pair_decode(p, sh.nocc, i, j);
  tpair_decode(tp, sh.ntiles, A, B);
}

template <int SCHEME>
__global__ void __launch_bounds__(NTHREADS, 1)
    energy_tc_kernel(const uint16_t* __restrict__ S, const double* __restrict__ eps,
                     const float* __restrict__ sc, const float* __restrict__ dg,
                     const double* __restrict__ scale, EnergyShape sh, int nkb, uint32_t idesc,
                     double* __restrict__ partials, int* status) {
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
    if (lane == 0) {
      int st = 0;
      uint32_t ph = 0;
      uint32_t last_ph[STAGES];
      bool has[STAGES];
      for (int s = 0; s < STAGES; ++s) has[s] = false;
      bool ok = true;
      for (long long u = blockIdx.x; u < sh.nunits && ok; u += gridDim.x) {
        int i, j, A, B;
        unit_decode(u, sh, &i, &j, &A, &B);
        const int nph = (i == j || A == B) ? 1 : 2;
        for (int phs = 0; phs < nph && ok; ++phs) {
          const int x = phs == 0 ? i : j;  // row operand slab
          const int y = phs == 0 ? j : i;  // column operand slab
          for (int kb = 0; kb < nkb; ++kb) {
            if (!mbar_wait(&ctl->empty[st], ph ^ 1, abort, status)) {
              ok = false;
              break;
            }
            uint64_t* bar = &ctl->full[st];
            mbar_expect_tx(bar, STAGE_BYTES);
            uint8_t* sb = tiles + (size_t)st * STAGE_BYTES;
#pragma unroll
            for (int l = 0; l < 3; ++l) {
              bulk_load(sb + (2 * l) * TILE_BYTES,
                        S + slice_tile_offset(l, x, kb, A, o, nkb, sh.ntiles), TILE_BYTES, bar);
              bulk_load(sb + (2 * l + 1) * TILE_BYTES,
                        S + slice_tile_offset(l, y, kb, B, o, nkb, sh.ntiles), TILE_BYTES, bar);
            }
            has[st] = true;
            last_ph[st] = ph;
            if (++st == STAGES) {
              st = 0;
              ph ^= 1;
            }
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
      uint32_t nuse = 0;
      bool ok = true;
      for (long long u = blockIdx.x; u < sh.nunits && ok; u += gridDim.x) {
        int i, j, A, B;
        unit_decode(u, sh, &i, &j, &A, &B);
        const int nph = (i == j || A == B) ? 1 : 2;
        for (int phs = 0; phs < nph && ok; ++phs) {
          if (!mbar_wait(&ctl->aempty, (nuse & 1) ^ 1, abort, status)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t c0 = tmem, c1 = tmem + 128u, c2 = tmem + 256u;
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
              uint64_t r[3], q[3];
#pragma unroll
              for (int l = 0; l < 3; ++l) {
                r[l] = smem_desc(sb + (uint32_t)(2 * l) * TILE_BYTES + off, 16, 512, SW64);
                q[l] = smem_desc(sb + (uint32_t)(2 * l + 1) * TILE_BYTES + off, 16, 512, SW64);
              }
              const uint32_t acc = (kb | kk) ? 1u : 0u;
              issue_digit_mmas<SCHEME>(c0, c1, c2, r, q, idesc, acc);
            }
            tc_commit(&ctl->empty[st]);  // stage reusable once these MMAs finish
            if (++st == STAGES) {
              st = 0;
              ph ^= 1;
            }
          }
          if (ok) tc_commit(&ctl->afull);
          ++nuse;
        }
      }
      tc_commit(&ctl->fin);  // wait until every MMA this thread issued has retired
      int never = 0;
      mbar_wait(&ctl->fin, 0, &never, status);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;           // TMEM lane quarter of this warp
    const int et = threadIdx.x - 64;  // 0..127
    const int arow = 32 * q + lane;   // accumulator row = TMEM lane
    const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16);
    const float inv_l = (float)scale[1];
    const float inv_l2 = inv_l * inv_l;
    double tot_os = 0.0, tot_ss = 0.0;
    bool dead = false;
    uint32_t nuse = 0;
    for (long long u = blockIdx.x; u < sh.nunits; u += gridDim.x) {
      int i, j, A, B;
      unit_decode(u, sh, &i, &j, &A, &B);
      const int A0 = A * TILE, B0 = B * TILE;
      const bool same = (i == j);
      {
        // phase 1: rows from slab i, columns from slab j
        const int b = B0 + et;
        ctl->db[et] = b < v ? (float)(eps[o + b] - eps[j]) : __int_as_float(0x7f800000);
        ctl->scb[et] = b < v ? sc[(size_t)j * v + b] : 0.0f;
      }
      named_bar(1, 128);
      const int a = A0 + arow;
      const float da = a < v ? (float)(eps[o + a] - eps[i]) : __int_as_float(0x7f800000);
      const float sca1 = a < v ? sc[(size_t)i * v + a] : 0.0f;
      const float sca2 = a < v ? sc[(size_t)j * v + a] : 0.0f;
      const bool diag_tile = same && (A == B);
      const float dga = (diag_tile && a < v) ? dg[(size_t)i * v + a] : 0.0f;
      double uos = 0.0, uss = 0.0;

      // ---- phase 1: D1
      // The outcome of the wait is made uniform over the four epilogue warps
      // (named barriers below must be reached by all of them or none).
      bool got = !dead && __all_sync(0xffffffffu,
                                     mbar_wait(&ctl->afull, nuse & 1, abort, status));
      if (lane == 0) ctl->wok[nuse & 1][q] = got ? 1 : 0;
      named_bar(1, 128);
      got = ctl->wok[nuse & 1][0] & ctl->wok[nuse & 1][1] & ctl->wok[nuse & 1][2] &
            ctl->wok[nuse & 1][3];
      if (!got) dead = true;
      if (!dead) {
        tc_fence_after();
        if (same) {
          // D2 == D1: fold straight into the energy
#pragma unroll 1
          for (int c = 0; c < TILE; c += 32) {
            float d1[32];
            load_level_sum<SCHEME>(tq, c, inv_l, inv_l2, sca1, ctl->scb, d1);
            float fos = 0.f;
#pragma unroll
            for (int k = 0; k < 32; ++k) {
              const float x = (diag_tile && c + k == arow) ? dga : d1[k];
              const float r = __frcp_rn(da + ctl->db[c + k]);
              fos = fmaf(2.0f * x * x, r, fos);
            }
            uos += (double)fos;
          }
        } else if (A == B) {
          // Diagonal tile pair: D2 = D1^T.  Four rounds; in round k warp q
          // publishes its D1 block of column chunk (q+k)%4 and takes the block
          // of warp (q-k)%4, which is the D1^T block of column chunk (q-k)%4.
#pragma unroll 1
          for (int k = 0; k < 4; ++k) {
            float d[32];
            const int cw = 32 * ((q + k) & 3);
            load_level_sum<SCHEME>(tq, cw, inv_l, inv_l2, sca1, ctl->scb, d);
#pragma unroll
            for (int x = 0; x < 32; ++x) ctl->tbuf[q][lane][x] = d[x];
            named_bar(1, 128);
            const int wr = (q - k) & 3;
            const int cr = 32 * wr;
            float d2[32];
#pragma unroll
            for (int x = 0; x < 32; ++x) d2[x] = ctl->tbuf[wr][x][lane];
            load_level_sum<SCHEME>(tq, cr, inv_l, inv_l2, sca1, ctl->scb, d);
            float fos = 0.f, fss = 0.f;
#pragma unroll
            for (int x = 0; x < 32; ++x) {
              const float r = __frcp_rn(da + ctl->db[cr + x]);
              const float y1 = d[x], y2 = d2[x];
              fos = fmaf(fmaf(y1, y1, y2 * y2), r, fos);
              const float df = y1 - y2;
              fss = fmaf(df * df, r, fss);
            }
            uos += (double)fos;
            uss += (double)fss;
            named_bar(1, 128);  // tbuf is rewritten in the next round
          }
        } else {
#pragma unroll 1
          for (int c = 0; c < TILE; c += 32) {
            float d1[32];
            load_level_sum<SCHEME>(tq, c, inv_l, inv_l2, sca1, ctl->scb, d1);
            tmem_st32(tq + COL_STASH + (uint32_t)c, d1);
          }
          tc_wait_st();
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&ctl->aempty);
      }
      ++nuse;

      // ---- phase 2: D2 (i != j, A != B): rows from slab j, columns from slab i
      if (!same && A != B) {
        named_bar(1, 128);  // everyone is done with the phase-1 column scales
        if (B0 + et < v) ctl->scb[et] = sc[(size_t)i * v + B0 + et];
        named_bar(1, 128);
        got = !dead && __all_sync(0xffffffffu, mbar_wait(&ctl->afull, nuse & 1, abort, status));
        if (lane == 0) ctl->wok[nuse & 1][q] = got ? 1 : 0;
        named_bar(1, 128);
        got = ctl->wok[nuse & 1][0] & ctl->wok[nuse & 1][1] & ctl->wok[nuse & 1][2] &
              ctl->wok[nuse & 1][3];
        if (!got) dead = true;
        if (!dead) {
          tc_fence_after();
#pragma unroll 1
          for (int c = 0; c < TILE; c += 32) {
            float d2[32], d1[32];
            load_level_sum<SCHEME>(tq, c, inv_l, inv_l2, sca2, ctl->scb, d2);
            tmem_ld32(tq + COL_STASH + (uint32_t)c, d1);
            tc_wait_ld();
            float fos = 0.f, fss = 0.f;
#pragma unroll
            for (int k = 0; k < 32; ++k) {
              const float r = __frcp_rn(da + ctl->db[c + k]);
              const float x = d1[k], y = d2[k];
              fos = fmaf(fmaf(x, x, y * y), r, fos);
              const float df = x - y;
              fss = fmaf(df * df, r, fss);
            }
            uos += (double)fos;
            uss += (double)fss;
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ctl->aempty);
        }
        ++nuse;
      }
      const double fw = (A < B ? 2.0 : 1.0) * (same ? 0.5 : 1.0);
      tot_os -= fw * uos;
      tot_ss -= fw * uss;
      named_bar(1, 128);  // smem db/scb are rewritten by the next unit
    }
    tot_os = warp_sum(tot_os);
    tot_ss = warp_sum(tot_ss);
    if (lane == 0) {
      ctl->red[0][warp - 2] = tot_os;
      ctl->red[1][warp - 2] = tot_ss;
    }
    named_bar(1, 128);
    if (et == 0) {
      partials[2 * blockIdx.x] =
          (ctl->red[0][0] + ctl->red[0][1]) + (ctl->red[0][2] + ctl->red[0][3]);
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

cudaError_t prepare_energy_tc() {
  cudaError_t e = cudaFuncSetAttribute(energy_tc_kernel<kSchemeDigits3>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSmemBytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(energy_tc_kernel<kSchemeKara>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
}

cudaError_t launch_energy_tc(const uint16_t* S, const double* eps, const float* sc,
                             const float* dg, const double* scale, const EnergyShape& sh, int Qp,
                             int fmt, int scheme, double* partials, int grid, int* status,
                             cudaStream_t s) {
  const uint32_t idesc = idesc_f16((uint32_t)fmt, TILE, TILE);
  if (scheme == kSchemeKara)
    energy_tc_kernel<kSchemeKara><<<grid, NTHREADS, kSmemBytes, s>>>(
        S, eps, sc, dg, scale, sh, Qp / KB, idesc, partials, status);
  else
    energy_tc_kernel<kSchemeDigits3><<<grid, NTHREADS, kSmemBytes, s>>>(
        S, eps, sc, dg, scale, sh, Qp / KB, idesc, partials, status);
  return cudaGetLastError();
}

}  // namespace corr
