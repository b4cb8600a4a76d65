// Batched precision-form RI-MP2 energies: many independent instances of uneven
// (nocc, nvir, naux) in one persistent launch fed by a device work queue.
//
// Every instance is sliced by the pre-pass of split.cu into its own region; a
// device table holds per instance the shape, the pointers of its row factors
// and orbital energies, its first global unit and its TMA map (the maps live in
// device memory, 64-byte aligned).  Units (instance, i<=j, A<=B) are numbered
// instance after instance in the order the host chose (the autotuned policy).
// The producer thread of each CTA takes the next unit from a global atomic
// counter and hands the unit number to the MMA thread and to the epilogue
// warps through a 4-slot ring in shared memory (mbarriers ufull/uempty); a
// negative number ends the CTA.  The per-unit work is that of energy_tc.cu
// (three exact digit levels in TMEM, D1 parked while D2 accumulates, D2 = D1^T
// through shared memory on diagonal tile pairs, FP64 diagonal).  Each unit
// writes its weighted {E_OS, E_SS} partial to unit_part[u]; a second kernel
// sums them per instance in a fixed order, so results are deterministic for
// any scheduling.  All waits are bounded (common.cuh).
#include "batch.h"
#include "common.cuh"
#include "kernels.h"
#include "tc_common.cuh"

namespace corr {

namespace {

constexpr int TILE = kTcTile;
constexpr int KB = kSliceQ;
constexpr int TILE_BYTES = TILE * KB * 2;
// a stage = the NPL digit planes of the row and of the column operand
template <int SCHEME>
__host__ __device__ constexpr int stage_bytes() {
  return 2 * planes_for_scheme(SCHEME) * TILE_BYTES;
}
constexpr int NTHREADS = 192;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t COL_STASH = 384;
constexpr uint32_t SW128 = 2;
constexpr int RING = 4;

template <int STAGES>
struct BCtl {
  uint64_t full[STAGES];
  uint64_t empty[STAGES];
  uint64_t afull;
  uint64_t aempty;
  uint64_t fin;
  uint64_t ufull[RING];
  uint64_t uempty[RING];
  long long uring[RING];
  uint32_t tmem;
  int abort;
  float db[TILE];
  float scb[TILE];
  double red[2][4];
  float tbuf[4][32][33];
  int wok[2][4];
};

template <int STAGES, int SCHEME>
constexpr size_t batch_smem_bytes() {
  return (size_t)STAGES * stage_bytes<SCHEME>() + sizeof(BCtl<STAGES>) + 1024;
}

// Instance of global unit u: last instance whose first unit is <= u.
__device__ __forceinline__ int find_instance(const BatchInst* __restrict__ in, int n, long long u) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (in[mid].unit_begin <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct UnitInfo {
  int inst, i, j, A, B;
};

__device__ __forceinline__ UnitInfo unit_info(const BatchInst* __restrict__ in, int n, long long u) {
  UnitInfo r;
  r.inst = find_instance(in, n, u);
  const BatchInst& b = in[r.inst];
  unit_decode_cost(u - b.unit_begin, b.o, b.ntiles, b.ntpairs, &r.i, &r.j, &r.A, &r.B);
  return r;
}

template <int STAGES, int SCHEME>
__global__ void __launch_bounds__(NTHREADS, 1)
    energy_batch_kernel(const BatchInst* __restrict__ insts,
                        int ninst, long long total, unsigned long long* __restrict__ queue,
                        uint32_t idesc, double* __restrict__ unit_part, int* status) {
  using Ctl = BCtl<STAGES>;
  constexpr int NPL = planes_for_scheme(SCHEME);
  constexpr int STAGE_BYTES = stage_bytes<SCHEME>();
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  Ctl* ctl = reinterpret_cast<Ctl*>(tiles + (size_t)STAGES * STAGE_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&ctl->full[s], 1);
      mbar_init(&ctl->empty[s], 1);
    }
    for (int s = 0; s < RING; ++s) {
      mbar_init(&ctl->ufull[s], 1);
      mbar_init(&ctl->uempty[s], 2);
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
    // Lane 0 takes units from the queue and paces the stages; lanes 0 and 1
    // copy a stage's row and column operand (three adjacent planes each).
    {
      int st = 0;
      uint32_t ph = 0;
      uint32_t last_ph[STAGES];
      bool has[STAGES];
      for (int s = 0; s < STAGES; ++s) has[s] = false;
      bool ok = true;
      const bool colop = (lane & 1) != 0;
      for (long long t = 0; ok; ++t) {
        const int slot = (int)(t % RING);
        const uint32_t use = (uint32_t)(t / RING);
        long long u = -2;  // -2: wait failed, -1: queue drained
        if (lane == 0) {
          if (mbar_wait(&ctl->uempty[slot], (use & 1) ^ 1, abort, status)) {
            u = (long long)atomicAdd(queue, 1ull);
            if (u >= total) u = -1;
            ctl->uring[slot] = u;
            mbar_arrive(&ctl->ufull[slot]);
          }
        }
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u < 0) break;
        const UnitInfo ui = unit_info(insts, ninst, u);
        const BatchInst& bi = insts[ui.inst];
        const int nph = (ui.i == ui.j || ui.A == ui.B) ? 1 : 2;
        for (int phs = 0; phs < nph && ok; ++phs) {
          const int x = phs == 0 ? ui.i : ui.j;
          const int y = phs == 0 ? ui.j : ui.i;
          const int slab = colop ? y : x, tile = colop ? ui.B : ui.A;
          for (int kb = 0; kb < bi.nkb; ++kb) {
            bool got = true;
            if (lane == 0) got = mbar_wait(&ctl->empty[st], ph ^ 1, abort, status);
            if (!__shfl_sync(0xffffffffu, got ? 1 : 0, 0)) {
              ok = false;
              break;
            }
            uint64_t* bar = &ctl->full[st];
            if (lane == 0) mbar_expect_tx(bar, STAGE_BYTES);
            __syncwarp();
            if (lane < 2)  // the NPL adjacent planes of the row / column operand
              bulk_load(tiles + (size_t)st * STAGE_BYTES + NPL * (colop ? 1 : 0) * TILE_BYTES,
                        bi.S + slice_tile_offset(0, slab, kb, tile, bi.nkb, bi.ntiles, NPL),
                        NPL * TILE_BYTES, bar);
            has[st] = true;
            last_ph[st] = ph;
            if (++st == STAGES) {
              st = 0;
              ph ^= 1;
            }
          }
        }
      }
      if (lane == 0) {
        int never = 0;
        for (int s = 0; s < STAGES; ++s)
          if (has[s]) mbar_wait(&ctl->full[s], last_ph[s], &never, status);
      }
      __syncwarp();
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int st = 0;
      uint32_t ph = 0;
      uint32_t nuse = 0;
      bool ok = true;
      const uint64_t dbase = smem_desc(smem_u32(tiles), 16, 1024, SW128);  // tile 0, stage 0
      for (long long t = 0; ok; ++t) {
        const int slot = (int)(t % RING);
        const uint32_t use = (uint32_t)(t / RING);
        if (!mbar_wait(&ctl->ufull[slot], use & 1, abort, status)) break;
        const long long u = ctl->uring[slot];
        mbar_arrive(&ctl->uempty[slot]);
        if (u < 0) break;
        const UnitInfo ui = unit_info(insts, ninst, u);
        const int nkb = insts[ui.inst].nkb;
        const int nph = (ui.i == ui.j || ui.A == ui.B) ? 1 : 2;
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
            const uint64_t ds = dbase + (uint64_t)(((uint32_t)st * STAGE_BYTES) >> 4);
#pragma unroll
            for (int kk = 0; kk < KB / 16; ++kk) {
              uint64_t r[NPL], q[NPL];
#pragma unroll
              for (int l = 0; l < NPL; ++l) {
                r[l] = ds + (uint64_t)((l * TILE_BYTES + kk * 32) >> 4);
                q[l] = ds + (uint64_t)(((NPL + l) * TILE_BYTES + kk * 32) >> 4);
              }
              const uint32_t acc = (kb | kk) ? 1u : 0u;
              issue_digit_mmas<SCHEME>(c0, c1, c2, r, q, idesc, acc);
            }
            tc_commit(&ctl->empty[st]);
            if (++st == STAGES) {
              st = 0;
              ph ^= 1;
            }
          }
          if (ok) tc_commit(&ctl->afull);
          ++nuse;
        }
      }
      tc_commit(&ctl->fin);
      int never = 0;
      mbar_wait(&ctl->fin, 0, &never, status);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;
    const int et = threadIdx.x - 64;
    const int arow = 32 * q + lane;
    const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16);
    bool dead = false;
    uint32_t nuse = 0;
    for (long long t = 0;; ++t) {
      const int slot = (int)(t % RING);
      const uint32_t use = (uint32_t)(t / RING);
      // unit number: every epilogue thread waits, reads, then one releases the slot
      const bool gotu = __all_sync(0xffffffffu, mbar_wait(&ctl->ufull[slot], use & 1, abort, status));
      if (lane == 0) ctl->wok[nuse & 1][q] = gotu ? 1 : 0;
      const long long u = gotu ? ctl->uring[slot] : -1;
      named_bar(1, 128);
      const bool all = ctl->wok[nuse & 1][0] & ctl->wok[nuse & 1][1] & ctl->wok[nuse & 1][2] &
                       ctl->wok[nuse & 1][3];
      named_bar(1, 128);
      if (et == 0 && all) mbar_arrive(&ctl->uempty[slot]);
      if (!all || u < 0) break;  // uniform: every thread read the same slot
      const UnitInfo ui = unit_info(insts, ninst, u);
      const BatchInst& bi = insts[ui.inst];
      const int o = bi.o, v = bi.v, i = ui.i, j = ui.j, A = ui.A, B = ui.B;
      const double* eps = bi.eps;
      const float* sc = bi.sc;
      const float inv_l = (float)bi.scale[1], inv_l2 = inv_l * inv_l;
      const int A0 = A * TILE, B0 = B * TILE;
      const bool same = (i == j);
      {
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
      const float dga = (diag_tile && a < v) ? bi.dg[(size_t)i * v + a] : 0.0f;
      double uos = 0.0, uss = 0.0;

      bool got = !dead && __all_sync(0xffffffffu, mbar_wait(&ctl->afull, nuse & 1, abort, status));
      if (lane == 0) ctl->wok[nuse & 1][q] = got ? 1 : 0;
      named_bar(1, 128);
      got = ctl->wok[nuse & 1][0] & ctl->wok[nuse & 1][1] & ctl->wok[nuse & 1][2] &
            ctl->wok[nuse & 1][3];
      if (!got) dead = true;
      if (!dead) {
        tc_fence_after();
        // phase-1 result to the stash columns; the accumulators go back to
        // the MMA issuer before the energy arithmetic (energy_tc.cu)
#pragma unroll 1
        for (int c = 0; c < TILE; c += 32) {
          float d1[32];
          load_level_sum<SCHEME>(tq, c, inv_l, inv_l2, sca1, ctl->scb, d1);
          tmem_st32(tq + COL_STASH + (uint32_t)c, d1);
        }
        tc_wait_st();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&ctl->aempty);
        if (same) {
#pragma unroll 1
          for (int c = 0; c < TILE; c += 32) {
            float d1[32];
            tmem_ld32(tq + COL_STASH + (uint32_t)c, d1);
            tc_wait_ld();
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
#pragma unroll 1
          for (int k = 0; k < 4; ++k) {
            float d[32];
            const int cw = 32 * ((q + k) & 3);
            tmem_ld32(tq + COL_STASH + (uint32_t)cw, d);
            tc_wait_ld();
#pragma unroll
            for (int x = 0; x < 32; ++x) ctl->tbuf[q][lane][x] = d[x];
            named_bar(1, 128);
            const int wr = (q - k) & 3;
            const int cr = 32 * wr;
            float d2[32];
#pragma unroll
            for (int x = 0; x < 32; ++x) d2[x] = ctl->tbuf[wr][x][lane];
            tmem_ld32(tq + COL_STASH + (uint32_t)cr, d);
            tc_wait_ld();
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
            named_bar(1, 128);
          }
        }
      }
      ++nuse;

      if (!same && A != B) {
        named_bar(1, 128);
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
          float d2a[TILE];
#pragma unroll
          for (int c = 0; c < TILE; c += 16)
            load_level_sum16<SCHEME>(tq, c, inv_l, inv_l2, sca2, ctl->scb, d2a + c);
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ctl->aempty);
#pragma unroll
          for (int c = 0; c < TILE; c += 32) {
            float d1[32];
            tmem_ld32(tq + COL_STASH + (uint32_t)c, d1);
            tc_wait_ld();
            float fos = 0.f, fss = 0.f;
#pragma unroll
            for (int k = 0; k < 32; ++k) {
              const float r = __frcp_rn(da + ctl->db[c + k]);
              const float x = d1[k], y = d2a[c + k];
              fos = fmaf(fmaf(x, x, y * y), r, fos);
              const float df = x - y;
              fss = fmaf(df * df, r, fss);
            }
            uos += (double)fos;
            uss += (double)fss;
          }
        }
        ++nuse;
      }
      // unit partial (weighted), reduced over the 128 epilogue threads
      const double fw = (A < B ? 2.0 : 1.0) * (same ? 0.5 : 1.0);
      double pos = warp_sum(-fw * uos), pss = warp_sum(-fw * uss);
      if (lane == 0) {
        ctl->red[0][q] = pos;
        ctl->red[1][q] = pss;
      }
      named_bar(1, 128);
      if (et == 0) {
        unit_part[2 * u] = (ctl->red[0][0] + ctl->red[0][1]) + (ctl->red[0][2] + ctl->red[0][3]);
        unit_part[2 * u + 1] =
            (ctl->red[1][0] + ctl->red[1][1]) + (ctl->red[1][2] + ctl->red[1][3]);
      }
      named_bar(1, 128);  // db/scb/red are rewritten by the next unit
    }
  }

  __syncwarp();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, TMEM_COLS);
}

// Per instance: fixed-order compensated sum of its unit partials, times the
// instance's energy scale, into out[4*k .. 4*k+3] = {E_SS, E_OS, E, E_SCS}.
__global__ void batch_reduce_kernel(const BatchInst* __restrict__ insts,
                                    const double* __restrict__ unit_part,
                                    const int* __restrict__ out_index, double* __restrict__ out) {
  const BatchInst b = insts[blockIdx.x];
  __shared__ double s_os[256], s_ss[256];
  double os = 0.0, ss = 0.0, cos_ = 0.0, css = 0.0;
  for (long long k = threadIdx.x; k < b.nunits; k += 256) {
    const long long u = b.unit_begin + k;
    double y = unit_part[2 * u] - cos_;
    double t = os + y;
    cos_ = (t - os) - y;
    os = t;
    y = unit_part[2 * u + 1] - css;
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
    const double sc = b.scale ? b.scale[0] : 1.0;
    const double eos = s_os[0] * sc, ess = s_ss[0] * sc;
    double* o = out + 4 * (size_t)out_index[blockIdx.x];
    o[0] = ess;
    o[1] = eos;
    o[2] = ess + eos;
    o[3] = ess / 3.0 + eos * 6.0 / 5.0;
  }
}

}  // namespace

size_t batch_kernel_smem(int stages) {
  return stages == 2 ? batch_smem_bytes<2, kSchemeDigits3>() : batch_smem_bytes<3, kSchemeDigits2>();
}

template <int STAGES, int SCHEME>
static cudaError_t set_batch_attr() {
  return cudaFuncSetAttribute(energy_batch_kernel<STAGES, SCHEME>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)batch_smem_bytes<STAGES, SCHEME>());
}

cudaError_t prepare_energy_batch() {
  cudaError_t e = set_batch_attr<2, kSchemeDigits3>();
  if (e == cudaSuccess) e = set_batch_attr<2, kSchemeDigits2>();
  if (e == cudaSuccess) e = set_batch_attr<3, kSchemeDigits2>();
  return e;
}

template <int STAGES, int SCHEME>
static void launch_batch_variant(const BatchInst* insts, int ninst,
                                 long long total, unsigned long long* queue, uint32_t idesc,
                                 int grid, double* unit_part, int* status, cudaStream_t s) {
  energy_batch_kernel<STAGES, SCHEME><<<grid, NTHREADS, batch_smem_bytes<STAGES, SCHEME>(), s>>>(
      insts, ninst, total, queue, idesc, unit_part, status);
}

// stages: 2 or 3 (the three-plane form fits two stages only and always runs 2)
cudaError_t launch_energy_batch(const BatchInst* insts, int ninst,
                                long long total, unsigned long long* queue, int fmt, int scheme,
                                int stages, int grid, double* unit_part, int* status,
                                cudaStream_t s) {
  const uint32_t idesc = idesc_f16((uint32_t)fmt, TILE, TILE);
  if (scheme != kSchemeDigits2)
    launch_batch_variant<2, kSchemeDigits3>(insts, ninst, total, queue, idesc, grid, unit_part,
                                            status, s);
  else if (stages == 3)
    launch_batch_variant<3, kSchemeDigits2>(insts, ninst, total, queue, idesc, grid, unit_part,
                                            status, s);
  else
    launch_batch_variant<2, kSchemeDigits2>(insts, ninst, total, queue, idesc, grid, unit_part,
                                            status, s);
  return cudaGetLastError();
}

cudaError_t launch_batch_reduce(const BatchInst* insts, int ninst, const double* unit_part,
                                const int* out_index, double* out, cudaStream_t s) {
  batch_reduce_kernel<<<ninst, 256, 0, s>>>(insts, unit_part, out_index, out);
  return cudaGetLastError();
}

}  // namespace corr
