// Precision-form fused RI-MP2 energy on the 5th-generation tensor cores, for
// one instance or for a batch of independent instances in one launch (the
// same kernel template; the batch form looks each unit's instance up in a
// device table).
//
// Input: the 16-bit integer digit planes of B (split.cu; three in scheme 0,
// two in scheme 1) in the tiled layout of kernels.h: every 128 x 64 operand
// tile is one contiguous, pre-swizzled (128-byte swizzle) 16 KB block fetched
// with a linear bulk copy (whole 128-byte lines from L2).
// Work unit = (instance, occupied pair i<=j, virtual tile pair A<=B), tiles of
// 128 rows.  Units are numbered instance after instance; within an instance
// in cost order (two-phase units first, tc_common.cuh).
//
// Phase 1 forms D1[a][b] = (ia|jb) for a in A, b in B; phase 2 forms
// D2[a][b] = (ib|ja).  Each phase accumulates three exact integer sums in
// TMEM (split.cu), by scheme:
//   0: acc_m = sum_{k+l=m} s_k(row) . s_l(col)^T   (m = 0..2, six MMAs per K=16)
//   1: acc_0 = s0.s0', acc_1 = s0.s1' + s1.s0', acc_2 = s1.s1'   (four MMAs per K=16)
// and the epilogue forms d = sc_row sc_col (acc_0 + acc_1/L + acc_2/L^2) in
// FP32 (tc_common.cuh).  D1 is parked in TMEM columns 384-511 while D2
// accumulates in 0-383.  For i == j, D2 == D1 and phase 2 is skipped; for
// A == B, D2 = D1^T is obtained by a 32x32-block exchange through shared
// memory instead of a second pass.  On the (i==j, A==B) diagonal the element
// (ia|ia) is replaced by its FP64 value.
//
// Every tile runs 128 wide: the padded columns of the last virtual tile are
// zeros in the digit layout and get column scale 0.  (A narrower last tile
// needs a second MMA instruction descriptor, and on the issue path, which
// runs in step with the tensor pipe, any descriptor that is not a kernel
// parameter, a second copy of the issue loop, or predicated descriptor pairs
// each cost more than the padded columns: 0.663 / 0.728 / 0.99 ms against
// 0.613 ms for nocc=40, nvir=360, naux=1200.)
//
// Energy arithmetic (tc_common.cuh, pair_terms2): the denominators
// D = (e_a - e_i) + (e_b - e_j) come from the FP64 orbital energies as
// float-float pairs, 1/D is taken to ~2^-44 relative (one float-float
// Newton-Raphson step), the squares and products are error-free (FMA
// residuals), and the terms are summed in float-float over 32 columns, then
// in FP64: the only rounding of FP32 size left in the energy is that of the
// (ia|jb) values themselves.  Two columns per packed FP32 instruction.
//
// CTA = 6 warps, persistent, one CTA per SM, units from a device work queue:
//   warp 0     bulk-copy producer (lane 0 takes units and paces the stages;
//              lane 2l + c copies digit plane l of the row (c = 0) or column
//              (c = 1) operand), 2 stages of 96 KB (scheme 0) or 2-3 of 64 KB
//   warp 1     TMEM owner + MMA issuer (one thread), tcgen05.mma kind::f16
//   warps 2..  epilogue: EG groups of four warps (one per TMEM lane quarter),
//              group g owning the 32-column chunks c with c % EG == g
// Every unit writes its own {E_OS, E_SS} partial, summed afterwards in unit
// order, so results do not depend on which CTA took which unit.  Every wait
// is bounded (common.cuh); on a timeout the CTA winds down and the host sees
// CORR_ERR_DEVICE_TIMEOUT.
#include "common.cuh"
#include "kernels.h"
#include "tc_common.cuh"

namespace corr {

namespace {

constexpr int TILE = kTcTile;                 // 128
constexpr int KB = kSliceQ;                   // Q per stage (128-byte tile rows)
constexpr int TILE_BYTES = TILE * KB * 2;     // 16 KB
// Epilogue groups: EG groups of four warps (one per TMEM lane quarter); group
// g owns the 32-column chunks c with c % EG == g of every tile.
constexpr int EG = 1;
constexpr int NEPI = 128 * EG;                // epilogue threads
constexpr int NCH = 4 / EG;                   // column chunks per group
constexpr int NTHREADS = 64 + NEPI;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t COL_STASH = 384;           // parked D1
constexpr uint32_t SW128 = 2;                 // descriptor layout type: 128B swizzle
constexpr int RING = 4;                       // unit numbers in flight

template <int SCHEME, int STAGES>
struct Geo {
  static constexpr int NPL = planes_for_scheme(SCHEME);
  static constexpr int STAGE_BYTES = 2 * NPL * TILE_BYTES;  // row + column operand planes
  static constexpr int RING_BYTES = STAGES * STAGE_BYTES;
};

template <int STAGES>
struct Ctl {
  uint64_t full[STAGES];
  uint64_t empty[STAGES];
  uint64_t ufull[RING];   // unit ring: producer -> MMA thread and epilogue
  uint64_t uempty[RING];
  long long uring[RING];
  int unph[RING];         // the unit's MMA phases and Q blocks, for the MMA role
  int unkb[RING];
  uint64_t afull;
  uint64_t aempty;
  uint64_t fin;
  uint32_t tmem;
  int abort;
  int wu[2][4 * EG];      // per-warp outcome of the epilogue's unit wait
  int wok[2][4 * EG];     // per-warp outcome of the accumulator wait
  float2 db[TILE];        // column denominators e_b - e_j (float-float)
  float scb[TILE];        // column scales
  double red[2][4 * EG];
  float tbuf[EG][NCH][32][33];  // D1 -> D1^T exchange on diagonal tile pairs (per group)
};

template <int SCHEME, int STAGES>
constexpr size_t smem_bytes() {
  return (size_t)Geo<SCHEME, STAGES>::RING_BYTES + sizeof(Ctl<STAGES>) + 1024;
}
static_assert(smem_bytes<1, 3>() <= 227 * 1024, "shared memory");
static_assert(smem_bytes<0, 2>() <= 227 * 1024, "shared memory");

struct Work {
  int i, j, A, B;  // occupied pair and tile pair of the instance
  int nph;         // MMA phases: 1 (D2 from D1) or 2
};

// Table index of the instance that owns global unit u (the last instance
// whose first unit is <= u).
__device__ __forceinline__ int find_instance(const TcInst* __restrict__ tab, int n, long long u) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tab[mid].unit_begin <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <bool BATCH>
__device__ __forceinline__ Work work_at(long long u, const TcInst& one,
                                        const TcInst* __restrict__ tab, int n, TcInst* in) {
  if (BATCH) *in = tab[find_instance(tab, n, u)];
  else *in = one;
  Work w;
  w.nph = unit_decode_cost(u - in->unit_begin, in->o, in->ntiles, in->ntpairs, &w.i, &w.j, &w.A,
                           &w.B);
  return w;
}

// The four epilogue warps agree on one outcome of a wait (named barriers
// below must be reached by all of them or none).
template <int STAGES>
__device__ __forceinline__ bool epi_agree(Ctl<STAGES>* ctl, int (*slot)[4 * EG], int par, int ew,
                                          int lane, bool mine) {
  const bool w = __all_sync(0xffffffffu, mine);
  if (lane == 0) slot[par][ew] = w ? 1 : 0;
  named_bar(1, NEPI);
  int all = 1;
#pragma unroll
  for (int k = 0; k < 4 * EG; ++k) all &= slot[par][k];
  return all != 0;
}

// Element e of 32-column chunk s of a register array a[32 * N] for a run-time
// s: N - 1 selects, so a stays in registers (e is a compile-time constant in
// the unrolled callers).
template <int N>
__device__ __forceinline__ float pick_chunk(const float* a, int s, int e) {
  float r = a[e];
#pragma unroll
  for (int t = 1; t < N; ++t) r = s == t ? a[32 * t + e] : r;
  return r;
}

// Energy terms of the 32 columns [cb, cb + 32) of this thread's row for a
// pair i != j: x = D1 from the stash at TMEM address xs (16 columns at a time,
// to keep few registers live), y(e) = D2 (a functor, so D2 can come from
// registers or from shared memory without a copy); the float-float sums go to
// FP64 at the end.
template <class Y>
__device__ __forceinline__ void chunk_pair_terms(uint32_t xs, Y y, float2 da, const float2* db,
                                                 int cb, FFSum2& os, FFSum2& ss) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float x[16];
    tmem_ld16(xs + 16u * h, x);
    tc_wait_ld();
    ld_ready<16>(x);
#pragma unroll
    for (int e = 0; e < 16; e += 2) {
      const float2 b0 = db[cb + 16 * h + e], b1 = db[cb + 16 * h + e + 1];
      float2 rh, rl;
      recip_ff2(da, make_float2(b0.x, b1.x), make_float2(b0.y, b1.y), &rh, &rl);
      pair_terms2(make_float2(x[e], x[e + 1]), make_float2(y(16 * h + e), y(16 * h + e + 1)), rh,
                  rl, os, ss);
    }
  }
  os.flush();
  ss.flush();
}

// Position in the operand ring: stage index and its mbarrier parity.
struct StagePos {
  int st;
  uint32_t ph;
};

// One MMA phase: every Q block of the unit from the operand ring into the
// level accumulators at TMEM columns tmem + {0, 128, 256}, each stage
// released to the producer once its MMAs finish.  False when a wait failed.
template <int SCHEME, int STAGES>
__device__ __forceinline__ bool mma_phase(Ctl<STAGES>* ctl, uint64_t dbase, uint32_t tmem, int nkb,
                                          uint32_t idesc, StagePos* pos, volatile int* abort,
                                          int* status) {
  using G = Geo<SCHEME, STAGES>;
  constexpr int NPL = G::NPL, STAGE_BYTES = G::STAGE_BYTES;
  const uint32_t c0 = tmem, c1 = tmem + 128u, c2 = tmem + 256u;
  int st = pos->st;
  uint32_t ph = pos->ph;
  bool ok = true;
  bool ready = false;  // the next stage's barrier, probed ahead of time
  for (int kb = 0; kb < nkb; ++kb) {
    if (!ready && !mbar_wait(&ctl->full[st], ph, abort, status)) {
      ok = false;
      break;
    }
    // (no tcgen05 fence: the bulk copies' mbarrier completion orders the
    // shared-memory operands)
    const uint64_t ds = dbase + (uint64_t)(((uint32_t)st * STAGE_BYTES) >> 4);
    const int nst = st + 1 == STAGES ? 0 : st + 1;
    const uint32_t nph = st + 1 == STAGES ? ph ^ 1 : ph;
    ready = false;
#pragma unroll
    for (int kk = 0; kk < KB / 16; ++kk) {
      uint64_t r[NPL], q[NPL];
#pragma unroll
      for (int p = 0; p < NPL; ++p) {
        r[p] = ds + (uint64_t)((p * TILE_BYTES + kk * 32) >> 4);
        q[p] = ds + (uint64_t)(((NPL + p) * TILE_BYTES + kk * 32) >> 4);
      }
      // while the MMAs queued so far run, probe the next stage (non-blocking),
      // so the stage boundary costs no barrier latency
      if (kk == KB / 16 - 1 && kb + 1 < nkb) ready = mbar_test_wait(&ctl->full[nst], nph);
      const uint32_t acc = (kb | kk) ? 1u : 0u;
      issue_digit_mmas<SCHEME>(c0, c1, c2, r, q, idesc, acc);
    }
    tc_commit(&ctl->empty[st]);  // stage reusable once these MMAs finish
    if (++st == STAGES) {
      st = 0;
      ph ^= 1;
    }
  }
  pos->st = st;
  pos->ph = ph;
  return ok;
}

template <int SCHEME, int STAGES, bool BATCH>
__global__ void __launch_bounds__(NTHREADS, 1)
    energy_tc_kernel(TcInst one, const TcInst* __restrict__ tab, int ninst, long long total,
                     uint32_t idesc, double* __restrict__ partials,
                     int* status, unsigned long long* __restrict__ queue) {
  using G = Geo<SCHEME, STAGES>;
  constexpr int NPL = G::NPL, STAGE_BYTES = G::STAGE_BYTES;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  Ctl<STAGES>* ctl = reinterpret_cast<Ctl<STAGES>*>(tiles + G::RING_BYTES);
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
    mbar_init(&ctl->aempty, 4 * EG);
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
    // The whole warp runs the loop: lane 0 takes the unit and waits for a
    // free stage, then lanes 0 .. 2 NPL - 1 issue the stage's copies in one
    // instruction (one copy per lane issues several times faster than the
    // same copies in sequence from one thread).
    int st = 0;
    uint32_t ph = 0;
    uint32_t last_ph[STAGES];
    bool has[STAGES];
    for (int s = 0; s < STAGES; ++s) has[s] = false;
    bool ok = true;
    const int l = lane >> 1;
    const bool colop = (lane & 1) != 0;
    for (long long t = 0; ok; ++t) {
      const int slot = (int)(t % RING);
      const uint32_t use = (uint32_t)(t / RING);
      long long u = -2;  // -2: wait failed, -1: queue drained
      if (lane == 0 && mbar_wait(&ctl->uempty[slot], (use & 1) ^ 1, abort, status)) {
        u = (long long)atomicAdd(queue, 1ull);
        if (u >= total) u = -1;
        // the MMA role needs only the phase and Q-block counts: decoded here,
        // off its issue path (which runs in step with the tensor pipe)
        int nph = 0, nkb = 0;
        if (u >= 0) {
          TcInst in0;
          nph = work_at<BATCH>(u, one, tab, ninst, &in0).nph;
          nkb = in0.nkb;
        }
        ctl->uring[slot] = u;
        ctl->unph[slot] = nph;
        ctl->unkb[slot] = nkb;
        mbar_arrive(&ctl->ufull[slot]);
      }
      u = __shfl_sync(0xffffffffu, u, 0);
      if (u == -2) ok = false;
      if (u < 0) break;
      TcInst in;
      const Work w = work_at<BATCH>(u, one, tab, ninst, &in);
      for (int phs = 0; phs < w.nph && ok; ++phs) {
        const int x = phs == 0 ? w.i : w.j;  // row operand slab
        const int y = phs == 0 ? w.j : w.i;  // column operand slab
        const int slab = colop ? y : x, tile = colop ? w.B : w.A;
        for (int kb = 0; kb < in.nkb; ++kb) {
          bool got = true;
          if (lane == 0) got = mbar_wait(&ctl->empty[st], ph ^ 1, abort, status);
          if (!__shfl_sync(0xffffffffu, got ? 1 : 0, 0)) {
            ok = false;
            break;
          }
          uint64_t* bar = &ctl->full[st];
          if (lane == 0) mbar_expect_tx(bar, (uint32_t)(2 * NPL * TILE_BYTES));
          __syncwarp();
          if (lane < 2 * NPL)
            bulk_load(tiles + (size_t)st * STAGE_BYTES + (NPL * (colop ? 1 : 0) + l) * TILE_BYTES,
                      in.S + slice_tile_offset(l, slab, kb, tile, in.nkb, in.ntiles, NPL), TILE_BYTES,
                      bar);
          has[st] = true;
          last_ph[st] = ph;
          if (++st == STAGES) {
            st = 0;
            ph ^= 1;
          }
        }
      }
    }
    // never leave with a bulk copy still landing in shared memory
    if (lane == 0) {
      int never = 0;
      for (int s = 0; s < STAGES; ++s)
        if (has[s]) mbar_wait(&ctl->full[s], last_ph[s], &never, status);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      StagePos ring{0, 0u};
      uint32_t nuse = 0;
      bool ok = true;
      // shared-memory descriptor of tile 0 of stage 0 (every tile address is
      // below 2^18, so offsets added to the 14-bit start field never carry out)
      const uint64_t dbase = smem_desc(smem_u32(tiles), 16, 1024, SW128);
      for (long long t = 0; ok; ++t) {
        const int slot = (int)(t % RING);
        const uint32_t use = (uint32_t)(t / RING);
        if (!mbar_wait(&ctl->ufull[slot], use & 1, abort, status)) break;
        const long long u = ctl->uring[slot];
        const int nph = ctl->unph[slot], nkb = ctl->unkb[slot];
        mbar_arrive(&ctl->uempty[slot]);
        if (u < 0) break;
        for (int phs = 0; phs < nph && ok; ++phs) {
          if (!mbar_wait(&ctl->aempty, (nuse & 1) ^ 1, abort, status)) {
            ok = false;
            break;
          }
          tc_fence_after();
          // the instruction descriptor stays a kernel parameter (see the header)
          const bool pok =
              mma_phase<SCHEME, STAGES>(ctl, dbase, tmem, nkb, idesc, &ring, abort, status);
          if (!pok) ok = false;
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
    const int ew = warp - 2;          // epilogue warp 0 .. 4 EG - 1
    const int g = ew >> 2;            // group: owns the column chunks c % EG == g
    const int q = warp & 3;           // TMEM lane quarter of this warp
    const int et = threadIdx.x - 64;  // 0 .. NEPI - 1
    const int arow = 32 * q + lane;   // accumulator row = TMEM lane
    const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16);
    bool dead = false;
    uint32_t nuse = 0;
    for (long long t = 0;; ++t) {
      if (dead) break;
      // unit number: every epilogue thread waits and reads, then one thread
      // releases the slot (after the barrier that ends the reads)
      const int slot = (int)(t % RING);
      const uint32_t use = (uint32_t)(t / RING);
      const bool gotu = mbar_wait(&ctl->ufull[slot], use & 1, abort, status);
      const long long u = gotu ? ctl->uring[slot] : -1;
      const bool all = epi_agree(ctl, ctl->wu, (int)(t & 1), ew, lane, gotu);
      named_bar(1, NEPI);
      if (et == 0 && all) mbar_arrive(&ctl->uempty[slot]);
      if (!all || u < 0) break;  // uniform: every thread read the same slot
      TcInst in;
      const Work w = work_at<BATCH>(u, one, tab, ninst, &in);
      const int o = in.o, v = in.v, i = w.i, j = w.j, A = w.A, B = w.B;
      const bool two = w.nph == 2, same = i == j;
      const float inv_l = (float)in.scale[1];
      const float inv_l2 = inv_l * inv_l;
      const int A0 = A * TILE, B0 = B * TILE;
      if (et < TILE) {
        // phase-1 columns come from slab j; padded columns get scale 0 and a
        // finite denominator
        const int b = B0 + et;
        const bool live = b < v;
        ctl->db[et] = live ? ff_split(in.eps[o + b] - in.eps[j]) : make_float2(1.0f, 0.0f);
        ctl->scb[et] = live ? in.sc[(size_t)j * v + b] : 0.0f;
      }
      named_bar(1, NEPI);
      const int a = A0 + arow;
      const bool alive = a < v;
      const float2 da = alive ? ff_split(in.eps[o + a] - in.eps[i]) : make_float2(1.0f, 0.0f);
      const float sca1 = alive ? in.sc[(size_t)i * v + a] : 0.0f;
      const float sca2 = alive ? in.sc[(size_t)j * v + a] : 0.0f;
      const bool diag_tile = same && (A == B);
      FFSum2 os, ss;  // flushed to FP64 after every 32 columns
      float d2a[32 * NCH];  // this group's chunks of D2 of a two-phase unit, this row

      // ---- phase 1: D1
      bool got = !dead && mbar_wait(&ctl->afull, nuse & 1, abort, status);
      got = epi_agree(ctl, ctl->wok, (int)(nuse & 1), ew, lane, got);
      if (!got) dead = true;
      if (!dead) {
        tc_fence_after();
        // Phase-1 result (scaled D1, FP32) of this group's chunks to the
        // stash columns, then the accumulators go back to the MMA issuer at
        // once: the rest of this unit's epilogue overlaps the next phase's MMAs.
#pragma unroll 1
        for (int s = 0; s < NCH; ++s) {
          const int c = 32 * (g + EG * s);
          float d1[32];
          load_level_sum16<SCHEME>(tq, c, inv_l, inv_l2, sca1, ctl->scb, d1);
          load_level_sum16<SCHEME>(tq, c + 16, inv_l, inv_l2, sca1, ctl->scb, d1 + 16);
          tmem_st32(tq + COL_STASH + (uint32_t)c, d1);
        }
        tc_wait_st();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&ctl->aempty);
        if (EG > 1 && !same && !two) {
          // the exchange below reads every chunk of the stash, some written by
          // the other groups
          named_bar(1, NEPI);
          tc_fence_after();
        }
        if (same) {
          // i == j: D2 == D1, E_OS only.  On a diagonal tile the element
          // (ia|ia) is the FP64 diagonal: its high part enters here, the
          // correction for its low part after the loop.
          const float2 dga = (diag_tile && alive) ? in.dg[(size_t)i * v + a] : make_float2(0.f, 0.f);
#pragma unroll 1
          for (int s = 0; s < NCH; ++s) {
            const int c = 32 * (g + EG * s);
            float d1[32];
            tmem_ld32(tq + COL_STASH + (uint32_t)c, d1);
            tc_wait_ld();
            ld_ready<32>(d1);
#pragma unroll
            for (int k = 0; k < 32; k += 2) {
              const float x0 = (diag_tile && c + k == arow) ? dga.x : d1[k];
              const float x1 = (diag_tile && c + k + 1 == arow) ? dga.x : d1[k + 1];
              const float2 b0 = ctl->db[c + k], b1 = ctl->db[c + k + 1];
              float2 rh, rl;
              recip_ff2(da, make_float2(b0.x, b1.x), make_float2(b0.y, b1.y), &rh, &rl);
              same_pair_term2(make_float2(x0, x1), rh, rl, os);
            }
            os.flush();
          }
          // 2 (xh + xl)^2 - 2 xh^2 = 4 xh xl + O(xl^2), by the group owning column arow
          if (diag_tile && alive && (q % EG) == g) {
            float rh, rl;
            recip_ff(da, ctl->db[arow], &rh, &rl);
            os.add(make_float2(4.0f * dga.x * dga.y * rh, 0.0f), make_float2(0.0f, 0.0f));
            os.flush();
          }
        }
      }
      ++nuse;

      // ---- phase 2: D2 (two-phase units): rows from slab j, columns from slab i
      if (two) {
        named_bar(1, NEPI);  // everyone is done with the phase-1 column scales
        if (B0 + et < v) ctl->scb[et] = in.sc[(size_t)i * v + B0 + et];
        named_bar(1, NEPI);
        got = !dead && mbar_wait(&ctl->afull, nuse & 1, abort, status);
        got = epi_agree(ctl, ctl->wok, (int)(nuse & 1), ew, lane, got);
        if (!got) dead = true;
        if (!dead) {
          tc_fence_after();
          // this group's chunks of D2 (scaled, FP32) into registers, then
          // release the accumulators
#pragma unroll
          for (int s = 0; s < NCH; ++s) {
            const int c = 32 * (g + EG * s);
            load_level_sum16<SCHEME>(tq, c, inv_l, inv_l2, sca2, ctl->scb, d2a + 32 * s);
            load_level_sum16<SCHEME>(tq, c + 16, inv_l, inv_l2, sca2, ctl->scb, d2a + 32 * s + 16);
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ctl->aempty);
        }
        ++nuse;
      }

      // ---- energy of a pair i != j, 32 columns at a time: x = D1 (stash),
      // y = D2 (registers, two-phase units) or D1^T (diagonal tile pairs,
      // A == B).  For D1^T, in round k every warp of the group whose lane
      // quarter c is one of the group's chunks publishes its D1 block of column
      // chunk (c+k)%4, and the warp of quarter q = (c+k)%4 takes it: the D1^T
      // block of its column chunk c.
      if (!dead && !same && two) {
#pragma unroll 1
        for (int s = 0; s < NCH; ++s) {
          const int cb = 32 * (g + EG * s);
          // D2 from registers: a compile-time register choice per column
          chunk_pair_terms(tq + COL_STASH + (uint32_t)cb,
                           [&](int e) { return pick_chunk<NCH>(d2a, s, e); }, da, ctl->db, cb, os,
                           ss);
        }
      } else if (!dead && !same) {
        // The terms of (a, b) and (b, a) are equal on a diagonal tile pair (the
        // denominator is symmetric, x and y swap), so the block pairs {q, q-k}
        // of round k (k = 1: four adjacent pairs; k = 2: pairs {0,2}, {1,3},
        // taken by quarters 0 and 1) count twice and round 3 repeats round 1.
        static_assert(EG == 1, "the round plan below assumes one group of four quarters");
        double w1_os = 0.0, w1_ss = 0.0;
#pragma unroll 1
        for (int k = 0; k < 3; ++k) {
          if (k == 1) {  // the diagonal blocks (weight 1) are in; the rest weigh 2
            w1_os = os.d;
            w1_ss = ss.d;
            os.d = 0.0;
            ss.d = 0.0;
          }
          if (q % EG == g) {  // publisher
            float x[32];
            const int cw = 32 * ((q + k) & 3);
            tmem_ld32(tq + COL_STASH + (uint32_t)cw, x);
            tc_wait_ld();
            ld_ready<32>(x);
#pragma unroll
            for (int e = 0; e < 32; ++e) ctl->tbuf[g][q / EG][lane][e] = x[e];
          }
          named_bar(2 + g, 128);
          const int wr = (q - k) & 3, cb = 32 * wr;
          if (wr % EG == g && (k < 2 || q < 2))  // reader
            chunk_pair_terms(tq + COL_STASH + (uint32_t)cb,
                             [&](int e) { return ctl->tbuf[g][wr / EG][e][lane]; }, da, ctl->db,
                             cb, os, ss);
          named_bar(2 + g, 128);  // tbuf is rewritten in the next round
        }
        os.d = w1_os + 2.0 * os.d;
        ss.d = w1_ss + 2.0 * ss.d;
      }
      // unit partial (weighted), reduced over the epilogue threads in a fixed
      // order; the host-side reduction sums the units in unit order
      const double fw = (A < B ? 2.0 : 1.0) * (same ? 0.5 : 1.0);
      const double pos = warp_sum(-fw * os.d), pss = warp_sum(-fw * ss.d);
      if (lane == 0) {
        ctl->red[0][ew] = pos;
        ctl->red[1][ew] = pss;
      }
      named_bar(1, NEPI);
      if (et == 0) {
        double s0 = 0.0, s1 = 0.0;
#pragma unroll
        for (int k = 0; k < 4 * EG; ++k) {
          s0 += ctl->red[0][k];
          s1 += ctl->red[1][k];
        }
        partials[2 * u] = s0;
        partials[2 * u + 1] = s1;
      }
      named_bar(1, NEPI);  // db/scb/red are rewritten by the next unit
    }
  }

  __syncwarp();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, TMEM_COLS);
}

template <int SCHEME, int STAGES, bool BATCH>
cudaError_t set_attr() {
  return cudaFuncSetAttribute(energy_tc_kernel<SCHEME, STAGES, BATCH>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem_bytes<SCHEME, STAGES>());
}

template <int SCHEME, int STAGES, bool BATCH>
cudaError_t launch_variant(const TcInst& one, const TcInst* tab, int n, long long total, int fmt,
                           int grid, double* partials, int* status, unsigned long long* queue,
                           cudaStream_t s) {
  const uint32_t idf = idesc_f16((uint32_t)fmt, TILE, TILE);
  energy_tc_kernel<SCHEME, STAGES, BATCH>
      <<<grid, NTHREADS, smem_bytes<SCHEME, STAGES>(), s>>>(one, tab, n, total, idf, partials,
                                                            status, queue);
  return cudaGetLastError();
}

template <bool BATCH>
cudaError_t dispatch(const TcInst& one, const TcInst* tab, int n, long long total, int fmt,
                     int scheme, int stages, int grid, double* partials, int* status,
                     unsigned long long* queue, cudaStream_t s) {
  if (scheme != kSchemeDigits2)  // three 32 KB planes per operand: two 96 KB stages fit
    return launch_variant<kSchemeDigits3, 2, BATCH>(one, tab, n, total, fmt, grid, partials,
                                                    status, queue, s);
  if (stages == 2)
    return launch_variant<kSchemeDigits2, 2, BATCH>(one, tab, n, total, fmt, grid, partials,
                                                    status, queue, s);
  return launch_variant<kSchemeDigits2, 3, BATCH>(one, tab, n, total, fmt, grid, partials, status,
                                                  queue, s);
}

}  // namespace

TcInst make_tc_inst(const SliceWork& sw, const double* eps, const EnergyShape& sh, int Qp,
                    long long unit_begin) {
  TcInst t;
  t.S = sw.S;
  t.eps = eps;
  t.sc = sw.sc;
  t.dg = sw.dg;
  t.scale = sw.scale;
  t.unit_begin = unit_begin;
  t.nunits = sh.nunits;
  t.o = sh.nocc;
  t.v = sh.nvir;
  t.ntiles = sh.ntiles;
  t.ntpairs = sh.ntpairs;
  t.nkb = Qp / kSliceQ;
  return t;
}

cudaError_t prepare_energy_tc() {
  cudaError_t e = set_attr<kSchemeDigits3, 2, false>();
  if (e == cudaSuccess) e = set_attr<kSchemeDigits3, 2, true>();
  if (e == cudaSuccess) e = set_attr<kSchemeDigits2, 2, false>();
  if (e == cudaSuccess) e = set_attr<kSchemeDigits2, 2, true>();
  if (e == cudaSuccess) e = set_attr<kSchemeDigits2, 3, false>();
  if (e == cudaSuccess) e = set_attr<kSchemeDigits2, 3, true>();
  return e;
}

cudaError_t launch_energy_tc(const TcInst& inst, int fmt, int scheme, int stages, int grid,
                             double* partials, int* status, unsigned long long* queue,
                             cudaStream_t s) {
  // the queue counter and, after it, the ticket of the final reduction
  cudaError_t e = cudaMemsetAsync(queue, 0, 2 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  return dispatch<false>(inst, nullptr, 1, inst.nunits, fmt, scheme, stages, grid, partials,
                         status, queue, s);
}

cudaError_t launch_energy_tc_batch(const TcInst* dtab, int n, long long total, int fmt, int scheme,
                                   int stages, int grid, double* partials, int* status,
                                   unsigned long long* queue, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(queue, 0, 2 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  TcInst none{};
  return dispatch<true>(none, dtab, n, total, fmt, scheme, stages, grid, partials, status, queue,
                        s);
}

}  // namespace corr
