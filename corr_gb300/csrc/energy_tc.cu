// Precision-form fused RI-MP2 energy on the 5th-generation tensor cores.
//
// Input: the 16-bit integer digit planes of B (split.cu; three in scheme 0,
// two in scheme 1) in the tiled layout of kernels.h: every 128 x 64 operand
// tile is one contiguous, pre-swizzled (128-byte swizzle) 16 KB block fetched
// with a linear bulk copy (whole 128-byte lines from L2).
// Work unit = (occupied pair i<=j, virtual tile pair A<=B), tiles of 128.
//
// Phase 1 forms D1[a][b] = (ia|jb) for a in A, b in B; phase 2 forms
// D2[a][b] = (ib|ja).  Each phase accumulates three exact integer sums in
// TMEM (split.cu), by scheme:
//   0: acc_m = sum_{k+l=m} s_k(row) . s_l(col)^T   (m = 0..2, six MMAs per K=16)
//   1: acc_0 = s0.s0', acc_1 = s0.s1' + s1.s0', acc_2 = s1.s1'   (four MMAs per K=16)
// Scheme 1 moves 4 KB of operands per 128x128x16 MMA (two planes of each
// operand for four MMAs), half of what three planes for three products would.
// The epilogue forms d = sc_row sc_col (value of the digits) in FP32 with
// round-to-nearest (tc_common.cuh).  Measured at nocc=40, nvir=360,
// naux=1200: the tensor pipe is active 73 % of the cycles while shared memory
// (banks 28 % read, 19 % write; tensor-core path 55 %), L2 (53 %) and DRAM
// (4 %) all have room: the gaps are the single issuing thread's hand-offs.
// D1 is parked in TMEM columns 384-511 while D2 accumulates in 0-383.  For
// i == j, D2 == D1 and phase 2 is skipped; for A == B, D2 = D1^T is obtained
// by a 32x32-block exchange through shared memory instead of a second pass.  On the (i==j, A==B) diagonal the
// element (ia|ia) is replaced by its FP64 value.  The energy epilogue is the
// one of energy_fp64.cu:
//   E_OS -= f w (D1^2 + D2^2)/D,  E_SS -= f w (D1 - D2)^2/D,
// with 1/D as an IEEE-rounded FP32 reciprocal and FP64 sums per unit.
//
// Cluster form (CL): 2 x 2 clusters of CTAs.  A cluster takes a block pair
// (a <= b) of occupied indices and a tile pair; CTA (r, c) of the cluster
// computes the pair (i, j) = (2a + r, 2b + c).  The D1 row tile (i, A) is
// needed by both CTAs of cluster row r and the column tile (j, B) by both
// CTAs of cluster column c (in phase 2 the roles swap: rows (j, A) per column,
// columns (i, B) per row), so each CTA copies one 64-row half of each shared
// tile and multicasts it to the CTAs that need it: half the L2 -> SM stream
// of the plain form.  A stage of CTA X is written by X and its two partners,
// so its `empty` barrier waits for three consumer releases (tcgen05.commit
// multicast).  All four CTAs run the same phase sequence: tile pairs A != B
// always take two phases (for i == j the second recomputes D2 = D1), pairs
// outside i <= j < nocc load their share and contribute with weight 0.
//
// CTA = 6 warps, persistent, one CTA per SM:
//   warp 0     bulk-copy producer (lane 0 paces; one lane per 16 KB operand tile:
//              the digit planes of the row and of the column operand), 2 stages
//              (scheme 0, 96 KB each) or 3 (scheme 1, 64 KB each)
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
constexpr int KB = kSliceQ;                   // 16-bit Q elements per tile row (128 B)
constexpr int KBS = 1;                        // Q blocks per pipeline stage
constexpr int TILE_BYTES = TILE * KB * 2;     // 16 KB
constexpr int HALF_BYTES = TILE_BYTES / 2;    // 64 rows of a tile (cluster form)
// Per scheme: NPL digit planes per operand, a stage = KBS x NPL planes x (row,
// column operand) in a 192 KB ring: 3 stages of two planes (64 KB), 2 of three.
template <int SCHEME>
struct Geo {
  static constexpr int NPL = planes_for_scheme(SCHEME);
  static constexpr int STAGES = NPL == 2 ? 3 : 2;
  static constexpr int NTILES = 2 * NPL * KBS;
  static constexpr int STAGE_BYTES = NTILES * TILE_BYTES;
};
constexpr int MAX_STAGES = 3;
constexpr size_t kRingBytes = (size_t)12 * TILE_BYTES;
static_assert(Geo<0>::STAGES * Geo<0>::STAGE_BYTES <= (int)kRingBytes, "ring");
static_assert(Geo<1>::STAGES * Geo<1>::STAGE_BYTES <= (int)kRingBytes, "ring");
constexpr int NTHREADS = 192;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t COL_STASH = 384;           // parked D1
constexpr uint32_t SW128 = 2;                 // descriptor layout type: 128B swizzle

constexpr int RING = 4;                       // unit numbers in flight (one-CTA form)

struct Ctl {
  uint64_t full[MAX_STAGES];
  uint64_t empty[MAX_STAGES];
  uint64_t ufull[RING];   // unit ring: producer -> MMA thread and epilogue
  uint64_t uempty[RING];
  long long uring[RING];
  int wu[2][4];           // per-warp outcome of the epilogue's unit wait
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

constexpr size_t kSmemBytes = kRingBytes + sizeof(Ctl) + 1024;

struct Unit {
  int i, j, A, B;  // occupied pair (clamped into range) and tile pair
  int nph;         // MMA phases: 1 (D2 from D1) or 2
  bool valid;      // contributes to the energy
};

// Work item k.  Queue form: unit k in cost order -- first the units with two
// MMA phases (i < j and A < B), then those with one (i == j, or A == B), so
// the last units handed out are the cheap ones.  Cluster form: super-unit
// k = (block pair, tile pair), this CTA's (r, c) member.
template <bool CL>
__device__ __forceinline__ Unit unit_at(long long k, const EnergyShape& sh, int r, int c) {
  Unit u;
  if (!CL) {
    u.nph = unit_decode_cost(k, sh.nocc, sh.ntiles, sh.ntpairs, &u.i, &u.j, &u.A, &u.B);
    u.valid = true;
  } else {
    const int tp = (int)(k % sh.ntpairs);
    tpair_decode(tp, sh.ntiles, &u.A, &u.B);
    int a, b;
    pair_decode((int)(k / sh.ntpairs), (sh.nocc + 1) / 2, &a, &b);
    const int i = 2 * a + r, j = 2 * b + c;
    u.valid = i < sh.nocc && j < sh.nocc && i <= j;
    u.i = i < sh.nocc ? i : sh.nocc - 1;
    u.j = j < sh.nocc ? j : sh.nocc - 1;
    u.nph = u.A == u.B ? 1 : 2;
  }
  return u;
}

template <bool CL>
__device__ __forceinline__ long long work_count(const EnergyShape& sh) {
  if (!CL) return sh.nunits;
  const long long nb = (sh.nocc + 1) / 2;
  return nb * (nb + 1) / 2 * sh.ntpairs;
}

template <int SCHEME, bool CL>
__global__ void __launch_bounds__(NTHREADS, 1)
    energy_tc_kernel(const uint16_t* __restrict__ S, const double* __restrict__ eps,
                     const float* __restrict__ sc, const float* __restrict__ dg,
                     const double* __restrict__ scale, EnergyShape sh, int nkb, uint32_t idesc,
                     double* __restrict__ partials, int* status,
                     unsigned long long* __restrict__ queue) {
  using G = Geo<SCHEME>;
  constexpr int STAGES = G::STAGES, STAGE_BYTES = G::STAGE_BYTES, NPL = G::NPL;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  Ctl* ctl = reinterpret_cast<Ctl*>(tiles + kRingBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int o = sh.nocc, v = sh.nvir;
  // cluster coordinates and multicast groups (rank q = 2r + c)
  const int q4 = CL ? (int)cluster_ctarank() : 0;
  const int cr = q4 >> 1, cc = q4 & 1;
  const uint16_t grow = (uint16_t)(3u << (2 * cr));  // CTAs of cluster row cr
  const uint16_t gcol = (uint16_t)(5u << cc);        // CTAs of cluster column cc
  const long long first = CL ? (long long)cluster_id_x() : (long long)blockIdx.x;
  const long long stride = CL ? (long long)cluster_count_x() : (long long)gridDim.x;
  const long long nwork = work_count<CL>(sh);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&ctl->full[s], 1);
      mbar_init(&ctl->empty[s], CL ? 3 : 1);
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
  if (CL) cluster_sync();  // partners' barriers exist before any multicast
  tc_fence_after();
  const uint32_t tmem = ctl->tmem;
  volatile int* abort = &ctl->abort;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    // The whole warp runs the loop: lane 0 waits for a free stage and arms
    // its barrier, then lanes 0-5 issue the stage's six copies in one
    // instruction (one copy per lane issues several times faster than six
    // copies in sequence from one thread).
    {
      int st = 0;
      uint32_t ph = 0;
      uint32_t last_ph[STAGES];
      bool has[STAGES];
      for (int s = 0; s < STAGES; ++s) has[s] = false;
      bool ok = true;
      // Shared-memory slots of a stage: [row operand planes][column operand
      // planes] per Q block.  Lane 2 NPL kbo + 2 l + colop copies plane l of
      // its operand (one-CTA form: the whole 16 KB tile; cluster form: its
      // 64-row half).
      const int kbo = lane / (2 * NPL);
      const int l = (lane % (2 * NPL)) >> 1;
      const bool colop = (lane & 1) != 0;
      const int ncopy = G::NTILES;
      for (long long t = 0; ok; ++t) {
        // next unit: the static sequence (cluster form) or the device queue
        long long k = first + t * stride;
        if (!CL) {
          const int slot = (int)(t % RING);
          const uint32_t use = (uint32_t)(t / RING);
          long long u = -2;  // -2: wait failed, -1: queue drained
          if (lane == 0 && mbar_wait(&ctl->uempty[slot], (use & 1) ^ 1, abort, status)) {
            u = (long long)atomicAdd(queue, 1ull);
            if (u >= nwork) u = -1;
            ctl->uring[slot] = u;
            mbar_arrive(&ctl->ufull[slot]);
          }
          k = __shfl_sync(0xffffffffu, u, 0);
          if (k == -2) ok = false;
          if (k < 0) break;
        } else if (k >= nwork) {
          break;
        }
        const Unit w = unit_at<CL>(k, sh, cr, cc);
        for (int phs = 0; phs < w.nph && ok; ++phs) {
          const int x = phs == 0 ? w.i : w.j;  // row operand slab
          const int y = phs == 0 ? w.j : w.i;  // column operand slab
          // cluster: the row tile is shared along the cluster row in phase 1
          // and along the cluster column in phase 2 (and the column tile the
          // other way); this CTA copies its half of each
          const uint16_t mrow = phs == 0 ? grow : gcol, mcol = phs == 0 ? gcol : grow;
          const int hrow = phs == 0 ? cc : cr, hcol = phs == 0 ? cr : cc;
          const int slab = colop ? y : x, tile = colop ? w.B : w.A;
          const uint16_t mask = colop ? mcol : mrow;
          const int half = colop ? hcol : hrow;
          for (int ks = 0; ks < nkb; ks += KBS) {
            const int kb = ks + kbo;
            bool got = true;
            if (lane == 0) got = mbar_wait(&ctl->empty[st], ph ^ 1, abort, status);
            if (!__shfl_sync(0xffffffffu, got ? 1 : 0, 0)) {
              ok = false;
              break;
            }
            uint64_t* bar = &ctl->full[st];
            if (lane == 0) mbar_expect_tx(bar, STAGE_BYTES);
            __syncwarp();
            uint8_t* sb =
                tiles + (size_t)st * STAGE_BYTES +
                (2 * NPL * kbo + NPL * (colop ? 1 : 0) + l) * TILE_BYTES;
            if (lane < ncopy) {
              const uint16_t* src = S + slice_tile_offset(l, slab, kb, tile, nkb, sh.ntiles, NPL);
              if (CL)
                bulk_load_mc(sb + half * HALF_BYTES, src + half * (HALF_BYTES / 2), HALF_BYTES,
                             bar, mask);
              else
                bulk_load(sb, src, TILE_BYTES, bar);
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
      // Never leave with a bulk copy still landing in shared memory; in the
      // cluster form also wait for the partners' releases of the last fills
      // (their remote arrivals target this CTA's barriers).
      if (lane == 0) {
        int never = 0;
        for (int s = 0; s < STAGES; ++s)
          if (has[s]) mbar_wait(&ctl->full[s], last_ph[s], &never, status);
        if (CL)
          for (int s = 0; s < STAGES; ++s)
            if (has[s]) mbar_wait(&ctl->empty[s], last_ph[s], &never, status);
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
      const uint16_t release = (uint16_t)(grow | gcol);  // this CTA and its two partners
      // shared-memory descriptor of tile 0 of stage 0 (every tile address is
      // below 2^18, so offsets added to the 14-bit start field never carry out)
      const uint64_t dbase = smem_desc(smem_u32(tiles), 16, 1024, SW128);
      for (long long t = 0; ok; ++t) {
        long long k = first + t * stride;
        if (!CL) {
          const int slot = (int)(t % RING);
          const uint32_t use = (uint32_t)(t / RING);
          if (!mbar_wait(&ctl->ufull[slot], use & 1, abort, status)) break;
          k = ctl->uring[slot];
          mbar_arrive(&ctl->uempty[slot]);
          if (k < 0) break;
        } else if (k >= nwork) {
          break;
        }
        const Unit w = unit_at<CL>(k, sh, cr, cc);
        for (int phs = 0; phs < w.nph && ok; ++phs) {
          if (!mbar_wait(&ctl->aempty, (nuse & 1) ^ 1, abort, status)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t c0 = tmem, c1 = tmem + 128u, c2 = tmem + 256u;
          bool ready = false;  // the next stage's barrier, probed ahead of time
          for (int ks = 0; ks < nkb; ks += KBS) {
            if (!ready && !mbar_wait(&ctl->full[st], ph, abort, status)) {
              ok = false;
              break;
            }
            // (no tcgen05 fence: the bulk copies' mbarrier completion orders
            // the shared-memory operands)
            // descriptor of this stage: the base descriptor plus the stage's
            // address offset in the 16-byte units of the start-address field
            const uint64_t ds = dbase + (uint64_t)(((uint32_t)st * STAGE_BYTES) >> 4);
            const int nst = st + 1 == STAGES ? 0 : st + 1;
            const uint32_t nph = st + 1 == STAGES ? ph ^ 1 : ph;
            ready = false;
#pragma unroll
            for (int j = 0; j < KBS * (KB / 16); ++j) {
              const int kbo = j / (KB / 16), kk = j % (KB / 16);
              uint64_t r[NPL], q[NPL];
#pragma unroll
              for (int l = 0; l < NPL; ++l) {
                r[l] = ds + (uint64_t)(((2 * NPL * kbo + l) * TILE_BYTES + kk * 32) >> 4);
                q[l] = ds + (uint64_t)(((2 * NPL * kbo + NPL + l) * TILE_BYTES + kk * 32) >> 4);
              }
              // while the MMAs queued so far run, probe the next stage
              // (non-blocking), so the stage boundary costs no barrier latency
              if (j == KBS * (KB / 16) - 1 && ks + KBS < nkb)
                ready = mbar_test_wait(&ctl->full[nst], nph);
              const uint32_t acc = (ks | j) ? 1u : 0u;
              issue_digit_mmas<SCHEME>(c0, c1, c2, r, q, idesc, acc);
            }
            // stage reusable once these MMAs finish (in every CTA that wrote it)
            if (CL)
              tc_commit_mc(&ctl->empty[st], release);
            else
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
    for (long long t = 0;; ++t) {
      long long k = first + t * stride;
      if (!CL) {
        // unit number: every epilogue thread waits and reads, then one
        // thread releases the slot (after the barrier that ends the reads)
        if (dead) break;
        const int slot = (int)(t % RING);
        const uint32_t use = (uint32_t)(t / RING);
        const bool gotu =
            __all_sync(0xffffffffu, mbar_wait(&ctl->ufull[slot], use & 1, abort, status));
        if (lane == 0) ctl->wu[t & 1][q] = gotu ? 1 : 0;
        k = gotu ? ctl->uring[slot] : -1;
        named_bar(1, 128);
        const bool all = ctl->wu[t & 1][0] & ctl->wu[t & 1][1] & ctl->wu[t & 1][2] &
                         ctl->wu[t & 1][3];
        named_bar(1, 128);
        if (et == 0 && all) mbar_arrive(&ctl->uempty[slot]);
        if (!all) dead = true;
        if (!all || k < 0) break;  // uniform: every thread read the same slot
      } else if (k >= nwork) {
        break;
      }
      const Unit w = unit_at<CL>(k, sh, cr, cc);
      const int i = w.i, j = w.j, A = w.A, B = w.B;
      const bool two = w.nph == 2;
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
        // Phase-1 result (scaled D1, FP32) to the stash columns, then the
        // accumulators go back to the MMA issuer at once: the rest of this
        // unit's epilogue overlaps the next phase's MMAs.
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
        if (!two && same) {
          // D2 == D1: fold straight into the energy
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
        } else if (!two) {
          // Diagonal tile pair (A == B): D2 = D1^T.  Four rounds; in round k warp q
          // publishes its D1 block of column chunk (q+k)%4 and takes the block
          // of warp (q-k)%4, which is the D1^T block of column chunk (q-k)%4.
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
            named_bar(1, 128);  // tbuf is rewritten in the next round
          }
        }
      }
      ++nuse;

      // ---- phase 2: D2 (two-phase units): rows from slab j, columns from slab i
      if (two) {
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
          // D2 (scaled, FP32) into registers, then release the accumulators
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
      const double fw = w.valid ? (A < B ? 2.0 : 1.0) * (same ? 0.5 : 1.0) : 0.0;
      if (CL) {
        tot_os -= fw * uos;
        tot_ss -= fw * uss;
      } else {
        // queue form: which CTA takes a unit varies from run to run, so each
        // unit writes its own partial (reduced over the 128 epilogue threads
        // in a fixed order) and the host-side reduction sums them in unit order
        const double pos = warp_sum(-fw * uos), pss = warp_sum(-fw * uss);
        if (lane == 0) {
          ctl->red[0][q] = pos;
          ctl->red[1][q] = pss;
        }
        named_bar(1, 128);
        if (et == 0) {
          partials[2 * k] = (ctl->red[0][0] + ctl->red[0][1]) + (ctl->red[0][2] + ctl->red[0][3]);
          partials[2 * k + 1] =
              (ctl->red[1][0] + ctl->red[1][1]) + (ctl->red[1][2] + ctl->red[1][3]);
        }
      }
      named_bar(1, 128);  // smem db/scb/red are rewritten by the next unit
    }
    if (CL) {  // static assignment: one partial per CTA
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
  }

  __syncwarp();
  tc_fence_before();
  __syncthreads();
  // no CTA of a cluster leaves while a partner may still address its shared memory
  if (CL) cluster_sync();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, TMEM_COLS);
}

}  // namespace

template <int SCHEME, bool CL>
static cudaError_t set_smem_attr() {
  return cudaFuncSetAttribute(energy_tc_kernel<SCHEME, CL>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
}

template <int SCHEME, bool CL>
static cudaError_t launch_variant(int grid, cudaStream_t s, const uint16_t* S, const double* eps,
                                  const float* sc, const float* dg, const double* scale,
                                  const EnergyShape& sh, int nkb, uint32_t idesc,
                                  double* partials, int* status, unsigned long long* queue) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(NTHREADS);
  cfg.dynamicSmemBytes = kSmemBytes;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL ? kTcCluster : 1;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = CL ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, energy_tc_kernel<SCHEME, CL>, S, eps, sc, dg, scale, sh, nkb,
                            idesc, partials, status, queue);
}

cudaError_t prepare_energy_tc(int* max_clusters) {
  cudaError_t e = set_smem_attr<kSchemeDigits3, false>();
  if (e == cudaSuccess) e = set_smem_attr<kSchemeDigits2, false>();
  if (e == cudaSuccess) e = set_smem_attr<kSchemeDigits3, true>();
  if (e == cudaSuccess) e = set_smem_attr<kSchemeDigits2, true>();
  if (e != cudaSuccess) return e;
  // how many 4-CTA clusters of this kernel fit on the device at once
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kTcCluster);
  cfg.blockDim = dim3(NTHREADS);
  cfg.dynamicSmemBytes = kSmemBytes;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kTcCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  e = cudaOccupancyMaxActiveClusters(&n, energy_tc_kernel<kSchemeDigits2, true>, &cfg);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    n = 0;  // no cluster form on this device
  }
  *max_clusters = n;
  return cudaSuccess;
}

long long energy_tc_cluster_work(const EnergyShape& sh) {
  const long long nb = (sh.nocc + 1) / 2;
  return nb * (nb + 1) / 2 * sh.ntpairs;
}

cudaError_t launch_energy_tc(const uint16_t* S, const double* eps, const float* sc,
                             const float* dg, const double* scale, const EnergyShape& sh, int Qp,
                             int fmt, int scheme, bool cluster, double* partials, int grid,
                             int* status, unsigned long long* queue, cudaStream_t s) {
  const uint32_t idesc = idesc_f16((uint32_t)fmt, TILE, TILE);
  const int nkb = Qp / KB;
  if (!cluster) {
    // the queue counter and, after it, the ticket of the final reduction
    cudaError_t e = cudaMemsetAsync(queue, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
  }
  if (scheme == kSchemeDigits2)
    return cluster ? launch_variant<kSchemeDigits2, true>(grid, s, S, eps, sc, dg, scale, sh, nkb,
                                                          idesc, partials, status, queue)
                   : launch_variant<kSchemeDigits2, false>(grid, s, S, eps, sc, dg, scale, sh,
                                                           nkb, idesc, partials, status, queue);
  return cluster ? launch_variant<kSchemeDigits3, true>(grid, s, S, eps, sc, dg, scale, sh, nkb,
                                                        idesc, partials, status, queue)
                 : launch_variant<kSchemeDigits3, false>(grid, s, S, eps, sc, dg, scale, sh, nkb,
                                                         idesc, partials, status, queue);
}

}  // namespace corr
