// tcgen05 epilogue helpers of the precision-form energy kernel (energy_tc.cu)
// and of its adjoint (adjoint_tc.cu).
#pragma once

#include "common.cuh"

namespace corr {

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
      "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
      "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
      "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
      "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])),
      "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])), "r"(__float_as_uint(v[20])),
      "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
      "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])),
      "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])),
      "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// After tcgen05.wait::ld: an empty asm that "modifies" each destination
// register, ordered after the wait (both are volatile), so no arithmetic on
// the loaded values can be scheduled before the load has completed.
template <int N>
__device__ __forceinline__ void ld_ready(float* v) {
#pragma unroll
  for (int k = 0; k < N; ++k) asm volatile("" : "+f"(v[k]));
}

__device__ __forceinline__ void tc_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Unit k of an energy problem with o occupied orbitals and nt virtual tiles
// (ntp = nt (nt + 1) / 2 tile pairs) in cost order: first the units with two
// MMA phases (i < j and A < B), then those with one (i == j, or A == B), so a
// work queue hands out the cheap units last.  Returns the number of phases.
__device__ __forceinline__ int unit_decode_cost(long long k, int o, int nt, int ntp, int* i,
                                                int* j, int* A, int* B) {
  const long long ps = (long long)o * (o - 1) / 2;    // pairs i < j
  const long long ts = (long long)nt * (nt - 1) / 2;  // tile pairs A < B
  int jj, bb;
  if (k < ps * ts) {
    pair_decode((int)(k / ts), o - 1, i, &jj);
    tpair_decode((int)(k % ts), nt - 1, A, &bb);
    *j = jj + 1;
    *B = bb + 1;
    return 2;
  }
  const long long v = k - ps * ts;
  if (v < (long long)o * ntp) {  // i == j, any tile pair
    *i = *j = (int)(v / ntp);
    tpair_decode((int)(v % ntp), nt, A, B);
  } else {  // i < j, A == B
    const long long w = v - (long long)o * ntp;
    pair_decode((int)(w / nt), o - 1, i, &jj);
    *j = jj + 1;
    *A = *B = (int)(w % nt);
  }
  return 1;
}

// 16 columns [c, c+16) of one phase's result in scaled FP32 units, from the
// three exact integer accumulators at columns tb, tb+128, tb+256 (levels 0, 1,
// 2 of either scheme): d = acc0 + acc1/L + acc2/L^2.  Every step rounds to
// nearest (CUDA cores), so no bias enters here.
template <int SCHEME>
__device__ __forceinline__ void load_level_sum16(uint32_t tb, int c, float inv_l, float inv_l2,
                                                 float sca, const float* scb, float* d) {
  float a0[16], a1[16], a2[16];
  tmem_ld16(tb + 0u + (uint32_t)c, a0);
  tmem_ld16(tb + 128u + (uint32_t)c, a1);
  tmem_ld16(tb + 256u + (uint32_t)c, a2);
  tc_wait_ld();
  ld_ready<16>(a0);
  ld_ready<16>(a1);
  ld_ready<16>(a2);
  // two columns per packed instruction (each lane as the scalar expression
  // fmaf(a2, inv_l2, fmaf(a1, inv_l, a0)) * (sca * scb))
#pragma unroll
  for (int k = 0; k < 16; k += 2) {
    const float2 t = __ffma2_rn(make_float2(a2[k], a2[k + 1]), make_float2(inv_l2, inv_l2),
                                __ffma2_rn(make_float2(a1[k], a1[k + 1]),
                                           make_float2(inv_l, inv_l),
                                           make_float2(a0[k], a0[k + 1])));
    const float2 sc = __fmul2_rn(make_float2(sca, sca), make_float2(scb[c + k], scb[c + k + 1]));
    const float2 r = __fmul2_rn(t, sc);
    d[k] = r.x;
    d[k + 1] = r.y;
  }
}

// ---- energy arithmetic with FP32 instructions only ----------------------
// GB300 runs FP64 at about 1/64 of its FP32 rate, so the per-element energy
// arithmetic uses float-float values (hi + lo, about 48 significand bits)
// built from error-free transformations: Knuth's TwoSum, the FMA residual of
// a product (x*x - RN(x*x) is exact as fmaf(x, x, -RN(x*x))), one
// Newton-Raphson step for the reciprocal, and a float-float running sum.

// s + e == a + b exactly (Knuth's TwoSum; no ordering of |a|, |b| needed).
__device__ __forceinline__ void two_sum(float a, float b, float* s, float* e) {
  const float t = a + b;
  const float bb = t - a;
  *e = (a - (t - bb)) + (b - bb);
  *s = t;
}

// An FP64 value as a float-float pair (hi = RN(d), lo = RN(d - hi)).
__device__ __forceinline__ float2 ff_split(double d) {
  const float hi = (float)d;
  return make_float2(hi, (float)(d - (double)hi));
}

// 1/(da + db) for float-float da, db as rh + rl: D = dh + dl by TwoSum of the
// high parts, r0 = rcp.approx(dh) (relative error below 2^-22), the residual
// e = 1 - D r0 by two FMAs, and 1/D = r0 / (1 - e) ~ r0 + r0 e (one
// Newton-Raphson step): relative error about e^2 + 2^-46, i.e. ~2^-44.
__device__ __forceinline__ void recip_ff(float2 da, float2 db, float* rh, float* rl) {
  float dh, dl;
  two_sum(da.x, db.x, &dh, &dl);
  dl += da.y + db.y;
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(dh));
  float e = fmaf(-dh, r0, 1.0f);
  e = fmaf(-dl, r0, e);
  *rh = r0;
  *rl = r0 * e;
}

// ---- two columns at once ---------------------------------------------------
// The per-element arithmetic runs on Blackwell's packed FP32 instructions
// (FADD2/FMUL2/FFMA2: two IEEE round-to-nearest operations per instruction,
// each lane exactly as the scalar operation), so the error-free
// transformations above hold per lane and the epilogue issues half the
// instructions.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2* s, float2* e) {
  const float2 t = __fadd2_rn(a, b);
  const float2 bb = __fadd2_rn(t, neg2(a));
  *e = __fadd2_rn(__fadd2_rn(a, neg2(__fadd2_rn(t, neg2(bb)))), __fadd2_rn(b, neg2(bb)));
  *s = t;
}

// 1/(da + db) for one row value da and two column values (bh + bl per lane).
__device__ __forceinline__ void recip_ff2(float2 da, float2 bh, float2 bl, float2* rh,
                                          float2* rl) {
  float2 dh, dl;
  two_sum2(dup2(da.x), bh, &dh, &dl);
  dl = __fadd2_rn(dl, __fadd2_rn(dup2(da.y), bl));
  float2 r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0.x) : "f"(dh.x));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0.y) : "f"(dh.y));
  float2 e = __ffma2_rn(neg2(dh), r0, dup2(1.0f));
  e = __ffma2_rn(neg2(dl), r0, e);
  *rh = r0;
  *rl = __fmul2_rn(r0, e);
}

// Running sum of float-float terms, two independent lanes: per lane h + l,
// with h updated by TwoSum (exact) and l collecting the TwoSum errors and the
// terms' low parts in FP32.  flush() adds both lanes to the FP64 total d and
// restarts: over m terms per lane the FP32 roundings of l stay below
// m^2 2^-48 of the sum, so callers flush every 32 columns (16 terms per lane)
// -- a compensated sum in the sense of Kahan's, carried to float-float
// accuracy (plain Kahan summation in FP32 only reaches ~2^-23).
struct FFSum2 {
  float2 h = make_float2(0.0f, 0.0f), l = make_float2(0.0f, 0.0f);
  double d = 0.0;
  __device__ __forceinline__ void add(float2 hi, float2 lo) {
    float2 t, e;
    two_sum2(h, hi, &t, &e);
    h = t;
    l = __fadd2_rn(l, __fadd2_rn(e, lo));
  }
  __device__ __forceinline__ void flush() {
    d += ((double)h.x + (double)h.y) + ((double)l.x + (double)l.y);
    h = make_float2(0.0f, 0.0f);
    l = make_float2(0.0f, 0.0f);
  }
};

// Terms of two elements (a, b) of a pair i != j with x = (ia|jb), y = (ib|ja)
// (scaled FP32 values) and 1/D = rh + rl, per lane:
//   E_OS += (x^2 + y^2)/D,  E_SS += (x - y)^2/D,
// the squares and the difference error-free (FMA residuals, TwoSum), the
// products with 1/D to float-float accuracy.
__device__ __forceinline__ void pair_terms2(float2 x, float2 y, float2 rh, float2 rl, FFSum2& os,
                                            FFSum2& ss) {
  const float2 px = __fmul2_rn(x, x), ex = __ffma2_rn(x, x, neg2(px));
  const float2 py = __fmul2_rn(y, y), ey = __ffma2_rn(y, y, neg2(py));
  float2 nh, nl;
  two_sum2(px, py, &nh, &nl);
  nl = __fadd2_rn(nl, __fadd2_rn(ex, ey));
  float2 dh, dl;
  two_sum2(x, neg2(y), &dh, &dl);
  const float2 mh = __fmul2_rn(dh, dh);
  const float2 ml = __ffma2_rn(__fmul2_rn(dup2(2.0f), dh), dl, __ffma2_rn(dh, dh, neg2(mh)));
  const float2 th = __fmul2_rn(nh, rh);
  os.add(th, __fadd2_rn(__ffma2_rn(nh, rh, neg2(th)), __ffma2_rn(nh, rl, __fmul2_rn(nl, rh))));
  const float2 uh = __fmul2_rn(mh, rh);
  ss.add(uh, __fadd2_rn(__ffma2_rn(mh, rh, neg2(uh)), __ffma2_rn(mh, rl, __fmul2_rn(ml, rh))));
}

// The terms of two elements of a pair i == j (D2 == D1 == x), per lane:
// E_OS += 2 x^2/D.
__device__ __forceinline__ void same_pair_term2(float2 x, float2 rh, float2 rl, FFSum2& os) {
  const float2 px = __fmul2_rn(x, x), ex = __ffma2_rn(x, x, neg2(px));
  const float2 th = __fmul2_rn(px, rh);
  const float2 tl = __fadd2_rn(__ffma2_rn(px, rh, neg2(th)), __ffma2_rn(px, rl, __fmul2_rn(ex, rh)));
  os.add(__fmul2_rn(dup2(2.0f), th), __fmul2_rn(dup2(2.0f), tl));
}

// The MMAs of one K=16 step: r[l], q[l] are the row/column descriptors of
// digit plane l; c0..c2 the three accumulators.  MMAs sharing a row operand
// run back to back and keep it in the tensor core's A collector buffer (one
// shared-memory read of each row plane per K step), and no two consecutive
// MMAs (within or across K steps) write the same accumulator.  The first MMA
// into each accumulator carries `acc` (0: overwrite at the start of a phase).
template <int SCHEME>
__device__ __forceinline__ void issue_digit_mmas(uint32_t c0, uint32_t c1, uint32_t c2,
                                                 const uint64_t* r, const uint64_t* q,
                                                 uint32_t idesc, uint32_t acc) {
  if (SCHEME == 1) {
    tc_mma_f16_ca<0>(c0, r[0], q[0], idesc, acc);  // s0.s0'
    tc_mma_f16_ca<2>(c1, r[0], q[1], idesc, acc);  // s0.s1'
    tc_mma_f16_ca<0>(c2, r[1], q[1], idesc, acc);  // s1.s1'
    tc_mma_f16_ca<2>(c1, r[1], q[0], idesc, 1u);   // + s1.s0'
  } else {
    tc_mma_f16_ca<0>(c1, r[0], q[1], idesc, acc);
    tc_mma_f16_ca<1>(c2, r[0], q[2], idesc, acc);
    tc_mma_f16_ca<2>(c0, r[0], q[0], idesc, acc);
    tc_mma_f16_ca<0>(c2, r[1], q[1], idesc, 1u);
    tc_mma_f16_ca<2>(c1, r[1], q[0], idesc, 1u);
    tc_mma_f16(c2, r[2], q[0], idesc, 1u);
  }
}

}  // namespace corr
