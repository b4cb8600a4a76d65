// tcgen05 epilogue helpers shared by the precision-form energy kernels
// (energy_tc.cu: one instance; energy_batch.cu: batched instances).
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

__device__ __forceinline__ void tc_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// 32 columns [c, c+32) of one phase's result in scaled FP32 units.
__device__ __forceinline__ void load_level_sum(uint32_t tb, int c, float inv_l, float inv_l2,
                                               float sca, const float* scb, float* d) {
  float a0[32], a1[32], a2[32];
  tmem_ld32(tb + 0u + (uint32_t)c, a0);
  tmem_ld32(tb + 128u + (uint32_t)c, a1);
  tmem_ld32(tb + 256u + (uint32_t)c, a2);
  tc_wait_ld();
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    // acc_0 is an exact integer; the sum is rounded once to nearest
    const float t = fmaf(a2[k], inv_l2, fmaf(a1[k], inv_l, a0[k]));
    d[k] = t * (sca * scb[c + k]);
  }
}


}  // namespace corr
