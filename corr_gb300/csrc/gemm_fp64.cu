// Batched FP64 GEMM on the FP64 tensor path (mma.sync m8n8k4 f64), TMA-fed.
//
//   C[b] = alpha * op(A[b]) * op(B[b]) + beta * C[b]      (row-major, FP64)
//
// op(A) is M x K: ta == 0 -> A stored M x K (K contiguous, lda >= K);
//                 ta == 1 -> A stored K x M (M contiguous, lda >= M).
// op(B) is K x N: tb == 0 -> B stored K x N (N contiguous, ldb >= N);
//                 tb == 1 -> B stored N x K (K contiguous, ldb >= K).
// Batch strides may be 0 (operand shared by every batch entry).
//
// Tiles of 64 x 64 x 16 per CTA (4 warps, 32 x 32 each), two shared-memory
// stages.  An operand whose base address and leading dimension are 16-byte
// aligned is fetched by TMA (3-D map: contiguous dim, other dim, batch) into
// a dense tile; otherwise the CTA loads it with bounds-checked plain loads
// into the same layout.  Out-of-range rows/columns are zero-filled, so any
// M, N, K works.  This kernel is the building block of every FP64 contraction
// of the hot path: build_FMo, the four MOtrans quarter transforms, transform_ri,
// the RI B build and the J^-1/2 assembly.
#include "common.cuh"
#include "gemm_fp64.h"

namespace corr {

namespace {

constexpr int BM = 64, BN = 64, BK = 16;
constexpr int NT = 128;

struct Tiles {
  double a[2][BM * BK];
  double b[2][BK * BN];
  uint64_t bar[2];
};

__device__ __forceinline__ void dmma(double (&d)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(d[0]), "+d"(d[1])
               : "d"(a), "d"(b));
}

// Plain bounds-checked fill of one operand tile in the TMA layout
// ([outer][inner], inner = the operand's contiguous dimension).
__device__ __forceinline__ void fill_tile(double* dst, const double* base, long long ld,
                                          int inner0, int inner_n, int inner_box, int outer0,
                                          int outer_n, int outer_box) {
  for (int idx = threadIdx.x; idx < inner_box * outer_box; idx += NT) {
    int oi = idx / inner_box, ii = idx % inner_box;
    int go = outer0 + oi, gi = inner0 + ii;
    dst[idx] = (go < outer_n && gi < inner_n) ? base[(long long)go * ld + gi] : 0.0;
  }
}

template <int TA, int TB>
__global__ void __launch_bounds__(NT) gemm_f64_kernel(const __grid_constant__ CUtensorMap tmA,
                                                      const __grid_constant__ CUtensorMap tmB,
                                                      GemmF64 g, int tmaA, int tmaB,
                                                      int* status) {
  __shared__ __align__(128) Tiles sm;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int gq = lane >> 2, tq = lane & 3;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN, bz = blockIdx.z;
  const double* Ab = g.A + (long long)bz * g.sa;
  const double* Bb = g.B + (long long)bz * g.sb;
  double* Cb = g.C + (long long)bz * g.sc;
  const int nk = (g.K + BK - 1) / BK;
  __shared__ int abort_flag;

  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](int kb, int s) {
    const int k0 = kb * BK;
    if (tid == 0 && (tmaA || tmaB)) {
      uint32_t bytes = (tmaA ? BM * BK * 8 : 0) + (tmaB ? BK * BN * 8 : 0);
      mbar_expect_tx(&sm.bar[s], bytes);
      if (tmaA) {
        if (TA == 0) tma_load_3d(sm.a[s], &tmA, &sm.bar[s], k0, m0, g.sa ? bz : 0);
        else tma_load_3d(sm.a[s], &tmA, &sm.bar[s], m0, k0, g.sa ? bz : 0);
      }
      if (tmaB) {
        if (TB == 0) tma_load_3d(sm.b[s], &tmB, &sm.bar[s], n0, k0, g.sb ? bz : 0);
        else tma_load_3d(sm.b[s], &tmB, &sm.bar[s], k0, n0, g.sb ? bz : 0);
      }
    }
    if (!tmaA) {
      if (TA == 0) fill_tile(sm.a[s], Ab, g.lda, k0, g.K, BK, m0, g.M, BM);
      else fill_tile(sm.a[s], Ab, g.lda, m0, g.M, BM, k0, g.K, BK);
    }
    if (!tmaB) {
      if (TB == 0) fill_tile(sm.b[s], Bb, g.ldb, n0, g.N, BN, k0, g.K, BK);
      else fill_tile(sm.b[s], Bb, g.ldb, k0, g.K, BK, n0, g.N, BN);
    }
  };

  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

  uint32_t ph[2] = {0, 0};
  bool pending[2] = {false, false};
  issue(0, 0);
  pending[0] = true;
  bool aborted = false;
  for (int kb = 0; kb < nk; ++kb) {
    const int s = kb & 1;
    if (kb + 1 < nk) {
      issue(kb + 1, s ^ 1);
      pending[s ^ 1] = true;
    }
    bool ok = true;
    if (tmaA || tmaB) {
      ok = mbar_wait(&sm.bar[s], ph[s], &abort_flag, status);
      if (ok) {
        ph[s] ^= 1;
        pending[s] = false;
      }
    } else {
      pending[s] = false;
    }
    // block-uniform: a timed-out wait in any thread stops every thread
    if (__syncthreads_or(!ok)) {
      aborted = true;
      break;
    }
    const double* As = sm.a[s];
    const double* Bs = sm.b[s];
#pragma unroll
    for (int k4 = 0; k4 < BK; k4 += 4) {
      const int k = k4 + tq;
      double af[4], bf[4];
#pragma unroll
      for (int mi = 0; mi < 4; ++mi) {
        const int m = wm * 32 + mi * 8 + gq;
        af[mi] = TA == 0 ? As[m * BK + k] : As[k * BM + m];
      }
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        const int n = wn * 32 + ni * 8 + gq;
        bf[ni] = TB == 0 ? Bs[k * BN + n] : Bs[n * BK + k];
      }
#pragma unroll
      for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) dmma(acc[mi][ni], af[mi], bf[ni]);
    }
    __syncthreads();  // stage s is refilled by the next iteration's issue
  }
  if (aborted && tid == 0 && (tmaA || tmaB)) {
    // let every issued bulk copy land before the CTA's shared memory is released
    int never = 0;
    for (int s = 0; s < 2; ++s)
      if (pending[s]) mbar_wait(&sm.bar[s], ph[s], &never, status);
  }

#pragma unroll
  for (int mi = 0; mi < 4; ++mi) {
    const int m = m0 + wm * 32 + mi * 8 + gq;
    if (m >= g.M) continue;
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int n = n0 + wn * 32 + ni * 8 + 2 * tq + e;
        if (n >= g.N) continue;
        double* c = Cb + (long long)m * g.ldc + n;
        const double v = g.alpha * acc[mi][ni][e];
        *c = g.beta == 0.0 ? v : v + g.beta * (*c);
      }
  }
}

bool aligned16(const void* p, long long ld) {
  return ((uintptr_t)p % 16 == 0) && ((ld * 8) % 16 == 0);
}

}  // namespace

int gemm_f64(const GemmF64& g, int* status, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return CORR_OK;
  CUtensorMap ta{}, tb{};
  // TMA needs 16-byte aligned base/leading dimension and batch strides
  bool tmaA = aligned16(g.A, g.lda) && (g.sa * 8) % 16 == 0 && g.K > 0;
  bool tmaB = aligned16(g.B, g.ldb) && (g.sb * 8) % 16 == 0 && g.K > 0;
  if (tmaA) {
    uint64_t inner = g.ta == 0 ? g.K : g.M, outer = g.ta == 0 ? g.M : g.K;
    uint64_t dims[3] = {inner, outer, (uint64_t)(g.sa ? g.batch : 1)};
    uint64_t strides[2] = {(uint64_t)g.lda * 8, (uint64_t)(g.sa ? g.sa : g.lda * outer) * 8};
    uint32_t box[3] = {(uint32_t)(g.ta == 0 ? BK : BM), (uint32_t)(g.ta == 0 ? BM : BK), 1};
    if (encode_tmap(&ta, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, (void*)g.A, dims, strides, box,
                    CU_TENSOR_MAP_SWIZZLE_NONE) != CORR_OK)
      tmaA = false;
  }
  if (tmaB) {
    uint64_t inner = g.tb == 0 ? g.N : g.K, outer = g.tb == 0 ? g.K : g.N;
    uint64_t dims[3] = {inner, outer, (uint64_t)(g.sb ? g.batch : 1)};
    uint64_t strides[2] = {(uint64_t)g.ldb * 8, (uint64_t)(g.sb ? g.sb : g.ldb * outer) * 8};
    uint32_t box[3] = {(uint32_t)(g.tb == 0 ? BN : BK), (uint32_t)(g.tb == 0 ? BK : BN), 1};
    if (encode_tmap(&tb, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, (void*)g.B, dims, strides, box,
                    CU_TENSOR_MAP_SWIZZLE_NONE) != CORR_OK)
      tmaB = false;
  }
  dim3 grid((g.M + BM - 1) / BM, (g.N + BN - 1) / BN, g.batch);
  if (grid.y > 65535 || grid.z > 65535) {
    set_error("gemm_f64: grid too large (N=%d, batch=%d)", g.N, g.batch);
    return CORR_ERR_BAD_ARG;
  }
  const int a = tmaA ? 1 : 0, b = tmaB ? 1 : 0;
  if (g.ta == 0 && g.tb == 0) gemm_f64_kernel<0, 0><<<grid, NT, 0, s>>>(ta, tb, g, a, b, status);
  else if (g.ta == 0) gemm_f64_kernel<0, 1><<<grid, NT, 0, s>>>(ta, tb, g, a, b, status);
  else if (g.tb == 0) gemm_f64_kernel<1, 0><<<grid, NT, 0, s>>>(ta, tb, g, a, b, status);
  else gemm_f64_kernel<1, 1><<<grid, NT, 0, s>>>(ta, tb, g, a, b, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("gemm_f64 launch: %s", cudaGetErrorString(e));
    return CORR_ERR_CUDA;
  }
  return CORR_OK;
}

}  // namespace corr
