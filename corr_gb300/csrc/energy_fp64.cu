// Plain FP64 fused RI-MP2 energy on the FP64 tensor path (mma.sync m8n8k4 f64).
//
// Work unit = (occupied pair i<=j, virtual tile pair A<=B).  A unit forms two
// 64x64 tiles of the exchange-paired integrals
//   D1[a][b] = (ia|jb) = sum_Q B^Q_ia B^Q_jb          (a in A, b in B)
//   D2[a][b] = (ib|ja) = sum_Q B^Q_ja B^Q_ib
// in registers and folds them straight into the energy:
//   E_OS -= f w (D1^2 + D2^2) / D,   E_SS -= f w (D1 - D2)^2 / D,
// D = e_a + e_b - e_i - e_j, f = 2 if A<B else 1, w = 1 if i<j else 1/2.
// Summed over units this is exactly the reference's double sum over ordered
// (i,j) and all (a,b) (can_mp2.cc:82-97): the (j,i) term equals the (i,j) term
// with a and b swapped, and the (b,a) element of a pair pairs with (a,b).
// No (ia|jb) value ever reaches global memory.
#include "common.cuh"
#include "kernels.h"

namespace corr {

namespace {

constexpr int T = kF64Tile;  // 64
constexpr int KB = 16;       // Q rows per step
constexpr int LD = T + 4;    // padded smem row (doubles): conflict-free fragment loads

__device__ __forceinline__ void dmma(double (&d)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(d[0]), "+d"(d[1])
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(128) energy_fp64_kernel(const double* __restrict__ bia,
                                                          const double* __restrict__ eps,
                                                          EnergyShape sh,
                                                          double* __restrict__ partials) {
  __shared__ double s_iA[KB][LD], s_jB[KB][LD], s_jA[KB][LD], s_iB[KB][LD];
  __shared__ double red[2][4];
  const int o = sh.nocc, v = sh.nvir, X = sh.naux;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int g = lane >> 2, t = lane & 3;
  const long long rowQ = (long long)o * v;  // stride between Q rows

  double tot_os = 0.0, tot_ss = 0.0;

  for (long long u = blockIdx.x; u < sh.nunits; u += gridDim.x) {
    int p = (int)(u / sh.ntpairs), tp = (int)(u % sh.ntpairs);
    int i, j, A, B;
    pair_decode(p, o, &i, &j);
    tpair_decode(tp, sh.ntiles, &A, &B);
    const int A0 = A * T, B0 = B * T;

    double acc1[4][4][2], acc2[4][4][2];
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        acc1[mi][ni][0] = acc1[mi][ni][1] = 0.0;
        acc2[mi][ni][0] = acc2[mi][ni][1] = 0.0;
      }

    for (int q0 = 0; q0 < X; q0 += KB) {
#pragma unroll
      for (int e = 0; e < (KB * T) / 128; ++e) {
        int idx = tid + 128 * e;
        int r = idx / T, c = idx % T;
        int q = q0 + r;
        bool qok = q < X;
        const double* base = bia + (long long)q * rowQ;
        int a = A0 + c, b = B0 + c;
        s_iA[r][c] = (qok && a < v) ? base[(long long)i * v + a] : 0.0;
        s_jA[r][c] = (qok && a < v) ? base[(long long)j * v + a] : 0.0;
        s_jB[r][c] = (qok && b < v) ? base[(long long)j * v + b] : 0.0;
        s_iB[r][c] = (qok && b < v) ? base[(long long)i * v + b] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int k0 = 0; k0 < KB; k0 += 4) {
        double a1[4], a2[4], b1[4], b2[4];
#pragma unroll
        for (int mi = 0; mi < 4; ++mi) {
          a1[mi] = s_iA[k0 + t][wm * 32 + mi * 8 + g];
          a2[mi] = s_jA[k0 + t][wm * 32 + mi * 8 + g];
        }
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
          b1[ni] = s_jB[k0 + t][wn * 32 + ni * 8 + g];
          b2[ni] = s_iB[k0 + t][wn * 32 + ni * 8 + g];
        }
#pragma unroll
        for (int mi = 0; mi < 4; ++mi)
#pragma unroll
          for (int ni = 0; ni < 4; ++ni) {
            dmma(acc1[mi][ni], a1[mi], b1[ni]);
            dmma(acc2[mi][ni], a2[mi], b2[ni]);
          }
      }
      __syncthreads();
    }

    // fused epilogue: denominators and pair energies in FP64
    const double ei = eps[i], ej = eps[j];
    double los = 0.0, lss = 0.0;
#pragma unroll
    for (int mi = 0; mi < 4; ++mi) {
      int a = A0 + wm * 32 + mi * 8 + g;
      if (a >= v) continue;
      double ea = eps[o + a];
#pragma unroll
      for (int ni = 0; ni < 4; ++ni)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          int b = B0 + wn * 32 + ni * 8 + 2 * t + e;
          if (b >= v) continue;
          double den = ((ea + eps[o + b]) - ei) - ej;
          double d1 = acc1[mi][ni][e], d2 = acc2[mi][ni][e];
          double r = 1.0 / den;
          los += (d1 * d1 + d2 * d2) * r;
          double df = d1 - d2;
          lss += df * df * r;
        }
    }
    double fw = (A < B ? 2.0 : 1.0) * (i < j ? 1.0 : 0.5);
    tot_os -= fw * los;
    tot_ss -= fw * lss;
  }

  tot_os = warp_sum(tot_os);
  tot_ss = warp_sum(tot_ss);
  if (lane == 0) {
    red[0][warp] = tot_os;
    red[1][warp] = tot_ss;
  }
  __syncthreads();
  if (tid == 0) {
    partials[2 * blockIdx.x] = (red[0][0] + red[0][1]) + (red[0][2] + red[0][3]);
    partials[2 * blockIdx.x + 1] = (red[1][0] + red[1][1]) + (red[1][2] + red[1][3]);
  }
}

}  // namespace

cudaError_t launch_energy_fp64(const double* bia, const double* eps, const EnergyShape& sh,
                               double* partials, int grid, cudaStream_t s) {
  energy_fp64_kernel<<<grid, 128, 0, s>>>(bia, eps, sh, partials);
  return cudaGetLastError();
}

}  // namespace corr
