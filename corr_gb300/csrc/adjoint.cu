// RI-MP2 adjoint: dE/dB^Q_ia and dE/d eps (no reference counterpart; the
// reference has no gradient code).
//
// With M^{ij}_ab = sum_Q B^Q_ia B^Q_jb and D = e_a + e_b - e_i - e_j,
//   E = -sum_{ijab} (2 M_ab - M_ba) M_ab / D                  (can_mp2.cc:82-97)
//   G^{ij}_ab = dE/dM^{ij}_ab = -(4 M_ab - 2 M_ba) / D
//   dE/dB^Q_ia = 2 sum_{jb} G^{ij}_ab B^Q_jb
//   W^{ij}_ab = (2 M_ab - M_ba) M_ab / D^2,
//   dE/de_c = +sum of W over (a == c) and (b == c),  dE/de_k = -sum of W over (i == k), (j == k).
//
// For a block I of occupied orbitals the panel kernel recomputes the tiles
// M^{ij}[A,B] and M^{ij}[B,A] (A <= B) on the FP64 tensor path, writes the
// gradient panel P[i-i0][a][j][b] = G^{ij}_ab (a transient buffer of |I| o v^2
// doubles, never the whole amplitude tensor) and folds W into dE/de with FP64
// atomics; then dB[Q][i][a] (i in I) = 2 sum_{(j,b)} B[Q][(j,b)] P[(i,a)][(j,b)]
// is one FP64 GEMM (gemm_fp64.cu).
#include <algorithm>

#include "common.cuh"
#include "dgemm_tc.h"
#include "gemm_fp64.h"
#include "kernels.h"

namespace corr {

namespace {

constexpr int T = kF64Tile;  // 64
constexpr int KB = 16;
constexpr int LD = T + 4;

__device__ __forceinline__ void dmma(double (&d)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(d[0]), "+d"(d[1])
               : "d"(a), "d"(b));
}

struct PanelArgs {
  const double* bia;
  const double* eps;
  double* panel;  // [bi][v][o][v]
  double* deps;   // [o+v], accumulated
  double* part;   // per-CTA energy partials {E, 0}
  int o, v, X, i0, bi, ntiles, ntp;
  long long nunits;  // bi * o * ntp
};

__global__ void __launch_bounds__(128) adjoint_panel_kernel(PanelArgs g) {
  __shared__ double s_iA[KB][LD], s_jB[KB][LD], s_jA[KB][LD], s_iB[KB][LD];
  __shared__ double red[4], red2[4];
  __shared__ double roww[T], colw[T];
  const int o = g.o, v = g.v, X = g.X;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int gq = lane >> 2, tq = lane & 3;
  const long long rowQ = (long long)o * v;
  double etot = 0.0;

  for (long long u = blockIdx.x; u < g.nunits; u += gridDim.x) {
    const int tp = (int)(u % g.ntp);
    const long long ij = u / g.ntp;
    const int j = (int)(ij % o);
    const int il = (int)(ij / o);
    const int i = g.i0 + il;
    int A, B;
    tpair_decode(tp, g.ntiles, &A, &B);
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
        const int idx = tid + 128 * e;
        const int r = idx / T, c = idx % T;
        const int q = q0 + r;
        const bool qok = q < X;
        const double* base = g.bia + (long long)q * rowQ;
        const int a = A0 + c, b = B0 + c;
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
          a1[mi] = s_iA[k0 + tq][wm * 32 + mi * 8 + gq];
          a2[mi] = s_jA[k0 + tq][wm * 32 + mi * 8 + gq];
        }
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
          b1[ni] = s_jB[k0 + tq][wn * 32 + ni * 8 + gq];
          b2[ni] = s_iB[k0 + tq][wn * 32 + ni * 8 + gq];
        }
#pragma unroll
        for (int mi = 0; mi < 4; ++mi)
#pragma unroll
          for (int ni = 0; ni < 4; ++ni) {
            dmma(acc1[mi][ni], a1[mi], b1[ni]);  // M^{ij}_ab
            dmma(acc2[mi][ni], a2[mi], b2[ni]);  // M^{ji}_ab = M^{ij}_ba
          }
      }
      __syncthreads();
    }

    // epilogue: gradient panel, W sums (reduced in shared memory per unit), energy
    if (tid < T) {
      roww[tid] = 0.0;
      colw[tid] = 0.0;
    }
    __syncthreads();
    const double ei = g.eps[i], ej = g.eps[j];
    const bool diag = (A == B);
    double* P = g.panel + (size_t)il * v * o * v;
    double wsum = 0.0, eu = 0.0;
#pragma unroll
    for (int mi = 0; mi < 4; ++mi) {
      const int a = A0 + wm * 32 + mi * 8 + gq;
      if (a >= v) continue;
      const double ea = g.eps[o + a];
      double wa = 0.0;
#pragma unroll
      for (int ni = 0; ni < 4; ++ni)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int b = B0 + wn * 32 + ni * 8 + 2 * tq + e;
          if (b >= v) continue;
          const double den = ((ea + g.eps[o + b]) - ei) - ej;
          const double r = 1.0 / den;
          const double mab = acc1[mi][ni][e], mba = acc2[mi][ni][e];
          const double tab = 2.0 * mab - mba, tba = 2.0 * mba - mab;
          P[((size_t)a * o + j) * v + b] = -2.0 * tab * r;  // G^{ij}_ab
          P[((size_t)b * o + j) * v + a] = -2.0 * tba * r;  // G^{ij}_ba
          double w = tab * mab * r * r;
          eu -= tab * mab * r;
          if (!diag) {
            const double wba = tba * mba * r * r;
            eu -= tba * mba * r;
            w += wba;
          }
          wa += w;
          wsum += w;
          atomicAdd(&colw[b - B0], w);
        }
      atomicAdd(&roww[a - A0], wa);
    }
    wsum = warp_sum(wsum);
    if (lane == 0) red2[warp] = wsum;
    __syncthreads();
    if (tid < T) {
      if (A0 + tid < v) atomicAdd(&g.deps[o + A0 + tid], roww[tid]);
      if (B0 + tid < v) atomicAdd(&g.deps[o + B0 + tid], colw[tid]);
    }
    if (tid == 0) {
      const double ws = (red2[0] + red2[1]) + (red2[2] + red2[3]);
      atomicAdd(&g.deps[i], -ws);
      atomicAdd(&g.deps[j], -ws);
    }
    etot += eu;
  }
  etot = warp_sum(etot);
  if (lane == 0) red[warp] = etot;
  __syncthreads();
  if (tid == 0) {
    g.part[2 * blockIdx.x] = (red[0] + red[1]) + (red[2] + red[3]);
    g.part[2 * blockIdx.x + 1] = 0.0;
  }
}

// Tensor-core form, step 2: the panel P[(il, a)][(j, b)] holds M^{ij}_ab for
// the occupied block i = i0 + il; one CTA per (il, j) replaces every element
// by G^{ij}_ab = -(4 M_ab - 2 M_ba) / D (in place: one thread owns the pair
// (a, b), (b, a)), accumulates W = (2 M_ab - M_ba) M_ab / D^2 into dE/d eps
// (per-CTA sums in shared memory, then atomics) and writes the pair block's
// energy -sum (2 M_ab - M_ba) M_ab / D to its own partial.
__global__ void __launch_bounds__(256) grad_panel_kernel(double* __restrict__ P,
                                                         const double* __restrict__ eps, int o,
                                                         int v, int i0, double* __restrict__ deps,
                                                         double* __restrict__ part) {
  extern __shared__ double wv[];  // [v]: W summed into dE/d eps_(o+c)
  __shared__ double red[2][8];
  const int il = blockIdx.x / o, j = blockIdx.x % o, i = i0 + il;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int c = threadIdx.x; c < v; c += blockDim.x) wv[c] = 0.0;
  __syncthreads();
  const long long ld = (long long)o * v;
  double* Pi = P + (long long)il * v * ld + (long long)j * v;  // row a at Pi + a * ld
  const double eij = eps[i] + eps[j];
  double wsum = 0.0, esum = 0.0;
  for (int a = warp; a < v; a += nw) {
    const double ea = eps[o + a];
    double wa = 0.0;
    for (int b = a + lane; b < v; b += 32) {
      const double r = 1.0 / ((ea + eps[o + b]) - eij);
      double* pab = Pi + (long long)a * ld + b;
      double* pba = Pi + (long long)b * ld + a;
      const double mab = *pab, mba = *pba;
      const double tab = 2.0 * mab - mba, tba = 2.0 * mba - mab;
      double w, e;
      if (a == b) {
        w = 2.0 * tab * mab * r * r;  // (a == c) and (b == c)
        e = tab * mab * r;
        *pab = -2.0 * tab * r;
      } else {
        const double wab = (tab * mab + tba * mba) * r * r;
        w = wab;
        e = (tab * mab + tba * mba) * r;
        *pab = -2.0 * tab * r;
        *pba = -2.0 * tba * r;
        atomicAdd(&wv[b], wab);
      }
      wa += w;
      wsum += (a == b) ? 0.5 * w : w;
      esum -= e;
    }
    for (int off = 16; off > 0; off >>= 1) wa += __shfl_xor_sync(0xffffffffu, wa, off);
    if (lane == 0) atomicAdd(&wv[a], wa);
  }
  wsum = warp_sum(wsum);
  esum = warp_sum(esum);
  if (lane == 0) {
    red[0][warp] = wsum;
    red[1][warp] = esum;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < v; c += blockDim.x)
    if (wv[c] != 0.0) atomicAdd(&deps[o + c], wv[c]);
  if (threadIdx.x == 0) {
    double ws = 0.0, es = 0.0;
    for (int k = 0; k < nw; ++k) {
      ws += red[0][k];
      es += red[1][k];
    }
    atomicAdd(&deps[i], -ws);
    atomicAdd(&deps[j], -ws);
    part[2 * blockIdx.x] = es;
    part[2 * blockIdx.x + 1] = 0.0;
  }
}

}  // namespace

size_t rimp2_gradient_workspace(int o, int v, int sms, size_t panel_budget);

// Enqueue the whole FP64 gradient on c->stream.  bia, eps device; dbia
// [X][o][v] and deps [o+v] device outputs (overwritten); energy -> c->dres.
int rimp2_gradient_fp64(corr_context* c, Carver& w, int o, int v, int X, const double* bia,
                        const double* eps, double* dbia, double* deps, size_t panel_budget) {
  const size_t per_i = (size_t)v * o * v * 8;
  int bi = (int)(panel_budget / per_i);
  if (bi < 1) bi = 1;
  if (bi > o) bi = o;
  double* panel = static_cast<double*>(w.take(per_i * bi));
  const int grid = c->sms * 2;
  double* part = static_cast<double*>(w.take((size_t)grid * 16 * ((o + bi - 1) / bi)));
  CORR_CUDA(cudaMemsetAsync(deps, 0, (size_t)(o + v) * 8, c->stream));
  const int nt = (v + T - 1) / T;
  const int nblocks = (o + bi - 1) / bi;
  for (int blk = 0; blk < nblocks; ++blk) {
    PanelArgs a;
    a.bia = bia;
    a.eps = eps;
    a.panel = panel;
    a.deps = deps;
    a.part = part + (size_t)blk * grid * 2;
    a.o = o;
    a.v = v;
    a.X = X;
    a.i0 = blk * bi;
    a.bi = (a.i0 + bi <= o) ? bi : (o - a.i0);
    a.ntiles = nt;
    a.ntp = nt * (nt + 1) / 2;
    a.nunits = (long long)a.bi * o * a.ntp;
    adjoint_panel_kernel<<<grid, 128, 0, c->stream>>>(a);
    CORR_CUDA(cudaGetLastError());
    // dB[Q][(i,a)], i in the block = 2 * B[Q][(j,b)] . P[(i,a)][(j,b)]^T
    GemmF64 gm = gemm_args(bia, panel, dbia + (size_t)a.i0 * v, X, a.bi * v, o * v, (long long)o * v,
                           (long long)o * v, (long long)o * v, 0, 1);
    gm.alpha = 2.0;
    CORR_TRY(gemm_f64(gm, &c->dres->status, c->stream));
    c->launches += 2;
  }
  CORR_CUDA(launch_energy_reduce(part, grid * nblocks, nullptr, c->dres->e, c->stream));
  c->launches += 1;
  return CORR_OK;
}

size_t rimp2_gradient_workspace(int o, int v, int sms, size_t panel_budget) {
  const size_t per_i = (size_t)v * o * v * 8;
  int bi = (int)(panel_budget / per_i);
  if (bi < 1) bi = 1;
  if (bi > o) bi = o;
  return per_i * bi + (size_t)sms * 2 * 16 * ((o + bi - 1) / bi) + 512;
}

// The adjoint on the tensor cores: per block of bi occupied orbitals the
// panel M[(i, a)][(j, b)] = sum_Q B^Q_ia B^Q_jb (i in the block, all j) by the
// FP64-accurate digit GEMM (dgemm_tc.cu), G, W and E by grad_panel_kernel,
// then dB[Q][(i, a)] = 2 sum_(j,b) B[Q][(j, b)] G[(i, a)][(j, b)] by the digit
// GEMM.  FP64 accuracy (bounds of the digit GEMM), tensor-core speed.
size_t rimp2_gradient_tc_workspace(int o, int v, int X, size_t panel_budget, int* bi_out) {
  const size_t per_i = (size_t)v * o * v * 8;
  int bi = (int)(panel_budget / per_i);
  bi = std::max(1, std::min(bi, o));
  if (bi_out) *bi_out = bi;
  const int ov = o * v;
  const size_t ws = std::max(dgemm_tc_workspace(bi * v, ov, X), dgemm_tc_workspace(X, bi * v, ov));
  return per_i * bi + ws + (size_t)o * o * 16 + 1024;
}

int rimp2_gradient_tc(corr_context* c, Carver& w, int o, int v, int X, const double* bia,
                      const double* eps, double* dbia, double* deps, size_t panel_budget) {
  CORR_CHECK_ARG(v <= 6144, "corr_rimp2_gradient_tc: nvir %d above 6144", v);
  int bi = 1;
  rimp2_gradient_tc_workspace(o, v, X, panel_budget, &bi);
  const int ov = o * v;
  double* panel = static_cast<double*>(w.take((size_t)v * o * v * 8 * bi));
  void* dws = w.take(std::max(dgemm_tc_workspace(bi * v, ov, X),
                              dgemm_tc_workspace(X, bi * v, ov)));
  double* part = static_cast<double*>(w.take((size_t)o * o * 16));
  CORR_CUDA(cudaMemsetAsync(deps, 0, (size_t)(o + v) * 8, c->stream));
  for (int i0 = 0; i0 < o; i0 += bi) {
    const int nb = std::min(bi, o - i0);
    DgemmTc m;
    m.A = mat_view(bia + (size_t)i0 * v, 1, ov);  // rows (i, a) of the block, over Q
    m.B = mat_view(bia, 1, ov);                   // rows (j, b), over Q
    m.C = out_view(panel, ov, 1);
    m.M = nb * v;
    m.N = ov;
    m.K = X;
    m.alpha = 1.0;
    m.accumulate = false;
    m.a_lower = false;
    CORR_TRY(dgemm_tc(c, m, dws));
    grad_panel_kernel<<<nb * o, 256, (size_t)v * 8, c->stream>>>(panel, eps, o, v, i0, deps,
                                                                  part + (size_t)i0 * o * 2);
    CORR_CUDA(cudaGetLastError());
    DgemmTc d;
    d.A = mat_view(bia, ov, 1);    // rows Q, over (j, b)
    d.B = mat_view(panel, ov, 1);  // rows (i, a) of the block, over (j, b)
    d.C = out_view(dbia + (size_t)i0 * v, ov, 1);
    d.M = X;
    d.N = nb * v;
    d.K = ov;
    d.alpha = 2.0;
    d.accumulate = false;
    d.a_lower = false;
    CORR_TRY(dgemm_tc(c, d, dws));
    c->launches += 1;
  }
  CORR_CUDA(launch_energy_reduce(part, o * o, nullptr, c->dres->e, c->stream));
  c->launches += 1;
  return CORR_OK;
}

}  // namespace corr

using namespace corr;

static int rimp2_gradient_call(corr_context* c, int nocc, int nvir, int naux, const double* bia,
                               const double* eps, double* dbia, double* deps,
                               corr_mp2_energy* e_out, bool tc) {
  CORR_CHECK_ARG(c && bia && eps && dbia && deps, "corr_rimp2_gradient: null pointer argument");
  CORR_CHECK_ARG(nocc >= 1 && nvir >= 1 && naux >= 1, "corr_rimp2_gradient: bad sizes");
  CORR_CHECK_ARG((long long)nocc * nvir <= 0x7fffffffLL, "corr_rimp2_gradient: nocc*nvir too large");
  CORR_CUDA(cudaSetDevice(c->device));
  const size_t nb = (size_t)naux * nocc * nvir, ne = (size_t)nocc + nvir;
  const bool bdev = is_device_ptr(bia), edev = is_device_ptr(eps);
  const bool odb = is_device_ptr(dbia), ode = is_device_ptr(deps);
  const size_t budget = (size_t)1 << 30;  // gradient panel of at most ~1 GiB per i-block
  auto plan = [&](Carver& w, void** sb, void** se, double** db, double** de) {
    *sb = bdev ? nullptr : w.take(nb * 8);
    *se = edev ? nullptr : w.take(ne * 8);
    *db = odb ? dbia : static_cast<double*>(w.take(nb * 8));
    *de = ode ? deps : static_cast<double*>(w.take(ne * 8));
  };
  void *sb, *se;
  double *db, *de;
  Carver cv{nullptr, 0};
  plan(cv, &sb, &se, &db, &de);
  cv.take(tc ? rimp2_gradient_tc_workspace(nocc, nvir, naux, budget, nullptr)
             : rimp2_gradient_workspace(nocc, nvir, c->sms, budget));
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  plan(w, &sb, &se, &db, &de);
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_b = static_cast<const double*>(stage_in(c, bia, nb * 8, sb));
  const double* d_e = static_cast<const double*>(stage_in(c, eps, ne * 8, se));
  CORR_CHECK_ARG(d_b && d_e, "host-to-device copy failed");
  mark(c, 1);
  if (tc)
    CORR_TRY(rimp2_gradient_tc(c, w, nocc, nvir, naux, d_b, d_e, db, de, budget));
  else
    CORR_TRY(rimp2_gradient_fp64(c, w, nocc, nvir, naux, d_b, d_e, db, de, budget));
  mark(c, 2);
  CORR_TRY(stage_out(c, dbia, db, nb * 8));
  CORR_TRY(stage_out(c, deps, de, ne * 8));
  CORR_TRY(finish_results(c, 3));
  if (e_out) {
    e_out->e_total = c->hres->e[2];
    e_out->e_os = e_out->e_ss = e_out->e_scs = 0.0;  // the gradient call reports E only
  }
  return CORR_OK;
}

extern "C" int corr_rimp2_gradient(corr_context* c, int nocc, int nvir, int naux,
                                   const double* bia, const double* eps, double* dbia,
                                   double* deps, corr_mp2_energy* e_out) {
  return rimp2_gradient_call(c, nocc, nvir, naux, bia, eps, dbia, deps, e_out, false);
}

extern "C" int corr_rimp2_gradient_tc(corr_context* c, int nocc, int nvir, int naux,
                                      const double* bia, const double* eps, double* dbia,
                                      double* deps, corr_mp2_energy* e_out) {
  return rimp2_gradient_call(c, nocc, nvir, naux, bia, eps, dbia, deps, e_out, true);
}
