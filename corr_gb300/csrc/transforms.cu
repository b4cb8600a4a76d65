// FP64 transforms of the hot path and the canonical MP2 energy:
//   build_FMo          (src/POSTHF/motrans.cc:8-32)    two GEMMs
//   MOtrans            (src/POSTHF/motrans.cc:35-503)  packed-ERI unpack + 4 quarter GEMMs
//   run_canonical_mp2  (src/POSTHF/can_mp2.cc:11-49)   fused FP64 reduction
//   transform_ri       (src/POSTHF/ri.cc:147-172)      batched + flat GEMM
//   B build            (src/POSTHF/ri.cc:102-103)      one GEMM
// Every contraction runs through gemm_fp64.cu (FP64 tensor path, TMA-fed).
#include "common.cuh"
#include "gemm_fp64.h"
#include "kernels.h"

namespace corr {

namespace {

// Dense (ab|cd) from the reference's packed list: each entry scatters the
// permutations of its class (motrans.cc:341-403) into a zeroed N^4 array.
__global__ void unpack_eri_kernel(int N, long long n, const long long* __restrict__ sc,
                                  const double* __restrict__ val,
                                  const unsigned short* __restrict__ num,
                                  double* __restrict__ eri) {
  const size_t N1 = N, N2 = N1 * N1, N3 = N2 * N1;
  const long long s0 = sc[0], s1 = sc[1], s2 = sc[2], s3 = sc[3];
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
       x += (long long)gridDim.x * blockDim.x) {
    const size_t a = num[4 * x], b = num[4 * x + 1], c = num[4 * x + 2], d = num[4 * x + 3];
    const double v = val[x];
#define AT(p, q, r, s) atomicAdd(&eri[(p) * N3 + (q) * N2 + (r) * N1 + (s)], v)
    AT(a, b, c, d);
    if (x < s0) continue;
    if (x < s1) {
      AT(c, d, a, b);
      continue;
    }
    if (x < s2) {
      AT(a, b, d, c);
      AT(b, a, c, d);
      AT(b, a, d, c);
      continue;
    }
    if (x < s3) {
      AT(a, b, d, c);
      AT(c, d, a, b);
      AT(d, c, a, b);
      continue;
    }
    AT(a, b, d, c);
    AT(b, a, c, d);
    AT(b, a, d, c);
    AT(c, d, a, b);
    AT(d, c, a, b);
    AT(c, d, b, a);
    AT(d, c, b, a);
#undef AT
  }
}

// Canonical MP2 (can_mp2.cc:26-35) over (ia|jb), read either from the full
// [N][N][N][N] tensor (full != 0) or from an [o][v][o][v] block.
__global__ void canonical_mp2_kernel(const double* __restrict__ t, int full, int N, int o, int v,
                                     const double* __restrict__ eps, double* __restrict__ part) {
  const long long total = (long long)o * o * v * v;
  double os = 0.0, ss = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(e % v);
    const int a = (int)((e / v) % v);
    const int j = (int)((e / ((long long)v * v)) % o);
    const int i = (int)(e / ((long long)v * v * o));
    double iajb, ibja;
    if (full) {
      const size_t n1 = N;
      iajb = t[(((size_t)i * n1 + (o + a)) * n1 + j) * n1 + (o + b)];
      ibja = t[(((size_t)i * n1 + (o + b)) * n1 + j) * n1 + (o + a)];
    } else {
      iajb = t[(((size_t)i * v + a) * o + j) * v + b];
      ibja = t[(((size_t)i * v + b) * o + j) * v + a];
    }
    const double den = ((eps[o + a] + eps[o + b]) - eps[i]) - eps[j];
    os += -(iajb * iajb) / den;
    ss += -(iajb - ibja) * iajb / den;
  }
  os = warp_sum(os);
  ss = warp_sum(ss);
  __shared__ double r[2][32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    r[0][w] = os;
    r[1][w] = ss;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      a += r[0][k];
      b += r[1][k];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

__global__ void diag_kernel(const double* __restrict__ f, int N, double* __restrict__ d) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < N) d[p] = f[(size_t)p * N + p];
}

int grid_for(long long n, int sms) {
  long long g = (n + 255) / 256;
  long long cap = (long long)sms * 8;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

// One quarter transform: out[r][p] = sum_a in[a][r] C[p][a] for the nout rows
// of C starting at `crow` (in: K x M with K = N).
int quarter(corr_context* c, const double* in, const double* mos, int N, int crow, int nout,
            long long M, double* out) {
  if (M > 0x7fffffffLL) {
    set_error("quarter transform: %lld rows exceed the GEMM row limit", M);
    return CORR_ERR_BAD_ARG;
  }
  GemmF64 g = gemm_args(in, mos + (size_t)crow * N, out, (int)M, nout, N, M, N, nout, 1, 1);
  return gemm_f64(g, &c->dres->status, c->stream);
}

int launch_unpack(corr_context* c, int N, long long n, const long long* sc, const double* val,
                  const unsigned short* num, double* eri) {
  size_t n4 = (size_t)N * N * N * N;
  CORR_CUDA(cudaMemsetAsync(eri, 0, n4 * 8, c->stream));
  if (n > 0) {
    unpack_eri_kernel<<<grid_for(n, c->sms), 256, 0, c->stream>>>(N, n, sc, val, num, eri);
    CORR_CUDA(cudaGetLastError());
    c->launches += 1;
  }
  return CORR_OK;
}

int launch_canonical(corr_context* c, const double* t, int full, int N, int o, int v,
                     const double* eps, double* part, int grid) {
  canonical_mp2_kernel<<<grid, 256, 0, c->stream>>>(t, full, N, o, v, eps, part);
  CORR_CUDA(cudaGetLastError());
  CORR_CUDA(launch_energy_reduce(part, grid, nullptr, c->dres->e, c->stream));
  c->launches += 2;
  return CORR_OK;
}

int launch_diag(corr_context* c, const double* f, int N, double* d) {
  diag_kernel<<<(N + 255) / 256, 256, 0, c->stream>>>(f, N, d);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  return CORR_OK;
}

int canonical_grid(corr_context* c, long long total) { return grid_for(total, c->sms); }

}  // namespace corr
