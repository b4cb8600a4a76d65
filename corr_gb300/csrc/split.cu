// Split pre-pass of the RI-MP2 precision form and the final energy reduction.
//
// B^Q_ia (FP64, the reference's [Q][i][a] layout, ri.cc:147-172) is
// transposed to the K-major [i][a][Qp] layout the tcgen05 kernel reads with
// TMA and split into a 16-bit pair hi + lo, after a power-of-two pre-scale g
// that puts max|B| g in [2^13, 2^14): hi = rn(g B), lo = rn(g B - hi).  Every
// product hi*hi', hi*lo', lo*hi' is exact in FP32; the energy kernel undoes g
// with one multiplication by g^-4 of the pair-energy sums (exact).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"
#include "kernels.h"

namespace corr {

namespace {

__global__ void maxabs_kernel(const double* __restrict__ x, long long n,
                              unsigned long long* dmax) {
  double m = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x)
    m = fmax(m, fabs(x[k]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double wm[32];
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) wm[w] = m;
  __syncthreads();
  if (w == 0) {
    m = l < (int)(blockDim.x >> 5) ? wm[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    // non-negative doubles order like their bit patterns
    if (l == 0) atomicMax(dmax, (unsigned long long)__double_as_longlong(m));
  }
}

__device__ __forceinline__ double prescale(const unsigned long long* dmax) {
  double m = __longlong_as_double((long long)*dmax);
  if (!(m > 0.0) || !isfinite(m)) return 1.0;
  return ldexp(1.0, 13 - ilogb(m));
}

template <int FMT>
__global__ void split_kernel(const double* __restrict__ b, int naux, long long R, int Qp,
                             const unsigned long long* dmax, uint16_t* __restrict__ hi,
                             uint16_t* __restrict__ lo, double* scale_out) {
  __shared__ double tile[32][33];
  const double g = prescale(dmax);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long r0 = (long long)blockIdx.x * 32;
  const int q0 = blockIdx.y * 32;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int q = q0 + ty + 8 * k;
    long long r = r0 + tx;
    tile[ty + 8 * k][tx] = (q < naux && r < R) ? b[(long long)q * R + r] : 0.0;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    long long r = r0 + ty + 8 * k;
    int q = q0 + tx;
    if (r < R) {
      double v = tile[tx][ty + 8 * k] * g;
      uint16_t h, l;
      if (FMT == 0) {
        __half hh = __double2half(v);
        __half ll = __double2half(v - (double)__half2float(hh));
        h = __half_as_ushort(hh);
        l = __half_as_ushort(ll);
      } else {
        __nv_bfloat16 hh = __double2bfloat16(v);
        __nv_bfloat16 ll = __double2bfloat16(v - (double)__bfloat162float(hh));
        h = __bfloat16_as_ushort(hh);
        l = __bfloat16_as_ushort(ll);
      }
      hi[r * Qp + q] = h;
      lo[r * Qp + q] = l;
    }
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && tx == 0 && ty == 0) {
    double ig = 1.0 / g;  // power of two: exact
    scale_out[0] = ig * ig * ig * ig;
  }
}

__global__ void energy_reduce_kernel(const double* __restrict__ part, int n,
                                     const double* __restrict__ scale, double* out) {
  __shared__ double s_os[256], s_ss[256];
  double os = 0.0, ss = 0.0, cos_ = 0.0, css = 0.0;
  for (int k = threadIdx.x; k < n; k += 256) {  // compensated, fixed order
    double y = part[2 * k] - cos_;
    double t = os + y;
    cos_ = (t - os) - y;
    os = t;
    y = part[2 * k + 1] - css;
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
    double sc = scale ? scale[0] : 1.0;
    double eos = s_os[0] * sc, ess = s_ss[0] * sc;
    out[0] = ess;
    out[1] = eos;
    out[2] = ess + eos;
    out[3] = ess / 3.0 + eos * 6.0 / 5.0;
  }
}

}  // namespace

cudaError_t launch_maxabs(const double* x, long long n, unsigned long long* dmax, int sms,
                          cudaStream_t s) {
  long long want = (n + 255) / 256;
  int grid = (int)(want < (long long)sms * 8 ? (want > 0 ? want : 1) : (long long)sms * 8);
  maxabs_kernel<<<grid, 256, 0, s>>>(x, n, dmax);
  return cudaGetLastError();
}

cudaError_t launch_split(const double* b, int naux, long long R, int Qp, int fmt,
                         const unsigned long long* dmax, void* hi, void* lo, double* scale_out,
                         cudaStream_t s) {
  dim3 grid((unsigned)((R + 31) / 32), (unsigned)(Qp / 32));
  dim3 block(32, 8);
  if (fmt == 0)
    split_kernel<0><<<grid, block, 0, s>>>(b, naux, R, Qp, dmax, (uint16_t*)hi, (uint16_t*)lo,
                                           scale_out);
  else
    split_kernel<1><<<grid, block, 0, s>>>(b, naux, R, Qp, dmax, (uint16_t*)hi, (uint16_t*)lo,
                                           scale_out);
  return cudaGetLastError();
}

cudaError_t launch_energy_reduce(const double* partials, int n, const double* scale, double* out,
                                 cudaStream_t s) {
  energy_reduce_kernel<<<1, 256, 0, s>>>(partials, n, scale, out);
  return cudaGetLastError();
}

}  // namespace corr
