// Internal interface between the C-ABI layer (abi.cu) and the kernel files.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace corr {

// Per-unit work description of the fused RI-MP2 energy kernels.
//   pairs (i<=j) of occupied orbitals x tile pairs (A<=B) of virtual tiles.
struct EnergyShape {
  int nocc, nvir, naux;
  int tile;     // virtual tile edge (rows of a / cols of b)
  int ntiles;   // ceil(nvir / tile)
  int npairs;   // nocc (nocc+1) / 2
  int ntpairs;  // ntiles (ntiles+1) / 2
  long long nunits;
};

EnergyShape make_energy_shape(int nocc, int nvir, int naux, int tile);

// ---- split pre-pass (split.cu) ---------------------------------------------
// maxabs of n doubles -> *dmax (as ordered uint64 bits; *dmax must start at 0).
cudaError_t launch_maxabs(const double* x, long long n, unsigned long long* dmax, int sms,
                          cudaStream_t s);
// B[Q][r] (r = i*nvir + a, R = nocc*nvir) -> hi/lo[r][Qp] (16-bit), scaled by the
// power of two derived from *dmax; Q >= naux is zero padding.  fmt 0 fp16, 1 bf16.
cudaError_t launch_split(const double* b, int naux, long long R, int Qp, int fmt,
                         const unsigned long long* dmax, void* hi, void* lo, double* scale_out,
                         cudaStream_t s);
// Sum per-CTA partial pairs {os, ss} in fixed order, times `scale` (device),
// into out[4] = {E_SS, E_OS, E, E_SCS}.
cudaError_t launch_energy_reduce(const double* partials, int n, const double* scale, double* out,
                                 cudaStream_t s);

// ---- fused energy kernels ---------------------------------------------------
// tcgen05 split form (energy_tc.cu).  tmap_hi/tmap_lo: 3-D maps over
// [nocc][nvir][Qp] 16-bit arrays, box {32, 128, 1}, 64B swizzle.
cudaError_t launch_energy_tc(const CUtensorMap& tmap_hi, const CUtensorMap& tmap_lo,
                             const double* eps, const EnergyShape& sh, int Qp, int fmt,
                             double* partials, int grid, int* status, cudaStream_t s);
constexpr int kTcTile = 128;

// FP64 form on the FP64 tensor path (energy_fp64.cu).
cudaError_t launch_energy_fp64(const double* bia, const double* eps, const EnergyShape& sh,
                               double* partials, int grid, cudaStream_t s);
constexpr int kF64Tile = 64;

}  // namespace corr
