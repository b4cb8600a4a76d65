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

// ---- slice pre-pass (split.cu) ---------------------------------------------
// Device buffers of the precision form's pre-pass (R = nocc*nvir rows).
// Tiled digit layout read by the energy kernels: occupied i, 64-wide Q block
// kb, 128-row virtual tile A, digit plane l -> one 16 KB tile of 128 rows x
// 64 Q (16-bit), stored as the 128-byte-swizzled shared-memory image the
// tensor-core descriptors read (the 16-byte chunk c of row r sits at chunk
// c ^ (r & 7)).  The npl planes of one (i, kb, A) are adjacent (npl x 16 KB),
// so an operand of a pipeline stage is one copy.  Offsets in elements.
constexpr int kSliceQ = 64;                          // Q per tile row (128 bytes)
constexpr int kSliceTileElems = 128 * kSliceQ;       // 8192 elements, 16 KB
__host__ __device__ inline size_t slice_tile_offset(int l, int i, int kb, int A, int nkb,
                                                    int ntiles, int npl) {
  return ((((size_t)i * nkb + kb) * ntiles + A) * npl + l) * kSliceTileElems;
}
__host__ __device__ inline size_t slice_chunk_offset(int row, int chunk) {
  return (size_t)row * kSliceQ + (size_t)((chunk ^ (row & 7)) * 8);
}
// naux padded for the tensor-core forms (whole 64-wide Q blocks)
inline int padded_naux(int naux) { return ((naux + kSliceQ - 1) / kSliceQ) * kSliceQ; }
// bytes of the digit planes (sized for three planes, enough for either scheme)
inline size_t slice_bytes(int nocc, int nvir, int Qp) {
  return (size_t)3 * nocc * (Qp / kSliceQ) * ((nvir + 127) / 128) * (kSliceTileElems * 2);
}

struct SliceWork {
  uint16_t* S;     // digit planes in the tiled layout (fp16 or bf16 encoding)
  int* erow;       // [R] row exponents
  double* diag;    // [R] FP64 sum_Q B^2
  float* sc;       // [R] 2^(e_r - e_ref)
  float2* dg;      // [R] FP64 diag in scaled units as float-float (hi, lo)
  int* eref;       // [2] {e_ref, level exponent k (scheme 1)}
  double* scale;   // [2] {global energy factor 2^(4 e_ref), 1/L}
  int* x20;        // [naux][R] fixed-point values at the row scale (scheme 1), or null:
                   // written by the row statistics, read by the slice (row_stats_stage_x20)
};
// Whether the scheme-1 row statistics of this naux run in the shared-memory
// form, which can hand the 20-bit fixed-point values on to the slice (SliceWork::x20).
bool row_stats_stage_x20(int naux);
// Slice schemes (split.cu).  0: three BF16 digits, six products per K step
// (levels 0..2).  1: two FP16 digits, four products per K step into three
// accumulators (s0.s0', s0.s1' + s1.s0', s1.s1').
constexpr int kSchemeDigits3 = 0;
constexpr int kSchemeDigits2 = 1;
__host__ __device__ constexpr int planes_for_scheme(int scheme) {
  return scheme == kSchemeDigits2 ? 2 : 3;
}
inline int scheme_for_precision(int precision) {
  return precision == 1 /* CORR_PREC_SPLIT_FP16 */ ? kSchemeDigits2 : kSchemeDigits3;
}
inline int format_for_scheme(int scheme) { return scheme == kSchemeDigits2 ? 0 : 1; }  // 0 FP16
int slice_bits_for(int Qp);
cudaError_t launch_slices(const double* b, int naux, int nocc, int nvir, int Qp, int scheme,
                          int fmt, int p, SliceWork w, cudaStream_t s);
// The same in parts (for row statistics that follow rows arriving in chunks):
// reset the reductions, row statistics of rows [rbeg, rend) (rbeg a multiple
// of 32), then the digit planes once every row is done.
cudaError_t reset_row_stats(SliceWork w, cudaStream_t s);
// After the row statistics of the two-digit scheme: halve L (error estimate).
cudaError_t coarsen_level(SliceWork w, cudaStream_t s);
cudaError_t launch_row_stats(const double* b, int naux, int nocc, int nvir, int scheme, int p,
                             SliceWork w, long long rbeg, long long rend, cudaStream_t s);
cudaError_t launch_slice_planes(const double* b, int naux, int nocc, int nvir, int Qp,
                                int scheme, int fmt, int p, SliceWork w, cudaStream_t s);
// Sum per-CTA partial pairs {os, ss} in fixed order, times `scale` (device),
// into out[4] = {E_SS, E_OS, E, E_SCS}.
// The same for many pairs (one per unit): kReduceBlocks blocks sum fixed
// chunks into scratch (kReduceBlocks pairs) and the last block to finish sums
// those in chunk order (one launch; *ticket, a device counter, must be 0).
// Returns the kernels launched (1), or -1 on a launch error.
constexpr int kReduceBlocks = 64;
int launch_unit_reduce(const double* partials, int n, const double* scale, double* out,
                       double* scratch, unsigned* ticket, cudaStream_t s);
cudaError_t launch_energy_reduce(const double* partials, int n, const double* scale, double* out,
                                 cudaStream_t s);

// ---- fused energy kernels ---------------------------------------------------
// One RI-MP2 instance as the tcgen05 precision-form kernel (energy_tc.cu) reads
// it: its digit planes and row factors (SliceWork), orbital energies, shape,
// and its first unit in the launch's global unit numbering.  The batch form
// holds an array of these in device memory.
constexpr int kTcTile = 128;
struct TcInst {
  const uint16_t* S;     // digit planes in the tiled layout
  const double* eps;     // [o+v]
  const float* sc;       // [o*v] row factors 2^(e_r - e_ref)
  const float2* dg;      // [o*v] FP64 diagonal (ia|ia) in scaled units (float-float)
  const double* scale;   // [2] {energy factor 2^(4 e_ref), 1/L of the digits}
  long long unit_begin;  // first global unit of this instance
  long long nunits;
  int o, v, ntiles, ntpairs, nkb;
};
TcInst make_tc_inst(const SliceWork& sw, const double* eps, const EnergyShape& sh, int Qp,
                    long long unit_begin);
// Shared-memory attributes of every kernel variant (once per device, outside
// stream capture).
cudaError_t prepare_energy_tc();
// One instance: units 0 .. nunits-1 from the device counter `queue` (16
// bytes, zeroed here on the stream before the launch; the second word is the
// ticket of launch_unit_reduce).  partials: {os, ss} per unit.  stages: 2 or
// 3 (scheme 1; scheme 0 always runs 2).
cudaError_t launch_energy_tc(const TcInst& inst, int fmt, int scheme, int stages, int grid,
                             double* partials, int* status, unsigned long long* queue,
                             cudaStream_t s);
// A batch: dtab[n] in device memory with consecutive unit ranges (total units).
cudaError_t launch_energy_tc_batch(const TcInst* dtab, int n, long long total, int fmt,
                                   int scheme, int stages, int grid, double* partials,
                                   int* status, unsigned long long* queue, cudaStream_t s);
// Per instance k of the table: the fixed-order sum of its unit partials times
// its energy scale, into out[4 out_index[k] + {0,1,2,3}] = {E_SS, E_OS, E, E_SCS}.
cudaError_t launch_batch_reduce(const TcInst* dtab, int n, const double* partials,
                                const int* out_index, double* out, cudaStream_t s);

// FP64 form on the FP64 tensor path (energy_fp64.cu).
cudaError_t launch_energy_fp64(const double* bia, const double* eps, const EnergyShape& sh,
                               double* partials, int grid, cudaStream_t s);
constexpr int kF64Tile = 64;

}  // namespace corr
