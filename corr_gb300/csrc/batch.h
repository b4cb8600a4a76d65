// Batched precision-form RI-MP2 (energy_batch.cu, batch.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace corr {

// Device-side description of one instance of a batch.
struct BatchInst {
  const uint16_t* S;    // digit planes in the tiled layout (kernels.h)
  const double* eps;    // [o+v]
  const float* sc;      // [o*v] row factors 2^(e_r - e_ref)
  const float* dg;      // [o*v] FP64 diagonal in scaled units
  const double* scale;  // [2] {energy factor 2^(4 e_ref), 1/L of the digits}
  long long unit_begin; // first global unit of this instance
  long long nunits;
  int o, v, ntiles, ntpairs, nkb;
};

size_t batch_kernel_smem(int stages);
cudaError_t prepare_energy_batch();
cudaError_t launch_energy_batch(const BatchInst* insts, int ninst,
                                long long total, unsigned long long* queue, int fmt, int scheme,
                                int stages, int grid, double* unit_part, int* status,
                                cudaStream_t s);
cudaError_t launch_batch_reduce(const BatchInst* insts, int ninst, const double* unit_part,
                                const int* out_index, double* out, cudaStream_t s);

}  // namespace corr
