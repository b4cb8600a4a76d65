// Context internals shared by the C-ABI translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/corr_gb300.h"

namespace corr {

// Small result block the kernels write and one D2H copy brings back.
struct ResultBlock {
  double e[8];
  int status;  // bit flags raised by device code (CORR_ERR_DEVICE_TIMEOUT)
  int pad;
};

struct Workspace {
  void* ptr = nullptr;
  size_t cap = 0;
  int reserve(size_t bytes);
};

// Bump allocator over a workspace (base == nullptr: size pass only).
struct Carver {
  void* base;
  size_t used;
  void* take(size_t bytes);
};

bool is_device_ptr(const void* p);
int encode_tmap(CUtensorMap* m, CUtensorMapDataType dt, int rank, void* base, const uint64_t* dims,
                const uint64_t* strides_bytes, const uint32_t* box, CUtensorMapSwizzle swz);

}  // namespace corr

struct corr_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sms = 0;
  corr::Workspace ws;
  corr::ResultBlock* dres = nullptr;  // device
  corr::ResultBlock* hres = nullptr;  // pinned host
  bool timing = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float t_prepass = 0.f, t_kernel = 0.f, t_total = 0.f;
  long long launches = 0;
  bool attrs_set = false;  // one-time kernel attributes (kept out of graph capture)
  int fp64_strict = 0;     // 1: the plain-form metric calls use FP64 GEMMs and Jacobi only
  // batched driver
  int batch_order = 1;   // 0 input order, 1 cost-descending
  int batch_stages = 3;
  int batch_tiles = 1;
  corr::Workspace batch_out;
  void* pinned = nullptr;
  // chunked upload of host inputs (created on first use)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t cev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // side streams of the batched pre-pass (instances sliced concurrently) and
  // their fork/join events (the last one marks the fork on the context stream)
  static constexpr int kPreStreams = 8;
  cudaStream_t pre_stream[kPreStreams] = {};
  cudaEvent_t pre_ev[kPreStreams + 1] = {};
  // instantiated Jacobi sweep graphs, reused while the order and the work
  // buffers (workspace addresses) repeat; kind 0 = FP64 sweep, 1 = FP32 block sweep
  struct SweepGraph {
    int kind = -1;
    int n = 0;
    const void* ptr[5] = {};
    cudaGraphExec_t exec = nullptr;
  };
  static constexpr int kSweepGraphs = 4;
  SweepGraph sweep_graph[kSweepGraphs];
  int sweep_graph_next = 0;
  size_t pinned_cap = 0;
  // pinned chunk buffers of the file readers (io.cu), created on first use
  void* io_pinned[2] = {nullptr, nullptr};
  cudaEvent_t io_ev[2] = {nullptr, nullptr};
};

namespace corr {
const void* stage_in(corr_context* c, const void* p, size_t bytes, void* slot);
int stage_out(corr_context* c, void* dst, const void* src, size_t bytes);
int finish_results(corr_context* c, int nres);
// Record timing event k (0 start, 1 before the main kernel, 2 after it, 3 end).
void mark(corr_context* c, int k);
// Enqueue an RI-MP2 energy; results go to `res` (device, 4 doubles; NULL =
// the context's result block).
int rimp2_energy_device(corr_context* c, int nocc, int nvir, int naux, const double* bia,
                        const double* eps, int precision, double* res = nullptr);
// Scratch bytes of the energy stage, and the stage itself on device-resident
// inputs, carving from `w` (already backed by reserved workspace).
size_t energy_scratch_bytes(corr_context* c, int nocc, int nvir, int naux, int precision);
// host_b (optional): B still in host memory; the precision forms upload it
// into d_b in row chunks on the context's copy stream, each chunk's row
// statistics starting as soon as it has landed; the FP64 form copies it first.
int rimp2_energy_core(corr_context* c, Carver& w, int nocc, int nvir, int naux, const double* d_b,
                      const double* d_e, int precision, double* res,
                      const double* host_b = nullptr, int coarse = 0);
}  // namespace corr
