// C-ABI layer: context, status/error reporting, host/device argument staging,
// TMA descriptor encoding and dispatch of the RI-MP2 energy kernels.
#include <algorithm>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "abi_internal.h"
#include "common.cuh"
#include "kernels.h"

namespace corr {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

EnergyShape make_energy_shape(int nocc, int nvir, int naux, int tile) {
  EnergyShape s;
  s.nocc = nocc;
  s.nvir = nvir;
  s.naux = naux;
  s.tile = tile;
  s.ntiles = (nvir + tile - 1) / tile;
  s.npairs = nocc * (nocc + 1) / 2;
  s.ntpairs = s.ntiles * (s.ntiles + 1) / 2;
  s.nunits = (long long)s.npairs * s.ntpairs;
  return s;
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// ---------------------------------------------------------------------------
// workspace: one grow-only device buffer per context, carved per call
// ---------------------------------------------------------------------------
int Workspace::reserve(size_t bytes) {
  if (bytes <= cap) return CORR_OK;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  size_t want = bytes + bytes / 8;
  if (cudaMalloc(&ptr, want) != cudaSuccess) {
    cudaGetLastError();
    set_error("device allocation of %zu bytes failed", want);
    return CORR_ERR_OOM;
  }
  cap = want;
  return CORR_OK;
}

void* Carver::take(size_t bytes) {
  size_t at = (used + 255) & ~(size_t)255;
  used = at + bytes;
  return base ? static_cast<char*>(base) + at : nullptr;
}

// Stage a caller array on the device: device pointers pass through, host
// pointers are copied into `slot` on the context stream.
const void* stage_in(corr_context* c, const void* p, size_t bytes, void* slot) {
  if (is_device_ptr(p)) return p;
  if (cudaMemcpyAsync(slot, p, bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
    return nullptr;
  return slot;
}

int stage_out(corr_context* c, void* dst, const void* src, size_t bytes) {
  if (dst == src) return CORR_OK;
  CORR_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream));
  return CORR_OK;
}

PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    cudaGetLastError();
  });
  return fn;
}

int encode_tmap(CUtensorMap* m, CUtensorMapDataType dt, int rank, void* base,
                const uint64_t* dims, const uint64_t* strides_bytes, const uint32_t* box,
                CUtensorMapSwizzle swz) {
  auto enc = tmap_encoder();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled unavailable");
    return CORR_ERR_CUDA;
  }
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUresult r = enc(m, dt, (cuuint32_t)rank, base, (const cuuint64_t*)dims,
                   (const cuuint64_t*)strides_bytes, (const cuuint32_t*)box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return CORR_ERR_CUDA;
  }
  return CORR_OK;
}

// Finish a call: copy the small result block back, synchronise, check the
// device status word and the finiteness of the results.
void mark(corr_context* c, int k) {
  if (!c->timing) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(c->stream, &cs);
  if (cs == cudaStreamCaptureStatusNone) cudaEventRecord(c->ev[k], c->stream);
}

int finish_results(corr_context* c, int nres) {
  mark(c, 3);
  CORR_CUDA(cudaMemcpyAsync(c->hres, c->dres, sizeof(ResultBlock), cudaMemcpyDeviceToHost,
                            c->stream));
  CORR_CUDA(cudaStreamSynchronize(c->stream));
  if (c->timing) {
    cudaEventElapsedTime(&c->t_prepass, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&c->t_kernel, c->ev[1], c->ev[2]);
    cudaEventElapsedTime(&c->t_total, c->ev[0], c->ev[3]);
    cudaGetLastError();
  }
  if (c->hres->status & CORR_ERR_DEVICE_TIMEOUT) {
    set_error("a device-side wait exceeded its time limit");
    return CORR_ERR_DEVICE_TIMEOUT;
  }
  for (int k = 0; k < nres; ++k)
    if (!std::isfinite(c->hres->e[k])) {
      set_error("non-finite energy (zero denominator or non-finite input)");
      return CORR_ERR_NUMERIC;
    }
  return CORR_OK;
}

}  // namespace corr

using namespace corr;

extern "C" {

const char* corr_version(void) { return "corr_gb300 0.1.0 (sm_103a)"; }

const char* corr_last_error(void) { return g_err; }

int corr_create(corr_context** out, int device, void* stream) {
  CORR_CHECK_ARG(out != nullptr, "corr_create: null output pointer");
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("no CUDA device visible");
    return CORR_ERR_NO_DEVICE;
  }
  CORR_CHECK_ARG(device >= 0 && device < n, "corr_create: device %d out of range", device);
  cudaDeviceProp prop;
  CORR_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3) {
    set_error("device %d is sm_%d%d; this library is built for sm_103a", device, prop.major,
              prop.minor);
    return CORR_ERR_NO_DEVICE;
  }
  CORR_CUDA(cudaSetDevice(device));
  corr_context* c = new corr_context();
  c->device = device;
  c->stream = static_cast<cudaStream_t>(stream);
  c->sms = prop.multiProcessorCount;
  if (cudaMalloc(&c->dres, sizeof(ResultBlock)) != cudaSuccess ||
      cudaMallocHost(&c->hres, sizeof(ResultBlock)) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    set_error("corr_create: allocation failed");
    return CORR_ERR_OOM;
  }
  *out = c;
  return CORR_OK;
}

int corr_destroy(corr_context* c) {
  if (!c) return CORR_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);  // uploads into the workspace
  for (int k = 0; k < corr_context::kPreStreams; ++k)
    if (c->pre_stream[k]) cudaStreamSynchronize(c->pre_stream[k]);
  if (c->ws.ptr) cudaFree(c->ws.ptr);
  if (c->batch_out.ptr) cudaFree(c->batch_out.ptr);
  if (c->pinned) cudaFreeHost(c->pinned);
  for (int k = 0; k < 2; ++k) {
    if (c->io_pinned[k]) cudaFreeHost(c->io_pinned[k]);
    if (c->io_ev[k]) cudaEventDestroy(c->io_ev[k]);
  }
  if (c->dres) cudaFree(c->dres);
  if (c->hres) cudaFreeHost(c->hres);
  for (int k = 0; k < 4; ++k)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  for (int k = 0; k < 5; ++k)
    if (c->cev[k]) cudaEventDestroy(c->cev[k]);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  for (int k = 0; k < corr_context::kPreStreams; ++k)
    if (c->pre_stream[k]) cudaStreamDestroy(c->pre_stream[k]);
  for (int k = 0; k <= corr_context::kPreStreams; ++k)
    if (c->pre_ev[k]) cudaEventDestroy(c->pre_ev[k]);
  for (auto& g : c->sweep_graph)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  delete c;
  return CORR_OK;
}

int corr_set_stream(corr_context* c, void* stream) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  c->stream = static_cast<cudaStream_t>(stream);
  return CORR_OK;
}

int corr_device_sm_count(const corr_context* c) { return c ? c->sms : 0; }

int corr_rimp2_energy_async(corr_context* c, int nocc, int nvir, int naux, const double* bia,
                            const double* eps, int precision, double* energies_dev) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(bia && eps && energies_dev, "corr_rimp2_energy_async: null pointer argument");
  CORR_CHECK_ARG(nocc >= 1 && nvir >= 1 && naux >= 1, "corr_rimp2_energy_async: bad sizes");
  CORR_CHECK_ARG(precision >= CORR_PREC_FP64 && precision <= CORR_PREC_SPLIT_BF16,
                 "corr_rimp2_energy_async: unknown precision %d", precision);
  CORR_CHECK_ARG(is_device_ptr(bia) && is_device_ptr(eps) && is_device_ptr(energies_dev),
                 "corr_rimp2_energy_async: bia, eps and energies_dev must be device pointers");
  CORR_CUDA(cudaSetDevice(c->device));
  return rimp2_energy_device(c, nocc, nvir, naux, bia, eps, precision, energies_dev);
}

int corr_sync(corr_context* c) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CUDA(cudaSetDevice(c->device));
  int st = 0;
  CORR_CUDA(cudaMemcpyAsync(&c->hres->status, &c->dres->status, sizeof(int),
                            cudaMemcpyDeviceToHost, c->stream));
  CORR_CUDA(cudaStreamSynchronize(c->stream));
  st = c->hres->status;
  CORR_CUDA(cudaMemsetAsync(&c->dres->status, 0, sizeof(int), c->stream));
  if (st & CORR_ERR_DEVICE_TIMEOUT) {
    set_error("a device-side wait exceeded its time limit");
    return CORR_ERR_DEVICE_TIMEOUT;
  }
  return CORR_OK;
}

int corr_set_fp64_strict(corr_context* c, int strict) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(strict == 0 || strict == 1, "corr_set_fp64_strict: strict must be 0 or 1");
  c->fp64_strict = strict;
  return CORR_OK;
}

// Kept for callers of the earlier tile policy: both values now run every tile
// 128 wide (energy_tc.cu says why).
int corr_set_energy_tiles(corr_context* c, int tiles) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(tiles == 0 || tiles == 1,
                 "corr_set_energy_tiles: tiles must be 0 (128 wide) or 1 (narrow last tile)");
  return CORR_OK;
}

int corr_set_timing(corr_context* c, int enable) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  if (enable && !c->ev[0])
    for (int k = 0; k < 4; ++k) CORR_CUDA(cudaEventCreate(&c->ev[k]));
  c->timing = enable != 0;
  return CORR_OK;
}

int corr_get_timing(const corr_context* c, corr_timing* out) {
  CORR_CHECK_ARG(c != nullptr && out != nullptr, "null argument");
  out->prepass_ms = c->t_prepass;
  out->kernel_ms = c->t_kernel;
  out->total_ms = c->t_total;
  out->launches_total = c->launches;
  return CORR_OK;
}

int corr_rimp2_energy_estimate(corr_context* c, int nocc, int nvir, int naux, const double* bia,
                               const double* eps, int precision, corr_mp2_energy* out,
                               double* err) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(out != nullptr && err != nullptr && bia != nullptr && eps != nullptr,
                 "corr_rimp2_energy_estimate: null pointer argument");
  CORR_CHECK_ARG(nocc >= 1 && nvir >= 1 && naux >= 1,
                 "corr_rimp2_energy_estimate: sizes must be positive");
  CORR_CHECK_ARG(precision >= CORR_PREC_FP64 && precision <= CORR_PREC_SPLIT_BF16,
                 "corr_rimp2_energy_estimate: unknown precision %d", precision);
  CORR_CHECK_ARG((long long)nocc * nvir <= (1ll << 31) && nocc <= 46000,
                 "corr_rimp2_energy_estimate: nocc*nvir too large");
  CORR_CUDA(cudaSetDevice(c->device));
  if (precision == CORR_PREC_FP64) {  // the reference's own arithmetic: no estimate
    CORR_TRY(corr_rimp2_energy(c, nocc, nvir, naux, bia, eps, precision, out));
    *err = 0.0;
    return CORR_OK;
  }
  const size_t nb = (size_t)naux * nocc * nvir, ne = (size_t)nocc + nvir;
  const bool b_dev = is_device_ptr(bia), e_dev = is_device_ptr(eps);
  Carver cv{nullptr, 0};
  if (!b_dev) cv.take(nb * 8);
  if (!e_dev) cv.take(ne * 8);
  const size_t head = cv.used;
  CORR_TRY(c->ws.reserve(head + energy_scratch_bytes(c, nocc, nvir, naux, precision)));
  Carver w{c->ws.ptr, 0};
  void* b_slot = b_dev ? nullptr : w.take(nb * 8);
  void* e_slot = e_dev ? nullptr : w.take(ne * 8);
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  const double* d_b = b_dev ? bia : static_cast<const double*>(b_slot);
  const double* d_e = static_cast<const double*>(stage_in(c, eps, ne * 8, e_slot));
  if (!d_e) {
    set_error("host-to-device copy failed: %s", cudaGetErrorString(cudaGetLastError()));
    return CORR_ERR_CUDA;
  }
  // the energy, then the same evaluation one bit coarser per digit (B already
  // on the device; the scratch carved again from the same offset)
  Carver w2 = w;
  CORR_TRY(rimp2_energy_core(c, w, nocc, nvir, naux, d_b, d_e, precision, c->dres->e,
                             b_dev ? nullptr : bia, 0));
  CORR_TRY(rimp2_energy_core(c, w2, nocc, nvir, naux, d_b, d_e, precision, c->dres->e + 4,
                             nullptr, 1));
  CORR_TRY(finish_results(c, 8));
  out->e_ss = c->hres->e[0];
  out->e_os = c->hres->e[1];
  out->e_total = c->hres->e[2];
  out->e_scs = c->hres->e[3];
  // two digits: the difference of the two grids' representations has 6 times
  // the variance of the fine grid's rounding error; three digits, one bit
  // coarser each: 8 times the error, nearly independent (1 + 64)
  const double ratio = precision == CORR_PREC_SPLIT_FP16 ? 6.0 : 65.0;
  *err = fabs(c->hres->e[6] - c->hres->e[2]) / sqrt(ratio);
  return CORR_OK;
}

int corr_rimp2_energy(corr_context* c, int nocc, int nvir, int naux, const double* bia,
                      const double* eps, int precision, corr_mp2_energy* out) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(out != nullptr && bia != nullptr && eps != nullptr,
                 "corr_rimp2_energy: null pointer argument");
  CORR_CHECK_ARG(nocc >= 1 && nvir >= 1 && naux >= 1,
                 "corr_rimp2_energy: sizes must be positive (nocc=%d nvir=%d naux=%d)", nocc, nvir,
                 naux);
  CORR_CHECK_ARG(precision >= CORR_PREC_FP64 && precision <= CORR_PREC_SPLIT_BF16,
                 "corr_rimp2_energy: unknown precision %d", precision);
  CORR_CHECK_ARG((long long)nocc * nvir <= (1ll << 31) && nocc <= 46000,
                 "corr_rimp2_energy: nocc*nvir too large");
  CORR_CUDA(cudaSetDevice(c->device));
  int st = rimp2_energy_device(c, nocc, nvir, naux, bia, eps, precision);
  if (st != CORR_OK) return st;
  CORR_TRY(finish_results(c, 4));
  out->e_ss = c->hres->e[0];
  out->e_os = c->hres->e[1];
  out->e_total = c->hres->e[2];
  out->e_scs = c->hres->e[3];
  return CORR_OK;
}

}  // extern "C"

namespace corr {

// Scratch of the energy stage for device-resident B and eps.
static void energy_carve(Carver& w, int nocc, int nvir, int Qp, bool tc, bool x20, int grid,
                         SliceWork* sw, double** partials, unsigned long long** queue = nullptr,
                         double** red_scratch = nullptr) {
  const long long R = (long long)nocc * nvir;
  if (tc && x20) sw->x20 = static_cast<int*>(w.take((size_t)Qp * R * 4));
  if (tc) {
    sw->S = static_cast<uint16_t*>(w.take(slice_bytes(nocc, nvir, Qp)));
    sw->erow = static_cast<int*>(w.take((size_t)R * 4));
    sw->diag = static_cast<double*>(w.take((size_t)R * 8));
    sw->sc = static_cast<float*>(w.take((size_t)R * 4));
    sw->dg = static_cast<float2*>(w.take((size_t)R * 8));
    sw->eref = static_cast<int*>(w.take(16));
    sw->scale = static_cast<double*>(w.take(16));
  }
  *partials = static_cast<double*>(w.take((size_t)grid * 16));
  unsigned long long* qp = static_cast<unsigned long long*>(w.take(16));  // work-queue counter
  if (queue) *queue = qp;
  double* rs = static_cast<double*>(w.take((size_t)kReduceBlocks * 16));  // reduction stage 1
  if (red_scratch) *red_scratch = rs;
}

// split_fp16 hands the row statistics' fixed-point values to the slice (one
// extra 4-byte array of naux x nocc x nvir) when the statistics run in shared memory.
static bool stage_x20(int precision, int naux) {
  return precision == CORR_PREC_SPLIT_FP16 && row_stats_stage_x20(naux);
}

static int energy_grid(corr_context* c, const EnergyShape& sh, bool tc) {
  int grid = tc ? c->sms : c->sms * 2;
  if ((long long)grid > sh.nunits) grid = (int)sh.nunits;
  return grid;
}

size_t energy_scratch_bytes(corr_context* c, int nocc, int nvir, int naux, int precision) {
  const bool tc = precision != CORR_PREC_FP64;
  const int Qp = padded_naux(naux);
  const EnergyShape sh = make_energy_shape(nocc, nvir, naux, tc ? kTcTile : kF64Tile);
  SliceWork sw{};
  double* part;
  Carver cv{nullptr, 0};
  energy_carve(cv, nocc, nvir, Qp, tc, stage_x20(precision, naux),
               (int)std::max<long long>(2 * c->sms, sh.nunits), &sw,
               &part);  // partials of any grid or one per unit
  return cv.used + 256;
}

// Enqueue the energy of device-resident B/eps, carving scratch from `w`
// (which must already be backed by reserved workspace); results to `res`
// (device, 4 doubles; NULL = the context's result block).
// Upload B [naux][R] from host memory into d_b in row chunks on the copy
// stream and run each chunk's row statistics on the context stream once it has
// landed: the statistics pass runs under the transfer instead of after it.
static int upload_with_row_stats(corr_context* c, const double* host_b, double* d_b, int naux,
                                 int nocc, int nvir, int scheme, int p, SliceWork sw) {
  constexpr int kChunks = 4;
  if (!c->copy_stream) {
    CORR_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < kChunks + 1; ++k)
      CORR_CUDA(cudaEventCreateWithFlags(&c->cev[k], cudaEventDisableTiming));
  }
  const long long R = (long long)nocc * nvir;
  const long long per = ((R + kChunks - 1) / kChunks + 31) / 32 * 32;  // rows, multiple of 32
  CORR_CUDA(reset_row_stats(sw, c->stream));
  // the slot may still be read by earlier work on the context stream
  CORR_CUDA(cudaEventRecord(c->cev[kChunks], c->stream));
  CORR_CUDA(cudaStreamWaitEvent(c->copy_stream, c->cev[kChunks], 0));
  for (int k = 0; k < kChunks; ++k) {
    const long long lo = k * per, hi = std::min(R, lo + per);
    if (lo >= hi) break;
    CORR_CUDA(cudaMemcpy2DAsync(d_b + lo, (size_t)R * 8, host_b + lo, (size_t)R * 8,
                                (size_t)(hi - lo) * 8, (size_t)naux, cudaMemcpyHostToDevice,
                                c->copy_stream));
    CORR_CUDA(cudaEventRecord(c->cev[k], c->copy_stream));
    CORR_CUDA(cudaStreamWaitEvent(c->stream, c->cev[k], 0));
    CORR_CUDA(launch_row_stats(d_b, naux, nocc, nvir, scheme, p, sw, lo, hi, c->stream));
    c->launches += 1;
  }
  return CORR_OK;
}

int rimp2_energy_core(corr_context* c, Carver& w, int nocc, int nvir, int naux, const double* d_b,
                      const double* d_e, int precision, double* res, const double* host_b,
                      int coarse) {
  double* out_e = res ? res : c->dres->e;
  const bool tc = precision != CORR_PREC_FP64;
  const int Qp = padded_naux(naux);
  const EnergyShape sh = make_energy_shape(nocc, nvir, naux, tc ? kTcTile : kF64Tile);
  const int grid = energy_grid(c, sh, tc);
  SliceWork sw{};
  double* partials;
  unsigned long long* queue;
  double* red_scratch;
  energy_carve(w, nocc, nvir, Qp, tc, stage_x20(precision, naux),
               (int)std::max<long long>(2 * c->sms, sh.nunits), &sw, &partials, &queue,
               &red_scratch);
  if (!tc) {
    if (host_b)
      CORR_CUDA(cudaMemcpyAsync(const_cast<double*>(d_b), host_b,
                                (size_t)naux * nocc * nvir * 8, cudaMemcpyHostToDevice,
                                c->stream));
    mark(c, 1);
    CORR_CUDA(launch_energy_fp64(d_b, d_e, sh, partials, grid, c->stream));
    mark(c, 2);
    CORR_CUDA(launch_energy_reduce(partials, grid, nullptr, out_e, c->stream));
    c->launches += 2;
    return CORR_OK;
  }
  const int scheme = scheme_for_precision(precision);
  const int fmt = format_for_scheme(scheme);
  // coarse: the same evaluation on a grid one bit coarser per digit (the
  // error estimate of corr_rimp2_energy_estimate)
  const int p = std::max(1, slice_bits_for(Qp) - (scheme == kSchemeDigits3 ? coarse : 0));
  if (host_b) {
    CORR_TRY(upload_with_row_stats(c, host_b, const_cast<double*>(d_b), naux, nocc, nvir, scheme,
                                   p, sw));
  } else {
    CORR_CUDA(reset_row_stats(sw, c->stream));
    CORR_CUDA(launch_row_stats(d_b, naux, nocc, nvir, scheme, p, sw, 0, (long long)nocc * nvir,
                               c->stream));
    c->launches += 1;
  }
  if (coarse && scheme == kSchemeDigits2) {
    CORR_CUDA(coarsen_level(sw, c->stream));
    c->launches += 1;
  }
  CORR_CUDA(launch_slice_planes(d_b, naux, nocc, nvir, Qp, scheme, fmt, p, sw, c->stream));
  c->launches += 1;
  if (!c->attrs_set) {
    CORR_CUDA(prepare_energy_tc());
    c->attrs_set = true;
  }
  const TcInst inst = make_tc_inst(sw, d_e, sh, Qp, 0);
  mark(c, 1);
  CORR_CUDA(launch_energy_tc(inst, fmt, scheme, 3, grid, partials, &c->dres->status, queue,
                             c->stream));
  mark(c, 2);
  const int nred = launch_unit_reduce(partials, (int)sh.nunits, sw.scale, out_e, red_scratch,
                                      reinterpret_cast<unsigned*>(queue + 1), c->stream);
  if (nred < 0) {
    set_error("energy reduction launch failed");
    return CORR_ERR_CUDA;
  }
  c->launches += 1 + nred;  // energy, reduction
  return CORR_OK;
}

// Enqueue the whole energy evaluation on the context stream (host or device
// inputs); results land in `res` or the context's result block.
int rimp2_energy_device(corr_context* c, int nocc, int nvir, int naux, const double* bia,
                        const double* eps, int precision, double* res) {
  const size_t nb = (size_t)naux * nocc * nvir;
  const size_t ne = (size_t)nocc + nvir;
  const bool b_dev = is_device_ptr(bia), e_dev = is_device_ptr(eps);
  Carver cv{nullptr, 0};
  if (!b_dev) cv.take(nb * 8);
  if (!e_dev) cv.take(ne * 8);
  const size_t head = cv.used;
  CORR_TRY(c->ws.reserve(head + energy_scratch_bytes(c, nocc, nvir, naux, precision)));
  Carver w{c->ws.ptr, 0};
  void* b_slot = b_dev ? nullptr : w.take(nb * 8);
  void* e_slot = e_dev ? nullptr : w.take(ne * 8);
  if (!res) CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  // B: device arrays are used in place; host arrays go to b_slot inside the
  // energy stage (in row chunks for the precision forms)
  const double* d_b = b_dev ? bia : static_cast<const double*>(b_slot);
  const double* d_e = static_cast<const double*>(stage_in(c, eps, ne * 8, e_slot));
  if (!d_e) {
    set_error("host-to-device copy failed: %s", cudaGetErrorString(cudaGetLastError()));
    return CORR_ERR_CUDA;
  }
  return rimp2_energy_core(c, w, nocc, nvir, naux, d_b, d_e, precision, res,
                           b_dev ? nullptr : bia);
}

}  // namespace corr
