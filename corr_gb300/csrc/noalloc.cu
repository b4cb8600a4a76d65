// Allocation-free RI-MP2 energy.
//
// Some callers cannot call cudaMalloc: a host program that hands all device
// memory out through its own pool (a framework's caching allocator, a fixed
// arena sized at start-up), or a latency-critical loop in which an allocation
// and the device synchronisation it may imply are not allowed.  For them,
// corr_rimp2_energy_noalloc runs the same kernels as corr_rimp2_energy but
// keeps all of its scratch in kScratchBytes of device memory compiled into the
// library (g_scratch below).  Every GPU that loads the library holds that
// array until the process exits.
//
// Host code must not pass g_scratch to a kernel: in host code the name is a
// stand-in, not a device address.  The device address is looked up once per
// device with cudaGetSymbolAddress, with that device current, on the entry
// point's first call on the device (which also sets the energy kernel's
// shared-memory attribute there); make that first call before any stream
// capture on the device.  Every call is synchronous: it waits for its stream
// to finish the work before it returns the energies.  All calls share the one
// array, which keeps the previous call's contents: every value a call reads is
// written or cleared by the same call first.  Calls whose GPU work overlaps
// (different streams or threads on one device) race on the array and must be
// serialised by the caller.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "abi_internal.h"
#include "common.cuh"
#include "kernels.h"

namespace corr {

namespace {

constexpr size_t kScratchBytes = 32ull << 20;  // 32 MiB
constexpr int kMaxDevices = 64;
constexpr int kMaxGrid = 1024;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct DeviceScratch {
  void* ptr = nullptr;  // device address of g_scratch on this device
  int sms = 0;
};
std::mutex g_setup_mu;
DeviceScratch g_dev[kMaxDevices];

// Once per device, with the device current.
int setup_device(int device, DeviceScratch* out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceScratch& d = g_dev[device];
  if (!d.ptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error("corr_rimp2_energy_noalloc: cudaGetSymbolAddress failed: %s",
                cudaGetErrorString(e));
      cudaGetLastError();
      return CORR_ERR_CUDA;
    }
    int sms = 0;
    CORR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    CORR_CUDA(prepare_energy_tc());
    d.sms = sms;
    d.ptr = p;
  }
  *out = d;
  return CORR_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

struct Header {  // first 256 bytes of the scratch
  double e[8];
  int status;
};

}  // namespace

}  // namespace corr

using namespace corr;

extern "C" int corr_rimp2_energy_noalloc(int device, void* stream, int nocc, int nvir, int naux,
                                         const double* bia, const double* eps, int precision,
                                         corr_mp2_energy* out) {
  CORR_CHECK_ARG(out && bia && eps, "corr_rimp2_energy_noalloc: null pointer argument");
  CORR_CHECK_ARG(nocc >= 1 && nvir >= 1 && naux >= 1,
                 "corr_rimp2_energy_noalloc: sizes must be positive");
  CORR_CHECK_ARG(precision >= CORR_PREC_FP64 && precision <= CORR_PREC_SPLIT_BF16,
                 "corr_rimp2_energy_noalloc: unknown precision %d", precision);
  CORR_CHECK_ARG((long long)nocc * nvir <= (1ll << 31) && nocc <= 46000,
                 "corr_rimp2_energy_noalloc: nocc*nvir too large");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device visible");
    return CORR_ERR_NO_DEVICE;
  }
  CORR_CHECK_ARG(device >= 0 && device < ndev && device < kMaxDevices,
                 "corr_rimp2_energy_noalloc: device %d out of range", device);
  DeviceGuard guard(device);
  CORR_CHECK_ARG(is_device_ptr(bia) && is_device_ptr(eps),
                 "corr_rimp2_energy_noalloc: bia and eps must be device pointers");
  DeviceScratch ds;
  CORR_TRY(setup_device(device, &ds));
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  const bool tc = precision != CORR_PREC_FP64;
  const int Qp = padded_naux(naux);
  const long long R = (long long)nocc * nvir;
  const EnergyShape sh = make_energy_shape(nocc, nvir, naux, tc ? kTcTile : kF64Tile);
  int grid = tc ? ds.sms : 2 * ds.sms;
  if (grid > kMaxGrid) grid = kMaxGrid;
  if ((long long)grid > sh.nunits) grid = (int)sh.nunits;

  // carve the static scratch (same order for the size check and the real pass)
  auto carve = [&](Carver& w, Header** hdr, double** partials, unsigned long long** queue,
                   double** red_scratch, SliceWork* sw) {
    *hdr = static_cast<Header*>(w.take(256));
    // the FP64 form writes one partial per CTA, the precision forms one per unit
    *partials = static_cast<double*>(w.take((size_t)(tc ? sh.nunits : kMaxGrid) * 16));
    *queue = static_cast<unsigned long long*>(w.take(16));
    *red_scratch = static_cast<double*>(w.take((size_t)kReduceBlocks * 16));
    if (tc) {
      sw->erow = static_cast<int*>(w.take((size_t)R * 4));
      sw->diag = static_cast<double*>(w.take((size_t)R * 8));
      sw->sc = static_cast<float*>(w.take((size_t)R * 4));
      sw->dg = static_cast<float2*>(w.take((size_t)R * 8));
      sw->eref = static_cast<int*>(w.take(16));
      sw->scale = static_cast<double*>(w.take(16));
      sw->S = static_cast<uint16_t*>(w.take(slice_bytes(nocc, nvir, Qp)));
    }
  };
  Header* hdr;
  double* partials;
  unsigned long long* queue;
  double* red_scratch;
  SliceWork sw{};
  Carver size_pass{nullptr, 0};
  carve(size_pass, &hdr, &partials, &queue, &red_scratch, &sw);
  if (size_pass.used > kScratchBytes) {
    set_error(
        "corr_rimp2_energy_noalloc: nocc=%d nvir=%d naux=%d needs %zu bytes of scratch; the "
        "allocation-free entry point has %zu (precision forms: about 6*nocc*nvir*naux bytes); "
        "use corr_rimp2_energy for larger problems",
        nocc, nvir, naux, size_pass.used, kScratchBytes);
    return CORR_ERR_BAD_ARG;
  }
  Carver w{ds.ptr, 0};
  carve(w, &hdr, &partials, &queue, &red_scratch, &sw);

  CORR_CUDA(cudaMemsetAsync(hdr, 0, sizeof(Header), s));  // status and results start at zero
  if (!tc) {
    CORR_CUDA(launch_energy_fp64(bia, eps, sh, partials, grid, s));
    CORR_CUDA(launch_energy_reduce(partials, grid, nullptr, hdr->e, s));
  } else {
    const int scheme = scheme_for_precision(precision);
    const int fmt = format_for_scheme(scheme);
    const int p = slice_bits_for(Qp);
    CORR_CUDA(launch_slices(bia, naux, nocc, nvir, Qp, scheme, fmt, p, sw, s));
    const TcInst inst = make_tc_inst(sw, eps, sh, Qp, 0);
    CORR_CUDA(launch_energy_tc(inst, fmt, scheme, 3, grid, partials, &hdr->status, queue, s));
    if (launch_unit_reduce(partials, (int)sh.nunits, sw.scale, hdr->e, red_scratch,
                           reinterpret_cast<unsigned*>(queue + 1), s) < 0) {
      set_error("corr_rimp2_energy_noalloc: energy reduction launch failed");
      return CORR_ERR_CUDA;
    }
  }
  Header h;
  CORR_CUDA(cudaMemcpyAsync(&h, hdr, sizeof(Header), cudaMemcpyDeviceToHost, s));
  CORR_CUDA(cudaStreamSynchronize(s));
  if (h.status & CORR_ERR_DEVICE_TIMEOUT) {
    set_error("a device-side wait exceeded its time limit");
    return CORR_ERR_DEVICE_TIMEOUT;
  }
  for (int k = 0; k < 4; ++k)
    if (!std::isfinite(h.e[k])) {
      set_error("non-finite energy (zero denominator or non-finite input)");
      return CORR_ERR_NUMERIC;
    }
  out->e_ss = h.e[0];
  out->e_os = h.e[1];
  out->e_total = h.e[2];
  out->e_scs = h.e[3];
  return CORR_OK;
}
