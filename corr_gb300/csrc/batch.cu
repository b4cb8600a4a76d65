// Host side of the batched RI-MP2 driver: instance table, per-instance slicing,
// unit-order policies, the synchronous/asynchronous entry points, the
// per-instance reduction and the autotuner that picks the launch variant
// (unit order x pipeline depth x tile shape) by timing them on the caller's
// batch.  The kernel itself is the precision-form energy kernel of
// energy_tc.cu in its table-driven form.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "abi_internal.h"
#include "common.cuh"
#include "kernels.h"

namespace corr {

namespace {

// Per instance k of the table: Kahan-compensated sum of its unit partials in
// unit order, a fixed tree over the 256 threads, times the instance's energy
// scale, into out[4 out_index[k] + {0,1,2,3}] = {E_SS, E_OS, E, E_SCS}.
__global__ void batch_reduce_kernel(const TcInst* __restrict__ insts,
                                    const double* __restrict__ unit_part,
                                    const int* __restrict__ out_index, double* __restrict__ out) {
  const TcInst b = insts[blockIdx.x];
  __shared__ double s_os[256], s_ss[256];
  double os = 0.0, ss = 0.0, cos_ = 0.0, css = 0.0;
  for (long long k = threadIdx.x; k < b.nunits; k += 256) {
    const long long u = b.unit_begin + k;
    double y = unit_part[2 * u] - cos_;
    double t = os + y;
    cos_ = (t - os) - y;
    os = t;
    y = unit_part[2 * u + 1] - css;
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
    const double sc = b.scale ? b.scale[0] : 1.0;
    const double eos = s_os[0] * sc, ess = s_ss[0] * sc;
    double* o = out + 4 * (size_t)out_index[blockIdx.x];
    o[0] = ess;
    o[1] = eos;
    o[2] = ess + eos;
    o[3] = ess / 3.0 + eos * 6.0 / 5.0;
  }
}

double instance_cost(const corr_rimp2_instance& x) {
  return 2.0 * x.nocc * (double)x.nocc * x.nvir * (double)x.nvir * x.naux;
}

int grow_pinned(corr_context* c, size_t bytes) {
  if (bytes <= c->pinned_cap) return CORR_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(c->stream, &cs);
  if (cs != cudaStreamCaptureStatusNone) {
    set_error("batched call inside stream capture needs a first call outside capture");
    return CORR_ERR_BAD_ARG;
  }
  if (c->pinned) cudaFreeHost(c->pinned);
  c->pinned = nullptr;
  c->pinned_cap = 0;
  if (cudaMallocHost(&c->pinned, bytes * 2) != cudaSuccess) {
    cudaGetLastError();
    set_error("pinned host allocation failed");
    return CORR_ERR_OOM;
  }
  c->pinned_cap = bytes * 2;
  return CORR_OK;
}

// Enqueue one batched evaluation; energies (4 per caller instance) to `out`.
int batch_enqueue(corr_context* c, int n, const corr_rimp2_instance* in, int precision,
                  double* out, int order_policy, int stages) {
  const bool tc = precision != CORR_PREC_FP64;
  // ---- plan: order and per-instance shapes
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  if (order_policy == 1)
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      return instance_cost(in[a]) > instance_cost(in[b]);
    });
  struct Shape {
    int Qp, p;
    long long R;
    EnergyShape sh;
  };
  std::vector<Shape> shp(n);
  Carver cv{nullptr, 0};
  long long total = 0;
  for (int k = 0; k < n; ++k) {
    const corr_rimp2_instance& x = in[order[k]];
    Shape& s = shp[k];
    s.Qp = padded_naux(x.naux);
    s.p = slice_bits_for(s.Qp);
    s.R = (long long)x.nocc * x.nvir;
    s.sh = make_energy_shape(x.nocc, x.nvir, x.naux, tc ? kTcTile : kF64Tile);
    total += s.sh.nunits;
  }
  // ---- workspace
  auto carve = [&](Carver& w, std::vector<SliceWork>& sws, double** unit_part, TcInst** dtab,
                   int** dorder, unsigned long long** queue) {
    sws.resize(n);
    for (int k = 0; k < n; ++k) {
      if (!tc) continue;
      const Shape& s = shp[k];
      SliceWork& sw = sws[k];
      sw.S = static_cast<uint16_t*>(w.take(slice_bytes(in[order[k]].nocc, in[order[k]].nvir, s.Qp)));
      sw.erow = static_cast<int*>(w.take((size_t)s.R * 4));
      sw.diag = static_cast<double*>(w.take((size_t)s.R * 8));
      sw.sc = static_cast<float*>(w.take((size_t)s.R * 4));
      sw.dg = static_cast<float2*>(w.take((size_t)s.R * 8));
      sw.eref = static_cast<int*>(w.take(16));
      sw.scale = static_cast<double*>(w.take(16));
    }
    *unit_part = static_cast<double*>(w.take((size_t)(tc ? total : (long long)c->sms * 2 * n) * 16));
    *dtab = static_cast<TcInst*>(w.take(sizeof(TcInst) * n));
    *dorder = static_cast<int*>(w.take(sizeof(int) * n));
    *queue = static_cast<unsigned long long*>(w.take(16));
  };
  std::vector<SliceWork> sws;
  double* unit_part;
  TcInst* dtab;
  int* dorder;
  unsigned long long* queue;
  carve(cv, sws, &unit_part, &dtab, &dorder, &queue);
  if (c->ws.cap < cv.used || (tc && !c->pre_stream[0])) {  // workspace or side streams to create
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(c->stream, &cs);
    if (cs != cudaStreamCaptureStatusNone) {
      set_error("batched call inside stream capture needs a first call outside capture");
      return CORR_ERR_BAD_ARG;
    }
  }
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  carve(w, sws, &unit_part, &dtab, &dorder, &queue);

  if (!tc) {
    // FP64 comparison form: one fused kernel per instance
    const int grid = c->sms * 2;
    for (int k = 0; k < n; ++k) {
      const corr_rimp2_instance& x = in[order[k]];
      EnergyShape sh = shp[k].sh;
      int g = grid;
      if ((long long)g > sh.nunits) g = (int)sh.nunits;
      double* part = unit_part + (size_t)k * grid * 2;
      CORR_CUDA(launch_energy_fp64(x.bia, x.eps, sh, part, g, c->stream));
      CORR_CUDA(launch_energy_reduce(part, g, nullptr, out + 4 * (size_t)order[k], c->stream));
    }
    c->launches += 2LL * n;
    return CORR_OK;
  }

  // ---- per-instance slicing and the host copy of the table
  const int scheme = scheme_for_precision(precision);
  const int fmt = format_for_scheme(scheme);
  const size_t hbytes = sizeof(TcInst) * n + sizeof(int) * n + 256;
  CORR_TRY(grow_pinned(c, hbytes));
  char* hp = static_cast<char*>(c->pinned);
  TcInst* htab = reinterpret_cast<TcInst*>(hp);
  int* horder = reinterpret_cast<int*>(hp + ((sizeof(TcInst) * n + 127) & ~(size_t)127));
  // The instances' pre-passes are independent and mostly small (a few blocks
  // each): they run on kPreStreams side streams forked from and joined back
  // into the context stream (parallel branches when the call is captured).
  constexpr int K = corr_context::kPreStreams;
  if (!c->pre_stream[0]) {
    for (int k = 0; k < K; ++k)
      CORR_CUDA(cudaStreamCreateWithFlags(&c->pre_stream[k], cudaStreamNonBlocking));
    for (int k = 0; k <= K; ++k)
      CORR_CUDA(cudaEventCreateWithFlags(&c->pre_ev[k], cudaEventDisableTiming));
  }
  const int nside = n < K ? n : K;
  CORR_CUDA(cudaEventRecord(c->pre_ev[K], c->stream));
  for (int k = 0; k < nside; ++k) CORR_CUDA(cudaStreamWaitEvent(c->pre_stream[k], c->pre_ev[K], 0));
  long long ub = 0;
  for (int k = 0; k < n; ++k) {
    const corr_rimp2_instance& x = in[order[k]];
    const Shape& s = shp[k];
    CORR_CUDA(launch_slices(x.bia, x.naux, x.nocc, x.nvir, s.Qp, scheme, fmt, s.p, sws[k],
                            c->pre_stream[k % nside]));
    htab[k] = make_tc_inst(sws[k], x.eps, s.sh, s.Qp, ub);
    horder[k] = order[k];
    ub += s.sh.nunits;
  }
  c->launches += 2LL * n;  // row statistics and slice per instance
  for (int k = 0; k < nside; ++k) {
    CORR_CUDA(cudaEventRecord(c->pre_ev[k], c->pre_stream[k]));
    CORR_CUDA(cudaStreamWaitEvent(c->stream, c->pre_ev[k], 0));
  }
  CORR_CUDA(cudaMemcpyAsync(dtab, htab, sizeof(TcInst) * n, cudaMemcpyHostToDevice, c->stream));
  CORR_CUDA(cudaMemcpyAsync(dorder, horder, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
  if (!c->attrs_set) {
    CORR_CUDA(prepare_energy_tc());
    c->attrs_set = true;
  }
  int grid = c->sms;
  if ((long long)grid > total) grid = (int)total;
  mark(c, 1);
  CORR_CUDA(launch_energy_tc_batch(dtab, n, total, fmt, scheme, stages, grid, unit_part,
                                   &c->dres->status, queue, c->stream));
  mark(c, 2);
  CORR_CUDA(launch_batch_reduce(dtab, n, unit_part, dorder, out, c->stream));
  c->launches += 2;
  return CORR_OK;
}

int check_batch(corr_context* c, int n, const corr_rimp2_instance* in, int precision) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(n >= 1 && in != nullptr, "batched RI-MP2: need n >= 1 instances");
  CORR_CHECK_ARG(precision >= CORR_PREC_FP64 && precision <= CORR_PREC_SPLIT_BF16,
                 "batched RI-MP2: unknown precision %d", precision);
  for (int k = 0; k < n; ++k) {
    const corr_rimp2_instance& x = in[k];
    CORR_CHECK_ARG(x.nocc >= 1 && x.nvir >= 1 && x.naux >= 1, "instance %d: bad sizes", k);
    CORR_CHECK_ARG(is_device_ptr(x.bia) && is_device_ptr(x.eps),
                   "instance %d: bia and eps must be device pointers", k);
  }
  return CORR_OK;
}

}  // namespace

cudaError_t launch_batch_reduce(const TcInst* dtab, int n, const double* partials,
                                const int* out_index, double* out, cudaStream_t s) {
  batch_reduce_kernel<<<n, 256, 0, s>>>(dtab, partials, out_index, out);
  return cudaGetLastError();
}

}  // namespace corr

using namespace corr;

extern "C" {

int corr_set_batch_policy(corr_context* c, int order, int stages, int tiles) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(order == 0 || order == 1, "order policy must be 0 (input) or 1 (cost-descending)");
  CORR_CHECK_ARG(stages == 2 || stages == 3, "stages must be 2 or 3");
  CORR_CHECK_ARG(tiles == 0 || tiles == 1, "tiles must be 0 (128 wide) or 1 (narrow last tile)");
  c->batch_order = order;
  c->batch_stages = stages;
  c->batch_tiles = tiles;
  return CORR_OK;
}

int corr_rimp2_energy_batched_async(corr_context* c, int n, const corr_rimp2_instance* inst,
                                    int precision, double* energies_dev) {
  CORR_TRY(check_batch(c, n, inst, precision));
  CORR_CHECK_ARG(is_device_ptr(energies_dev), "energies_dev must be a device pointer");
  CORR_CUDA(cudaSetDevice(c->device));
  return batch_enqueue(c, n, inst, precision, energies_dev, c->batch_order, c->batch_stages);
}

int corr_rimp2_energy_batched(corr_context* c, int n, const corr_rimp2_instance* inst,
                              int precision, corr_mp2_energy* out) {
  CORR_TRY(check_batch(c, n, inst, precision));
  CORR_CHECK_ARG(out != nullptr, "null output");
  CORR_CUDA(cudaSetDevice(c->device));
  CORR_TRY(c->batch_out.reserve((size_t)n * 32));
  double* dout = static_cast<double*>(c->batch_out.ptr);
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  CORR_TRY(batch_enqueue(c, n, inst, precision, dout, c->batch_order, c->batch_stages));
  std::vector<double> h((size_t)n * 4);
  CORR_CUDA(cudaMemcpyAsync(h.data(), dout, (size_t)n * 32, cudaMemcpyDeviceToHost, c->stream));
  CORR_TRY(finish_results(c, 0));
  for (int k = 0; k < n; ++k) {
    out[k].e_ss = h[4 * k];
    out[k].e_os = h[4 * k + 1];
    out[k].e_total = h[4 * k + 2];
    out[k].e_scs = h[4 * k + 3];
    if (!std::isfinite(out[k].e_total)) {
      set_error("instance %d: non-finite energy", k);
      return CORR_ERR_NUMERIC;
    }
  }
  return CORR_OK;
}

int corr_rimp2_batch_autotune(corr_context* c, int n, const corr_rimp2_instance* inst,
                              int precision, int* order_out, int* stages_out, int* tiles_out,
                              float* ms_out) {
  CORR_TRY(check_batch(c, n, inst, precision));
  CORR_CUDA(cudaSetDevice(c->device));
  CORR_TRY(c->batch_out.reserve((size_t)n * 32));
  double* dout = static_cast<double*>(c->batch_out.ptr);
  cudaEvent_t e0, e1;
  CORR_CUDA(cudaEventCreate(&e0));
  CORR_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bo = c->batch_order, bs = c->batch_stages;
  const int bt = c->batch_tiles;  // no effect on the launch: reported back as set
  // the three-digit form always runs 2 stages: one stage value to try
  const int orders[2] = {0, 1}, stages[2] = {3, 2};
  const int nst = precision == CORR_PREC_SPLIT_FP16 ? 2 : 1;
  int st = CORR_OK;
  for (int oi = 0; oi < 2 && st == CORR_OK; ++oi)
    for (int si = 0; si < nst && st == CORR_OK; ++si) {
      const int so = orders[oi], ss = nst == 2 ? stages[si] : 2;
      // one untimed warm-up, then the median of three timed runs
      st = batch_enqueue(c, n, inst, precision, dout, so, ss);
      float t[3] = {0.f, 0.f, 0.f};
      for (int r = 0; r < 3 && st == CORR_OK; ++r) {
        if (cudaEventRecord(e0, c->stream) != cudaSuccess) st = CORR_ERR_CUDA;
        if (st == CORR_OK) st = batch_enqueue(c, n, inst, precision, dout, so, ss);
        if (st == CORR_OK && (cudaEventRecord(e1, c->stream) != cudaSuccess ||
                              cudaEventSynchronize(e1) != cudaSuccess ||
                              cudaEventElapsedTime(&t[r], e0, e1) != cudaSuccess))
          st = CORR_ERR_CUDA;
      }
      if (st != CORR_OK) break;
      std::sort(t, t + 3);
      if (t[1] < best) {
        best = t[1];
        bo = so;
        bs = ss;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == CORR_ERR_CUDA) {
    set_error("batched autotune: %s", cudaGetErrorString(cudaGetLastError()));
    return st;
  }
  if (st != CORR_OK) return st;
  CORR_TRY(corr_sync(c));  // a device-side timeout in any variant
  c->batch_order = bo;
  c->batch_stages = bs;
  if (order_out) *order_out = bo;
  if (stages_out) *stages_out = bs;
  if (tiles_out) *tiles_out = bt;
  if (ms_out) *ms_out = best;
  return CORR_OK;
}

}  // extern "C"
