// Readers of the reference's binary hand-off files (src/IO/ops_io.cc) that load
// straight into the GPU path, and the writer of the HF wavefunction file.
//
// File layouts (all native-endian, as the reference writes and reads them):
//   PREFIX.sys    int nroe, nroa, nroao, naux_1, naux_2; long long nrofint,
//                 nrofaux, nrofaux2; double coord[3 nroa], charges[nroa],
//                 zeff[nroa], mass[nroa]; char basis names[3][32]
//                 (read_system, ops_io.cc:63-109)
//   PREFIX.oei    double H, T, S, V [nroao^2 each]        (read_oei, ops_io.cc:112-121)
//   PREFIX.tei    long long sortcount[4]; double intval[nrofint];
//                 unsigned short intnums[4 nrofint]        (read_tei, ops_io.cc:203-212)
//   PREFIX.ahfw   int nroao; double MOens[nroao], MOs[nroao^2]
//                 (read_wav_HF, ops_io.cc:283-299; write_wav_HF, ops_io.cc:259-267)
//   PREFIX.rimp2  double BPQ[naux][nroao][nroao]          (read_transform_ri, ri.cc:109-119)
//
// Every array argument may be host or device memory.  Host arrays are read
// directly; device arrays stream through two pinned chunk buffers of the
// context: while one chunk is copied to the device on the context stream the
// next is read from the file into the other buffer, so reading and the
// host-to-device transfer overlap and no full-size host copy exists.  Unlike
// the reference (which does not check that a file opened or holds enough
// data), a missing or short file is an error: CORR_ERR_IO.  Trailing bytes
// are ignored, as they are there.
#include <cstdio>
#include <cstring>
#include <string>

#include "abi_internal.h"
#include "common.cuh"

namespace corr {

namespace {

constexpr size_t kIoChunk = 8u << 20;  // bytes per pinned staging buffer

struct File {
  FILE* f = nullptr;
  std::string path;
  ~File() {
    if (f) fclose(f);
  }
};

int open_file(File* fl, const std::string& path, const char* mode) {
  fl->path = path;
  fl->f = fopen(path.c_str(), mode);
  if (!fl->f) {
    set_error("cannot open %s", path.c_str());
    return CORR_ERR_IO;
  }
  return CORR_OK;
}

int read_host(File* fl, void* dst, size_t bytes) {
  if (bytes && fread(dst, 1, bytes, fl->f) != bytes) {
    set_error("%s is shorter than its header says", fl->path.c_str());
    return CORR_ERR_IO;
  }
  return CORR_OK;
}

int ensure_io_buffers(corr_context* c) {
  if (c->io_pinned[0]) return CORR_OK;
  for (int k = 0; k < 2; ++k) {
    if (cudaMallocHost(&c->io_pinned[k], kIoChunk) != cudaSuccess) {
      cudaGetLastError();
      set_error("pinned staging allocation failed");
      return CORR_ERR_OOM;
    }
    CORR_CUDA(cudaEventCreateWithFlags(&c->io_ev[k], cudaEventDisableTiming));
  }
  return CORR_OK;
}

// `bytes` from the file into dst (host or device of the context).
int read_to(corr_context* c, File* fl, void* dst, size_t bytes) {
  if (bytes == 0) return CORR_OK;
  if (!is_device_ptr(dst)) return read_host(fl, dst, bytes);
  CORR_CHECK_ARG(c != nullptr, "a device destination needs a context");
  CORR_CUDA(cudaSetDevice(c->device));
  CORR_TRY(ensure_io_buffers(c));
  bool used[2] = {false, false};
  size_t off = 0;
  for (int k = 0; off < bytes; k ^= 1) {
    const size_t n = bytes - off < kIoChunk ? bytes - off : kIoChunk;
    if (used[k]) CORR_CUDA(cudaEventSynchronize(c->io_ev[k]));  // its previous copy is done
    CORR_TRY(read_host(fl, c->io_pinned[k], n));
    CORR_CUDA(cudaMemcpyAsync(static_cast<char*>(dst) + off, c->io_pinned[k], n,
                              cudaMemcpyHostToDevice, c->stream));
    CORR_CUDA(cudaEventRecord(c->io_ev[k], c->stream));
    used[k] = true;
    off += n;
  }
  CORR_CUDA(cudaStreamSynchronize(c->stream));
  return CORR_OK;
}

void name_field(const char* raw, char* out) {
  int n = 0;
  while (n < 32 && raw[n] != '\0' && raw[n] != ' ' && raw[n] != '\n' && raw[n] != '\t') {
    out[n] = raw[n];
    ++n;
  }
  out[n] = '\0';
}

}  // namespace

}  // namespace corr

using namespace corr;

extern "C" {

int corr_read_system(const char* prefix, corr_system_info* info, double* coord, double* charges,
                     double* zeff, double* mass) {
  CORR_CHECK_ARG(prefix != nullptr && info != nullptr, "corr_read_system: null argument");
  File fl;
  CORR_TRY(open_file(&fl, std::string(prefix) + ".sys", "rb"));
  int h[5];
  long long c[3];
  CORR_TRY(read_host(&fl, h, sizeof(h)));
  CORR_TRY(read_host(&fl, c, sizeof(c)));
  info->nroe = h[0];
  info->nroa = h[1];
  info->nroao = h[2];
  info->naux_1 = h[3];
  info->naux_2 = h[4];
  info->nrofint = c[0];
  info->nrofaux = c[1];
  info->nrofaux2 = c[2];
  info->basis_ob[0] = info->basis_jk[0] = info->basis_ri[0] = '\0';
  CORR_CHECK_ARG(info->nroa >= 0 && info->nroa < (1 << 24), "%s: implausible atom count %d",
                 fl.path.c_str(), info->nroa);
  if (!coord && !charges && !zeff && !mass) return CORR_OK;  // sizes only
  CORR_CHECK_ARG(coord && charges && zeff && mass,
                 "corr_read_system: give all four atom arrays or none");
  const size_t na = (size_t)info->nroa;
  CORR_TRY(read_host(&fl, coord, 3 * na * sizeof(double)));
  CORR_TRY(read_host(&fl, charges, na * sizeof(double)));
  CORR_TRY(read_host(&fl, zeff, na * sizeof(double)));
  CORR_TRY(read_host(&fl, mass, na * sizeof(double)));
  char raw[96];
  std::memset(raw, 0, sizeof(raw));
  fread(raw, 1, sizeof(raw), fl.f);  // as the reference: whatever of the 96 bytes is there
  name_field(raw, info->basis_ob);
  name_field(raw + 32, info->basis_jk);
  name_field(raw + 64, info->basis_ri);
  return CORR_OK;
}

int corr_read_oei(corr_context* ctx, const char* prefix, int nroao, double* hmat, double* tmat,
                  double* smat, double* vmat) {
  CORR_CHECK_ARG(prefix && hmat && tmat && smat && vmat, "corr_read_oei: null argument");
  CORR_CHECK_ARG(nroao >= 1, "corr_read_oei: bad nroao %d", nroao);
  File fl;
  CORR_TRY(open_file(&fl, std::string(prefix) + ".oei", "rb"));
  const size_t n2 = (size_t)nroao * nroao * sizeof(double);
  CORR_TRY(read_to(ctx, &fl, hmat, n2));
  CORR_TRY(read_to(ctx, &fl, tmat, n2));
  CORR_TRY(read_to(ctx, &fl, smat, n2));
  return read_to(ctx, &fl, vmat, n2);
}

int corr_read_tei(corr_context* ctx, const char* prefix, long long nrofint, long long* sortcount,
                  double* intval, unsigned short* intnums) {
  CORR_CHECK_ARG(prefix && sortcount && intval && intnums, "corr_read_tei: null argument");
  CORR_CHECK_ARG(nrofint >= 0, "corr_read_tei: bad nrofint %lld", nrofint);
  File fl;
  CORR_TRY(open_file(&fl, std::string(prefix) + ".tei", "rb"));
  long long sc[4];
  CORR_TRY(read_host(&fl, sc, sizeof(sc)));
  if (is_device_ptr(sortcount)) {
    CORR_CHECK_ARG(ctx != nullptr, "a device destination needs a context");
    CORR_CUDA(cudaMemcpy(sortcount, sc, sizeof(sc), cudaMemcpyHostToDevice));
  } else {
    std::memcpy(sortcount, sc, sizeof(sc));
  }
  CORR_TRY(read_to(ctx, &fl, intval, (size_t)nrofint * sizeof(double)));
  return read_to(ctx, &fl, intnums, (size_t)nrofint * 4 * sizeof(unsigned short));
}

int corr_read_wav_hf(corr_context* ctx, const char* prefix, int nroao, double* moens,
                     double* mos) {
  CORR_CHECK_ARG(prefix && moens && mos, "corr_read_wav_hf: null argument");
  File fl;
  CORR_TRY(open_file(&fl, std::string(prefix) + ".ahfw", "rb"));
  int n = 0;
  CORR_TRY(read_host(&fl, &n, sizeof(int)));
  if (n != nroao) {  // the reference prints an error and exits (ops_io.cc:290-293)
    set_error("%s holds a wavefunction of %d orbitals, not %d", fl.path.c_str(), n, nroao);
    return CORR_ERR_BAD_ARG;
  }
  CORR_TRY(read_to(ctx, &fl, moens, (size_t)nroao * sizeof(double)));
  CORR_TRY(read_to(ctx, &fl, mos, (size_t)nroao * nroao * sizeof(double)));
  return CORR_OK;
}

int corr_write_wav_hf(const char* path, int nroao, const double* moens, const double* mos) {
  CORR_CHECK_ARG(path && moens && mos && nroao >= 1, "corr_write_wav_hf: bad argument");
  CORR_CHECK_ARG(!is_device_ptr(moens) && !is_device_ptr(mos),
                 "corr_write_wav_hf: moens and mos must be host arrays");
  File fl;
  CORR_TRY(open_file(&fl, path, "wb"));
  const size_t n = (size_t)nroao;
  if (fwrite(&nroao, sizeof(int), 1, fl.f) != 1 || fwrite(moens, sizeof(double), n, fl.f) != n ||
      fwrite(mos, sizeof(double), n * n, fl.f) != n * n) {
    set_error("writing %s failed", path);
    return CORR_ERR_IO;
  }
  return CORR_OK;
}

int corr_read_rimp2(corr_context* ctx, const char* prefix, int naux, int nroao, double* bpq) {
  CORR_CHECK_ARG(prefix && bpq && naux >= 1 && nroao >= 1, "corr_read_rimp2: bad argument");
  File fl;
  CORR_TRY(open_file(&fl, std::string(prefix) + ".rimp2", "rb"));
  return read_to(ctx, &fl, bpq, (size_t)naux * nroao * nroao * sizeof(double));
}

}  // extern "C"
