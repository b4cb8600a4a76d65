// Drop-in implementations of the reference's hot-path entry points on the
// corr_gb300 C ABI.  Same signatures, same allocation ownership (build_FMo and
// MOtrans allocate with new[]), same printed result blocks
// (src/POSTHF/can_mp2.cc:37-46, 115-125).  Any nonzero status aborts with the
// library's error message: the reference has no error channel either.
//
// Environment:
//   CORR_DEVICE              CUDA device of the process-wide context (default 0)
//   CORR_RIMP2_PRECISION     fp64 (default) | split_fp16 | split_bf16
#include "corr_shim.h"

#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <mutex>
#include <vector>

#include "../../include/corr_gb300.h"

#define PWIDTH_L 12
#define PWIDTH_R 16

namespace {

corr_context* g_ctx = nullptr;
std::once_flag g_once;

corr_context* ctx() {
  std::call_once(g_once, [] {
    const char* d = std::getenv("CORR_DEVICE");
    int dev = d ? std::atoi(d) : 0;
    int st = corr_create(&g_ctx, dev, nullptr);
    if (st != CORR_OK) {
      std::cerr << "corr_gb300: " << corr_last_error() << '\n';
      std::abort();
    }
  });
  return g_ctx;
}

void check(int st, const char* what) {
  if (st != CORR_OK) {
    std::cerr << "corr_gb300: " << what << " failed (" << st << "): " << corr_last_error()
              << '\n';
    std::abort();
  }
}

int precision_from_env() {
  const char* p = std::getenv("CORR_RIMP2_PRECISION");
  if (!p || !std::strcmp(p, "fp64")) return CORR_PREC_FP64;
  if (!std::strcmp(p, "split_fp16")) return CORR_PREC_SPLIT_FP16;
  if (!std::strcmp(p, "split_bf16")) return CORR_PREC_SPLIT_BF16;
  std::cerr << "corr_gb300: unknown CORR_RIMP2_PRECISION=" << p << '\n';
  std::abort();
}

std::vector<double> fmo_diagonal(const double* fmo, int n) {
  std::vector<double> e(n);
  for (int p = 0; p < n; ++p) e[p] = fmo[(size_t)p * n + p];
  return e;
}

void print_block(const char* title, const char* rule, const char* scs_title,
                 const char* scs_rule, const corr_mp2_energy& e) {
  std::cout << title;
  std::cout << rule;
  std::cout << std::setw(PWIDTH_L) << "EMP2_SS:" << std::setw(PWIDTH_R) << e.e_ss << '\n';
  std::cout << std::setw(PWIDTH_L) << "EMP2_OS:" << std::setw(PWIDTH_R) << e.e_os << '\n';
  std::cout << std::setw(PWIDTH_L) << "EMP2:" << std::setw(PWIDTH_R) << e.e_total << '\n';
  std::cout << scs_title;
  std::cout << scs_rule;
  std::cout << std::setw(PWIDTH_L) << "EMP2_SS:" << std::setw(PWIDTH_R) << e.e_ss / 3.0 << '\n';
  std::cout << std::setw(PWIDTH_L) << "EMP2_OS:" << std::setw(PWIDTH_R) << e.e_os * 6.0 / 5.0
            << '\n';
  std::cout << std::setw(PWIDTH_L) << "EMP2(SCS):" << std::setw(PWIDTH_R) << e.e_scs << '\n';
}

}  // namespace

void build_FMo(systeminfo* sysinfo, OEints* onemats, pHF* postHF) {
  const int n = sysinfo->nroao;
  postHF->FMo = new double[(size_t)n * n];
  check(corr_build_fmo(ctx(), n, onemats->MOs, onemats->Fmat, postHF->FMo), "build_FMo");
}

void MOtrans(systeminfo* sysinfo, OEints* onemats, TEints* twomats, pHF* postHF) {
  const long long n = sysinfo->nroao;
  const long long prec_mem = n * n * n * n;
  std::cout << "Need " << prec_mem * sizeof(double) << " bytes ("
            << prec_mem * sizeof(double) / 1024 / 1024 << " MB) for precalculation\n";
  postHF->prec_ints = new double[prec_mem];
  check(corr_motrans(ctx(), sysinfo->nroe, (int)n, onemats->MOs, sysinfo->nrofint,
                     twomats->sortcount, twomats->intval, twomats->intnums, postHF->prec_ints),
        "MOtrans");
}

void run_canonical_mp2(systeminfo* sysinfo, pHF* postHF) {
  const int n = sysinfo->nroao;
  std::vector<double> eps = fmo_diagonal(postHF->FMo, n);
  corr_mp2_energy e;
  check(corr_canonical_mp2(ctx(), sysinfo->nroe, n, postHF->prec_ints, eps.data(), &e),
        "run_canonical_mp2");
  print_block("\nMP2-Results:\n", "------------\n", "\nSCS-MP2-Results:\n", "------------\n", e);
}

void transform_ri(systeminfo* sysinfo, OEints* onemats, pHF* postHF) {
  check(corr_transform_ri(ctx(), sysinfo->nroe, sysinfo->nroao, sysinfo->naux_2, onemats->MOs,
                          postHF->BPQ, postHF->Bia),
        "transform_ri");
}

void run_canonical_mp2_ri(systeminfo* sysinfo, pHF* postHF) {
  const int n = sysinfo->nroao, nocc = sysinfo->nroe / 2;
  std::vector<double> eps = fmo_diagonal(postHF->FMo, n);
  corr_mp2_energy e;
  check(corr_rimp2_energy(ctx(), nocc, n - nocc, sysinfo->naux_2, postHF->Bia, eps.data(),
                          precision_from_env(), &e),
        "run_canonical_mp2_ri");
  print_block("\nRI-MP2-Results:\n", "---------------\n", "\nSCS-RI-MP2-Results:\n",
              "-------------------\n", e);
}

void calculate_ri_from_integrals(int naux, int nroao, const double* J, const double* Pmn,
                                 double* BPQ) {
  check(corr_calculate_ri(ctx(), naux, nroao, J, Pmn, BPQ), "calculate_ri");
}

void read_transform_ri(std::string prefix, int nroe, int nroao, int naux_2, double* MOs,
                       double* Bia) {
  const size_t n = (size_t)naux_2 * nroao * nroao;
  std::vector<double> bpq(n);
  std::ifstream f(prefix + ".rimp2", std::ios::binary);
  if (!f || !f.read(reinterpret_cast<char*>(bpq.data()), (std::streamsize)(n * sizeof(double)))) {
    std::cerr << "corr_gb300: read_transform_ri cannot read " << n << " doubles from " << prefix
              << ".rimp2\n";
    std::abort();
  }
  check(corr_transform_ri(ctx(), nroe, nroao, naux_2, MOs, bpq.data(), Bia), "read_transform_ri");
}

// ---- src/MATH/ops_mat.cc ----------------------------------------------------

namespace {

int dim(long long np, const char* what) {
  if (np < 1 || np > INT_MAX) {
    std::cerr << "corr_gb300: " << what << ": matrix size " << np << " out of range\n";
    std::abort();
  }
  return (int)np;
}

// f = op(a) op(b), n x n row-major
void square_gemm(int n, int ta, int tb, const double* a, const double* b, double* f,
                 const char* what) {
  check(corr_dgemm(ctx(), ta, tb, n, n, n, 1.0, a, n, b, n, 0.0, f, n), what);
}

}  // namespace

// ops_mat.cc:21-45: dsyev(JOBZ='V', UPLO='U') of a row-major array, i.e. its
// lower triangle; vals ascending, vecs[k*n + i] = component i of vector k.
void diag_mat(int nroao, double* mat, double* vals, double* vecs) {
  check(corr_syev(ctx(), nroao, mat, vals, vecs), "diag_mat");
}

// ops_mat.cc:53-69: dummat = tmat mat, mat = dummat tmat.
void symmortho_mat(int nroao, double* mat, double* tmat, double* dummat) {
  square_gemm(nroao, 0, 0, tmat, mat, dummat, "symmortho_mat");
  square_gemm(nroao, 0, 0, dummat, tmat, mat, "symmortho_mat");
}

// ops_mat.cc:75-88: MOs <- MOs tmat^T row by row; tmpvec keeps the last row.
void transform_MOs(int nroao, double* MOs, double* tmat, double* tmpvec) {
  const size_t n = (size_t)nroao;
  std::vector<double> out(n * n);
  square_gemm(nroao, 0, 1, MOs, tmat, out.data(), "transform_MOs");
  std::memcpy(MOs, out.data(), n * n * sizeof(double));
  std::memcpy(tmpvec, out.data() + (n - 1) * n, n * sizeof(double));
}

// mat_f = mat_i1 mat_i2 (declared at ops_mat.h:5 and :8, used by the
// commented-out trans_mat of ops_mat.cc:159-190)
void mat_mat(int np, double* mat_i1, double* mat_i2, double* mat_f) {
  square_gemm(dim(np, "mat_mat"), 0, 0, mat_i1, mat_i2, mat_f, "mat_mat");
}
void mat_mat(long long int np, double* mat_i1, double* mat_i2, double* mat_f) {
  square_gemm(dim(np, "mat_mat"), 0, 0, mat_i1, mat_i2, mat_f, "mat_mat");
}

// ops_mat.cc:93-105, :122-134: mat_f = mat_i1 mat_i2^T
void mat_mat_T(int np, double* mat_i1, double* mat_i2, double* mat_f) {
  square_gemm(dim(np, "mat_mat_T"), 0, 1, mat_i1, mat_i2, mat_f, "mat_mat_T");
}
void mat_mat_T(long long int np, double* mat_i1, double* mat_i2, double* mat_f) {
  square_gemm(dim(np, "mat_mat_T"), 0, 1, mat_i1, mat_i2, mat_f, "mat_mat_T");
}

// ops_mat.cc:107-119, :136-148: mat_f = mat_i1^T mat_i2
void mat_T_mat(int np, double* mat_i1, double* mat_i2, double* mat_f) {
  square_gemm(dim(np, "mat_T_mat"), 1, 0, mat_i1, mat_i2, mat_f, "mat_T_mat");
}
void mat_T_mat(long long int np, double* mat_i1, double* mat_i2, double* mat_f) {
  square_gemm(dim(np, "mat_T_mat"), 1, 0, mat_i1, mat_i2, mat_f, "mat_T_mat");
}

// ops_mat.cc:155-190 (declared at ops_mat.h:11-12): dir == 0: tmpmat = mat
// trans, mat = trans^T tmpmat; otherwise tmpmat = trans mat, mat = tmpmat trans^T.
void trans_mat(long long int np, double* mat, double* trans, double* tmpmat, int dir) {
  const int n = dim(np, "trans_mat");
  if (dir == 0) {
    square_gemm(n, 0, 0, mat, trans, tmpmat, "trans_mat");
    square_gemm(n, 1, 0, trans, tmpmat, mat, "trans_mat");
  } else {
    square_gemm(n, 0, 0, trans, mat, tmpmat, "trans_mat");
    square_gemm(n, 0, 1, tmpmat, trans, mat, "trans_mat");
  }
}
void trans_mat(int np, double* mat, double* trans, double* tmpmat, int dir) {
  trans_mat((long long int)np, mat, trans, tmpmat, dir);
}

// ops_mat.cc:192-198: vo = mat vi
void pmv(double* mat, double* vi, double* vo, int nroao) {
  check(corr_dgemm(ctx(), 0, 0, nroao, 1, nroao, 1.0, mat, nroao, vi, 1, 0.0, vo, 1), "pmv");
}

// ---- RHF (src/SCF) -----------------------------------------------------------

void build_Fmat(int nroao, double* Fmat, double* Pmat, double* Hmat, double* intval,
                unsigned short* intnums, long long int* sortcount, long long int nrofint) {
  check(corr_build_fmat(ctx(), nroao, Pmat, Hmat, nrofint, sortcount, intval, intnums, Fmat),
        "build_Fmat");
}

#ifdef CORR_SHIM_USE_REFERENCE_HEADERS
void run_scf(systeminfo* sysinfo, OEints* onemats, TEints* twomats) {
  std::cout << "\nSCF:\n----" << '\n';
  double e[3];
  int iters = 0;
  check(corr_run_scf(ctx(), sysinfo->nroe, sysinfo->nroao, sysinfo->ion_rep, onemats->Smat,
                     onemats->Hmat, sysinfo->nrofint, twomats->sortcount, twomats->intval,
                     twomats->intnums, sysinfo->scfiter, onemats->MOs, onemats->Fmat,
                     onemats->MOens, e, &iters, onemats->Pmat),
        "run_scf");
  std::cout << "iterations: " << iters << '\n';
  std::cout << "\nHF-Results:\n";
  std::cout << "-----------\n";
  std::cout << std::setw(PWIDTH_L) << "  ONE E:" << std::setw(PWIDTH_R) << e[1] << '\n';
  std::cout << std::setw(PWIDTH_L) << "  TWO E:" << std::setw(PWIDTH_R) << e[2] << '\n';
  std::cout << std::setw(PWIDTH_L) << "TOTAL E:" << std::setw(PWIDTH_R) << e[0] << '\n';
}
#endif

// ---- hand-off files (src/IO/ops_io.cc) --------------------------------------

void write_wav_HF(std::string wavfile, int nroao, double* MOens, double* MOs) {
  check(corr_write_wav_hf(wavfile.c_str(), nroao, MOens, MOs), "write_wav_HF");
}

#ifdef CORR_SHIM_USE_REFERENCE_HEADERS
void read_system(systeminfo* sysinfo) {
  corr_system_info info;
  check(corr_read_system(sysinfo->prefix.c_str(), &info, nullptr, nullptr, nullptr, nullptr),
        "read_system");
  const int na = info.nroa;
  sysinfo->nroe = info.nroe;
  sysinfo->nroa = na;
  sysinfo->nroao = info.nroao;
  sysinfo->naux_1 = info.naux_1;
  sysinfo->naux_2 = info.naux_2;
  sysinfo->nrofint = info.nrofint;
  sysinfo->nrofaux = info.nrofaux;
  sysinfo->nrofaux2 = info.nrofaux2;
  sysinfo->coord = new double[3 * na];
  sysinfo->charges = new double[na];
  sysinfo->zeff = new double[na];
  sysinfo->mass = new double[na];
  check(corr_read_system(sysinfo->prefix.c_str(), &info, sysinfo->coord, sysinfo->charges,
                         sysinfo->zeff, sysinfo->mass),
        "read_system");
  sysinfo->basisNameOB = info.basis_ob;
  sysinfo->basisNameJK = info.basis_jk;
  sysinfo->basisNameRI = info.basis_ri;
  sysinfo->atoms.resize(na);
  for (int i = 0; i < na; ++i) {
    sysinfo->atoms[i].atomic_number = sysinfo->charges[i];
    sysinfo->atoms[i].x = sysinfo->coord[3 * i + 0];
    sysinfo->atoms[i].y = sysinfo->coord[3 * i + 1];
    sysinfo->atoms[i].z = sysinfo->coord[3 * i + 2];
  }
}

void read_oei(systeminfo* sysinfo, OEints* onemats) {
  check(corr_read_oei(nullptr, sysinfo->prefix.c_str(), sysinfo->nroao, onemats->Hmat,
                      onemats->Tmat, onemats->Smat, onemats->Vmat),
        "read_oei");
}

void read_tei(systeminfo* sysinfo, TEints* twomats) {
  check(corr_read_tei(nullptr, sysinfo->prefix.c_str(), sysinfo->nrofint, twomats->sortcount,
                      twomats->intval, twomats->intnums),
        "read_tei");
}

void read_wav_HF(systeminfo* sysinfo, OEints* onemats) {
  check(corr_read_wav_hf(nullptr, sysinfo->prefix.c_str(), sysinfo->nroao, onemats->MOens,
                         onemats->MOs),
        "read_wav_HF");
}
#endif
