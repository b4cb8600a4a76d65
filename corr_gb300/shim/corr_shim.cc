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

#include <cstdio>
#include <cstdlib>
#include <cstring>
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
