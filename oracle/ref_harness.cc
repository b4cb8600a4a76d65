// Test infrastructure: the reference-oracle harness.
//
// Compiled together with the reference's own, unmodified sources
// (src/POSTHF/{motrans,can_mp2,ri}.cc, src/SCF/{ops_rhf,scf}.cc,
// src/MATH/ops_mat.cc, src/IO/ops_io.cc) into oracle/_ref/libcorr_ref.so by
// oracle/Makefile.  Each extern "C" entry point fills the reference's structs
// (src/UTIL/util.h:7-65), calls one reference function, captures what it
// prints at 17 significant digits and copies its outputs into caller buffers.
// Only the tests and the golden-fixture script load this library; it is the
// checker, never the product.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <cstdio>
#include <sstream>
#include <string>
#include <vector>

#include "IO/ops_io.h"
#include "MATH/ops_mat.h"
#include "POSTHF/can_mp2.h"
#include "POSTHF/ccsd.h"
#include "POSTHF/motrans.h"
#include "POSTHF/ri.h"
#include "SCF/ops_rhf.h"
#include "SCF/scf.h"
#include "UTIL/util.h"

namespace corr_oracle_tables {
int N = 0, X = 0;
const double* S = nullptr;
const double* T = nullptr;
const double* V = nullptr;
const double* eri = nullptr;
const double* J = nullptr;
const double* P3 = nullptr;
}  // namespace corr_oracle_tables

// Fortran LAPACK/BLAS names the reference declares itself (ops_mat.h:14,
// scf.cc:13-31), forwarded to scipy's prefixed OpenBLAS exports.
extern "C" {
void scipy_dsyev_(char*, char*, int*, double*, int*, double*, double*, int*, int*);
void scipy_dgels_(char*, int*, int*, int*, double*, int*, double*, int*, double*, int*, int*);
int scipy_dgemm_(char*, char*, int*, int*, int*, double*, double*, int*, double*, int*, double*,
                 double*, int*);
int scipy_daxpy_(int*, double*, double*, int*, double*, int*);
double scipy_ddot_(int*, double*, int*, double*, int*);
void scipy_dgesv_(int*, int*, double*, int*, int*, double*, int*, int*);
void scipy_openblas_set_num_threads(int);

void dsyev_(char* a, char* b, int* n, double* A, int* lda, double* w, double* work, int* lwork,
            int* info) {
  scipy_dsyev_(a, b, n, A, lda, w, work, lwork, info);
}
void dgels_(char* m, int* a, int* b, int* c, double* A, int* lda, double* B, int* ldb, double* w,
            int* lw, int* info) {
  scipy_dgels_(m, a, b, c, A, lda, B, ldb, w, lw, info);
}
int dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* al, double* A, int* lda, double* B,
           int* ldb, double* be, double* C, int* ldc) {
  return scipy_dgemm_(ta, tb, m, n, k, al, A, lda, B, ldb, be, C, ldc);
}
int daxpy_(int* n, double* a, double* x, int* ix, double* y, int* iy) {
  return scipy_daxpy_(n, a, x, ix, y, iy);
}
double ddot_(int* n, double* x, int* ix, double* y, int* iy) { return scipy_ddot_(n, x, ix, y, iy); }
void dgesv_(int* n, int* r, double* a, int* lda, int* p, double* b, int* ldb, int* info) {
  scipy_dgesv_(n, r, a, lda, p, b, ldb, info);
}
}

namespace {

// Redirect std::cout into a buffer for the duration of one reference call.
struct Capture {
  std::ostringstream buf;
  std::streambuf* old;
  std::ios_base::fmtflags flags;
  std::streamsize prec;
  Capture() {
    old = std::cout.rdbuf(buf.rdbuf());
    flags = std::cout.flags();
    prec = std::cout.precision();
    std::cout.unsetf(std::ios_base::floatfield);
    std::cout.precision(17);
  }
  ~Capture() {
    std::cout.rdbuf(old);
    std::cout.flags(flags);
    std::cout.precision(prec);
  }
};

// Value printed after `key` that follows the first occurrence of `block`.
double grab(const std::string& text, const char* block, const char* key) {
  size_t p = text.find(block);
  if (p == std::string::npos) return 0.0;
  p = text.find(key, p);
  if (p == std::string::npos) return 0.0;
  return std::strtod(text.c_str() + p + std::strlen(key), nullptr);
}

std::string g_last_output;

}  // namespace

// defined with external linkage in src/POSTHF/ccsd.cc (:509, :11), not declared in ccsd.h
void calc_ints_so(cc_helper* CC, pHF* postHF);
void form_fock(cc_helper* CC, pHF* postHF);

extern "C" {

void ref_set_threads(int n) { scipy_openblas_set_num_threads(n); }

const char* ref_last_output() { return g_last_output.c_str(); }

// src/POSTHF/can_mp2.cc:53 run_canonical_mp2_ri.  Bia[Q][i][a]; eps has nroao
// entries and becomes the diagonal of FMo.  out = {EMP2_SS, EMP2_OS, EMP2}.
void ref_rimp2_energy(int nocc, int nvir, int naux, const double* Bia, const double* eps,
                      double* out) {
  int nroao = nocc + nvir;
  systeminfo si;
  si.nroe = 2 * nocc;
  si.nroao = nroao;
  si.naux_2 = naux;
  std::vector<double> fmo((size_t)nroao * nroao, 0.0);
  for (int p = 0; p < nroao; ++p) fmo[(size_t)p * nroao + p] = eps[p];
  pHF ph;
  ph.FMo = fmo.data();
  ph.Bia = const_cast<double*>(Bia);
  std::string text;
  {
    Capture c;
    run_canonical_mp2_ri(&si, &ph);
    text = c.buf.str();
  }
  g_last_output = text;
  out[0] = grab(text, "RI-MP2-Results", "EMP2_SS:");
  out[1] = grab(text, "RI-MP2-Results", "EMP2_OS:");
  out[2] = grab(text, "RI-MP2-Results", "EMP2:");
}

// src/POSTHF/can_mp2.cc:11 run_canonical_mp2 on a full [N][N][N][N] MO tensor.
void ref_canonical_mp2(int nroe, int nroao, const double* prec_ints, const double* fmo,
                       double* out) {
  systeminfo si;
  si.nroe = nroe;
  si.nroao = nroao;
  pHF ph;
  ph.FMo = const_cast<double*>(fmo);
  ph.prec_ints = const_cast<double*>(prec_ints);
  std::string text;
  {
    Capture c;
    run_canonical_mp2(&si, &ph);
    text = c.buf.str();
  }
  g_last_output = text;
  out[0] = grab(text, "MP2-Results", "EMP2_SS:");
  out[1] = grab(text, "MP2-Results", "EMP2_OS:");
  out[2] = grab(text, "MP2-Results", "EMP2:");
}

// src/POSTHF/motrans.cc:8 build_FMo.
void ref_build_fmo(int nroao, const double* mos, const double* fmat, double* fmo_out) {
  systeminfo si;
  si.nroao = nroao;
  OEints oe;
  oe.MOs = const_cast<double*>(mos);
  oe.Fmat = const_cast<double*>(fmat);
  pHF ph;
  build_FMo(&si, &oe, &ph);
  std::memcpy(fmo_out, ph.FMo, sizeof(double) * nroao * nroao);
  delete[] ph.FMo;
}

// src/SCF/ops_rhf.cc:618 calculate_libint_tei (screening, unique selection)
// followed by its resort_integrals (ops_rhf.cc:750).  Two calls: with
// intval == nullptr only the count is returned.
static std::vector<double> g_intval;
static std::vector<unsigned short> g_intnums;
static long long g_sortcount[4];

long long ref_pack_eri(int nroao, const double* eri) {
  corr_oracle_tables::N = nroao;
  corr_oracle_tables::eri = eri;
  libint2::BasisSet obs(0, nroao);
  systeminfo si;
  si.nroao = nroao;
  TEints te;
  {
    Capture c;
    calculate_libint_tei(&si, obs, &te);
  }
  g_intval.assign(te.intval, te.intval + si.nrofint);
  g_intnums.assign(te.intnums, te.intnums + 4 * si.nrofint);
  for (int k = 0; k < 4; ++k) g_sortcount[k] = te.sortcount[k];
  delete[] te.intval;
  delete[] te.intnums;
  return si.nrofint;
}

void ref_packed_copy(double* intval, unsigned short* intnums, long long* sortcount) {
  std::memcpy(intval, g_intval.data(), sizeof(double) * g_intval.size());
  std::memcpy(intnums, g_intnums.data(), sizeof(unsigned short) * g_intnums.size());
  for (int k = 0; k < 4; ++k) sortcount[k] = g_sortcount[k];
}

// src/POSTHF/motrans.cc:35 MOtrans.  Its mo2int_op keeps function-static
// buffers sized by the first nroao seen, so one process may only use one
// nroao (the golden script runs each case in its own process).
void ref_motrans(int nroe, int nroao, const double* mos, long long nrofint,
                 const long long* sortcount, const double* intval, const unsigned short* intnums,
                 double* prec_out) {
  systeminfo si;
  si.nroe = nroe;
  si.nroao = nroao;
  si.nrofint = nrofint;
  OEints oe;
  oe.MOs = const_cast<double*>(mos);
  TEints te;
  te.intval = const_cast<double*>(intval);
  te.intnums = const_cast<unsigned short*>(intnums);
  for (int k = 0; k < 4; ++k) te.sortcount[k] = sortcount[k];
  pHF ph;
  {
    Capture c;
    MOtrans(&si, &oe, &te, &ph);
  }
  size_t n4 = (size_t)nroao * nroao * nroao * nroao;
  std::memcpy(prec_out, ph.prec_ints, sizeof(double) * n4);
  delete[] ph.prec_ints;
}

// src/POSTHF/motrans.cc:286 calc_mo2int_bf (single element, brute force).
double ref_mo2int_bf(int i, int j, int k, int l, int nroao, const double* mos, long long nrofint,
                     const long long* sortcount, const double* intval,
                     const unsigned short* intnums) {
  return calc_mo2int_bf(i, j, k, l, nroao, const_cast<double*>(mos), nrofint,
                        const_cast<long long*>(sortcount), const_cast<double*>(intval),
                        const_cast<unsigned short*>(intnums));
}

// src/POSTHF/ri.cc:7 calculate_ri on registered (P|Q) and (P|mn) tables:
// dsyev, the 1e-10 relative eigenvalue cutoff, J^-1/2 and BPQ = J^-1/2 (Q|mn).
void ref_calculate_ri(int naux, int nroao, const double* J, const double* P3, double* bpq_out) {
  corr_oracle_tables::N = nroao;
  corr_oracle_tables::X = naux;
  corr_oracle_tables::J = J;
  corr_oracle_tables::P3 = P3;
  libint2::BasisSet obs(0, nroao), dfbs(1, naux);
  calculate_ri(obs, dfbs, bpq_out);
}

// src/POSTHF/ri.cc:147 transform_ri.  Bia[Q][i][a].
void ref_transform_ri(int nroe, int nroao, int naux, const double* mos, const double* bpq,
                      double* bia_out) {
  systeminfo si;
  si.nroe = nroe;
  si.nroao = nroao;
  si.naux_2 = naux;
  OEints oe;
  oe.MOs = const_cast<double*>(mos);
  pHF ph;
  ph.BPQ = const_cast<double*>(bpq);
  ph.Bia = bia_out;
  transform_ri(&si, &oe, &ph);
}

// src/POSTHF/ri.cc:109 read_transform_ri: BPQ read from prefix + ".rimp2".
void ref_read_transform_ri(const char* prefix, int nroe, int nroao, int naux, const double* mos,
                           double* bia_out) {
  read_transform_ri(std::string(prefix), nroe, nroao, naux, const_cast<double*>(mos), bia_out);
}

// The reference's RHF (src/main.cc:102-117): calc_S12, core guess
// (check_initial_guess, ops_rhf.cc:15), run_scf (scf.cc:145) with 100
// iterations.  Inputs S, T, V (H = T + V) and the packed ERIs; outputs the MO
// coefficients [p][mu], the final Fock matrix and the MO energies.
// out_e = {total HF energy}.
void ref_rhf(int nroe, int nroao, double ion_rep, const double* S, const double* T,
             const double* V, long long nrofint, const long long* sortcount, const double* intval,
             const unsigned short* intnums, double* mos_out, double* fmat_out, double* moens_out,
             double* out_e) {
  systeminfo si;
  si.nroe = nroe;
  si.nroao = nroao;
  si.nrofint = nrofint;
  si.ion_rep = ion_rep;
  si.scfiter = 100;
  OEints oe;
  allocate_onemats(&si, &oe);
  size_t n2 = (size_t)nroao * nroao;
  for (size_t x = 0; x < n2; ++x) {
    oe.Smat[x] = S[x];
    oe.Tmat[x] = T[x];
    oe.Vmat[x] = V[x];
    oe.Hmat[x] = T[x] + V[x];
    oe.MOs[x] = 0.0;
    oe.Pmat[x] = 0.0;
    oe.Fmat[x] = 0.0;
  }
  TEints te;
  te.intval = const_cast<double*>(intval);
  te.intnums = const_cast<unsigned short*>(intnums);
  for (int k = 0; k < 4; ++k) te.sortcount[k] = sortcount[k];
  std::string text;
  {
    Capture c;
    calc_S12(&si, &oe);
    check_initial_guess(&si, &oe);
    run_scf(&si, &oe, &te);
    std::cout.unsetf(std::ios_base::floatfield);
    std::cout.precision(17);
    text = c.buf.str();
  }
  g_last_output = text;
  std::memcpy(mos_out, oe.MOs, sizeof(double) * n2);
  std::memcpy(fmat_out, oe.Fmat, sizeof(double) * n2);
  std::memcpy(moens_out, oe.MOens, sizeof(double) * nroao);
  out_e[0] = grab(text, "HF-Results", "TOTAL E:");
  delete[] oe.Hmat;  // allocate_onemats hands out one block starting at Hmat
}

// src/SCF/ops_rhf.cc:549 build_Fmat: the Fock matrix of density pmat from the
// packed unique integrals.
void ref_build_fmat(int nroao, const double* pmat, const double* hmat, long long nrofint,
                    const long long* sortcount, const double* intval,
                    const unsigned short* intnums, double* fmat_out) {
  long long sc[4];
  for (int k = 0; k < 4; ++k) sc[k] = sortcount[k];
  build_Fmat(nroao, fmat_out, const_cast<double*>(pmat), const_cast<double*>(hmat),
             const_cast<double*>(intval), const_cast<unsigned short*>(intnums), sc, nrofint);
}

// src/POSTHF/ccsd.cc:509 calc_ints_so: ints_so[norb^4] (norb = 2 nroao) from
// the spatial MO integrals prec_ints[N^4].
void ref_ints_so(int nroe, int nroao, const double* prec, double* out) {
  cc_helper cc;
  cc.nocc = nroe;
  cc.nroao = nroao;
  cc.norb = 2 * nroao;
  cc.nvir = cc.norb - nroe;
  pHF ph;
  ph.prec_ints = const_cast<double*>(prec);
  calc_ints_so(&cc, &ph);
  const size_t n = (size_t)cc.norb * cc.norb * cc.norb * cc.norb;
  std::memcpy(out, ph.ints_so, sizeof(double) * n);
  delete[] ph.ints_so;
}

// src/POSTHF/ccsd.cc:11 form_fock: spin-orbital h and f (norb x norb) from the
// MO coefficients, the AO core Hamiltonian and prec_ints.
void ref_form_fock(int nroe, int nroao, const double* mos, const double* hmat, const double* prec,
                   double* h_out, double* f_out) {
  cc_helper cc;
  cc.nocc = nroe;
  cc.nroao = nroao;
  cc.norb = 2 * nroao;
  cc.nvir = cc.norb - nroe;
  cc.MOs = const_cast<double*>(mos);
  cc.Hmat = const_cast<double*>(hmat);
  pHF ph;
  ph.prec_ints = const_cast<double*>(prec);
  form_fock(&cc, &ph);
  const size_t n = (size_t)cc.norb * cc.norb;
  std::memcpy(h_out, cc.h, sizeof(double) * n);
  std::memcpy(f_out, cc.f, sizeof(double) * n);
  delete[] cc.h;
  delete[] cc.f;
}

// src/IO/ops_io.cc:63 read_system.  ints = {nroe, nroa, nroao, naux_1,
// naux_2}, lls = {nrofint, nrofaux, nrofaux2}; atoms (caller-sized by a first
// call with coord == NULL) and the three basis names, each into 33 bytes.
void ref_read_system(const char* prefix, int* ints, long long* lls, double* coord,
                     double* charges, double* zeff, double* mass, char* names) {
  systeminfo si;
  si.prefix = prefix;
  read_system(&si);
  ints[0] = si.nroe;
  ints[1] = si.nroa;
  ints[2] = si.nroao;
  ints[3] = si.naux_1;
  ints[4] = si.naux_2;
  lls[0] = si.nrofint;
  lls[1] = si.nrofaux;
  lls[2] = si.nrofaux2;
  if (coord) {
    std::memcpy(coord, si.coord, sizeof(double) * 3 * si.nroa);
    std::memcpy(charges, si.charges, sizeof(double) * si.nroa);
    std::memcpy(zeff, si.zeff, sizeof(double) * si.nroa);
    std::memcpy(mass, si.mass, sizeof(double) * si.nroa);
    std::snprintf(names, 33, "%s", si.basisNameOB.c_str());
    std::snprintf(names + 33, 33, "%s", si.basisNameJK.c_str());
    std::snprintf(names + 66, 33, "%s", si.basisNameRI.c_str());
  }
  delete[] si.coord;
  delete[] si.charges;
  delete[] si.zeff;
  delete[] si.mass;
}

// src/IO/ops_io.cc:112 read_oei into the caller's four nroao^2 arrays.
void ref_read_oei(const char* prefix, int nroao, double* H, double* T, double* S, double* V) {
  systeminfo si;
  si.prefix = prefix;
  si.nroao = nroao;
  OEints oe;
  oe.Hmat = H;
  oe.Tmat = T;
  oe.Smat = S;
  oe.Vmat = V;
  read_oei(&si, &oe);
}

// src/IO/ops_io.cc:203 read_tei into caller arrays.
void ref_read_tei(const char* prefix, long long nrofint, long long* sortcount, double* intval,
                  unsigned short* intnums) {
  systeminfo si;
  si.prefix = prefix;
  si.nrofint = nrofint;
  TEints te;
  te.intval = intval;
  te.intnums = intnums;
  read_tei(&si, &te);
  for (int k = 0; k < 4; ++k) sortcount[k] = te.sortcount[k];
}

// src/IO/ops_io.cc:283 read_wav_HF and :259 write_wav_HF.
void ref_read_wav_hf(const char* prefix, int nroao, double* moens, double* mos) {
  systeminfo si;
  si.prefix = prefix;
  si.nroao = nroao;
  OEints oe;
  oe.MOens = moens;
  oe.MOs = mos;
  read_wav_HF(&si, &oe);
}

void ref_write_wav_hf(const char* path, int nroao, double* moens, double* mos) {
  write_wav_HF(std::string(path), nroao, moens, mos);
}

}  // extern "C"
