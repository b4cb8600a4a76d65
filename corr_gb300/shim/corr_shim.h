// Drop-in C++ layer: the reference's hot-path functions with their exact C++
// signatures, implemented on the corr_gb300 C ABI (include/corr_gb300.h).
//
// Built inside the reference tree (define CORR_SHIM_USE_REFERENCE_HEADERS and
// put the reference's src/ on the include path) it uses the reference's own
// src/UTIL/util.h.  Built standalone it declares the hand-off structs below,
// whose leading members have the reference's layout (src/UTIL/util.h:7-65);
// the shim reads only those leading members, never sizeof(systeminfo).
#ifndef CORR_SHIM_H
#define CORR_SHIM_H

#include <string>

#ifdef CORR_SHIM_USE_REFERENCE_HEADERS
#include "UTIL/util.h"
#include "MATH/ops_mat.h"
#include "POSTHF/motrans.h"
#else
struct pHF {  // src/UTIL/util.h:7-13
  double* FMo;
  double* prec_ints;
  double* ints_so;
  double* BPQ;
  double* Bia;
};

struct systeminfo {  // src/UTIL/util.h:16-45, leading members only
  int nroe;
  int nroao;
  int nroa;
  int naux_1;
  int naux_2;
  long long int nrofint;
  long long int nrofaux;
  long long int nrofaux2;
};

struct OEints {  // src/UTIL/util.h:47-59
  double* Hmat;
  double* Tmat;
  double* Smat;
  double* Som12;
  double* Vmat;
  double* MOens;
  double* MOs;
  double* Pmat;
  double* Fmat;
};

struct TEints {  // src/UTIL/util.h:61-65
  double* intval;
  unsigned short* intnums;
  long long int sortcount[4];
};
#endif

// src/POSTHF/motrans.h:22 -- allocates postHF->FMo (new[], as the reference)
void build_FMo(systeminfo* sysinfo, OEints* onemats, pHF* postHF);
// src/POSTHF/motrans.h:5 -- allocates postHF->prec_ints (new[], N^4 doubles)
void MOtrans(systeminfo* sysinfo, OEints* onemats, TEints* twomats, pHF* postHF);
// src/POSTHF/can_mp2.h:4
void run_canonical_mp2(systeminfo* sysinfo, pHF* postHF);
// src/POSTHF/ri.h:9 -- writes the caller-allocated postHF->Bia
void transform_ri(systeminfo* sysinfo, OEints* onemats, pHF* postHF);
// src/POSTHF/can_mp2.h:5
void run_canonical_mp2_ri(systeminfo* sysinfo, pHF* postHF);
// The GPU part of calculate_ri (src/POSTHF/ri.cc:50-69, 102-103): the host
// integral engine fills J[P][Q] = (P|Q) and Pmn[P][mu][nu] = (P|mu nu), this
// call writes BPQ (caller-allocated naux*nroao*nroao, as main.cc:151 does).
void calculate_ri_from_integrals(int naux, int nroao, const double* J, const double* Pmn,
                                 double* BPQ);
// src/POSTHF/motrans.h:12 (defined at ri.cc:109-144): BPQ[naux_2][nroao][nroao]
// read raw from prefix + ".rimp2", transformed into the caller's Bia.  A
// missing or short file aborts (the reference would transform uninitialised
// memory).
void read_transform_ri(std::string prefix, int nroe, int nroao, int naux_2, double* MOs,
                       double* Bia);

// src/IO/ops_io.h:33 -- writes nroao, MOens, MOs to `wavfile` (host arrays).
void write_wav_HF(std::string wavfile, int nroao, double* MOens, double* MOs);
#ifdef CORR_SHIM_USE_REFERENCE_HEADERS
// The readers need systeminfo::prefix, a member the standalone layout above
// does not declare: they exist in the build against the reference's util.h.
void read_system(systeminfo* sysinfo);                   // ops_io.h:37, allocates as the reference
void read_oei(systeminfo* sysinfo, OEints* onemats);      // ops_io.h:38, caller-allocated arrays
void read_tei(systeminfo* sysinfo, TEints* twomats);      // ops_io.h:39, caller-allocated arrays
void read_wav_HF(systeminfo* sysinfo, OEints* onemats);   // ops_io.h:34, caller-allocated arrays
#endif

// RHF (src/SCF).  ops_rhf.h:22 -- F = H + sum P ((mn|ls) - 1/2 (ml|ns)) from the
// packed unique integrals, host arrays.
void build_Fmat(int nroao, double* Fmat, double* Pmat, double* Hmat, double* intval,
                unsigned short* intnums, long long int* sortcount, long long int nrofint);
#ifdef CORR_SHIM_USE_REFERENCE_HEADERS
// scf.h:5 -- the whole iteration on the GPU (needs systeminfo::ion_rep and
// ::scfiter, members the standalone layout does not declare); S^-1/2 is formed
// on the device, onemats->Som12 is not read; MOs, MOens, Pmat and Fmat are
// written as the reference leaves them, and the HF-Results block is printed.
void run_scf(systeminfo* sysinfo, OEints* onemats, TEints* twomats);
#endif

// Dense FP64 helpers of src/MATH/ops_mat.h, row-major np x np, on the GPU.
void diag_mat(int nroao, double* mat, double* vals, double* vecs);          // ops_mat.h:3
void symmortho_mat(int nroao, double* mat, double* tmat, double* dummat);   // ops_mat.h:4
void transform_MOs(int nroao, double* MOs, double* tmat, double* tmpvec);   // ops_mat.cc:75
void mat_mat(int np, double* mat_i1, double* mat_i2, double* mat_f);        // ops_mat.h:5
void mat_mat_T(int np, double* mat_i1, double* mat_i2, double* mat_f);      // ops_mat.h:6
void mat_T_mat(int np, double* mat_i1, double* mat_i2, double* mat_f);      // ops_mat.h:7
void mat_mat(long long int np, double* mat_i1, double* mat_i2, double* mat_f);    // ops_mat.h:8
void mat_mat_T(long long int np, double* mat_i1, double* mat_i2, double* mat_f);  // ops_mat.h:9
void mat_T_mat(long long int np, double* mat_i1, double* mat_i2, double* mat_f);  // ops_mat.h:10
void trans_mat(int np, double* mat, double* trans, double* tmpmat, int dir);      // ops_mat.h:11
void trans_mat(long long int np, double* mat, double* trans, double* tmpmat, int dir);  // :12
void pmv(double* mat, double* vi, double* vo, int nroao);                   // ops_mat.h:13

#endif
