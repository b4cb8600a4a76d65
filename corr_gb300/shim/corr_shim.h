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

#ifdef CORR_SHIM_USE_REFERENCE_HEADERS
#include "UTIL/util.h"
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

#endif
