/*
 * corr_gb300 -- GB300 (sm_103a) implementation of the correlation hot path of
 * Masterluke87/corr: build_FMo, the AO->MO 4-index transform, canonical MP2,
 * the RI metric J^-1/2 and B build, the RI transform and the RI-MP2 energy,
 * plus an RI-MP2 adjoint and a batched RI-MP2 driver.
 *
 * Plain C ABI: opaque context handle, int status codes, caller-owned buffers
 * given as plain pointers with explicit sizes.  Every array argument may live
 * in host memory (pageable or pinned) or in device memory of the context's
 * GPU; the library detects which and stages host data through its own device
 * buffers.  Layouts are row-major and follow the reference's arrays:
 *   mos[p*N + mu]            MO coefficients, one MO per row (OEints::MOs)
 *   fmat, fmo [N*N]          Fock matrix in AO / MO basis (OEints::Fmat, pHF::FMo)
 *   bpq[(P*N + mu)*N + nu]   B^P_mu,nu                     (pHF::BPQ)
 *   bia[(Q*nocc + i)*nvir+a] B^Q_ia                        (pHF::Bia)
 *   prec[((i*N+j)*N+k)*N+l]  MO integrals (ij|kl)          (pHF::prec_ints)
 *   intval[n], intnums[4n], sortcount[4]  packed AO ERIs   (TEints)
 * Orbital energies eps[p] are the diagonal FMo[p*N+p] the reference reads.
 *
 * There is no CPU fallback: every entry point runs on the GPU or returns an
 * error status (CORR_ERR_NO_DEVICE when no GPU is visible).
 */
#ifndef CORR_GB300_H
#define CORR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum corr_status {
  CORR_OK = 0,
  CORR_ERR_BAD_ARG = 1,        /* invalid size, null pointer, bad enum value   */
  CORR_ERR_OOM = 2,            /* device allocation failed                     */
  CORR_ERR_NOT_PD = 3,         /* RI metric has no positive eigenvalue         */
  CORR_ERR_DEVICE_TIMEOUT = 4, /* a bounded device-side wait gave up           */
  CORR_ERR_CUDA = 5,           /* any other CUDA runtime error                 */
  CORR_ERR_NO_DEVICE = 6,      /* no usable sm_103 GPU                          */
  CORR_ERR_NUMERIC = 7,        /* non-finite input or zero energy denominator  */
  CORR_ERR_IO = 8              /* a file is missing, short or not writable     */
};

/* Arithmetic of the RI-MP2 contraction (ia|jb) = sum_Q B^Q_ia B^Q_jb. */
enum corr_precision {
  CORR_PREC_FP64 = 0,       /* FP64 end to end (FP64 mma.sync)                   */
  CORR_PREC_SPLIT_FP16 = 1, /* each row (i,a) of B scaled by a power of two and
                               split into two integer digits s0 + s1/L stored as
                               FP16 (|digit| <= 2048); the products s0.s0',
                               s0.s1' + s1.s0', s1.s1' on tcgen05 with exact
                               FP32 integer accumulation in TMEM; (ia|ia) to
                               FP64 accuracy; FP64 pair-energy sums.  The fast
                               form.                                             */
  CORR_PREC_SPLIT_BF16 = 2  /* three 7-bit integer digits per element stored as
                               BF16; the six digit products of orders 0-2 on
                               tcgen05, exact accumulation, (ia|ia) in FP64     */
};

typedef struct corr_context corr_context;

/* Closed-shell MP2 energy pieces, as printed by the reference
 * (can_mp2.cc:36-46, 114-125): E_SS, E_OS, E = E_SS + E_OS and the
 * spin-component-scaled E_SCS = E_SS/3 + 6/5 E_OS. */
typedef struct corr_mp2_energy {
  double e_ss;
  double e_os;
  double e_total;
  double e_scs;
} corr_mp2_energy;

/* ---- context ----------------------------------------------------------- */

/* Library version string. */
const char* corr_version(void);

/* Create a context bound to CUDA device `device`.  `stream` is a
 * cudaStream_t (NULL = the legacy default stream); all work of the context
 * is ordered on it.  Returns CORR_ERR_NO_DEVICE without a usable GPU. */
int corr_create(corr_context** ctx, int device, void* stream);

/* Release the context and every device buffer it owns. */
int corr_destroy(corr_context* ctx);

/* Re-bind the context to another stream. */
int corr_set_stream(corr_context* ctx, void* stream);

/* Human-readable description of the last error raised on this thread. */
const char* corr_last_error(void);

/* Number of SMs of the context's GPU. */
int corr_device_sm_count(const corr_context* ctx);

/* Per-call device timings (no reference counterpart; the reference only
 * prints wall-clock totals, src/main.cc:212-214).  With timing enabled every
 * call records CUDA events on the context stream around its stages. */
typedef struct corr_timing {
  float prepass_ms; /* input staging + slice pre-pass                          */
  float kernel_ms;  /* the dominant kernel of the call                         */
  float total_ms;   /* whole call on the device                                */
  long long launches_total; /* kernels this context has launched so far     */
} corr_timing;

int corr_set_timing(corr_context* ctx, int enable);
int corr_get_timing(const corr_context* ctx, corr_timing* out);

/* ---- RI-MP2 energy ----------------------------------------------------- */

/* Replaces run_canonical_mp2_ri (src/POSTHF/can_mp2.cc:53-132, declared at
 * src/POSTHF/can_mp2.h:5): E_OS = -sum (ia|jb)^2 / D,
 * E_SS = -sum [(ia|jb)-(ib|ja)](ia|jb) / D, D = e_a + e_b - e_i - e_j, with
 * (ia|jb) = sum_Q B^Q_ia B^Q_jb.  bia[(Q*nocc+i)*nvir+a] (pHF::Bia),
 * eps[nocc+nvir] (the diagonal of pHF::FMo).  The (ia|jb) tiles live only in
 * registers/TMEM; no 4-index tensor is stored.  `precision` is a
 * corr_precision. */
int corr_rimp2_energy(corr_context* ctx, int nocc, int nvir, int naux, const double* bia,
                      const double* eps, int precision, corr_mp2_energy* out);

/* corr_rimp2_energy plus an error estimate for the precision forms (no
 * reference counterpart: the reference computes in FP64): *err estimates the
 * deviation of E from the FP64 energy of the same inputs (one standard
 * deviation).  The deviation of a precision form is the rounding of B to its
 * digit grid, to first order sum_r delta_r . dE/dB_r; the call evaluates the
 * energy a second time on a grid one bit coarser per digit and scales the
 * difference by the variance ratio of the two roundings (sqrt 6 for
 * CORR_PREC_SPLIT_FP16, sqrt 65 for CORR_PREC_SPLIT_BF16).  Twice the cost of
 * corr_rimp2_energy.  CORR_PREC_FP64: *err = 0. */
int corr_rimp2_energy_estimate(corr_context* ctx, int nocc, int nvir, int naux, const double* bia,
                               const double* eps, int precision, corr_mp2_energy* out,
                               double* err);

/* Asynchronous form of corr_rimp2_energy for device-resident data (no
 * reference counterpart): bia and eps must be device pointers; the call only
 * enqueues work on the context stream and writes {E_SS, E_OS, E, E_SCS} to
 * the device buffer energies_dev[4].  It performs no host synchronisation,
 * so it can be captured into a CUDA graph once a first call with the same
 * sizes has sized the context workspace.  Device-side failures (a timed-out
 * wait) are reported by the next corr_sync. */
int corr_rimp2_energy_async(corr_context* ctx, int nocc, int nvir, int naux, const double* bia,
                            const double* eps, int precision, double* energies_dev);

/* Synchronise the context stream and return the device status accumulated
 * by asynchronous calls since the last corr_sync (CORR_OK or
 * CORR_ERR_DEVICE_TIMEOUT); clears it. */
int corr_sync(corr_context* ctx);

/* ---- batched RI-MP2 (no counterpart in the reference) ------------------- */

/* One independent RI-MP2 problem of a batch; bia [naux][nocc][nvir] and eps
 * [nocc+nvir] in device memory. */
typedef struct corr_rimp2_instance {
  int nocc, nvir, naux;
  const double* bia;
  const double* eps;
} corr_rimp2_instance;

/* Energies of n independent instances of uneven sizes.  The precision forms
 * run every instance's units through one persistent tcgen05 launch fed by a
 * device work queue (run_canonical_mp2_ri, src/POSTHF/can_mp2.cc:53, per
 * instance); the FP64 form runs the fused FP64 kernel per instance.  out[n]. */
int corr_rimp2_energy_batched(corr_context* ctx, int n, const corr_rimp2_instance* inst,
                              int precision, corr_mp2_energy* out);

/* Enqueue-only form, energies_dev[4*k+{0,1,2,3}] = {E_SS, E_OS, E, E_SCS} of
 * instance k.  After a first call with the same batch (which sizes the
 * workspaces) it can be captured into a CUDA graph. */
int corr_rimp2_energy_batched_async(corr_context* ctx, int n, const corr_rimp2_instance* inst,
                                    int precision, double* energies_dev);

/* Diagnostic (no counterpart in the reference): run the kernels' bounded-wait
 * path on purpose.  One CTA waits on an mbarrier phase that nothing completes,
 * with the same primitive every tcgen05-kernel wait uses, for limit_ms
 * (1..2000) milliseconds; the call then returns CORR_ERR_DEVICE_TIMEOUT and
 * the context remains usable. */
int corr_selftest_wait_timeout(corr_context* ctx, int limit_ms);

/* Tile shape of the tcgen05 energy kernel (no counterpart in the reference).
 * Accepts 0 or 1 and has no effect: every tile runs 128 wide, the padded
 * columns of the last virtual tile being zeros.  (A narrower last tile needs
 * a second MMA descriptor, which costs more on the issue path than the padded
 * columns save.) */
int corr_set_energy_tiles(corr_context* ctx, int tiles);

/* FP64 arithmetic of the plain-form metric calls (no counterpart in the
 * reference).  0 (the default): corr_ri_metric_inv_sqrt and corr_calculate_ri
 * compute J^-1/2 of a certified metric by Newton-Schulz and BPQ = J^-1/2 (Q|mn)
 * on the FP64-accurate digit GEMM (corr_dgemm_tc; 5e-11 from LAPACK's J^-1/2
 * on the 20-water cluster).  1: every product on the FP64 pipe and J^-1/2 by
 * the eigendecomposition -- IEEE FP64 end to end, several times slower. */
int corr_set_fp64_strict(corr_context* ctx, int strict);

/* Launch variant of the batched kernel: unit order (0 = input order,
 * 1 = costliest instance first) and shared-memory pipeline depth in stages of
 * one 64-wide Q block (2 or 3; the three-digit form always runs 2).  tiles (0
 * or 1) is accepted and has no effect, as in corr_set_energy_tiles. */
int corr_set_batch_policy(corr_context* ctx, int order, int stages, int tiles);

/* Time every launch variant on this batch (order x stages; median of three
 * runs after a warm-up), keep the fastest in the context and report it (any
 * output pointer may be NULL; *tiles reports the value last set). */
int corr_rimp2_batch_autotune(corr_context* ctx, int n, const corr_rimp2_instance* inst,
                              int precision, int* order, int* stages, int* tiles, float* ms);

/* RI-MP2 adjoint (no counterpart in the reference, which has no gradients):
 * dbia[(Q*nocc+i)*nvir+a] = dE/dB^Q_ia and deps[p] = dE/d eps_p for
 * E = E_OS + E_SS of corr_rimp2_energy, in FP64.  The (ia|jb) tiles are
 * recomputed, never stored: per block of occupied orbitals a transient panel
 * G^{ij}_ab = -(4 (ia|jb) - 2 (ib|ja)) / D (at most ~1 GiB) feeds one GEMM
 * dB = 2 B G^T; dE/d eps comes from W = (2(ia|jb) - (ib|ja))(ia|jb)/D^2.
 * e_out (optional) receives E in e_total. */
int corr_rimp2_gradient(corr_context* ctx, int nocc, int nvir, int naux, const double* bia,
                        const double* eps, double* dbia, double* deps, corr_mp2_energy* e_out);

/* corr_rimp2_gradient on the tensor cores: per block of occupied orbitals the
 * panel (ia|jb) by the FP64-accurate digit GEMM (corr_dgemm_tc), G, W and E
 * in place, and dB = 2 B G^T by the digit GEMM; the same outputs to the digit
 * GEMM's accuracy (~FP64), at tensor-core speed.  nvir <= 6144.  The adjoint
 * of the precision forms (the autograd backward of a split-precision
 * forward). */
int corr_rimp2_gradient_tc(corr_context* ctx, int nocc, int nvir, int naux, const double* bia,
                           const double* eps, double* dbia, double* deps, corr_mp2_energy* e_out);

/* Allocation-free RI-MP2 energy (no counterpart in the reference).  For
 * callers that cannot call cudaMalloc -- a host program whose device memory is
 * all handed out by its own pool allocator, or a latency-critical loop where an
 * allocation and its implicit synchronisation are not allowed.  Same kernels
 * and results as corr_rimp2_energy, but no context and no allocation: the
 * scratch is a fixed 32 MiB device array compiled into the library, which every
 * GPU that loads the library holds until the process exits.  Limit: the
 * precision forms need about 6*nocc*nvir*naux bytes of scratch and larger
 * problems are rejected with CORR_ERR_BAD_ARG; the FP64 form needs only a few
 * KB.  bia and eps must be device pointers of `device`; `stream` is a
 * cudaStream_t; the call returns after the stream has finished the work and
 * writes the energies to the host struct `out`.  Its first call on a device
 * looks up the array's device address and sets kernel attributes there: make
 * it before any stream capture on that device.  All calls share the array:
 * calls whose GPU work overlaps race and must be serialised by the caller. */
int corr_rimp2_energy_noalloc(int device, void* stream, int nocc, int nvir, int naux,
                              const double* bia, const double* eps, int precision,
                              corr_mp2_energy* out);

/* ---- FP64 transforms and canonical MP2 ---------------------------------- */

/* Replaces build_FMo (src/POSTHF/motrans.cc:8-32, declared at
 * src/POSTHF/motrans.h:22): fmo[i*N+j] = sum_{mu,nu} mos[i*N+mu] fmat[mu*N+nu]
 * mos[j*N+nu], as two FP64 GEMMs.  The caller owns fmo (N*N). */
int corr_build_fmo(corr_context* ctx, int nroao, const double* mos, const double* fmat,
                   double* fmo);

/* Replaces MOtrans (src/POSTHF/motrans.cc:35-211, declared at
 * src/POSTHF/motrans.h:21): prec[((i*N+j)*N+k)*N+l] = (ij|kl) over all MOs from
 * the reference's packed AO list (TEints: intval, intnums, sortcount as produced
 * by resort_integrals, src/SCF/ops_rhf.cc:750-900).  The caller owns prec (N^4
 * doubles; the reference allocated it inside MOtrans).  N <= 65535. */
int corr_motrans(corr_context* ctx, int nroe, int nroao, const double* mos, long long nrofint,
                 const long long* sortcount, const double* intval,
                 const unsigned short* intnums, double* prec);

/* The (ia|jb) block only, ovov[((i*nvir+a)*nocc+j)*nvir+b], through four
 * quarter transforms of cost 2oN^4 + 2ovN^3 + 2o^2vN^2 + 2o^2v^2N.  Same sums as
 * corr_motrans restricted to occupied/virtual index ranges. */
int corr_motrans_ovov(corr_context* ctx, int nroe, int nroao, const double* mos,
                      long long nrofint, const long long* sortcount, const double* intval,
                      const unsigned short* intnums, double* ovov);

/* Replaces run_canonical_mp2 (src/POSTHF/can_mp2.cc:11-49, declared at
 * src/POSTHF/can_mp2.h:4) on the full MO tensor prec (corr_motrans layout);
 * eps[nroao] = diagonal of FMo. */
int corr_canonical_mp2(corr_context* ctx, int nroe, int nroao, const double* prec,
                       const double* eps, corr_mp2_energy* out);

/* The same energy from an (ia|jb) block in corr_motrans_ovov layout. */
int corr_canonical_mp2_ovov(corr_context* ctx, int nocc, int nvir, const double* ovov,
                            const double* eps, corr_mp2_energy* out);

/* Replaces transform_ri (src/POSTHF/ri.cc:147-172, declared at
 * src/POSTHF/ri.h:9): bia[(Q*o+i)*v+a] = sum_{mu,nu} mos[i*N+mu]
 * bpq[(Q*N+mu)*N+nu] mos[(o+a)*N+nu], o = nroe/2, v = nroao - o.  naux <= 65535. */
int corr_transform_ri(corr_context* ctx, int nroe, int nroao, int naux, const double* mos,
                      const double* bpq, double* bia);

/* The B build of calculate_ri (src/POSTHF/ri.cc:102-103):
 * bpq[P][mu][nu] = sum_Q jm12[P][Q] pmn[Q][mu][nu]. */
int corr_ri_build_bpq(corr_context* ctx, int naux, int nroao, const double* jm12,
                      const double* pmn, double* bpq);

/* ---- RI metric ----------------------------------------------------------- */

/* The J^-1/2 part of calculate_ri (src/POSTHF/ri.cc:50-69): eigen-decompose
 * J (naux x naux, symmetric), zero every eigenvalue with lambda/lambda_max <
 * tol or lambda < 0 (the reference uses tol = 1e-10), take lambda^-1/2 of the
 * rest and return jm12 = V diag V^T.  FP64 throughout (parallel Jacobi
 * eigensolver).  *ncut (optional) receives the number of eigenvalues cut.
 * CORR_ERR_NOT_PD when J has no positive eigenvalue. */
int corr_ri_metric_inv_sqrt(corr_context* ctx, int naux, const double* J, double tol,
                            double* jm12, int* ncut);

/* Replaces calculate_ri (src/POSTHF/ri.cc:7-106, declared at src/POSTHF/ri.h:8)
 * downstream of the integral engine: given the 2-index metric J[P][Q] = (P|Q)
 * and the 3-index integrals pmn[P][mu][nu] = (P|mu nu) (the reference computes
 * both with libint inside calculate_ri, ri.cc:25-47, 70-100), returns
 * bpq = J^-1/2 (Q|mu nu) with the reference's eigenvalue cutoff. */
int corr_calculate_ri(corr_context* ctx, int naux, int nroao, const double* J, const double* pmn,
                      double* bpq);

/* out[P][k] = sum_Q jm12[P][Q] in[Q][k] for k < ncols: the metric step of
 * ri.cc:102-103 applied after the MO transform, on (P|ia) (ncols = nocc*nvir)
 * instead of (P|mu nu) -- 2 naux^2 nocc nvir flops instead of 2 naux^2 N^2.
 * No reference counterpart (the reference applies J^-1/2 in the AO basis). */
int corr_ri_apply_metric(corr_context* ctx, int naux, long long ncols, const double* jm12,
                         const double* in, double* out);

/* A basis of contracted Gaussian shells, as a libint2::BasisSet holds it:
 * shell s has angular momentum l[s] (0..3), nprim[s] primitives with
 * exponents exps[poff[s] + k] and contraction coefficients coefs[poff[s] + k]
 * of normalised primitives (the numbers of a basis-set file), centred at
 * center[3s..3s+2] (bohr).  Its functions are the real solid harmonics
 * m = -l..l of each shell in shell order, each normalised to one; Cartesian
 * components are ordered lx = l..0, ly = l-lx..0. */
typedef struct corr_basis {
  int nsh;
  const int* l;
  const int* nprim;
  const int* poff;
  const double* center;
  const double* exps;
  const double* coefs;
} corr_basis;

/* The integrals calculate_ri computes with libint (src/POSTHF/ri.cc:25-47,
 * 70-100; the psi4 plugin's syshfwplug/plugin.cc:478-503), on the GPU:
 * J[P][Q] = (P|Q) over the auxiliary basis and pmn[P][mu][nu] = (P|mu nu)
 * (orbital shells up to d), McMurchie-Davidson in FP64.  Either output may be
 * NULL; obs may be NULL when pmn is.  The outputs feed
 * corr_rimp2_energy_from_3index / corr_calculate_ri directly (keep them on the
 * device: (P|mu nu) is the largest hand-off of the RI path). */
int corr_ri_integrals(corr_context* ctx, const corr_basis* obs, const corr_basis* aux, double* J,
                      double* pmn);

/* The RI-MP2 energy from integrals, all on the GPU: (P|ia) from
 * pmn[P][mu][nu] = (P|mu nu) and the MO coefficients (the contractions of
 * transform_ri, ri.cc:147-172), J^-1/2 with the reference's cutoff
 * (ri.cc:50-69), B = J^-1/2 (P|ia), and the energy of run_canonical_mp2_ri
 * (can_mp2.cc:53) in `precision`.  Equals calculate_ri + transform_ri +
 * run_canonical_mp2_ri whenever no eigenvalue is cut. *ncut optional. */
int corr_rimp2_energy_from_3index(corr_context* ctx, int nroe, int nroao, int naux,
                                  const double* mos, const double* eps, const double* J,
                                  const double* pmn, int precision, corr_mp2_energy* out,
                                  int* ncut);

/* ---- RHF on the GPU (src/SCF) ------------------------------------------- */

/* Replaces build_Fmat (src/SCF/ops_rhf.cc:549-591): the closed-shell Fock
 * matrix fmat = hmat + sum_ls pmat[ls] ((mn|ls) - 1/2 (ml|ns)) from the packed
 * unique integrals (intval, intnums, sortcount: the .tei layout that
 * corr_motrans reads).  Every array may be host or device memory.  The
 * integral list is expanded once into the dense nroao^4 tensor on the device
 * (nroao^4 doubles of workspace); each F_mn is a fixed-order sum. */
int corr_build_fmat(corr_context* ctx, int nroao, const double* pmat, const double* hmat,
                    long long nrofint, const long long* sortcount, const double* intval,
                    const unsigned short* intnums, double* fmat);

/* Replaces run_scf (src/SCF/scf.cc:145-321) with its fixed settings: damped
 * density (damp 0.5, P = 2(1-damp) C_occ C_occ^T + damp P), Fock build, DIIS
 * over 8 Fock/error pairs (error S P F - F P S, started once the mean |error|
 * is below 1e-3 from the 8th iteration on, damping then off; dgels-style
 * least-squares solve), symmetric orthogonalisation with S^-1/2 (calc_S12,
 * ops_rhf.cc:342-378) and diagonalisation (diag_Fmat, ops_rhf.cc:425-431),
 * until |dE| <= 1e-8 or maxiter iterations.  mos (nroao x nroao, orbitals as
 * rows) is the guess on entry; when |sum_i mos[i][i]| < 0.1 the core guess
 * (diagonalised hmat, check_initial_guess, ops_rhf.cc:15-36) replaces it.  On
 * return: mos, fmat (rebuilt from the final density, scf.cc:289-290), moens
 * (the last diagonalisation's orbital energies; unchanged when none ran),
 * energies[3] = {TOTAL E, ONE E, TWO E} as run_scf prints them
 * (scf.cc:305-314) and, if pmat is non-null, that final density (onemats->Pmat
 * of the reference).  *iterations optional.  The overlap must be positive
 * definite (CORR_ERR_BAD_ARG otherwise; the reference would divide by the
 * square root of a non-positive eigenvalue).  Runs all on the device; host or
 * device arrays; nroao <= 2048; its own device allocation of nroao^4 +
 * 28 nroao^2 doubles plus the integral list. */
int corr_run_scf(corr_context* ctx, int nroe, int nroao, double ion_rep, const double* smat,
                 const double* hmat, long long nrofint, const long long* sortcount,
                 const double* intval, const unsigned short* intnums, int maxiter, double* mos,
                 double* fmat, double* moens, double* energies, int* iterations, double* pmat);

/* ---- dense FP64 helpers (src/MATH/ops_mat.cc) ---------------------------- */

/* C = alpha op(A) op(B) + beta C, all row-major FP64: op(A) is m x k (A stored
 * m x k with lda >= k, or k x m with lda >= m when transa = 1), op(B) is k x n
 * (B stored k x n, ldb >= n, or n x k, ldb >= k when transb = 1), ldc >= n.
 * One kernel on the FP64 tensor path.  Covers the reference's mat_mat_T
 * (ops_mat.cc:93-105, :122-134: transb = 1), mat_T_mat (ops_mat.cc:107-119,
 * :136-148: transa = 1), symmortho_mat (ops_mat.cc:53-69: two calls),
 * transform_MOs (ops_mat.cc:75-88: mos tmat^T) and pmv (ops_mat.cc:192-198:
 * n = 1).  When C is a host pointer and beta != 0 it is read first. */
int corr_dgemm(corr_context* ctx, int transa, int transb, int m, int n, int k, double alpha,
               const double* A, int lda, const double* B, int ldb, double beta, double* C,
               int ldc);

/* corr_dgemm on the tensor cores, FP64-accurate: both operands are split
 * exactly into eight balanced 7-bit integer digits per row of op(A) and per
 * column of op(B) (scaled by the row's / column's largest binary exponent),
 * the 36 digit products of significance up to 2^-56 run as BF16 tcgen05 MMAs
 * whose level sums are exact in FP32 (K in passes of 512), and the levels are
 * recombined in 64-bit integers with one rounding to FP64.  Error per element
 * <= ~2^-53 sqrt(k) max|A row| max|B column| -- comparable to an FP64 GEMM for
 * data without a wide range inside a row; elements much smaller than their
 * row/column scales carry a larger relative error than in FP64.  Inputs must
 * be finite.  Same arguments as corr_dgemm. */
int corr_dgemm_tc(corr_context* ctx, int transa, int transb, int m, int n, int k, double alpha,
                  const double* A, int lda, const double* B, int ldb, double beta, double* C,
                  int ldc);

/* Replaces diag_mat (ops_mat.cc:21-45, LAPACK dsyev with JOBZ='V'): the
 * eigenvalues of the symmetric n x n matrix A in ascending order in w[n], and
 * vecs[k*n + i] = component i of the eigenvector of w[k] (dsyev's column-major
 * output read row-major).  Cyclic Jacobi in FP64 on the GPU; each eigenvector's
 * sign is arbitrary, as LAPACK's.  A is not modified.  n <= 32768. */
int corr_syev(corr_context* ctx, int n, const double* A, double* w, double* vecs);

/* ---- CCSD consumer of the MO integrals (src/POSTHF/ccsd.cc) -------------- */

/* Replaces calc_ints_so (src/POSTHF/ccsd.cc:509-535, with get_integral,
 * ccsd.cc:6-9): the antisymmetrized spin-orbital integrals
 * ints_so[((i*M + j)*M + k)*M + l] = <ij||kl>, M = 2 nroao spin orbitals
 * (spin p % 2, spatial orbital p / 2), from prec (corr_motrans layout; keep it
 * on the device to skip the N^4 host round trip).  16 nroao^4 doubles out. */
int corr_ints_so(corr_context* ctx, int nroao, const double* prec, double* ints_so);

/* Replaces form_fock (ccsd.cc:11-48): the spin-orbital core Hamiltonian
 * h_so[p*M + q] = (C H C^T)_{p/2,q/2} [same spin] and Fock matrix
 * f_so = h_so + sum_{j < nroe} <pj||qj>, from mos[p*N + mu], hmat[N*N] and
 * prec; M = 2 nroao. */
int corr_cc_fock(corr_context* ctx, int nroe, int nroao, const double* mos, const double* hmat,
                 const double* prec, double* h_so, double* f_so);

/* ---- on-disk hand-off files (src/IO/ops_io.cc) --------------------------- */

/* System description of PREFIX.sys. */
typedef struct corr_system_info {
  int nroe, nroa, nroao, naux_1, naux_2;
  long long nrofint, nrofaux, nrofaux2;
  char basis_ob[33], basis_jk[33], basis_ri[33];
} corr_system_info;

/* Replaces read_system (src/IO/ops_io.cc:63-109, declared at src/IO/ops_io.h:37):
 * the sizes of PREFIX.sys into *info; with coord[3 nroa], charges, zeff and
 * mass[nroa] (host arrays, all four or none) also the atoms and the three
 * 32-byte basis-name fields.  Call once with NULL arrays to learn nroa. */
int corr_read_system(const char* prefix, corr_system_info* info, double* coord, double* charges,
                     double* zeff, double* mass);

/* Replaces read_oei (ops_io.cc:112-121, ops_io.h:38): H, T, S, V (nroao^2
 * each) from PREFIX.oei.  The files readers below take host or device arrays
 * (device arrays of ctx's GPU stream through pinned chunks; ctx may be NULL
 * when every array is host memory) and return CORR_ERR_IO for a missing or
 * short file. */
int corr_read_oei(corr_context* ctx, const char* prefix, int nroao, double* hmat, double* tmat,
                  double* smat, double* vmat);

/* Replaces read_tei (ops_io.cc:203-212, ops_io.h:39): the packed AO ERIs of
 * PREFIX.tei (sortcount[4], intval[nrofint], intnums[4 nrofint]), the input
 * of corr_motrans. */
int corr_read_tei(corr_context* ctx, const char* prefix, long long nrofint, long long* sortcount,
                  double* intval, unsigned short* intnums);

/* Replaces read_wav_HF (ops_io.cc:283-299, ops_io.h:34): MO energies and
 * coefficients from PREFIX.ahfw; CORR_ERR_BAD_ARG when the file holds another
 * orbital count (the reference exits there). */
int corr_read_wav_hf(corr_context* ctx, const char* prefix, int nroao, double* moens,
                     double* mos);

/* Replaces write_wav_HF (ops_io.cc:259-267, ops_io.h:33): writes the file
 * `path` (host arrays). */
int corr_write_wav_hf(const char* path, int nroao, const double* moens, const double* mos);

/* BPQ[naux][nroao][nroao] from PREFIX.rimp2, the file read_transform_ri reads
 * (src/POSTHF/ri.cc:109-119). */
int corr_read_rimp2(corr_context* ctx, const char* prefix, int naux, int nroao, double* bpq);

#ifdef __cplusplus
}
#endif
#endif /* CORR_GB300_H */
