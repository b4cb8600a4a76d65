/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A plain-C restatement of the reference's hot-path algorithms (Masterluke87/corr,
 * src/POSTHF and src/SCF), used only by tests/, the smoke check and the CPU
 * baseline leg of bench.py as the thing results are checked against.  Each
 * function names the reference lines it follows.  Parity of this restatement is
 * pinned against the reference's own compiled sources (oracle/_ref, built by
 * oracle/Makefile) through tests/test_oracle_pin.py and the committed golden
 * fixtures under tests/golden/.
 *
 * Layouts (all row-major, as in the reference):
 *   mos[p*N + mu]          MO coefficient C_mu,p   (pHF/OEints MOs, util.h:47-59)
 *   eri[((a*N+b)*N+c)*N+d] AO integral (ab|cd), chemist notation
 *   prec[((i*N+j)*N+k)*N+l] MO integral (ij|kl)    (motrans.cc:49-71)
 *   intval[n], intnums[4n], sortcount[4]           (util.h:61-65)
 *   bpq[(P*N+mu)*N+nu]     B^P_mu,nu               (ri.cc:102-103)
 *   bia[(Q*o+i)*v+a]       B^Q_ia                  (ri.cc:147-172)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef long long i64;
typedef unsigned short u16;

/* --------------------------------------------------------------------------
 * Packed AO-ERI list.
 * src/SCF/ops_rhf.cc:618-723 selects (ab|cd) with a>=b, c>=d,
 * a(a+1)/2+b >= c(c+1)/2+d and |v| > 1e-12 (after a Schwarz pre-screen of
 * shell pairs, ops_rhf.cc:680, which for one-function shells keeps every pair
 * whose diagonal product is >= 1e-12); loop order s2, s1>=s2, s4, s3>=s4.
 * ops_rhf.cc:750-900 then canonicalises the index order and partitions the list
 * into five permutation classes.
 * ------------------------------------------------------------------------ */
static void swap_entry(i64 x, i64 y, double* val, u16* num) {
  double tv = val[x];
  val[x] = val[y];
  val[y] = tv;
  for (int k = 0; k < 4; ++k) {
    u16 t = num[x * 4 + k];
    num[x * 4 + k] = num[y * 4 + k];
    num[y * 4 + k] = t;
  }
}

/* ops_rhf.cc:750-900 (resort_integrals). */
void oracle_resort(u16* num, double* val, i64 n, i64* sortcount) {
  for (i64 x = 0; x < n; ++x) {
    u16* q = num + 4 * x;
    u16 a = q[0], b = q[1], c = q[2], d = q[3];
    /* The eight in-place rewrites are applied one after another, each testing
     * the ORIGINAL a,b,c,d (ops_rhf.cc:756-817). */
    if (a == b && b == d && c != d) { q[0] = a; q[1] = a; q[2] = a; q[3] = c; }
    if (a != b && a == c && c == d) { q[0] = a; q[1] = a; q[2] = a; q[3] = b; }
    if (a != b && b == c && c == d) { q[0] = b; q[1] = b; q[2] = b; q[3] = a; }
    if (a == d && b == c && a != b) { q[0] = a; q[1] = b; q[2] = d; q[3] = c; }
    if (b == c && b != a && b != d && a != d) { q[0] = b; q[1] = a; q[2] = c; q[3] = d; }
    if (c == d && c != a && c != b && a != b) { q[0] = c; q[1] = c; q[2] = a; q[3] = b; }
    if (a == d && a != b && a != c && b != c) { q[0] = a; q[1] = b; q[2] = d; q[3] = c; }
    if (b == d && b != a && b != c && a != c) { q[0] = b; q[1] = a; q[2] = d; q[3] = c; }
  }
  i64 sorted = 0;
  for (i64 x = 0; x < n; ++x) { /* (aa|aa) */
    u16* q = num + 4 * x;
    if (q[0] == q[1] && q[1] == q[2] && q[2] == q[3]) swap_entry(x, sorted++, val, num);
  }
  sortcount[0] = sorted;
  for (i64 x = sorted; x < n; ++x) { /* (aa|cc) */
    u16* q = num + 4 * x;
    if (q[0] == q[1] && q[2] == q[3]) swap_entry(x, sorted++, val, num);
  }
  sortcount[1] = sorted;
  for (i64 x = sorted; x < n; ++x) { /* (ab|ab) */
    u16* q = num + 4 * x;
    if (q[0] == q[2] && q[1] == q[3]) swap_entry(x, sorted++, val, num);
  }
  sortcount[2] = sorted;
  for (i64 x = sorted; x < n; ++x) { /* (aa|cd) */
    u16* q = num + 4 * x;
    if (q[0] == q[1]) swap_entry(x, sorted++, val, num);
  }
  sortcount[3] = sorted;
}

/* Unique-integral selection of ops_rhf.cc:618-723 for one-function shells.
 * Returns the count; with val == NULL only counts. */
i64 oracle_pack_eri(int N, const double* eri, double* val, u16* num) {
  double* sw = (double*)malloc(sizeof(double) * (size_t)N * N);
  /* Schwarz estimate per pair: the reference tracks sqrt|(s1 s2|s3 s4)| of
   * the last shell quartet with s1==s3, s2==s4 (ops_rhf.cc:648-667).  For one
   * function per shell that is sqrt|(ab|ab)|. */
  for (int a = 0; a < N; ++a)
    for (int b = 0; b < N; ++b) {
      double v = fabs(eri[(((size_t)a * N + b) * N + a) * N + b]);
      sw[(size_t)a * N + b] = v > 0.0 ? sqrt(v) : 0.0;
    }
  i64 count = 0;
  for (int s2 = 0; s2 < N; ++s2)
    for (int s1 = s2; s1 < N; ++s1)
      for (int s4 = 0; s4 < N; ++s4)
        for (int s3 = s4; s3 < N; ++s3) {
          if (sw[(size_t)s1 * N + s2] * sw[(size_t)s3 * N + s4] < 1e-12) continue;
          i64 ab = (i64)s1 * (s1 + 1) / 2 + s2, cd = (i64)s3 * (s3 + 1) / 2 + s4;
          if (ab < cd) continue;
          double v = eri[(((size_t)s1 * N + s2) * N + s3) * N + s4];
          if (!(fabs(v) > 1e-12)) continue;
          if (val) {
            val[count] = v;
            num[4 * count + 0] = (u16)s1;
            num[4 * count + 1] = (u16)s2;
            num[4 * count + 2] = (u16)s3;
            num[4 * count + 3] = (u16)s4;
          }
          ++count;
        }
  free(sw);
  return count;
}

/* Dense (ab|cd) from the packed list: the permutation multiset that
 * motrans.cc:341-403 (trans_I) scatters for each class, added into a zeroed
 * N^4 array. */
void oracle_unpack_eri(int N, i64 n, const i64* sc, const double* val, const u16* num,
                       double* eri) {
  size_t N1 = (size_t)N, N2 = N1 * N1, N3 = N2 * N1;
  memset(eri, 0, sizeof(double) * N3 * N1);
#define AT(p, q, r, s) eri[(size_t)(p) * N3 + (size_t)(q) * N2 + (size_t)(r) * N1 + (size_t)(s)]
  for (i64 x = 0; x < n; ++x) {
    const u16* q = num + 4 * x;
    int a = q[0], b = q[1], c = q[2], d = q[3];
    double v = val[x];
    AT(a, b, c, d) += v;                        /* (1) every class */
    if (x < sc[0]) continue;
    if (x < sc[1]) { AT(c, d, a, b) += v; continue; }          /* PERM_15   */
    if (x < sc[2]) {                                            /* PERM_1234 */
      AT(a, b, d, c) += v; AT(b, a, c, d) += v; AT(b, a, d, c) += v;
      continue;
    }
    if (x < sc[3]) {                                            /* PERM_1256 */
      AT(a, b, d, c) += v; AT(c, d, a, b) += v; AT(d, c, a, b) += v;
      continue;
    }
    AT(a, b, d, c) += v; AT(b, a, c, d) += v; AT(b, a, d, c) += v;  /* PERM_ALL */
    AT(c, d, a, b) += v; AT(d, c, a, b) += v; AT(c, d, b, a) += v; AT(d, c, b, a) += v;
  }
#undef AT
}

/* One quarter transform: out[i][r][s][t] = sum_a C[i][a] in[a][r][s][t] with
 * the transformed index rotated to the back, so four calls produce (ij|kl). */
static void quarter(int N, const double* mos, const double* in, double* out) {
  size_t N1 = (size_t)N, N3 = N1 * N1 * N1;
  /* in viewed as [a][rest]; out[rest][i] = sum_a in[a][rest] * C[i][a] */
#pragma omp parallel for schedule(static)
  for (i64 r = 0; r < (i64)N3; ++r) {
    for (int i = 0; i < N; ++i) {
      double s = 0.0;
      for (int a = 0; a < N; ++a) s += in[(size_t)a * N3 + r] * mos[(size_t)i * N + a];
      out[(size_t)r * N + i] = s;
    }
  }
}

/* motrans.cc:35-71 + 341-503: prec[i][j][k][l] = sum C_ia C_jb C_kc C_ld (ab|cd),
 * from the packed list (dense unpack, then four quarter transforms). */
void oracle_motrans(int N, const double* mos, i64 n, const i64* sc, const double* val,
                    const u16* num, double* prec) {
  size_t N4 = (size_t)N * N * N * N;
  double* t0 = (double*)malloc(sizeof(double) * N4);
  double* t1 = (double*)malloc(sizeof(double) * N4);
  oracle_unpack_eri(N, n, sc, val, num, t0);
  quarter(N, mos, t0, t1); /* [b][c][d][i] */
  quarter(N, mos, t1, t0); /* [c][d][i][j] */
  quarter(N, mos, t0, t1); /* [d][i][j][k] */
  quarter(N, mos, t1, prec); /* [i][j][k][l] */
  free(t0);
  free(t1);
}

/* motrans.cc:286-327 calc_mo2int_bf (single element). */
double oracle_mo2int_bf(int i, int j, int k, int l, int N, const double* m, i64 n, const i64* sc,
                        const double* val, const u16* num) {
  const double *I = m + (size_t)i * N, *J = m + (size_t)j * N, *K = m + (size_t)k * N,
               *L = m + (size_t)l * N;
  double s = 0.0;
  for (i64 x = 0; x < n; ++x) {
    const u16* q = num + 4 * x;
    int a = q[0], b = q[1], c = q[2], d = q[3];
    double v = val[x];
    double t = I[a] * J[b] * K[c] * L[d];
    if (x >= sc[0] && x < sc[1]) t += I[c] * J[d] * K[a] * L[b];
    else if (x >= sc[1] && x < sc[2])
      t += I[a] * J[b] * K[d] * L[c] + I[b] * J[a] * K[c] * L[d] + I[b] * J[a] * K[d] * L[c];
    else if (x >= sc[2] && x < sc[3])
      t += I[a] * J[b] * K[d] * L[c] + I[c] * J[d] * K[a] * L[b] + I[d] * J[c] * K[a] * L[b];
    else if (x >= sc[3])
      t += I[a] * J[b] * K[d] * L[c] + I[b] * J[a] * K[c] * L[d] + I[b] * J[a] * K[d] * L[c] +
           I[c] * J[d] * K[a] * L[b] + I[d] * J[c] * K[a] * L[b] + I[c] * J[d] * K[b] * L[a] +
           I[d] * J[c] * K[b] * L[a];
    s += t * v;
  }
  return s;
}

/* can_mp2.cc:11-49 run_canonical_mp2: out = {E_SS, E_OS, E}. */
void oracle_canonical_mp2(int nroe, int N, const double* prec, const double* fmo, double* out) {
  int o = nroe / 2;
  size_t ks = (size_t)N, js = ks * N, is = js * N;
  double eos = 0.0, ess = 0.0;
  for (int i = 0; i < o; ++i)
    for (int j = 0; j < o; ++j)
      for (int a = o; a < N; ++a)
        for (int b = o; b < N; ++b) {
          double iajb = prec[i * is + a * js + j * ks + b];
          double ibja = prec[i * is + b * js + j * ks + a];
          double den = fmo[(size_t)a * N + a] + fmo[(size_t)b * N + b] - fmo[(size_t)i * N + i] -
                       fmo[(size_t)j * N + j];
          eos += -(iajb * iajb) / den;
          ess += -(iajb - ibja) * iajb / den;
        }
  out[0] = ess;
  out[1] = eos;
  out[2] = ess + eos;
}

/* Same energy from an (ia|jb) block stored [i][a][j][b] (o*v*o*v). */
void oracle_mp2_from_ovov(int o, int v, const double* ovov, const double* eps, double* out) {
  size_t V = (size_t)v, s3 = V * o * V;
  double eos = 0.0, ess = 0.0;
  for (int i = 0; i < o; ++i)
    for (int j = 0; j < o; ++j)
      for (int a = 0; a < v; ++a)
        for (int b = 0; b < v; ++b) {
          double iajb = ovov[i * s3 + a * (size_t)o * V + j * V + b];
          double ibja = ovov[i * s3 + b * (size_t)o * V + j * V + a];
          double den = eps[o + a] + eps[o + b] - eps[i] - eps[j];
          eos += -(iajb * iajb) / den;
          ess += -(iajb - ibja) * iajb / den;
        }
  out[0] = ess;
  out[1] = eos;
  out[2] = ess + eos;
}

/* motrans.cc:8-32 build_FMo: FMo[i][j] = sum_{mu,nu} C[i][mu] F[mu][nu] C[j][nu]. */
void oracle_build_fmo(int N, const double* mos, const double* f, double* fmo) {
  double* t = (double*)malloc(sizeof(double) * (size_t)N * N);
  for (int i = 0; i < N; ++i)
    for (int nu = 0; nu < N; ++nu) {
      double s = 0.0;
      for (int mu = 0; mu < N; ++mu) s += mos[(size_t)i * N + mu] * f[(size_t)mu * N + nu];
      t[(size_t)i * N + nu] = s;
    }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double s = 0.0;
      for (int nu = 0; nu < N; ++nu) s += t[(size_t)i * N + nu] * mos[(size_t)j * N + nu];
      fmo[(size_t)i * N + j] = s;
    }
  free(t);
}

/* ri.cc:147-172 transform_ri: BiQ[Q][i][nu] = sum_mu C[i][mu] BPQ[Q][mu][nu];
 * Bia[Q][i][a] = sum_nu C[o+a][nu] BiQ[Q][i][nu]. */
void oracle_transform_ri(int nroe, int N, int X, const double* mos, const double* bpq,
                         double* bia) {
  int o = nroe / 2, v = N - o;
#pragma omp parallel
  {
    double* biq = (double*)malloc(sizeof(double) * (size_t)o * N);
#pragma omp for schedule(static)
    for (int Q = 0; Q < X; ++Q) {
      const double* b = bpq + (size_t)Q * N * N;
      memset(biq, 0, sizeof(double) * (size_t)o * N);
      for (int i = 0; i < o; ++i)
        for (int mu = 0; mu < N; ++mu) {
          double c = mos[(size_t)i * N + mu];
          const double* row = b + (size_t)mu * N;
          double* dst = biq + (size_t)i * N;
          for (int nu = 0; nu < N; ++nu) dst[nu] += c * row[nu];
        }
      for (int i = 0; i < o; ++i)
        for (int a = 0; a < v; ++a) {
          double s = 0.0;
          const double* c = mos + (size_t)(o + a) * N;
          for (int nu = 0; nu < N; ++nu) s += c[nu] * biq[(size_t)i * N + nu];
          bia[((size_t)Q * o + i) * v + a] = s;
        }
    }
    free(biq);
  }
}
