/*
 * ORACLE -- test infrastructure, not product code.
 *
 * Gaussian integrals over contracted spherical shells (McMurchie-Davidson
 * scheme with Hermite Gaussians, as in Helgaker, Joergensen, Olsen,
 * "Molecular Electronic-Structure Theory", ch. 9; Boys function by series
 * plus downward recursion, large-argument asymptotics plus upward recursion).
 * It stands in for libint 2.4.2, which the reference uses
 * (src/SCF/ops_rhf.cc:66-253, 618-723; src/POSTHF/ri.cc:25-47, 70-100) and
 * which is not available here, to produce realistic molecular inputs for the
 * H2O and water-cluster workloads.  Integral values are not part of the
 * accelerated path and are not pinned to libint.
 *
 * Shells are passed as flat arrays: l[s], nprim[s], poff[s] (offset into
 * exps/coefs), center[3s].  Coefficients already include the primitive
 * radial normalisation; every spherical function is normalised afterwards by
 * the caller from its self-overlap.  Cartesian components are ordered
 * lx = l..0, ly = l-lx..0; spherical components m = -l..l.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define LMAX 3
#define HMAX 13 /* Hermite orders up to 12 */

static inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }

/* ------------------------------------------------------------------------ */
/* Boys function F_n(T), n = 0..nmax                                        */
/* ------------------------------------------------------------------------ */
static void boys(int nmax, double T, double* F) {
  if (T < 1e-14) {
    for (int n = 0; n <= nmax; ++n) F[n] = 1.0 / (2 * n + 1);
    return;
  }
  const double et = exp(-T);
  if (T < 35.0) {
    /* F_nmax = e^-T sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1)) */
    double term = 1.0 / (2 * nmax + 1), sum = term;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0 * T / (2 * nmax + 2 * k + 1);
      sum += term;
      if (term < 1e-17 * sum) break;
    }
    F[nmax] = et * sum;
    for (int n = nmax - 1; n >= 0; --n) F[n] = (2.0 * T * F[n + 1] + et) / (2 * n + 1);
  } else {
    F[0] = 0.5 * sqrt(M_PI / T) * erf(sqrt(T));
    for (int n = 0; n < nmax; ++n) F[n + 1] = ((2 * n + 1) * F[n] - et) / (2.0 * T);
  }
}

/* Hermite expansion coefficients E[i][j][t] of the 1-D product
 * x_A^i x_B^j exp(-a x_A^2 - b x_B^2), i <= la, j <= lb, t <= i+j. */
static void hermite_E(int la, int lb, double a, double b, double Xab,
                      double E[LMAX + 1][LMAX + 1][2 * LMAX + 2]) {
  const double p = a + b, mu = a * b / p;
  const double Xpa = -b / p * Xab, Xpb = a / p * Xab, h = 0.5 / p;
  memset(E, 0, sizeof(double) * (LMAX + 1) * (LMAX + 1) * (2 * LMAX + 2));
  E[0][0][0] = exp(-mu * Xab * Xab);
  for (int i = 0; i <= la; ++i)
    for (int j = 0; j <= lb; ++j) {
      if (i == 0 && j == 0) continue;
      for (int t = 0; t <= i + j; ++t) {
        double v;
        if (i > 0) {
          v = Xpa * E[i - 1][j][t];
          if (t > 0) v += h * E[i - 1][j][t - 1];
          if (t + 1 <= i - 1 + j) v += (t + 1) * E[i - 1][j][t + 1];
        } else {
          v = Xpb * E[i][j - 1][t];
          if (t > 0) v += h * E[i][j - 1][t - 1];
          if (t + 1 <= i + j - 1) v += (t + 1) * E[i][j - 1][t + 1];
        }
        E[i][j][t] = v;
      }
    }
}

/* R^0_{tuv}(alpha, X, Y, Z) for t+u+v <= L, stored R[t][u][v]. */
static void hermite_R(int L, double alpha, double X, double Y, double Z,
                      double R[HMAX][HMAX][HMAX]) {
  static __thread double Rn[HMAX][HMAX][HMAX][HMAX];
  double F[HMAX + 1];
  boys(L, alpha * (X * X + Y * Y + Z * Z), F);
  double fac = 1.0;
  for (int n = 0; n <= L; ++n) {
    Rn[n][0][0][0] = fac * F[n];
    fac *= -2.0 * alpha;
  }
  for (int N = 1; N <= L; ++N)
    for (int n = 0; n <= L - N; ++n)
      for (int t = 0; t <= N; ++t)
        for (int u = 0; u <= N - t; ++u) {
          const int v = N - t - u;
          double r;
          if (t > 0) {
            r = X * Rn[n + 1][t - 1][u][v];
            if (t > 1) r += (t - 1) * Rn[n + 1][t - 2][u][v];
          } else if (u > 0) {
            r = Y * Rn[n + 1][t][u - 1][v];
            if (u > 1) r += (u - 1) * Rn[n + 1][t][u - 2][v];
          } else {
            r = Z * Rn[n + 1][t][u][v - 1];
            if (v > 1) r += (v - 1) * Rn[n + 1][t][u][v - 2];
          }
          Rn[n][t][u][v] = r;
        }
  for (int t = 0; t <= L; ++t)
    for (int u = 0; u <= L - t; ++u)
      for (int v = 0; v <= L - t - u; ++v) R[t][u][v] = Rn[0][t][u][v];
}

/* ------------------------------------------------------------------------ */
/* Cartesian -> real spherical (regular solid harmonics, unnormalised)     */
/* ------------------------------------------------------------------------ */
static double SPH[LMAX + 1][2 * LMAX + 1][(LMAX + 1) * (LMAX + 2) / 2];
static int sph_ready = 0;

static double binom(int n, int k) {
  if (k < 0 || k > n) return 0.0;
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

static int cart_index(int l, int lx, int ly) {
  /* lx = l..0, ly = l-lx..0 */
  int idx = 0;
  for (int x = l; x > lx; --x) idx += l - x + 1;
  return idx + (l - lx - ly);
}

static void sph_init(void) {
  if (sph_ready) return;
  memset(SPH, 0, sizeof(SPH));
  for (int l = 0; l <= LMAX; ++l)
    for (int m = -l; m <= l; ++m) {
      const int am = abs(m), vm2 = m < 0 ? 1 : 0;
      for (int t = 0; t <= (l - am) / 2; ++t)
        for (int u = 0; u <= t; ++u)
          for (int v2 = vm2; v2 <= am; v2 += 2) {
            const int sgn = ((t + (v2 - vm2) / 2) & 1) ? -1 : 1;
            const double c = sgn * pow(0.25, t) * binom(l, t) * binom(l - t, am + t) *
                             binom(t, u) * binom(am, v2);
            const int lx = 2 * t + am - 2 * u - v2, ly = 2 * u + v2, lz = l - 2 * t - am;
            if (lx < 0 || lz < 0) continue;
            SPH[l][m + l][cart_index(l, lx, ly)] += c;
          }
    }
  sph_ready = 1;
}

static void cart_list(int l, int* lx, int* ly, int* lz) {
  int k = 0;
  for (int x = l; x >= 0; --x)
    for (int y = l - x; y >= 0; --y) {
      lx[k] = x;
      ly[k] = y;
      lz[k] = l - x - y;
      ++k;
    }
}

typedef struct {
  const int* l;
  const int* nprim;
  const int* poff;
  const double* center;
  const double* exps;
  const double* coefs;
  int nsh;
} basis_t;

static int bf_offsets(const basis_t* b, int* off) {
  int n = 0;
  for (int s = 0; s < b->nsh; ++s) {
    off[s] = n;
    n += 2 * b->l[s] + 1;
  }
  return n;
}

/* Cartesian block -> spherical block for a 2-index quantity. */
static void sph2(int la, int lb, const double* cart, double* out /* (2la+1)(2lb+1) */) {
  const int na = ncart(la), nb = ncart(lb);
  double tmp[(2 * LMAX + 1) * 10];
  for (int m = 0; m < 2 * la + 1; ++m)
    for (int j = 0; j < nb; ++j) {
      double s = 0.0;
      for (int i = 0; i < na; ++i) s += SPH[la][m][i] * cart[i * nb + j];
      tmp[m * nb + j] = s;
    }
  for (int m = 0; m < 2 * la + 1; ++m)
    for (int n = 0; n < 2 * lb + 1; ++n) {
      double s = 0.0;
      for (int j = 0; j < nb; ++j) s += tmp[m * nb + j] * SPH[lb][n][j];
      out[m * (2 * lb + 1) + n] = s;
    }
}

/* ------------------------------------------------------------------------ */
/* one-electron integrals: S, T, V (op = 0, 1, 2)                           */
/* ------------------------------------------------------------------------ */
static void one_block(const basis_t* b, int sa, int sb, int op, int natom, const double* Z,
                      const double* xyz, double* cart) {
  const int la = b->l[sa], lb = b->l[sb], na = ncart(la), nb = ncart(lb);
  int ax[10], ay[10], az[10], bx[10], by[10], bz[10];
  cart_list(la, ax, ay, az);
  cart_list(lb, bx, by, bz);
  const double* A = b->center + 3 * sa;
  const double* B = b->center + 3 * sb;
  memset(cart, 0, sizeof(double) * na * nb);
  double Ex[LMAX + 1][LMAX + 1][2 * LMAX + 2], Ey[LMAX + 1][LMAX + 1][2 * LMAX + 2],
      Ez[LMAX + 1][LMAX + 1][2 * LMAX + 2];
  static __thread double R[HMAX][HMAX][HMAX];
  for (int p = 0; p < b->nprim[sa]; ++p)
    for (int q = 0; q < b->nprim[sb]; ++q) {
      const double a = b->exps[b->poff[sa] + p], bb = b->exps[b->poff[sb] + q];
      const double cc = b->coefs[b->poff[sa] + p] * b->coefs[b->poff[sb] + q];
      const double pp = a + bb;
      if (op != 1) {
        hermite_E(la, lb, a, bb, A[0] - B[0], Ex);
        hermite_E(la, lb, a, bb, A[1] - B[1], Ey);
        hermite_E(la, lb, a, bb, A[2] - B[2], Ez);
      }
      if (op == 0) {
        const double f = pow(M_PI / pp, 1.5) * cc;
        for (int i = 0; i < na; ++i)
          for (int j = 0; j < nb; ++j)
            cart[i * nb + j] += f * Ex[ax[i]][bx[j]][0] * Ey[ay[i]][by[j]][0] * Ez[az[i]][bz[j]][0];
      } else if (op == 1) {
        /* 1-D overlaps s_ij = E^{ij}_0 sqrt(pi/p) for j up to lb+2 */
        double sx[LMAX + 1][LMAX + 3], sy[LMAX + 1][LMAX + 3], sz[LMAX + 1][LMAX + 3];
        const double rp = sqrt(M_PI / pp);
        for (int d = 0; d < 3; ++d) {
          /* E^{i,j}_0 for j <= lb+2 via the j-recursion on a local table */
          double Et[LMAX + 1][LMAX + 3][2 * LMAX + 4];
          memset(Et, 0, sizeof(Et));
          const double Xab = A[d] - B[d], mu = a * bb / pp;
          const double Xpa = -bb / pp * Xab, Xpb = a / pp * Xab, h = 0.5 / pp;
          Et[0][0][0] = exp(-mu * Xab * Xab);
          for (int i = 0; i <= la; ++i)
            for (int j = 0; j <= lb + 2; ++j) {
              if (i == 0 && j == 0) continue;
              for (int t = 0; t <= i + j; ++t) {
                double v;
                if (i > 0) {
                  v = Xpa * Et[i - 1][j][t];
                  if (t > 0) v += h * Et[i - 1][j][t - 1];
                  if (t + 1 <= i - 1 + j) v += (t + 1) * Et[i - 1][j][t + 1];
                } else {
                  v = Xpb * Et[i][j - 1][t];
                  if (t > 0) v += h * Et[i][j - 1][t - 1];
                  if (t + 1 <= i + j - 1) v += (t + 1) * Et[i][j - 1][t + 1];
                }
                Et[i][j][t] = v;
              }
            }
          for (int i = 0; i <= la; ++i)
            for (int j = 0; j <= lb + 2; ++j) {
              const double s = Et[i][j][0] * rp;
              if (d == 0) sx[i][j] = s;
              else if (d == 1) sy[i][j] = s;
              else sz[i][j] = s;
            }
        }
        for (int i = 0; i < na; ++i)
          for (int j = 0; j < nb; ++j) {
            /* <i| -1/2 d2/dx2 |j> with d2/dx2 x^j e^{-b x^2} =
               j(j-1) x^{j-2} - 2b(2j+1) x^j + 4b^2 x^{j+2} */
            double tx, ty, tz;
#define KIN(s, ii, jj)                                                                  \
  (((jj) >= 2 ? (jj) * ((jj)-1) * s[ii][(jj)-2] : 0.0) - 2.0 * bb * (2 * (jj) + 1) * s[ii][jj] + \
   4.0 * bb * bb * s[ii][(jj) + 2])
            tx = KIN(sx, ax[i], bx[j]);
            ty = KIN(sy, ay[i], by[j]);
            tz = KIN(sz, az[i], bz[j]);
#undef KIN
            const double Sx = sx[ax[i]][bx[j]], Sy = sy[ay[i]][by[j]], Sz = sz[az[i]][bz[j]];
            cart[i * nb + j] += -0.5 * cc * (tx * Sy * Sz + Sx * ty * Sz + Sx * Sy * tz);
          }
      } else {
        const double P[3] = {(a * A[0] + bb * B[0]) / pp, (a * A[1] + bb * B[1]) / pp,
                             (a * A[2] + bb * B[2]) / pp};
        for (int C = 0; C < natom; ++C) {
          hermite_R(la + lb, pp, P[0] - xyz[3 * C], P[1] - xyz[3 * C + 1], P[2] - xyz[3 * C + 2],
                    R);
          const double f = -Z[C] * 2.0 * M_PI / pp * cc;
          for (int i = 0; i < na; ++i)
            for (int j = 0; j < nb; ++j) {
              double s = 0.0;
              for (int t = 0; t <= ax[i] + bx[j]; ++t)
                for (int u = 0; u <= ay[i] + by[j]; ++u)
                  for (int v = 0; v <= az[i] + bz[j]; ++v)
                    s += Ex[ax[i]][bx[j]][t] * Ey[ay[i]][by[j]][u] * Ez[az[i]][bz[j]][v] * R[t][u][v];
              cart[i * nb + j] += f * s;
            }
        }
      }
    }
}

void ints_one(int nsh, const int* l, const int* nprim, const int* poff, const double* center,
              const double* exps, const double* coefs, int op, int natom, const double* Z,
              const double* xyz, double* out) {
  sph_init();
  basis_t b = {l, nprim, poff, center, exps, coefs, nsh};
  int* off = (int*)malloc(sizeof(int) * nsh);
  const int n = bf_offsets(&b, off);
#pragma omp parallel for schedule(dynamic)
  for (int sa = 0; sa < nsh; ++sa) {
    double cart[100], sph[49];
    for (int sb = 0; sb < nsh; ++sb) {
      one_block(&b, sa, sb, op, natom, Z, xyz, cart);
      sph2(l[sa], l[sb], cart, sph);
      for (int m = 0; m < 2 * l[sa] + 1; ++m)
        for (int k = 0; k < 2 * l[sb] + 1; ++k)
          out[(size_t)(off[sa] + m) * n + off[sb] + k] = sph[m * (2 * l[sb] + 1) + k];
    }
  }
  free(off);
}

/* ------------------------------------------------------------------------ */
/* two-electron integrals over (pair | pair); a pair may be a single shell  */
/* (second shell = -1: an s function of exponent 0 at the same centre).     */
/* ------------------------------------------------------------------------ */
typedef struct {
  int la, lb, na, nb;
  int ax[10], ay[10], az[10], bx[10], by[10], bz[10];
} pairinfo_t;

static void pair_info(const basis_t* b, int sa, int sb, pairinfo_t* pi) {
  pi->la = b->l[sa];
  pi->lb = sb >= 0 ? b->l[sb] : 0;
  pi->na = ncart(pi->la);
  pi->nb = ncart(pi->lb);
  cart_list(pi->la, pi->ax, pi->ay, pi->az);
  cart_list(pi->lb, pi->bx, pi->by, pi->bz);
}

/* Cartesian (ab|cd) block [na][nb][nc][nd]; basis b1 for the bra, b2 for the ket. */
static void eri_block(const basis_t* b1, int sa, int sb, const basis_t* b2, int sc, int sd,
                      double* cart) {
  pairinfo_t P, Q;
  pair_info(b1, sa, sb, &P);
  pair_info(b2, sc, sd, &Q);
  const int nab = P.na * P.nb, ncd = Q.na * Q.nb;
  memset(cart, 0, sizeof(double) * nab * ncd);
  const double* A = b1->center + 3 * sa;
  const double* B = sb >= 0 ? b1->center + 3 * sb : A;
  const double* C = b2->center + 3 * sc;
  const double* D = sd >= 0 ? b2->center + 3 * sd : C;
  const int L = P.la + P.lb + Q.la + Q.lb;
  double Eab[3][LMAX + 1][LMAX + 1][2 * LMAX + 2], Ecd[3][LMAX + 1][LMAX + 1][2 * LMAX + 2];
  static __thread double R[HMAX][HMAX][HMAX];
  const int npa = b1->nprim[sa], npb = sb >= 0 ? b1->nprim[sb] : 1;
  const int npc = b2->nprim[sc], npd = sd >= 0 ? b2->nprim[sd] : 1;
  for (int pa = 0; pa < npa; ++pa)
    for (int pb = 0; pb < npb; ++pb) {
      const double a = b1->exps[b1->poff[sa] + pa];
      const double bb = sb >= 0 ? b1->exps[b1->poff[sb] + pb] : 0.0;
      const double cab = b1->coefs[b1->poff[sa] + pa] * (sb >= 0 ? b1->coefs[b1->poff[sb] + pb] : 1.0);
      const double p = a + bb;
      for (int d = 0; d < 3; ++d) hermite_E(P.la, P.lb, a, bb, A[d] - B[d], Eab[d]);
      const double Pc[3] = {(a * A[0] + bb * B[0]) / p, (a * A[1] + bb * B[1]) / p,
                            (a * A[2] + bb * B[2]) / p};
      for (int pc = 0; pc < npc; ++pc)
        for (int pd = 0; pd < npd; ++pd) {
          const double c = b2->exps[b2->poff[sc] + pc];
          const double dd = sd >= 0 ? b2->exps[b2->poff[sd] + pd] : 0.0;
          const double ccd =
              b2->coefs[b2->poff[sc] + pc] * (sd >= 0 ? b2->coefs[b2->poff[sd] + pd] : 1.0);
          const double q = c + dd;
          for (int d = 0; d < 3; ++d) hermite_E(Q.la, Q.lb, c, dd, C[d] - D[d], Ecd[d]);
          const double Qc[3] = {(c * C[0] + dd * D[0]) / q, (c * C[1] + dd * D[1]) / q,
                                (c * C[2] + dd * D[2]) / q};
          const double alpha = p * q / (p + q);
          hermite_R(L, alpha, Pc[0] - Qc[0], Pc[1] - Qc[1], Pc[2] - Qc[2], R);
          const double pref = 2.0 * pow(M_PI, 2.5) / (p * q * sqrt(p + q)) * cab * ccd;
          for (int ic = 0; ic < Q.na; ++ic)
            for (int id = 0; id < Q.nb; ++id) {
              const int cx = Q.ax[ic] + Q.bx[id], cy = Q.ay[ic] + Q.by[id],
                        cz = Q.az[ic] + Q.bz[id];
              /* G[t][u][v] = sum_{tau nu phi} (-1)^{tau+nu+phi} E^cd R_{t+tau,u+nu,v+phi} */
              double G[2 * LMAX + 2][2 * LMAX + 2][2 * LMAX + 2];
              const int Lab = P.la + P.lb;
              for (int t = 0; t <= Lab; ++t)
                for (int u = 0; u <= Lab - t; ++u)
                  for (int v = 0; v <= Lab - t - u; ++v) {
                    double s = 0.0;
                    for (int tau = 0; tau <= cx; ++tau) {
                      const double ex = Ecd[0][Q.ax[ic]][Q.bx[id]][tau];
                      if (ex == 0.0) continue;
                      for (int nu = 0; nu <= cy; ++nu) {
                        const double ey = Ecd[1][Q.ay[ic]][Q.by[id]][nu];
                        if (ey == 0.0) continue;
                        for (int ph = 0; ph <= cz; ++ph) {
                          const double ez = Ecd[2][Q.az[ic]][Q.bz[id]][ph];
                          const double sg = ((tau + nu + ph) & 1) ? -1.0 : 1.0;
                          s += sg * ex * ey * ez * R[t + tau][u + nu][v + ph];
                        }
                      }
                    }
                    G[t][u][v] = s;
                  }
              for (int ia = 0; ia < P.na; ++ia)
                for (int ib = 0; ib < P.nb; ++ib) {
                  double s = 0.0;
                  for (int t = 0; t <= P.ax[ia] + P.bx[ib]; ++t) {
                    const double ex = Eab[0][P.ax[ia]][P.bx[ib]][t];
                    for (int u = 0; u <= P.ay[ia] + P.by[ib]; ++u) {
                      const double ey = Eab[1][P.ay[ia]][P.by[ib]][u];
                      for (int v = 0; v <= P.az[ia] + P.bz[ib]; ++v)
                        s += ex * ey * Eab[2][P.az[ia]][P.bz[ib]][v] * G[t][u][v];
                    }
                  }
                  cart[(ia * P.nb + ib) * ncd + ic * Q.nb + id] += pref * s;
                }
            }
        }
    }
}

/* Cartesian [na*nb][nc*nd] -> spherical [(2la+1)(2lb+1)][(2lc+1)(2ld+1)] */
static void sph4(const pairinfo_t* P, const pairinfo_t* Q, const double* cart, double* out) {
  const int na = P->na, nb = P->nb, nc = Q->na, nd = Q->nb;
  const int sa = 2 * P->la + 1, sb = 2 * P->lb + 1, sc = 2 * Q->la + 1, sd = 2 * Q->lb + 1;
  double* t1 = (double*)malloc(sizeof(double) * sa * nb * nc * nd);
  double* t2 = (double*)malloc(sizeof(double) * sa * sb * nc * nd);
  double* t3 = (double*)malloc(sizeof(double) * sa * sb * sc * nd);
  for (int m = 0; m < sa; ++m)
    for (int r = 0; r < nb * nc * nd; ++r) {
      double s = 0.0;
      for (int i = 0; i < na; ++i) s += SPH[P->la][m][i] * cart[(size_t)i * nb * nc * nd + r];
      t1[(size_t)m * nb * nc * nd + r] = s;
    }
  for (int m = 0; m < sa; ++m)
    for (int n = 0; n < sb; ++n)
      for (int r = 0; r < nc * nd; ++r) {
        double s = 0.0;
        for (int j = 0; j < nb; ++j)
          s += SPH[P->lb][n][j] * t1[((size_t)m * nb + j) * nc * nd + r];
        t2[((size_t)m * sb + n) * nc * nd + r] = s;
      }
  for (int mn = 0; mn < sa * sb; ++mn)
    for (int k = 0; k < sc; ++k)
      for (int d = 0; d < nd; ++d) {
        double s = 0.0;
        for (int c = 0; c < nc; ++c) s += SPH[Q->la][k][c] * t2[((size_t)mn * nc + c) * nd + d];
        t3[((size_t)mn * sc + k) * nd + d] = s;
      }
  for (int mnk = 0; mnk < sa * sb * sc; ++mnk)
    for (int q = 0; q < sd; ++q) {
      double s = 0.0;
      for (int d = 0; d < nd; ++d) s += SPH[Q->lb][q][d] * t3[(size_t)mnk * nd + d];
      out[(size_t)mnk * sd + q] = s;
    }
  free(t1);
  free(t2);
  free(t3);
}

/* Dense (mu nu|la si) over one basis, [N][N][N][N]. */
void ints_eri4(int nsh, const int* l, const int* nprim, const int* poff, const double* center,
               const double* exps, const double* coefs, double* out) {
  sph_init();
  basis_t b = {l, nprim, poff, center, exps, coefs, nsh};
  int* off = (int*)malloc(sizeof(int) * nsh);
  const size_t n = bf_offsets(&b, off);
#pragma omp parallel for schedule(dynamic) collapse(2)
  for (int sa = 0; sa < nsh; ++sa)
    for (int sb = 0; sb < nsh; ++sb) {
      double* cart = (double*)malloc(sizeof(double) * 10000);
      double* sph = (double*)malloc(sizeof(double) * 2401);
      pairinfo_t P, Q;
      pair_info(&b, sa, sb, &P);
      for (int sc = 0; sc < nsh; ++sc)
        for (int sd = 0; sd < nsh; ++sd) {
          pair_info(&b, sc, sd, &Q);
          eri_block(&b, sa, sb, &b, sc, sd, cart);
          sph4(&P, &Q, cart, sph);
          const int da = 2 * l[sa] + 1, db = 2 * l[sb] + 1, dc = 2 * l[sc] + 1,
                    dd = 2 * l[sd] + 1;
          for (int i = 0; i < da; ++i)
            for (int j = 0; j < db; ++j)
              for (int k = 0; k < dc; ++k)
                for (int m = 0; m < dd; ++m)
                  out[(((off[sa] + i) * n + off[sb] + j) * n + off[sc] + k) * n + off[sd] + m] =
                      sph[((i * db + j) * dc + k) * dd + m];
        }
      free(cart);
      free(sph);
    }
  free(off);
}

/* (P|Q) over an auxiliary basis, [X][X]. */
void ints_2c(int nsh, const int* l, const int* nprim, const int* poff, const double* center,
             const double* exps, const double* coefs, double* out) {
  sph_init();
  basis_t b = {l, nprim, poff, center, exps, coefs, nsh};
  int* off = (int*)malloc(sizeof(int) * nsh);
  const size_t n = bf_offsets(&b, off);
#pragma omp parallel for schedule(dynamic)
  for (int sa = 0; sa < nsh; ++sa) {
    double cart[1000], sph[1000];
    pairinfo_t P, Q;
    pair_info(&b, sa, -1, &P);
    for (int sc = 0; sc < nsh; ++sc) {
      pair_info(&b, sc, -1, &Q);
      eri_block(&b, sa, -1, &b, sc, -1, cart);
      sph4(&P, &Q, cart, sph);
      const int da = 2 * l[sa] + 1, dc = 2 * l[sc] + 1;
      for (int i = 0; i < da; ++i)
        for (int k = 0; k < dc; ++k) out[(off[sa] + i) * n + off[sc] + k] = sph[i * dc + k];
    }
  }
  free(off);
}

/* (P|mu nu), aux basis a (bra), orbital basis o (ket pair), [X][N][N].
 * Orbital shell pairs whose Schwarz factor sqrt|(ss'|ss')| max, times the
 * largest aux factor, falls below `screen` are skipped (left zero). */
void ints_3c(int nsa, const int* la, const int* npa, const int* pofa, const double* cena,
             const double* expa, const double* cofa, int nso, const int* lo, const int* npo,
             const int* pofo, const double* ceno, const double* expo, const double* cofo,
             const double* pair_schwarz /* [nso*nso] or NULL */, double screen, double* out) {
  sph_init();
  basis_t ba = {la, npa, pofa, cena, expa, cofa, nsa};
  basis_t bo = {lo, npo, pofo, ceno, expo, cofo, nso};
  int* offa = (int*)malloc(sizeof(int) * nsa);
  int* offo = (int*)malloc(sizeof(int) * nso);
  bf_offsets(&ba, offa);
  const size_t N = bf_offsets(&bo, offo);
#pragma omp parallel for schedule(dynamic)
  for (int sc = 0; sc < nso; ++sc) {
    double* cart = (double*)malloc(sizeof(double) * 10 * 100);
    double* sph = (double*)malloc(sizeof(double) * 7 * 49);
    pairinfo_t P, Q;
    for (int sd = 0; sd <= sc; ++sd) {
      if (pair_schwarz && pair_schwarz[sc * nso + sd] < screen) continue;
      pair_info(&bo, sc, sd, &Q);
      const int dc = 2 * lo[sc] + 1, dd = 2 * lo[sd] + 1;
      for (int sa = 0; sa < nsa; ++sa) {
        pair_info(&ba, sa, -1, &P);
        eri_block(&ba, sa, -1, &bo, sc, sd, cart);
        sph4(&P, &Q, cart, sph);
        const int da = 2 * la[sa] + 1;
        for (int i = 0; i < da; ++i)
          for (int k = 0; k < dc; ++k)
            for (int m = 0; m < dd; ++m) {
              const double v = sph[(i * dc + k) * dd + m];
              const size_t pidx = (size_t)(offa[sa] + i) * N * N;
              out[pidx + (size_t)(offo[sc] + k) * N + offo[sd] + m] = v;
              out[pidx + (size_t)(offo[sd] + m) * N + offo[sc] + k] = v;
            }
      }
    }
    free(cart);
    free(sph);
  }
  free(offa);
  free(offo);
}
