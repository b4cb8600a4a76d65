// Gaussian integrals of the RI path on the GPU: the 2-index metric
// J[P][Q] = (P|Q) and the 3-index integrals (P|mu nu), the inputs the
// reference computes with libint inside calculate_ri (src/POSTHF/ri.cc:25-47,
// 70-100) or the psi4 plugin writes (syshfwplug/plugin.cc:478-503).
//
// Method: McMurchie-Davidson (Helgaker, Joergensen, Olsen, "Molecular
// Electronic-Structure Theory", ch. 9): Hermite expansion coefficients E of
// each Gaussian product, Hermite Coulomb integrals R_tuv from the Boys
// function F_n by the vertical recursion, contracted Cartesian blocks, then
// real solid harmonics (m = -l..l) normalised to one.  Cartesian components
// are ordered lx = l..0, ly = l-lx..0.  FP64 throughout.
//
// Work decomposition: one kernel per angular-momentum class (aux l, and the
// two orbital l's), templated so every table has a compile-time size; one
// thread per (aux shell, orbital shell pair c >= d), both triangles of
// (P|mu nu) written.  (P|Q) runs through the same kernel with an s function
// of exponent 0 as the partner of Q.  Boys function: for T < 33 the series
// e^-T sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1)) for the highest order and
// downward recursion; above, F_0 = sqrt(pi/T) erf(sqrt T) / 2 and upward
// recursion.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "abi_internal.h"
#include "common.cuh"

namespace corr {

namespace {

constexpr int kLmax = 3;

struct ShellD {
  double x, y, z;
  int l, nprim, poff, bf;  // bf: index of the shell's first function
};

__constant__ double c_sph[kLmax + 1][2 * kLmax + 1][10];  // spherical <- Cartesian
__constant__ int c_cexp[kLmax + 1][10][3];                   // Cartesian exponents
constexpr int kTmax = 2 * kLmax + 2;                         // Hermite orders < kTmax
__constant__ int c_tuv[kTmax][kTmax][kTmax];                  // tuv_index table

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Cartesian exponent of component k of shell l along dim (0 x, 1 y, 2 z)
__host__ __device__ constexpr int cexp(int l, int k, int dim) {
  int idx = 0;
  for (int x = l; x >= 0; --x)
    for (int y = l - x; y >= 0; --y) {
      if (idx == k) return dim == 0 ? x : (dim == 1 ? y : l - x - y);
      ++idx;
    }
  return 0;
}

// (t, u, v) with t + u + v <= L: index in a compact table of binom(L+3, 3) entries
__host__ __device__ constexpr int tuv_count(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ constexpr int tuv_index(int t, int u, int v) {
  // orders m = t + u + v in increasing order, within an order the (u, v) pairs
  return tuv_count(t + u + v - 1 >= 0 ? t + u + v - 1 : -1) + ((u + v) * (u + v + 1)) / 2 + v;
}

// Boys function F_n(T), n <= NMAX: for T < kBoysTmax an 8-term Taylor
// expansion of F_NMAX about the nearest point of a tabulated grid (spacing
// 1/16, |dT| <= 1/32, truncation below 2^-55 relative) and downward
// recursion F_n = (2T F_{n+1} + e^-T) / (2n + 1); above, the asymptotic
// F_0 = sqrt(pi/T) / 2 (erf(sqrt T) = 1 to 1e-18) and upward recursion
// without the e^-T term (below 4e-18 relative).
constexpr int kBoysOrders = 16;                // tabulated n = 0..15
constexpr int kBoysPerUnit = 16;               // grid points per unit of T
constexpr double kBoysTmax = 40.0;
constexpr int kBoysPoints = (int)kBoysTmax * kBoysPerUnit + 1;
__device__ double d_boys[kBoysPoints][kBoysOrders];

template <int NMAX>
__device__ __forceinline__ void boys(double T, double* F) {
  static_assert(NMAX + 8 <= kBoysOrders, "Boys table orders");
  if (T < kBoysTmax) {
    const int i = __double2int_rn(T * kBoysPerUnit);
    const double x = (double)i * (1.0 / kBoysPerUnit) - T;  // -dT
    const double* f = d_boys[i] + NMAX;
    double s = f[7];
#pragma unroll
    for (int k = 6; k >= 0; --k) s = fma(s, x * (1.0 / (k + 1)), f[k]);
    F[NMAX] = s;
    const double et = exp(-T), t2 = 2.0 * T;
#pragma unroll
    for (int n = NMAX - 1; n >= 0; --n) F[n] = fma(t2, F[n + 1], et) * (1.0 / (2 * n + 1));
    return;
  }
  const double rt = 1.0 / T;
  F[0] = 0.886226925452758 * sqrt(rt);  // sqrt(pi) / 2
#pragma unroll
  for (int n = 0; n < NMAX; ++n) F[n + 1] = F[n] * ((n + 0.5) * rt);
}

// R^0_{tuv}(alpha, X, Y, Z), t + u + v <= L, into buf[0][tuv_index].  Ping-pong
// over the auxiliary order n between buf[0] and buf[1]: level n holds the
// orders <= L - n.
template <int L>
__device__ __forceinline__ void hermite_r(double alpha, double X, double Y, double Z,
                                          double (&buf)[2][tuv_count(L)]) {
  constexpr int NT = tuv_count(L);
  double F[L + 1];
  boys<L>(alpha * (X * X + Y * Y + Z * Z), F);
  // level L: only R^L_000
  double fac = 1.0;
  double fn[L + 1];
#pragma unroll
  for (int n = 0; n <= L; ++n) {
    fn[n] = fac * F[n];
    fac *= -2.0 * alpha;
  }
  buf[L & 1][0] = fn[L];
#pragma unroll
  for (int n = L - 1; n >= 0; --n) {
    const double* up = buf[(n + 1) & 1];
    double* cur = buf[n & 1];
    cur[0] = fn[n];
#pragma unroll
    for (int m = 1; m <= L - n; ++m)
#pragma unroll
      for (int t = m; t >= 0; --t)
#pragma unroll
        for (int u = m - t; u >= 0; --u) {
          const int v = m - t - u;
          double r;
          if (t > 0) {
            r = X * up[tuv_index(t - 1, u, v)];
            if (t > 1) r += (t - 1) * up[tuv_index(t - 2, u, v)];
          } else if (u > 0) {
            r = Y * up[tuv_index(t, u - 1, v)];
            if (u > 1) r += (u - 1) * up[tuv_index(t, u - 2, v)];
          } else {
            r = Z * up[tuv_index(t, u, v - 1)];
            if (v > 1) r += (v - 1) * up[tuv_index(t, u, v - 2)];
          }
          cur[tuv_index(t, u, v)] = r;
        }
  }
  (void)NT;
}

// Hermite coefficients E[i][j][t] (i <= LA, j <= LB, t <= i + j) of the 1-D
// product of exponents a, b separated by Xab = A - B, flattened.
template <int LA, int LB>
__device__ __forceinline__ void hermite_e(double a, double b, double Xab, double* E) {
  constexpr int NT = LA + LB + 1;
  const double p = a + b;
  const double Xpa = -b / p * Xab, Xpb = a / p * Xab, h = 0.5 / p;
#define EIDX(i, j, t) (((i) * (LB + 1) + (j)) * NT + (t))
#pragma unroll
  for (int k = 0; k < (LA + 1) * (LB + 1) * NT; ++k) E[k] = 0.0;
  E[EIDX(0, 0, 0)] = exp(-a * b / p * Xab * Xab);
#pragma unroll
  for (int i = 0; i <= LA; ++i)
#pragma unroll
    for (int j = 0; j <= LB; ++j) {
      if (i == 0 && j == 0) continue;
#pragma unroll
      for (int t = 0; t <= i + j; ++t) {
        double v;
        if (i > 0) {
          v = Xpa * E[EIDX(i - 1, j, t)];
          if (t > 0) v += h * E[EIDX(i - 1, j, t - 1)];
          if (t + 1 <= i - 1 + j) v += (t + 1) * E[EIDX(i - 1, j, t + 1)];
        } else {
          v = Xpb * E[EIDX(i, j - 1, t)];
          if (t > 0) v += h * E[EIDX(i, j - 1, t - 1)];
          if (t + 1 <= i + j - 1) v += (t + 1) * E[EIDX(i, j - 1, t + 1)];
        }
        E[EIDX(i, j, t)] = v;
      }
    }
#undef EIDX
}

// As hermite_e, from the pair's precomputed quantities: e0 = exp(-ab/p X^2)
// in this dimension, Xpa = P - A, Xpb = P - B, h = 1/(2p).
template <int LA, int LB>
__device__ __forceinline__ void hermite_e_pre(double e0, double Xpa, double Xpb, double h,
                                              double* E) {
  constexpr int NT = LA + LB + 1;
#define EIDX(i, j, t) (((i) * (LB + 1) + (j)) * NT + (t))
#pragma unroll
  for (int k = 0; k < (LA + 1) * (LB + 1) * NT; ++k) E[k] = 0.0;
  E[EIDX(0, 0, 0)] = e0;
#pragma unroll
  for (int i = 0; i <= LA; ++i)
#pragma unroll
    for (int j = 0; j <= LB; ++j) {
      if (i == 0 && j == 0) continue;
#pragma unroll
      for (int t = 0; t <= i + j; ++t) {
        double v;
        if (i > 0) {
          v = Xpa * E[EIDX(i - 1, j, t)];
          if (t > 0) v += h * E[EIDX(i - 1, j, t - 1)];
          if (t + 1 <= i - 1 + j) v += (t + 1) * E[EIDX(i - 1, j, t + 1)];
        } else {
          v = Xpb * E[EIDX(i, j - 1, t)];
          if (t > 0) v += h * E[EIDX(i, j - 1, t - 1)];
          if (t + 1 <= i + j - 1) v += (t + 1) * E[EIDX(i, j - 1, t + 1)];
        }
        E[EIDX(i, j, t)] = v;
      }
    }
#undef EIDX
}

// Per orbital primitive pair (host-computed): p = a + b, the centre P, the
// per-dimension Gaussian factors exp(-ab/p X_AB^2), c_a c_b / p and 1/(2p).
struct PairData {
  double p, px, py, pz, ex, ey, ez, cdp, h;
};

struct Basis3 {
  const ShellD* aux;   // bra shells (the auxiliary basis)
  const int* alist;    // bra shells of this class
  int nalist;
  const ShellD* obs;   // ket shells
  const int2* plist;   // ket shell pairs (c, d) of this class; d < 0: exponent-0 s partner
  const int2* prange;  // per ket pair: its primitive pairs pp[x .. y)
  const ushort2* pp;   // (primitive of c, primitive of d) that pass the screening
  const PairData* ppd; // their precomputed data (same index)
  const double* arq;   // per auxiliary primitive: c / gamma
  const double* ahq;   // per auxiliary primitive: 1 / (2 gamma)
  int nplist;
  const double* aexp;  // primitives of the bra basis (coefficients include the
  const double* acof;  // primitive normalisation)
  const double* oexp;
  const double* ocof;
  const double* anorm;  // per function
  const double* onorm;
  double* out;          // (P|mu nu) [X][N][N], or J [X][X] (two_center)
  int N;                // ket functions (leading dimension of out)
  int two_center;
};

// Contracted (P| c d) block for one bra shell and one ket pair of class
// (LP, LC, LD); spherical, normalised, written to out.
template <int LP, int LC, int LD>
__global__ void __launch_bounds__(128) eri3_kernel(Basis3 g) {
  constexpr int L = LP + LC + LD, LCD = LC + LD;
  constexpr int NP = ncart(LP), NC = ncart(LC), ND = ncart(LD);
  constexpr int NTB = tuv_count(LP);     // bra Hermite orders
  const long long total = (long long)g.nalist * g.nplist;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < total;
       w += (long long)gridDim.x * blockDim.x) {
    const int pi = (int)(w % g.nalist);
    const int ki = (int)(w / g.nalist);
    const ShellD sp = g.aux[g.alist[pi]];
    const int2 cd = g.plist[ki];
    const ShellD sc = g.obs[cd.x];
    const bool has_d = cd.y >= 0;
    const ShellD sd = has_d ? g.obs[cd.y] : sc;
    const int npd = has_d ? sd.nprim : 1;
    double cart[NP * NC * ND];
#pragma unroll
    for (int k = 0; k < NP * NC * ND; ++k) cart[k] = 0.0;
    const double Xcd = sc.x - sd.x, Ycd = sc.y - sd.y, Zcd = sc.z - sd.z;
    (void)npd;
    const int2 rg = g.prange[ki];
    for (int q = rg.x; q < rg.y; ++q) {
        const PairData pd = g.ppd[q];
        const double p = pd.p, Px = pd.px, Py = pd.py, Pz = pd.pz;
        double Ex[(LC + 1) * (LD + 1) * (LCD + 1)], Ey[(LC + 1) * (LD + 1) * (LCD + 1)],
            Ez[(LC + 1) * (LD + 1) * (LCD + 1)];
        hermite_e_pre<LC, LD>(pd.ex, Px - sc.x, Px - sd.x, pd.h, Ex);
        hermite_e_pre<LC, LD>(pd.ey, Py - sc.y, Py - sd.y, pd.h, Ey);
        hermite_e_pre<LC, LD>(pd.ez, Pz - sc.z, Pz - sd.z, pd.h, Ez);
        (void)Xcd;
        (void)Ycd;
        (void)Zcd;
        for (int ip = 0; ip < sp.nprim; ++ip) {
          const double gq = g.aexp[sp.poff + ip];
          // bra Hermite coefficients of a single Gaussian: EP[k][tau], same in x, y, z
          double EP[(LP + 1) * (LP + 1)];
#pragma unroll
          for (int k = 0; k < (LP + 1) * (LP + 1); ++k) EP[k] = 0.0;
          EP[0] = 1.0;
          const double hq = g.ahq[sp.poff + ip];
#pragma unroll
          for (int k = 1; k <= LP; ++k)
#pragma unroll
            for (int t = 0; t <= k; ++t) {
              double v = 0.0;
              if (t > 0) v += hq * EP[(k - 1) * (LP + 1) + t - 1];
              if (t + 1 <= k - 1) v += (t + 1) * EP[(k - 1) * (LP + 1) + t + 1];
              EP[k * (LP + 1) + t] = v;
            }
          const double rs = rsqrt(gq + p);          // (gq + p)^-1/2
          const double alpha = gq * p * (rs * rs);  // gq p / (gq + p)
          double Rbuf[2][tuv_count(L)];  // R^0_tuv ends in Rbuf[0]
          hermite_r<L>(alpha, sp.x - Px, sp.y - Py, sp.z - Pz, Rbuf);
          const double* R = Rbuf[0];
          // 2 pi^(5/2) / (p q sqrt(p + q)) times the contraction coefficients
          const double pref = 34.986836655249725 * g.arq[sp.poff + ip] * pd.cdp * rs;
          // ket Cartesian pair (kc, kd): G[tuv] = sum_{tau nu phi} (-1)^(tau+nu+phi)
          // E^cd_tau E^cd_nu E^cd_phi R_{t+tau, u+nu, v+phi} over the bra orders
          // t+u+v <= LP, then the bra Cartesian components.  Run-time loops
          // (uniform over the warp: one class per launch), index tables in
          // constant memory.
#pragma unroll 1
          for (int kc = 0; kc < NC; ++kc)
#pragma unroll 1
            for (int kd = 0; kd < ND; ++kd) {
              const int cx = c_cexp[LC][kc][0] + c_cexp[LD][kd][0];
              const int cy = c_cexp[LC][kc][1] + c_cexp[LD][kd][1];
              const int cz = c_cexp[LC][kc][2] + c_cexp[LD][kd][2];
              const double* ex = Ex + (c_cexp[LC][kc][0] * (LD + 1) + c_cexp[LD][kd][0]) * (LCD + 1);
              const double* ey = Ey + (c_cexp[LC][kc][1] * (LD + 1) + c_cexp[LD][kd][1]) * (LCD + 1);
              const double* ez = Ez + (c_cexp[LC][kc][2] * (LD + 1) + c_cexp[LD][kd][2]) * (LCD + 1);
              double G[NTB];
#pragma unroll
              for (int k = 0; k < NTB; ++k) G[k] = 0.0;
#pragma unroll 1
              for (int ta = 0; ta <= cx; ++ta)
#pragma unroll 1
                for (int nu = 0; nu <= cy; ++nu)
#pragma unroll 1
                  for (int ph = 0; ph <= cz; ++ph) {
                    double e = ex[ta] * ey[nu] * ez[ph];
                    if ((ta + nu + ph) & 1) e = -e;
#pragma unroll
                    for (int t = 0; t <= LP; ++t)
#pragma unroll
                      for (int u = 0; u <= LP - t; ++u)
#pragma unroll
                        for (int v = 0; v <= LP - t - u; ++v)
                          G[tuv_index(t, u, v)] += e * R[c_tuv[t + ta][u + nu][v + ph]];
                  }
#pragma unroll
              for (int kp = 0; kp < NP; ++kp) {
                const int px = cexp(LP, kp, 0), py = cexp(LP, kp, 1), pz = cexp(LP, kp, 2);
                double acc = 0.0;
#pragma unroll
                for (int t = 0; t <= px; ++t)
#pragma unroll
                  for (int u = 0; u <= py; ++u)
#pragma unroll
                    for (int v = 0; v <= pz; ++v)
                      acc += EP[px * (LP + 1) + t] * EP[py * (LP + 1) + u] *
                             EP[pz * (LP + 1) + v] * G[tuv_index(t, u, v)];
                cart[(kp * NC + kc) * ND + kd] += pref * acc;
              }
            }
        }
      }
    // spherical transform, normalisation, stores
    constexpr int SP = 2 * LP + 1, SC = 2 * LC + 1, SD = 2 * LD + 1;
#pragma unroll
    for (int mp = 0; mp < SP; ++mp) {
      double t1[NC * ND];
#pragma unroll
      for (int k = 0; k < NC * ND; ++k) {
        double s = 0.0;
#pragma unroll
        for (int kp = 0; kp < NP; ++kp) s += c_sph[LP][mp][kp] * cart[kp * NC * ND + k];
        t1[k] = s;
      }
      const int fp = sp.bf + mp;
      const double np_ = g.anorm[fp];
#pragma unroll
      for (int mc = 0; mc < SC; ++mc) {
        double t2[ND];
#pragma unroll
        for (int kd = 0; kd < ND; ++kd) {
          double s = 0.0;
#pragma unroll
          for (int kc = 0; kc < NC; ++kc) s += c_sph[LC][mc][kc] * t1[kc * ND + kd];
          t2[kd] = s;
        }
        const int fc = sc.bf + mc;
#pragma unroll
        for (int md = 0; md < SD; ++md) {
          double s = 0.0;
#pragma unroll
          for (int kd = 0; kd < ND; ++kd) s += c_sph[LD][md][kd] * t2[kd];
          if (g.two_center) {
            g.out[(size_t)fp * g.N + fc] = s * np_ * g.onorm[fc];
          } else {
            const int fd = sd.bf + md;
            const double v = s * np_ * g.onorm[fc] * g.onorm[fd];
            const size_t base = (size_t)fp * g.N * g.N;
            g.out[base + (size_t)fc * g.N + fd] = v;
            g.out[base + (size_t)fd * g.N + fc] = v;
          }
        }
      }
    }
  }
}

// ---- host side -------------------------------------------------------------
double binom(int n, int k) {
  if (k < 0 || k > n) return 0.0;
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

// Real regular solid harmonics S_lm (m = -l..l) as Cartesian polynomials,
// unnormalised (Helgaker, Joergensen, Olsen eq. 6.4.47-6.4.50):
// S_lm = sum_{t=0}^{(l-|m|)/2} sum_{u=0}^{t} sum_{v} C_tuv x^(2t+|m|-2(u+v)) y^(2(u+v)) z^(l-2t-|m|),
// C_tuv = (-1)^(t+v-vm) (1/4)^t binom(l,t) binom(l-t,|m|+t) binom(t,u) binom(|m|,2v),
// v = vm, vm+1, ..., with vm = 0 for m >= 0 and 1/2 for m < 0.
void build_sph(double sph[kLmax + 1][2 * kLmax + 1][10]) {
  std::memset(sph, 0, sizeof(double) * (kLmax + 1) * (2 * kLmax + 1) * 10);
  for (int l = 0; l <= kLmax; ++l)
    for (int m = -l; m <= l; ++m) {
      const int am = m < 0 ? -m : m;
      const int twovm = m < 0 ? 1 : 0;  // 2 vm
      for (int t = 0; t <= (l - am) / 2; ++t)
        for (int u = 0; u <= t; ++u)
          for (int twov = twovm; twov <= am; twov += 2) {
            const int sgn = ((t + (twov - twovm) / 2) & 1) ? -1 : 1;
            const double c = sgn * std::pow(0.25, t) * binom(l, t) * binom(l - t, am + t) *
                             binom(t, u) * binom(am, twov);
            const int lx = 2 * t + am - 2 * u - twov, ly = 2 * u + twov, lz = l - 2 * t - am;
            if (lx < 0 || lz < 0) continue;
            int k = 0;  // Cartesian index of (lx, ly, lz)
            for (int x = l; x > lx; --x) k += l - x + 1;
            k += l - lx - ly;
            sph[l][m + l][k] += c;
          }
    }
}

// F_n(T_i), T_i = i / kBoysPerUnit, by the series
// F_N(T) = e^-T sum_k (2T)^k / ((2N+1)(2N+3)...(2N+2k+1)) for the highest
// order (all terms positive) and downward recursion, in long double.
void build_boys(double* tab) {
  for (int i = 0; i < kBoysPoints; ++i) {
    const long double T = (long double)i / kBoysPerUnit;
    const int N = kBoysOrders - 1;
    long double term = 1.0L / (2 * N + 1), sum = term;
    for (int k = 1; k < 2000; ++k) {
      term *= 2.0L * T / (2 * N + 2 * k + 1);
      sum += term;
      if (term < 1e-22L * sum) break;
    }
    const long double et = expl(-T);
    long double f[kBoysOrders];
    f[N] = et * sum;
    for (int n = N - 1; n >= 0; --n) f[n] = (2.0L * T * f[n + 1] + et) / (2 * n + 1);
    for (int n = 0; n < kBoysOrders; ++n) tab[(size_t)i * kBoysOrders + n] = (double)f[n];
  }
}

double dfact(int n) {  // n!!, 1 for n <= 0
  double r = 1.0;
  for (int k = n; k > 1; k -= 2) r *= k;
  return r;
}

// Host copy of a basis: primitive-normalised coefficients and, per function,
// the factor that normalises its contracted spherical function.
struct HostBasis {
  std::vector<ShellD> sh;
  std::vector<double> exps, cofs, norm;
  int nbf = 0;
  int maxl = 0;
};

int make_basis(const corr_basis* b, const double sph[kLmax + 1][2 * kLmax + 1][10],
               HostBasis* out, const char* what) {
  CORR_CHECK_ARG(b && b->nsh >= 1 && b->l && b->nprim && b->poff && b->center && b->exps &&
                     b->coefs,
                 "corr_ri_integrals: bad %s basis", what);
  out->sh.resize(b->nsh);
  int nprim_total = 0;
  for (int s = 0; s < b->nsh; ++s) {
    CORR_CHECK_ARG(b->l[s] >= 0 && b->l[s] <= kLmax,
                   "corr_ri_integrals: %s shell %d has l = %d (supported: 0..%d)", what, s,
                   b->l[s], kLmax);
    CORR_CHECK_ARG(b->nprim[s] >= 1 && b->poff[s] >= 0,
                   "corr_ri_integrals: %s shell %d: bad primitives", what, s);
    nprim_total = std::max(nprim_total, b->poff[s] + b->nprim[s]);
  }
  out->exps.assign(b->exps, b->exps + nprim_total);
  out->cofs.assign(nprim_total, 0.0);
  int bf = 0;
  for (int s = 0; s < b->nsh; ++s) {
    const int l = b->l[s];
    ShellD& d = out->sh[s];
    d.x = b->center[3 * s];
    d.y = b->center[3 * s + 1];
    d.z = b->center[3 * s + 2];
    d.l = l;
    d.nprim = b->nprim[s];
    d.poff = b->poff[s];
    d.bf = bf;
    out->maxl = std::max(out->maxl, l);
    for (int k = 0; k < d.nprim; ++k) {
      const double a = b->exps[d.poff + k];
      CORR_CHECK_ARG(a > 0.0, "corr_ri_integrals: %s shell %d: exponent must be positive", what, s);
      // x^l exp(-a r^2) normalised: (2a/pi)^(3/4) (4a)^(l/2) / sqrt((2l-1)!!)
      out->cofs[d.poff + k] = b->coefs[d.poff + k] * std::pow(2.0 * a / M_PI, 0.75) *
                              std::pow(4.0 * a, 0.5 * l) / std::sqrt(dfact(2 * l - 1));
    }
    // self-overlap of the contracted spherical functions (one centre):
    // S_ij = sum_pq c_p c_q prod_dim m(e_i + e_j, a_p + a_q),
    // m(n, s) = (n-1)!! / (2s)^(n/2) sqrt(pi/s) for even n, 0 for odd n
    const int nc = ncart(l);
    std::vector<double> Sc(nc * nc, 0.0);
    for (int i = 0; i < nc; ++i)
      for (int j = 0; j < nc; ++j) {
        double s = 0.0;
        for (int p = 0; p < d.nprim; ++p)
          for (int q = 0; q < d.nprim; ++q) {
            const double sa = out->exps[d.poff + p] + out->exps[d.poff + q];
            double f = out->cofs[d.poff + p] * out->cofs[d.poff + q];
            for (int dim = 0; dim < 3; ++dim) {
              const int n = cexp(l, i, dim) + cexp(l, j, dim);
              if (n & 1) {
                f = 0.0;
                break;
              }
              f *= dfact(n - 1) / std::pow(2.0 * sa, 0.5 * n) * std::sqrt(M_PI / sa);
            }
            s += f;
          }
        Sc[i * nc + j] = s;
      }
    for (int m = 0; m < 2 * l + 1; ++m) {
      double ov = 0.0;
      for (int i = 0; i < nc; ++i)
        for (int j = 0; j < nc; ++j) ov += sph[l][m][i] * Sc[i * nc + j] * sph[l][m][j];
      CORR_CHECK_ARG(ov > 0.0, "corr_ri_integrals: %s shell %d has a null function", what, s);
      out->norm.push_back(1.0 / std::sqrt(ov));
    }
    bf += 2 * l + 1;
  }
  out->nbf = bf;
  return CORR_OK;
}

// Primitive screening of the 3-index integrals.  For primitive Gaussians
// (exponents a, b on centres A, B; coefficients with their normalisation)
// the Schwarz inequality |(P|ab)| <= (P|P)^1/2 (ab|ab)^1/2 with, for s
// functions, (ab|ab) = 2 pi^(5/2) / (p^2 sqrt(2p)) K_ab^2, p = a + b,
// K_ab = exp(-ab/p |AB|^2); the factor (1 + |AB|)^(la+lb) (1 + 1/sqrt p)^(la+lb)
// covers the polynomial parts of higher angular momenta.  A primitive pair
// whose bound times the largest auxiliary factor stays below kScreen is
// skipped (its contributions lie below 1e-15 of the unit-normalised
// integrals); a shell pair left with none is zero.
constexpr double kScreen = 1e-15;

double aux_schwarz_max(const HostBasis& hb) {
  double m = 0.0;
  for (const ShellD& sh : hb.sh)
    for (int k = 0; k < sh.nprim; ++k) {
      const double q = hb.exps[sh.poff + k];
      const double f = std::fabs(hb.cofs[sh.poff + k]) *
                       std::sqrt(2.0 * std::pow(M_PI, 2.5) / (q * q * std::sqrt(2.0 * q))) *
                       std::pow(1.0 + 1.0 / std::sqrt(q), sh.l);
      m = std::max(m, f);
    }
  return m;
}

void screen_pairs(const HostBasis& hb, int x, int y, double saux, std::vector<ushort2>* pp) {
  const ShellD& A = hb.sh[x];
  const ShellD& B = hb.sh[y];
  const double dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
  const double r2 = dx * dx + dy * dy + dz * dz, r = std::sqrt(r2);
  const int lsum = A.l + B.l;
  for (int i = 0; i < A.nprim; ++i)
    for (int j = 0; j < B.nprim; ++j) {
      const double a = hb.exps[A.poff + i], b = hb.exps[B.poff + j], p = a + b;
      const double kab = std::exp(-a * b / p * r2);
      const double bound = std::fabs(hb.cofs[A.poff + i] * hb.cofs[B.poff + j]) * kab *
                           std::sqrt(2.0 * std::pow(M_PI, 2.5) / (p * p * std::sqrt(2.0 * p))) *
                           std::pow((1.0 + r) * (1.0 + 1.0 / std::sqrt(p)), lsum) * saux;
      if (bound >= kScreen) pp->push_back(make_ushort2((unsigned short)i, (unsigned short)j));
    }
}

using Kern = void (*)(Basis3);

template <int LP, int LC, int LD>
Kern kern() {
  return eri3_kernel<LP, LC, LD>;
}

// class table: ket classes (LC, LD) used by the 3-index (LD <= LC <= 2) and
// the 2-index (LD = 0, LC <= 3) integrals
Kern class_kernel(int lp, int lc, int ld) {
#define KC(LP)                                                     \
  if (lp == LP) {                                                  \
    if (lc == 0 && ld == 0) return kern<LP, 0, 0>();               \
    if (lc == 1 && ld == 0) return kern<LP, 1, 0>();               \
    if (lc == 1 && ld == 1) return kern<LP, 1, 1>();               \
    if (lc == 2 && ld == 0) return kern<LP, 2, 0>();               \
    if (lc == 2 && ld == 1) return kern<LP, 2, 1>();               \
    if (lc == 2 && ld == 2) return kern<LP, 2, 2>();               \
    if (lc == 3 && ld == 0) return kern<LP, 3, 0>();               \
  }
  KC(0)
  KC(1)
  KC(2)
  KC(3)
#undef KC
  return nullptr;
}

}  // namespace

}  // namespace corr

using namespace corr;

extern "C" int corr_ri_integrals(corr_context* c, const corr_basis* obs, const corr_basis* aux,
                                 double* J, double* pmn) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(J || pmn, "corr_ri_integrals: nothing to compute (J and pmn both NULL)");
  CORR_CHECK_ARG(aux != nullptr && (obs != nullptr || !pmn),
                 "corr_ri_integrals: null basis argument");
  CORR_CUDA(cudaSetDevice(c->device));
  double sph[kLmax + 1][2 * kLmax + 1][10];
  build_sph(sph);
  HostBasis ha, ho;
  CORR_TRY(make_basis(aux, sph, &ha, "auxiliary"));
  if (pmn) {
    CORR_TRY(make_basis(obs, sph, &ho, "orbital"));
    CORR_CHECK_ARG(ho.maxl <= 2, "corr_ri_integrals: orbital shells up to d are supported");
  }
  const int X = ha.nbf, N = pmn ? ho.nbf : 0;
  // shell lists by angular momentum, ket pairs by class
  std::vector<std::vector<int>> alist(kLmax + 1);
  for (int s = 0; s < (int)ha.sh.size(); ++s) alist[ha.sh[s].l].push_back(s);
  std::vector<std::vector<int2>> plist3(9), plist2(kLmax + 1);  // 3c: lc*3 + ld ; 2c: lc
  // primitive pairs of every ket pair: all of them for (P|Q); for (P|cd) the
  // pairs whose Schwarz factor can reach kScreen (see screen_pairs)
  std::vector<std::vector<int2>> prange3(9), prange2(kLmax + 1);
  std::vector<ushort2> pp;
  std::vector<PairData> ppd;
  for (int s = 0; s < (int)ha.sh.size(); ++s) {
    const int b = (int)pp.size();
    for (int k = 0; k < ha.sh[s].nprim; ++k) {
      pp.push_back(make_ushort2((unsigned short)k, 0));
      const ShellD& A = ha.sh[s];
      const double a = ha.exps[A.poff + k];
      ppd.push_back(PairData{a, A.x, A.y, A.z, 1.0, 1.0, 1.0, ha.cofs[A.poff + k] / a, 0.5 / a});
    }
    plist2[ha.sh[s].l].push_back(make_int2(s, -1));
    prange2[ha.sh[s].l].push_back(make_int2(b, (int)pp.size()));
  }
  long long pairs_kept = 0, pairs_all = 0;
  if (pmn) {
    const double saux = aux_schwarz_max(ha);
    for (int cs = 0; cs < (int)ho.sh.size(); ++cs)
      for (int ds = 0; ds <= cs; ++ds) {
        int x = cs, y = ds;
        if (ho.sh[x].l < ho.sh[y].l) std::swap(x, y);  // lc >= ld
        const int b = (int)pp.size();
        screen_pairs(ho, x, y, saux, &pp);
        for (int q = b; q < (int)pp.size(); ++q) {
          const ShellD& A = ho.sh[x];
          const ShellD& B = ho.sh[y];
          const double a = ho.exps[A.poff + pp[q].x], bb = ho.exps[B.poff + pp[q].y];
          const double pe = a + bb, mu = a * bb / pe;
          const double dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
          ppd.push_back(PairData{pe, (a * A.x + bb * B.x) / pe, (a * A.y + bb * B.y) / pe,
                                 (a * A.z + bb * B.z) / pe, std::exp(-mu * dx * dx),
                                 std::exp(-mu * dy * dy), std::exp(-mu * dz * dz),
                                 ho.cofs[A.poff + pp[q].x] * ho.cofs[B.poff + pp[q].y] / pe,
                                 0.5 / pe});
        }
        pairs_all += (long long)ho.sh[x].nprim * ho.sh[y].nprim;
        pairs_kept += (long long)pp.size() - b;
        if ((int)pp.size() == b) continue;  // every integral of the pair is below the threshold
        plist3[ho.sh[x].l * 3 + ho.sh[y].l].push_back(make_int2(x, y));
        prange3[ho.sh[x].l * 3 + ho.sh[y].l].push_back(make_int2(b, (int)pp.size()));
      }
  }
  (void)pairs_all;
  (void)pairs_kept;
  // device copies (workspace): shells, primitives, norms, lists, staged outputs
  auto bytes_of = [](size_t n, size_t e) { return n * e; };
  size_t nal = 0, np3 = 0, np2 = 0;
  for (auto& v : alist) nal += v.size();
  for (auto& v : plist3) np3 += v.size();
  for (auto& v : plist2) np2 += v.size();
  const bool jdev = J && is_device_ptr(J), pdev = pmn && is_device_ptr(pmn);
  auto plan = [&](Carver& w, void** p) {
    p[0] = w.take(bytes_of(ha.sh.size(), sizeof(ShellD)));
    p[1] = w.take(bytes_of(ha.exps.size(), 8));
    p[2] = w.take(bytes_of(ha.cofs.size(), 8));
    p[3] = w.take(bytes_of(ha.norm.size(), 8));
    p[4] = w.take(bytes_of(nal, 4));
    p[5] = w.take(bytes_of(np2, 8));
    p[6] = pmn ? w.take(bytes_of(ho.sh.size(), sizeof(ShellD))) : nullptr;
    p[7] = pmn ? w.take(bytes_of(ho.exps.size(), 8)) : nullptr;
    p[8] = pmn ? w.take(bytes_of(ho.cofs.size(), 8)) : nullptr;
    p[9] = pmn ? w.take(bytes_of(ho.norm.size(), 8)) : nullptr;
    p[10] = pmn ? w.take(bytes_of(np3, 8)) : nullptr;
    p[11] = (J && !jdev) ? w.take((size_t)X * X * 8) : nullptr;
    p[12] = (pmn && !pdev) ? w.take((size_t)X * N * N * 8) : nullptr;
    p[13] = w.take(bytes_of(np2, 8));
    p[14] = pmn ? w.take(bytes_of(np3, 8)) : nullptr;
    p[15] = w.take(bytes_of(pp.size(), 4));
    p[16] = w.take(bytes_of(ppd.size(), sizeof(PairData)));
    p[17] = w.take(bytes_of(ha.exps.size(), 8));
    p[18] = w.take(bytes_of(ha.exps.size(), 8));
  };
  void* p[19];
  Carver cv{nullptr, 0};
  plan(cv, p);
  CORR_TRY(c->ws.reserve(cv.used));
  Carver w{c->ws.ptr, 0};
  plan(w, p);
  // host-side packing of the lists (contiguous per class)
  std::vector<int> aflat;
  std::vector<int> aoff(kLmax + 2, 0);
  for (int l = 0; l <= kLmax; ++l) {
    aoff[l] = (int)aflat.size();
    aflat.insert(aflat.end(), alist[l].begin(), alist[l].end());
  }
  aoff[kLmax + 1] = (int)aflat.size();
  std::vector<int2> p2flat, p3flat, r2flat, r3flat;
  std::vector<int> p2off(kLmax + 2, 0), p3off(10, 0);
  for (int l = 0; l <= kLmax; ++l) {
    p2off[l] = (int)p2flat.size();
    p2flat.insert(p2flat.end(), plist2[l].begin(), plist2[l].end());
    r2flat.insert(r2flat.end(), prange2[l].begin(), prange2[l].end());
  }
  p2off[kLmax + 1] = (int)p2flat.size();
  for (int k = 0; k < 9; ++k) {
    p3off[k] = (int)p3flat.size();
    p3flat.insert(p3flat.end(), plist3[k].begin(), plist3[k].end());
    r3flat.insert(r3flat.end(), prange3[k].begin(), prange3[k].end());
  }
  p3off[9] = (int)p3flat.size();
  auto up = [&](void* dst, const void* src, size_t n) -> int {
    if (n) CORR_CUDA(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, c->stream));
    return CORR_OK;
  };
  CORR_TRY(up(p[0], ha.sh.data(), ha.sh.size() * sizeof(ShellD)));
  CORR_TRY(up(p[1], ha.exps.data(), ha.exps.size() * 8));
  CORR_TRY(up(p[2], ha.cofs.data(), ha.cofs.size() * 8));
  CORR_TRY(up(p[3], ha.norm.data(), ha.norm.size() * 8));
  CORR_TRY(up(p[4], aflat.data(), aflat.size() * 4));
  CORR_TRY(up(p[5], p2flat.data(), p2flat.size() * 8));
  CORR_TRY(up(p[13], r2flat.data(), r2flat.size() * 8));
  CORR_TRY(up(p[15], pp.data(), pp.size() * 4));
  CORR_TRY(up(p[16], ppd.data(), ppd.size() * sizeof(PairData)));
  std::vector<double> arq(ha.exps.size()), ahq(ha.exps.size());
  for (size_t k = 0; k < ha.exps.size(); ++k) {
    arq[k] = ha.cofs[k] / ha.exps[k];
    ahq[k] = 0.5 / ha.exps[k];
  }
  CORR_TRY(up(p[17], arq.data(), arq.size() * 8));
  CORR_TRY(up(p[18], ahq.data(), ahq.size() * 8));
  if (pmn) {
    CORR_TRY(up(p[14], r3flat.data(), r3flat.size() * 8));
    CORR_TRY(up(p[6], ho.sh.data(), ho.sh.size() * sizeof(ShellD)));
    CORR_TRY(up(p[7], ho.exps.data(), ho.exps.size() * 8));
    CORR_TRY(up(p[8], ho.cofs.data(), ho.cofs.size() * 8));
    CORR_TRY(up(p[9], ho.norm.data(), ho.norm.size() * 8));
    CORR_TRY(up(p[10], p3flat.data(), p3flat.size() * 8));
  }
  CORR_CUDA(cudaMemcpyToSymbolAsync(c_sph, sph, sizeof(sph), 0, cudaMemcpyHostToDevice, c->stream));
  {
    static std::vector<double> boys_tab;
    static bool boys_done[64] = {};
    if (boys_tab.empty()) {
      boys_tab.resize((size_t)kBoysPoints * kBoysOrders);
      build_boys(boys_tab.data());
    }
    if (c->device < 0 || c->device >= 64 || !boys_done[c->device]) {
      CORR_CUDA(cudaMemcpyToSymbol(d_boys, boys_tab.data(), boys_tab.size() * 8));
      if (c->device >= 0 && c->device < 64) boys_done[c->device] = true;
    }
  }
  {
    static int ce[kLmax + 1][10][3], tv[kTmax][kTmax][kTmax];  // constant tables
    for (int l = 0; l <= kLmax; ++l)
      for (int k = 0; k < 10; ++k)
        for (int d = 0; d < 3; ++d) ce[l][k][d] = k < ncart(l) ? cexp(l, k, d) : 0;
    for (int t = 0; t < kTmax; ++t)
      for (int u = 0; u < kTmax; ++u)
        for (int v = 0; v < kTmax; ++v) tv[t][u][v] = tuv_index(t, u, v);
    CORR_CUDA(cudaMemcpyToSymbolAsync(c_cexp, ce, sizeof(ce), 0, cudaMemcpyHostToDevice,
                                      c->stream));
    CORR_CUDA(cudaMemcpyToSymbolAsync(c_tuv, tv, sizeof(tv), 0, cudaMemcpyHostToDevice,
                                      c->stream));
  }
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  mark(c, 0);
  mark(c, 1);
  CORR_CUDA(cudaGetLastError());
  // The largest classes keep their Cartesian block and Hermite tables in
  // local memory (up to ~8 KB per thread): raise this context's per-thread
  // stack limit to what the kernels of this call need, if it is lower.
  {
    size_t need = 0;
    for (int lp = 0; lp <= kLmax; ++lp)
      for (int lc = 0; lc <= kLmax; ++lc)
        for (int ld = 0; ld <= 2; ++ld) {
          Kern k = class_kernel(lp, lc, ld);
          if (!k) continue;
          cudaFuncAttributes fa{};
          CORR_CUDA(cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(k)));
          need = std::max(need, fa.localSizeBytes);
        }
    size_t have = 0;
    CORR_CUDA(cudaDeviceGetLimit(&have, cudaLimitStackSize));
    need = (need + 1023) / 1024 * 1024 + 1024;
    if (have < need) CORR_CUDA(cudaDeviceSetLimit(cudaLimitStackSize, need));
  }
  // The classes write disjoint blocks of J and (P|mu nu): they run on eight
  // side streams forked from (and joined back into) the context stream, so
  // the tails of the large classes overlap the small ones.
  constexpr int kSide = 8;
  struct Side {
    cudaStream_t st[kSide] = {};
    cudaEvent_t ev[kSide + 1] = {};
    ~Side() {
      for (cudaStream_t x : st)
        if (x) cudaStreamDestroy(x);
      for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    }
  } side;
  for (int k = 0; k < kSide; ++k) {
    CORR_CUDA(cudaStreamCreateWithFlags(&side.st[k], cudaStreamNonBlocking));
    CORR_CUDA(cudaEventCreateWithFlags(&side.ev[k], cudaEventDisableTiming));
  }
  CORR_CUDA(cudaEventCreateWithFlags(&side.ev[kSide], cudaEventDisableTiming));
  CORR_CUDA(cudaEventRecord(side.ev[kSide], c->stream));
  for (int k = 0; k < kSide; ++k) CORR_CUDA(cudaStreamWaitEvent(side.st[k], side.ev[kSide], 0));
  int next_stream = 0;
  auto launch = [&](Kern k, Basis3 g, int lp, int lc, int ld) -> int {
    const long long work = (long long)g.nalist * g.nplist;
    if (work <= 0) return CORR_OK;
    const int grid = (int)std::min<long long>((work + 127) / 128, (long long)c->sms * 32);
    k<<<grid, 128, 0, side.st[next_stream]>>>(g);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      cudaFuncAttributes fa{};
      cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(k));
      cudaGetLastError();
      size_t lim = 0;
      cudaDeviceGetLimit(&lim, cudaLimitStackSize);
      cudaGetLastError();
      set_error("corr_ri_integrals: launch of class (%d|%d %d) failed: %s (local %zu B, "
                "max threads per block %d, registers %d, stack limit %zu, grid %d)",
                lp, lc, ld, cudaGetErrorString(e), fa.localSizeBytes, fa.maxThreadsPerBlock,
                fa.numRegs, lim, grid);
      return CORR_ERR_CUDA;
    }
    c->launches += 1;
    return CORR_OK;
  };
  const ShellD* dA = static_cast<const ShellD*>(p[0]);
  double* Jout = J ? (jdev ? J : static_cast<double*>(p[11])) : nullptr;
  double* Pout = pmn ? (pdev ? pmn : static_cast<double*>(p[12])) : nullptr;
  if (Pout) CORR_CUDA(cudaMemsetAsync(Pout, 0, (size_t)X * N * N * 8, c->stream));
  // every class launch with a cost estimate (auxiliary primitives x orbital
  // primitive pairs x Cartesian components); launched largest first, each on
  // the side stream with the least estimated work so far
  struct Job {
    Kern k;
    Basis3 g;
    int lp, lc, ld;
    double cost;
  };
  std::vector<Job> jobs;
  auto pairs_of = [](const std::vector<int2>& r) {
    double n = 0.0;
    for (const int2& x : r) n += x.y - x.x;
    return n;
  };
  for (int lp = 0; lp <= kLmax; ++lp) {
    const int na = aoff[lp + 1] - aoff[lp];
    if (na == 0) continue;
    double aprim = 0.0;
    for (int sidx : alist[lp]) aprim += ha.sh[sidx].nprim;
    Basis3 g{};
    g.aux = dA;
    g.alist = static_cast<const int*>(p[4]) + aoff[lp];
    g.nalist = na;
    g.aexp = static_cast<const double*>(p[1]);
    g.acof = static_cast<const double*>(p[2]);
    g.anorm = static_cast<const double*>(p[3]);
    g.ppd = static_cast<const PairData*>(p[16]);
    g.arq = static_cast<const double*>(p[17]);
    g.ahq = static_cast<const double*>(p[18]);
    if (J) {  // (P|Q): the ket is the auxiliary basis with an exponent-0 s partner
      for (int lc = 0; lc <= kLmax; ++lc) {
        Basis3 h = g;
        h.obs = dA;
        h.plist = static_cast<const int2*>(p[5]) + p2off[lc];
        h.prange = static_cast<const int2*>(p[13]) + p2off[lc];
        h.pp = static_cast<const ushort2*>(p[15]);
        h.nplist = p2off[lc + 1] - p2off[lc];
        h.oexp = h.aexp;
        h.ocof = h.acof;
        h.onorm = h.anorm;
        h.out = Jout;
        h.N = X;
        h.two_center = 1;
        jobs.push_back({class_kernel(lp, lc, 0), h, lp, lc, 0,
                        aprim * pairs_of(prange2[lc]) * ncart(lp) * ncart(lc)});
      }
    }
    if (pmn) {
      for (int lc = 0; lc <= 2; ++lc)
        for (int ld = 0; ld <= lc; ++ld) {
          Basis3 h = g;
          h.obs = static_cast<const ShellD*>(p[6]);
          h.plist = static_cast<const int2*>(p[10]) + p3off[lc * 3 + ld];
          h.prange = static_cast<const int2*>(p[14]) + p3off[lc * 3 + ld];
          h.pp = static_cast<const ushort2*>(p[15]);
          h.nplist = p3off[lc * 3 + ld + 1] - p3off[lc * 3 + ld];
          h.oexp = static_cast<const double*>(p[7]);
          h.ocof = static_cast<const double*>(p[8]);
          h.onorm = static_cast<const double*>(p[9]);
          h.out = Pout;
          h.N = N;
          h.two_center = 0;
          jobs.push_back({class_kernel(lp, lc, ld), h, lp, lc, ld,
                          aprim * pairs_of(prange3[lc * 3 + ld]) * ncart(lp) * ncart(lc) *
                              ncart(ld)});
        }
    }
  }
  std::stable_sort(jobs.begin(), jobs.end(),
                   [](const Job& a, const Job& b) { return a.cost > b.cost; });
  double load[kSide] = {};
  for (const Job& jb : jobs) {
    int k = 0;
    for (int q = 1; q < kSide; ++q)
      if (load[q] < load[k]) k = q;
    load[k] += jb.cost;
    next_stream = k;
    CORR_TRY(launch(jb.k, jb.g, jb.lp, jb.lc, jb.ld));
  }
  for (int k = 0; k < kSide; ++k) {
    CORR_CUDA(cudaEventRecord(side.ev[k], side.st[k]));
    CORR_CUDA(cudaStreamWaitEvent(c->stream, side.ev[k], 0));
  }
  mark(c, 2);
  if (J && !jdev) CORR_TRY(stage_out(c, J, Jout, (size_t)X * X * 8));
  if (pmn && !pdev) CORR_TRY(stage_out(c, pmn, Pout, (size_t)X * N * N * 8));
  return finish_results(c, 0);
}
