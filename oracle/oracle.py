"""ORACLE -- test infrastructure, not product code.

CPU restatement of the reference's correlation hot path (Masterluke87/corr), used
only by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` as the checker.  Nothing in the ``corr_gb300`` package imports it.

* numpy restatements of the BLAS-shaped steps (RI-MP2 energy, J^-1/2, B build),
  each citing the reference lines it follows;
* ctypes front end of ``liboracle.so`` (oracle/corr_oracle.c: packed-ERI
  handling, MOtrans, canonical MP2, build_FMo, transform_ri);
* the seeded synthetic input generators (numpy ``PCG64``) every test and the
  bench share;
* an FP64 restatement of the RI-MP2 gradient (no reference counterpart: the
  reference has no gradient code), for the adjoint checks.

Parity of these restatements is pinned against the reference's own compiled
code (``oracle/_ref``) in tests/test_oracle_pin.py and through the committed
fixtures in tests/golden/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_longlong)
_u16p = ctypes.POINTER(ctypes.c_ushort)


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def build():
    """Compile liboracle.so (gcc; no reference checkout needed)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all", f"PY={sys.executable}"])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle_pack_eri.restype = ctypes.c_longlong
        L.oracle_mo2int_bf.restype = ctypes.c_double
        _LIB = L
    return _LIB


# ---------------------------------------------------------------------------
# Seeded synthetic inputs
# ---------------------------------------------------------------------------

def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def synth_rimp2(nocc, nvir, naux, seed, dtype=np.float64):
    """B^Q_ia = G_Qia * s_Q with G ~ N(0,1), s_Q = 0.05 exp(-Q/400);
    eps_occ ~ U[-1.5,-0.3] sorted, eps_vir ~ U[0.05,3.0] sorted.
    Returns (B[Q][i][a], eps[nocc+nvir])."""
    r = rng(seed)
    B = r.standard_normal((naux, nocc, nvir))
    B *= (0.05 * np.exp(-np.arange(naux) / 400.0))[:, None, None]
    eo = np.sort(r.uniform(-1.5, -0.3, nocc))
    ev = np.sort(r.uniform(0.05, 3.0, nvir))
    return np.ascontiguousarray(B, dtype=dtype), np.concatenate([eo, ev])


def synth_batch_sizes(count, seed):
    """nocc ~ U{5..60}, nvir = nocc * U{4..8}, naux = round(3.5 nvir)."""
    r = rng(seed)
    out = []
    for _ in range(count):
        o = int(r.integers(5, 61))
        v = o * int(r.integers(4, 9))
        out.append((o, v, int(round(3.5 * v))))
    return out


def synth_orbitals(N, seed):
    """A random orthogonal MO coefficient matrix mos[p][mu]."""
    q, _ = np.linalg.qr(rng(seed).standard_normal((N, N)))
    return np.ascontiguousarray(q.T)


def synth_eri(N, seed, rank=None, scale=0.1):
    """A dense AO ERI tensor with the 8-fold permutational symmetry of real
    integrals and positive semi-definite (ab|cd) metric: (ab|cd) = sum_P
    L_Pab L_Pcd with L_P symmetric.  Returns (eri[N^4], L[P][N][N])."""
    r = rng(seed)
    P = rank or 2 * N
    L = r.standard_normal((P, N, N)) * scale
    L = 0.5 * (L + L.transpose(0, 2, 1))
    eri = np.einsum("Pab,Pcd->abcd", L, L, optimize=True)
    return np.ascontiguousarray(eri), L


# ---------------------------------------------------------------------------
# RI-MP2 energy: src/POSTHF/can_mp2.cc:53-132
# ---------------------------------------------------------------------------

def rimp2_energy(B, eps, nocc, nvir):
    """Restates run_canonical_mp2_ri (can_mp2.cc:82-97): for every ordered
    (i,j), M = B_i^T B_j (dgemm, :88), X = 1/(e_a+e_b-e_i-e_j) (:91),
    MD = M - M^T (:92), tmp = M*X (:95), E_OS -= tmp.M, E_SS -= tmp.MD
    (:96-97).  Returns (E_SS, E_OS, E)."""
    naux = B.shape[0]
    Bv = np.asarray(B, dtype=np.float64).reshape(naux, nocc, nvir)
    ev = np.asarray(eps[nocc:nocc + nvir], dtype=np.float64)
    eab = ev[:, None] + ev[None, :]
    eos = ess = 0.0
    for i in range(nocc):
        Bi = Bv[:, i, :]
        for j in range(nocc):
            M = Bi.T @ Bv[:, j, :]
            X = 1.0 / ((eab - eps[i]) - eps[j])
            tmp = M * X
            eos -= float(np.dot(tmp.ravel(), M.ravel()))
            ess -= float(np.dot(tmp.ravel(), (M - M.T).ravel()))
    return ess, eos, ess + eos


def rimp2_energy_pairs(B, eps, nocc, nvir, pairs):
    """The same sum restricted to a list of ordered (i,j) pairs (a bounded
    sample of the full job, for timing)."""
    naux = B.shape[0]
    Bv = np.asarray(B).reshape(naux, nocc, nvir)
    ev = np.asarray(eps[nocc:nocc + nvir])
    eab = ev[:, None] + ev[None, :]
    eos = ess = 0.0
    for i, j in pairs:
        M = Bv[:, i, :].T @ Bv[:, j, :]
        X = 1.0 / ((eab - eps[i]) - eps[j])
        tmp = M * X
        eos -= float(np.dot(tmp.ravel(), M.ravel()))
        ess -= float(np.dot(tmp.ravel(), (M - M.T).ravel()))
    return ess, eos, ess + eos


def rimp2_gradient(B, eps, nocc, nvir):
    """FP64 gradient of E = E_OS + E_SS (no reference counterpart).

    With M^{ij}_ab = sum_Q B^Q_ia B^Q_jb and D = e_a+e_b-e_i-e_j:
      E = -sum_{ijab} (2 M_ab - M_ba) M_ab / D,
      G^{ij}_ab = dE/dM^{ij}_ab = -(4 M_ab - 2 M_ba) / D,
      dE/dB^Q_ia = 2 sum_{jb} G^{ij}_ab B^Q_jb,
      dE/de_c (virtual)  = +sum W over every (a or b) == c,
      dE/de_k (occupied) = -sum W over every (i or j) == k,
    where W^{ij}_ab = (2 M_ab - M_ba) M_ab / D^2.
    Returns (E, dB[Q][i][a], deps[nocc+nvir])."""
    naux = B.shape[0]
    Bv = np.asarray(B, dtype=np.float64).reshape(naux, nocc, nvir)
    ev = np.asarray(eps[nocc:nocc + nvir], dtype=np.float64)
    eab = ev[:, None] + ev[None, :]
    dB = np.zeros_like(Bv)
    deps = np.zeros(nocc + nvir)
    E = 0.0
    for i in range(nocc):
        Bi = Bv[:, i, :]
        for j in range(nocc):
            Bj = Bv[:, j, :]
            M = Bi.T @ Bj
            D = (eab - eps[i]) - eps[j]
            T = 2.0 * M - M.T
            E -= float(np.sum(T * M / D))
            G = -2.0 * T / D
            dB[:, i, :] += 2.0 * (Bj @ G.T)
            W = T * M / (D * D)
            sW = W.sum()
            deps[nocc:] += W.sum(axis=1) + W.sum(axis=0)
            deps[i] -= sW
            deps[j] -= sW
    return E, dB, deps


def rimp2_energy_local(B, eps, nocc, nvir, i, a):
    """The part of the RI-MP2 energy (can_mp2.cc:82-97 summed over all ordered
    (i,j)) that contains an integral with orbital pair (i,a): every term of the
    pairs (i,j) and (j,i) whose (c,d) has c == a or d == a.  It changes with
    B^Q_ia exactly as the full energy does, at O(nocc nvir naux) cost, so
    central differences of it equal those of the full energy."""
    naux = B.shape[0]
    Bv = np.asarray(B).reshape(naux, nocc, nvir)
    ev = np.asarray(eps[nocc:nocc + nvir])
    row = np.einsum("q,qjb->jb", Bv[:, i, a], Bv)        # M^{ij}_{a,b}
    col = np.einsum("qc,qj->jc", Bv[:, i, :], Bv[:, :, a])  # M^{ij}_{c,a}
    tot = 0.0
    for j in range(nocc):
        w = 1.0 if j == i else 2.0  # (j,i) mirrors (i,j)
        Dr = ((ev[a] + ev) - eps[i]) - eps[j]
        r, c = row[j], col[j]
        t_row = -((2.0 * r - c) * r / Dr).sum()   # (a, d):  M_ad, M_da = col[d]
        t_col = -((2.0 * c - r) * c / Dr).sum()   # (c, a):  M_ca = col[c], M_ac = row[c]
        t_aa = -((2.0 * r[a] - c[a]) * r[a] / Dr[a])
        tot += w * (t_row + t_col - t_aa)
    return tot


# ---------------------------------------------------------------------------
# RI metric and B build: src/POSTHF/ri.cc:50-69, 102-103
# ---------------------------------------------------------------------------

def ri_metric_inv_sqrt(J, tol=1e-10):
    """ri.cc:50-69: eigen-decompose J, zero every eigenvalue with
    lambda/lambda_max < tol or lambda < 0, otherwise lambda^-1/2, and return
    V diag V^T together with the number of eigenvalues cut."""
    w, V = np.linalg.eigh(np.asarray(J, dtype=np.float64))
    mx = w[-1]
    cut = (w / mx < tol) | (w < 0)
    inv = np.where(cut, 0.0, 1.0 / np.sqrt(np.where(cut, 1.0, w)))
    return (V * inv) @ V.T, int(cut.sum())


def ri_build_bpq(Jm12, P3):
    """ri.cc:102-103: BPQ[P][mu][nu] = sum_Q Jm12[P][Q] (Q|mu nu)."""
    X = Jm12.shape[0]
    return (Jm12 @ P3.reshape(X, -1)).reshape(P3.shape)


def transform_ri(nroe, mos, bpq):
    """ri.cc:147-172 via liboracle (two quarter transforms)."""
    X, N, _ = bpq.shape
    o = nroe // 2
    out = np.zeros((X, o, N - o))
    lib().oracle_transform_ri(nroe, N, X, _p(np.ascontiguousarray(mos)),
                              _p(np.ascontiguousarray(bpq)), _p(out))
    return out


def transform_ri_np(nocc, mos, bpq):
    """transform_ri restated with matmuls (same sums, BLAS order)."""
    X, N, _ = bpq.shape
    Co = mos[:nocc]
    Cv = mos[nocc:]
    biq = np.einsum("im,Qmn->Qin", Co, bpq, optimize=True)
    return np.einsum("an,Qin->Qia", Cv, biq, optimize=True)


# ---------------------------------------------------------------------------
# Canonical path: motrans.cc, can_mp2.cc:11-49, ops_rhf.cc:618-900
# ---------------------------------------------------------------------------

class Packed:
    """The reference's TEints (util.h:61-65): intval[n], intnums[4n] (uint16),
    sortcount[4]."""

    def __init__(self, intval, intnums, sortcount):
        self.intval = np.ascontiguousarray(intval, dtype=np.float64)
        self.intnums = np.ascontiguousarray(intnums, dtype=np.uint16)
        self.sortcount = np.ascontiguousarray(sortcount, dtype=np.int64)

    @property
    def nrofint(self):
        return int(self.intval.shape[0])


def pack_eri(eri):
    """ops_rhf.cc:618-723 unique selection + ops_rhf.cc:750-900 resort."""
    eri = np.ascontiguousarray(eri, dtype=np.float64)
    N = eri.shape[0]
    L = lib()
    n = L.oracle_pack_eri(N, _p(eri), None, None)
    val = np.zeros(n)
    num = np.zeros(4 * n, dtype=np.uint16)
    L.oracle_pack_eri(N, _p(eri), _p(val), _p(num, _u16p))
    sc = np.zeros(4, dtype=np.int64)
    L.oracle_resort(_p(num, _u16p), _p(val), ctypes.c_longlong(n), _p(sc, _i64p))
    return Packed(val, num, sc)


def unpack_eri(N, packed):
    out = np.zeros((N, N, N, N))
    lib().oracle_unpack_eri(N, ctypes.c_longlong(packed.nrofint), _p(packed.sortcount, _i64p),
                            _p(packed.intval), _p(packed.intnums, _u16p), _p(out))
    return out


def motrans(mos, packed):
    N = mos.shape[0]
    out = np.zeros((N, N, N, N))
    lib().oracle_motrans(N, _p(np.ascontiguousarray(mos)), ctypes.c_longlong(packed.nrofint),
                         _p(packed.sortcount, _i64p), _p(packed.intval),
                         _p(packed.intnums, _u16p), _p(out))
    return out


def mo2int_bf(i, j, k, l, mos, packed):
    N = mos.shape[0]
    return lib().oracle_mo2int_bf(i, j, k, l, N, _p(np.ascontiguousarray(mos)),
                                  ctypes.c_longlong(packed.nrofint),
                                  _p(packed.sortcount, _i64p), _p(packed.intval),
                                  _p(packed.intnums, _u16p))


def canonical_mp2(nroe, prec, fmo):
    N = fmo.shape[0]
    out = np.zeros(3)
    lib().oracle_canonical_mp2(nroe, N, _p(np.ascontiguousarray(prec)),
                               _p(np.ascontiguousarray(fmo)), _p(out))
    return tuple(out)


def mp2_from_ovov(ovov, eps, nocc, nvir):
    out = np.zeros(3)
    lib().oracle_mp2_from_ovov(nocc, nvir, _p(np.ascontiguousarray(ovov)),
                               _p(np.ascontiguousarray(eps, dtype=np.float64)), _p(out))
    return tuple(out)


# ---------------------------------------------------------------------------
# RHF: src/SCF/ops_rhf.cc, src/SCF/scf.cc
# ---------------------------------------------------------------------------

def build_fmat(pmat, hmat, packed):
    """build_Fmat (ops_rhf.cc:549-591): the five permutation-class loops over
    the unique integrals add up to F = H + sum_ls P_ls ((mn|ls) - 1/2 (ml|ns))."""
    N = pmat.shape[0]
    eri = unpack_eri(N, packed)
    J = np.einsum("mnls,ls->mn", eri, pmat, optimize=True)
    K = np.einsum("mlns,ls->mn", eri, pmat, optimize=True)
    return hmat + J - 0.5 * K


def _dgels(A, b):
    """LAPACK dgels ('N': QR least squares), the solver scf.cc:262-266 calls;
    A here is symmetric, so its column-major reading there is A itself."""
    from scipy.linalg import lapack

    _, x, info = lapack.dgels(A, b.reshape(-1, 1))
    assert info == 0, info
    return x[:, 0]


def run_scf(nroe, S, H, packed, ion_rep=0.0, maxiter=100, mos=None):
    """run_scf (scf.cc:145-321) step for step: calc_S12 (ops_rhf.cc:342),
    check_initial_guess (ops_rhf.cc:15; core guess when |sum_i C_ii| < 0.1),
    the damped density (build_Pmat, scf.cc:41-61), DIIS over 8 pairs with the
    bordered least-squares system (dgels), Calc_e_el, diag_Fmat
    (ops_rhf.cc:425).  Returns dict(mos [p][mu], fmat, moens, energy, one,
    two, iterations)."""
    N = S.shape[0]
    nocc = nroe // 2
    w, U = np.linalg.eigh(S)
    T = U @ np.diag(w ** -0.5) @ U.T

    def diag(F):
        e, V = np.linalg.eigh(T @ F @ T)
        return V.T @ T.T, e  # eigenvectors as rows, then transform_MOs

    C = np.zeros((N, N)) if mos is None else np.array(mos, dtype=np.float64)
    moens = np.zeros(N)
    if abs(np.trace(C)) < 0.1:
        C, moens = diag(H)

    def density(C, P, damp):
        Co = C[:nocc]
        return 2.0 * (1.0 - damp) * Co.T @ Co + damp * P

    P = density(C, np.zeros((N, N)), 0.0)
    eri = unpack_eri(N, packed)

    def fock(P):
        return H + np.einsum("mnls,ls->mn", eri, P) - 0.5 * np.einsum("mlns,ls->mn", eri, P)

    hist_f = [np.zeros((N, N))] * 8
    hist_e = [np.zeros((N, N))] * 8
    damp, Eold, DE, it = 0.5, 100.0, 10.0, 0
    while it < maxiter and abs(DE) > 1e-8:
        P = density(C, P, damp)
        F = fock(P)
        err = S @ P @ F - F @ P @ S
        hist_f = hist_f[1:] + [F]
        hist_e = hist_e[1:] + [err]
        if np.mean(np.abs(err)) < 1e-3 and it >= 8:
            damp = 0.0
            B = np.zeros((9, 9))
            B[:8, :8] = [[np.dot(a.ravel(), b.ravel()) for b in hist_e] for a in hist_e]
            B[:8, 8] = B[8, :8] = -1.0
            rhs = np.zeros(9)
            rhs[8] = -1.0
            c = _dgels(B, rhs)
            F = sum(c[j] * hist_f[j] for j in range(8))
        E = 0.5 * np.sum(P * (F + H))
        DE, Eold = E - Eold, E
        C, moens = diag(F)
        it += 1
    P = density(C, P, damp)
    F = fock(P)
    one, two = np.sum(P * H), np.sum(P * F)
    return {"mos": C, "fmat": F, "moens": moens, "energy": 0.5 * (one + two) + ion_rep,
            "one": one + ion_rep, "two": 0.5 * (two - one), "iterations": it}


def build_fmo(mos, fmat):
    N = mos.shape[0]
    out = np.zeros((N, N))
    lib().oracle_build_fmo(N, _p(np.ascontiguousarray(mos)), _p(np.ascontiguousarray(fmat)),
                           _p(out))
    return out


# ---------------------------------------------------------------------------
# Dense helpers: src/MATH/ops_mat.cc, and read_transform_ri (ri.cc:109-144)
# ---------------------------------------------------------------------------

def diag_mat(mat):
    """ops_mat.cc:21-45: dsyev(JOBZ='V', UPLO='U') of the row-major array,
    which LAPACK reads column-major, i.e. the row-major LOWER triangle.
    Returns (vals ascending, vecs) with vecs[k] = eigenvector of vals[k]."""
    A = np.tril(np.asarray(mat, dtype=np.float64))
    A = A + np.tril(A, -1).T
    w, V = np.linalg.eigh(A)
    return w, np.ascontiguousarray(V.T)


def symmortho_mat(mat, tmat):
    """ops_mat.cc:53-69: dummat = tmat mat, mat <- dummat tmat.  Returns
    (new mat, dummat)."""
    dum = tmat @ mat
    return dum @ tmat, dum


def transform_MOs(mos, tmat):
    """ops_mat.cc:75-88: MOs[x][y] <- sum_z tmat[y][z] MOs[x][z] = (MOs tmat^T);
    tmpvec ends as the last transformed row.  Returns (new MOs, tmpvec)."""
    out = mos @ tmat.T
    return out, out[-1].copy()


def mat_mat_T(a, b):
    """ops_mat.cc:93-105, :122-134: f = a b^T."""
    return a @ b.T


def mat_T_mat(a, b):
    """ops_mat.cc:107-119, :136-148: f = a^T b."""
    return a.T @ b


def pmv(mat, vi):
    """ops_mat.cc:192-198: vo = mat vi."""
    return mat @ vi


def read_transform_ri(path, nroe, nroao, naux, mos):
    """ri.cc:109-144: BPQ[naux][nroao][nroao] read raw (native doubles) from
    `path` (prefix + ".rimp2"), then the transform_ri contractions."""
    bpq = np.fromfile(path, dtype=np.float64, count=naux * nroao * nroao)
    return transform_ri(nroe, mos, bpq.reshape(naux, nroao, nroao))


# ---- CCSD consumer of the MO integrals (src/POSTHF/ccsd.cc) --------------------
def ints_so(prec):
    """Restates calc_ints_so (ccsd.cc:509-535) with get_integral (ccsd.cc:6-9):
    so[i,j,k,l] = (i/2 k/2 | j/2 l/2)[s_i=s_k][s_j=s_l]
                - (i/2 l/2 | j/2 k/2)[s_i=s_l][s_j=s_k],  s_p = p % 2."""
    prec = np.asarray(prec)
    N = prec.shape[0]
    T = prec.transpose(0, 2, 1, 3)  # T[a,b,c,d] = (a c | b d)
    A = T
    B = T.transpose(0, 1, 3, 2)     # B[a,b,c,d] = (a d | b c)
    for ax in range(4):
        A = A.repeat(2, axis=ax)
        B = B.repeat(2, axis=ax)
    s = np.arange(2 * N) % 2
    si, sj, sk, sl = (s[:, None, None, None], s[None, :, None, None], s[None, None, :, None],
                      s[None, None, None, :])
    return A * ((si == sk) & (sj == sl)) - B * ((si == sl) & (sj == sk))


def cc_fock(nroe, mos, hmat, prec):
    """Restates form_fock (ccsd.cc:11-48): h = spin-blocked C H C^T,
    f_pq = h_pq + sum_{j < nroe} <pj||qj>.  Returns (h, f)."""
    mos, hmat, prec = (np.asarray(x) for x in (mos, hmat, prec))
    N = mos.shape[0]
    M = 2 * N
    s = np.arange(M) % 2
    hs = mos @ hmat @ mos.T
    h = hs[np.ix_(np.arange(M) // 2, np.arange(M) // 2)] * (s[:, None] == s[None, :])
    p = np.arange(M)
    twoe = np.zeros((M, M))
    for j in range(nroe):
        a = prec[p[:, None] // 2, p[None, :] // 2, j // 2, j // 2] * (s[:, None] == s[None, :])
        b = prec[p[:, None] // 2, j // 2, j // 2, p[None, :] // 2] * (
            (s[:, None] == s[j]) & (s[j] == s[None, :]))
        twoe += a - b
    return h, h + twoe
