"""ORACLE -- test infrastructure, not product code.

ctypes front end of ``oracle/_ref/libcorr_ref.so``: the reference's own
src/POSTHF, src/SCF, src/MATH and src/IO sources compiled unmodified against the
shim headers in ``oracle/ref_shim`` (see ``oracle/Makefile`` and
``oracle/ref_harness.cc``).  It exists only where the reference checkout does;
tests that need it skip elsewhere, and the golden fixtures in tests/golden/
carry its outputs to machines without it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: CORR_REFERENCE_DIR, else a sibling of the repository
REF = os.environ.get("CORR_REFERENCE_DIR",
                     os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
SO = os.path.join(HERE, "_ref", "libcorr_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_longlong)
_u16p = ctypes.POINTER(ctypes.c_ushort)
_L = None


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def available():
    return os.path.exists(SO) or os.path.isdir(os.path.join(REF, "src"))


def build():
    if os.path.isdir(os.path.join(REF, "src")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={REF}",
                               f"PY={sys.executable}"])


def lib():
    global _L
    if _L is None:
        if not os.path.exists(SO):
            build()
        L = ctypes.CDLL(SO)
        L.ref_pack_eri.restype = ctypes.c_longlong
        L.ref_mo2int_bf.restype = ctypes.c_double
        L.ref_last_output.restype = ctypes.c_char_p
        _L = L
    return _L


def set_threads(n):
    lib().ref_set_threads(int(n))


def rimp2_energy(B, eps, nocc, nvir):
    """src/POSTHF/can_mp2.cc:53 -> (E_SS, E_OS, E)."""
    B = np.ascontiguousarray(B, dtype=np.float64)
    out = np.zeros(3)
    lib().ref_rimp2_energy(nocc, nvir, B.shape[0], _p(B),
                           _p(np.ascontiguousarray(eps, dtype=np.float64)), _p(out))
    return tuple(out)


def canonical_mp2(nroe, prec, fmo):
    out = np.zeros(3)
    lib().ref_canonical_mp2(nroe, fmo.shape[0], _p(np.ascontiguousarray(prec)),
                            _p(np.ascontiguousarray(fmo)), _p(out))
    return tuple(out)


def build_fmo(mos, fmat):
    N = mos.shape[0]
    out = np.zeros((N, N))
    lib().ref_build_fmo(N, _p(np.ascontiguousarray(mos)), _p(np.ascontiguousarray(fmat)), _p(out))
    return out


def pack_eri(eri):
    from oracle.oracle import Packed
    eri = np.ascontiguousarray(eri, dtype=np.float64)
    n = lib().ref_pack_eri(eri.shape[0], _p(eri))
    val = np.zeros(n)
    num = np.zeros(4 * n, dtype=np.uint16)
    sc = np.zeros(4, dtype=np.int64)
    lib().ref_packed_copy(_p(val), _p(num, _u16p), _p(sc, _i64p))
    return Packed(val, num, sc)


def motrans(nroe, mos, packed):
    """src/POSTHF/motrans.cc:35.  One nroao per process (function statics)."""
    N = mos.shape[0]
    out = np.zeros((N, N, N, N))
    lib().ref_motrans(nroe, N, _p(np.ascontiguousarray(mos)), ctypes.c_longlong(packed.nrofint),
                      _p(packed.sortcount, _i64p), _p(packed.intval), _p(packed.intnums, _u16p),
                      _p(out))
    return out


def mo2int_bf(i, j, k, l, mos, packed):
    N = mos.shape[0]
    return lib().ref_mo2int_bf(i, j, k, l, N, _p(np.ascontiguousarray(mos)),
                               ctypes.c_longlong(packed.nrofint), _p(packed.sortcount, _i64p),
                               _p(packed.intval), _p(packed.intnums, _u16p))


def calculate_ri(J, P3):
    """src/POSTHF/ri.cc:7 on tabulated (P|Q) and (P|mn) -> BPQ[P][mu][nu]."""
    X, N, _ = P3.shape
    out = np.zeros((X, N, N))
    lib().ref_calculate_ri(X, N, _p(np.ascontiguousarray(J)), _p(np.ascontiguousarray(P3)),
                           _p(out))
    return out


def transform_ri(nroe, mos, bpq):
    X, N, _ = bpq.shape
    o = nroe // 2
    out = np.zeros((X, o, N - o))
    lib().ref_transform_ri(nroe, N, X, _p(np.ascontiguousarray(mos)),
                           _p(np.ascontiguousarray(bpq)), _p(out))
    return out


def read_transform_ri(prefix, nroe, nroao, naux, mos):
    """src/POSTHF/ri.cc:109: Bia from the raw BPQ file prefix + ".rimp2"."""
    o = nroe // 2
    out = np.zeros((naux, o, nroao - o))
    lib().ref_read_transform_ri(str(prefix).encode(), nroe, nroao, naux,
                                _p(np.ascontiguousarray(mos)), _p(out))
    return out


def rhf(nroe, ion_rep, S, T, V, packed):
    """src/SCF: calc_S12, core guess, run_scf (100 iterations).
    Returns (mos[p][mu], Fmat, MOens, E_HF)."""
    N = S.shape[0]
    mos = np.zeros((N, N))
    f = np.zeros((N, N))
    e = np.zeros(N)
    eh = np.zeros(1)
    lib().ref_rhf(nroe, N, ctypes.c_double(ion_rep), _p(np.ascontiguousarray(S)),
                  _p(np.ascontiguousarray(T)), _p(np.ascontiguousarray(V)),
                  ctypes.c_longlong(packed.nrofint), _p(packed.sortcount, _i64p),
                  _p(packed.intval), _p(packed.intnums, _u16p), _p(mos), _p(f), _p(e), _p(eh))
    return mos, f, e, float(eh[0])


def build_fmat(pmat, hmat, packed):
    """src/SCF/ops_rhf.cc:549 build_Fmat -> F."""
    N = pmat.shape[0]
    f = np.zeros((N, N))
    lib().ref_build_fmat(N, _p(np.ascontiguousarray(pmat)), _p(np.ascontiguousarray(hmat)),
                         ctypes.c_longlong(packed.nrofint), _p(packed.sortcount, _i64p),
                         _p(packed.intval), _p(packed.intnums, _u16p), _p(f))
    return f


def rhf_iterations():
    """Iterations the last rhf() call ran: the rows of run_scf's table."""
    import re

    text = lib().ref_last_output().decode()
    return len(re.findall(r"^\s*\d+:", text, flags=re.M))


# ---- src/MATH/ops_mat.cc (mangled C++ symbols of the unmodified sources) ----

def _sq(*arrs):
    return [np.ascontiguousarray(a, dtype=np.float64) for a in arrs]


def diag_mat(mat):
    """ops_mat.cc:21 -> (vals, vecs)."""
    (m,) = _sq(mat)
    n = m.shape[0]
    vals, vecs = np.zeros(n), np.zeros((n, n))
    getattr(lib(), "_Z8diag_matiPdS_S_")(n, _p(m), _p(vals), _p(vecs))
    return vals, vecs


def symmortho_mat(mat, tmat):
    """ops_mat.cc:53 -> (mat, dummat)."""
    m, t = _sq(mat, tmat)
    m = m.copy()
    dum = np.zeros_like(m)
    getattr(lib(), "_Z13symmortho_matiPdS_S_")(m.shape[0], _p(m), _p(t), _p(dum))
    return m, dum


def transform_MOs(mos, tmat):
    """ops_mat.cc:75 -> (MOs, tmpvec)."""
    c, t = _sq(mos, tmat)
    c = c.copy()
    tmp = np.zeros(c.shape[0])
    getattr(lib(), "_Z13transform_MOsiPdS_S_")(c.shape[0], _p(c), _p(t), _p(tmp))
    return c, tmp


def _mm(sym, a, b, wide):
    a, b = _sq(a, b)
    f = np.zeros_like(a)
    fn = getattr(lib(), sym)
    fn.argtypes = [ctypes.c_longlong if wide else ctypes.c_int, _dp, _dp, _dp]
    fn(a.shape[0], _p(a), _p(b), _p(f))
    return f


def mat_mat_T(a, b, wide=False):
    """ops_mat.cc:93 (int) / :122 (long long)."""
    return _mm("_Z9mat_mat_TxPdS_S_" if wide else "_Z9mat_mat_TiPdS_S_", a, b, wide)


def mat_T_mat(a, b, wide=False):
    """ops_mat.cc:107 (int) / :136 (long long)."""
    return _mm("_Z9mat_T_matxPdS_S_" if wide else "_Z9mat_T_matiPdS_S_", a, b, wide)


def pmv(mat, vi):
    """ops_mat.cc:192."""
    m, v = _sq(mat, vi)
    vo = np.zeros(m.shape[0])
    getattr(lib(), "_Z3pmvPdS_S_i")(_p(m), _p(v), _p(vo), m.shape[0])
    return vo


# ---- hand-off files (src/IO/ops_io.cc) ------------------------------------
def read_system(prefix):
    """The reference's read_system: (ints[5], lls[3], coord, charges, zeff,
    mass, [three basis names])."""
    L = lib()
    ints = np.zeros(5, dtype=np.int32)
    lls = np.zeros(3, dtype=np.int64)
    names = ctypes.create_string_buffer(99)
    L.ref_read_system(prefix.encode(), ints.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                      _p(lls, _i64p), None, None, None, None, names)
    na = int(ints[1])
    coord, charges, zeff, mass = np.empty(3 * na), np.empty(na), np.empty(na), np.empty(na)
    L.ref_read_system(prefix.encode(), ints.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                      _p(lls, _i64p), _p(coord), _p(charges), _p(zeff), _p(mass), names)
    raw = names.raw
    nm = [raw[33 * k:33 * k + 33].split(b"\0")[0].decode() for k in range(3)]
    return ints, lls, coord.reshape(na, 3), charges, zeff, mass, nm


def read_oei(prefix, nroao):
    mats = [np.empty((nroao, nroao)) for _ in range(4)]
    lib().ref_read_oei(prefix.encode(), int(nroao), *[_p(m) for m in mats])
    return tuple(mats)


def read_tei(prefix, nrofint):
    sc = np.zeros(4, dtype=np.int64)
    iv = np.empty(int(nrofint))
    inum = np.empty((int(nrofint), 4), dtype=np.uint16)
    lib().ref_read_tei(prefix.encode(), ctypes.c_longlong(int(nrofint)), _p(sc, _i64p), _p(iv),
                       _p(inum, _u16p))
    return sc, iv, inum


def read_wav_hf(prefix, nroao):
    e = np.empty(nroao)
    c = np.empty((nroao, nroao))
    lib().ref_read_wav_hf(prefix.encode(), int(nroao), _p(e), _p(c))
    return e, c


def write_wav_hf(path, moens, mos):
    lib().ref_write_wav_hf(path.encode(), int(moens.shape[0]), _p(np.ascontiguousarray(moens)),
                           _p(np.ascontiguousarray(mos)))


# ---- CCSD consumer (src/POSTHF/ccsd.cc) -------------------------------------
def ints_so(nroe, prec):
    N = prec.shape[0]
    out = np.empty((2 * N,) * 4)
    lib().ref_ints_so(int(nroe), int(N), _p(np.ascontiguousarray(prec)), _p(out))
    return out


def cc_fock(nroe, mos, hmat, prec):
    N = mos.shape[0]
    h, f = np.empty((2 * N, 2 * N)), np.empty((2 * N, 2 * N))
    lib().ref_form_fock(int(nroe), int(N), _p(np.ascontiguousarray(mos)),
                        _p(np.ascontiguousarray(hmat)), _p(np.ascontiguousarray(prec)), _p(h),
                        _p(f))
    return h, f
