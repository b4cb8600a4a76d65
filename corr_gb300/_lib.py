"""ctypes binding of libcorr_gb300.so (the C ABI declared in include/corr_gb300.h).

The library is built in-tree (corr_gb300/build.py).  There is no fallback: if
the shared library is missing, loading raises.
"""
from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libcorr_gb300.so")
HEADER = os.path.join(ROOT, "include", "corr_gb300.h")

CORR_OK = 0
STATUS = {
    0: "CORR_OK", 1: "CORR_ERR_BAD_ARG", 2: "CORR_ERR_OOM", 3: "CORR_ERR_NOT_PD",
    4: "CORR_ERR_DEVICE_TIMEOUT", 5: "CORR_ERR_CUDA", 6: "CORR_ERR_NO_DEVICE",
    7: "CORR_ERR_NUMERIC", 8: "CORR_ERR_IO",
}
PRECISION = {"fp64": 0, "split_fp16": 1, "split_bf16": 2}


class CorrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class MP2Energy(ctypes.Structure):
    _fields_ = [("e_ss", ctypes.c_double), ("e_os", ctypes.c_double),
                ("e_total", ctypes.c_double), ("e_scs", ctypes.c_double)]

    def as_tuple(self):
        return (self.e_ss, self.e_os, self.e_total)

    def __repr__(self):
        return (f"MP2Energy(e_ss={self.e_ss!r}, e_os={self.e_os!r}, e_total={self.e_total!r}, "
                f"e_scs={self.e_scs!r})")


class Timing(ctypes.Structure):
    _fields_ = [("prepass_ms", ctypes.c_float), ("kernel_ms", ctypes.c_float),
                ("total_ms", ctypes.c_float), ("launches_total", ctypes.c_longlong)]


class SystemInfo(ctypes.Structure):
    _fields_ = [("nroe", ctypes.c_int), ("nroa", ctypes.c_int), ("nroao", ctypes.c_int),
                ("naux_1", ctypes.c_int), ("naux_2", ctypes.c_int),
                ("nrofint", ctypes.c_longlong), ("nrofaux", ctypes.c_longlong),
                ("nrofaux2", ctypes.c_longlong), ("basis_ob", ctypes.c_char * 33),
                ("basis_jk", ctypes.c_char * 33), ("basis_ri", ctypes.c_char * 33)]


class BasisC(ctypes.Structure):
    _fields_ = [("nsh", ctypes.c_int), ("l", ctypes.c_void_p), ("nprim", ctypes.c_void_p),
                ("poff", ctypes.c_void_p), ("center", ctypes.c_void_p),
                ("exps", ctypes.c_void_p), ("coefs", ctypes.c_void_p)]


class RIMP2Instance(ctypes.Structure):
    _fields_ = [("nocc", ctypes.c_int), ("nvir", ctypes.c_int), ("naux", ctypes.c_int),
                ("bia", ctypes.c_void_p), ("eps", ctypes.c_void_p)]


_vp = ctypes.c_void_p
_i = ctypes.c_int
_ll = ctypes.c_longlong
_d = ctypes.c_double

# name -> argtypes (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "corr_version": [],
    "corr_create": [ctypes.POINTER(_vp), _i, _vp],
    "corr_destroy": [_vp],
    "corr_set_stream": [_vp, _vp],
    "corr_last_error": [],
    "corr_device_sm_count": [_vp],
    "corr_set_timing": [_vp, _i],
    "corr_get_timing": [_vp, ctypes.POINTER(Timing)],
    "corr_rimp2_energy": [_vp, _i, _i, _i, _vp, _vp, _i, ctypes.POINTER(MP2Energy)],
    "corr_rimp2_energy_async": [_vp, _i, _i, _i, _vp, _vp, _i, _vp],
    "corr_rimp2_energy_estimate": [_vp, _i, _i, _i, _vp, _vp, _i, ctypes.POINTER(MP2Energy),
                                   ctypes.POINTER(_d)],
    "corr_sync": [_vp],
    "corr_rimp2_gradient": [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, ctypes.POINTER(MP2Energy)],
    "corr_rimp2_gradient_tc": [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, ctypes.POINTER(MP2Energy)],
    "corr_rimp2_energy_noalloc": [_i, _vp, _i, _i, _i, _vp, _vp, _i, ctypes.POINTER(MP2Energy)],
    "corr_rimp2_energy_batched": [_vp, _i, ctypes.POINTER(RIMP2Instance), _i,
                                  ctypes.POINTER(MP2Energy)],
    "corr_rimp2_energy_batched_async": [_vp, _i, ctypes.POINTER(RIMP2Instance), _i, _vp],
    "corr_set_batch_policy": [_vp, _i, _i, _i],
    "corr_set_energy_tiles": [_vp, _i],
    "corr_set_fp64_strict": [_vp, _i],
    "corr_selftest_wait_timeout": [_vp, _i],
    "corr_rimp2_batch_autotune": [_vp, _i, ctypes.POINTER(RIMP2Instance), _i, ctypes.POINTER(_i),
                                  ctypes.POINTER(_i), ctypes.POINTER(_i),
                                  ctypes.POINTER(ctypes.c_float)],
    "corr_build_fmo": [_vp, _i, _vp, _vp, _vp],
    "corr_motrans": [_vp, _i, _i, _vp, _ll, _vp, _vp, _vp, _vp],
    "corr_motrans_ovov": [_vp, _i, _i, _vp, _ll, _vp, _vp, _vp, _vp],
    "corr_canonical_mp2": [_vp, _i, _i, _vp, _vp, ctypes.POINTER(MP2Energy)],
    "corr_canonical_mp2_ovov": [_vp, _i, _i, _vp, _vp, ctypes.POINTER(MP2Energy)],
    "corr_transform_ri": [_vp, _i, _i, _i, _vp, _vp, _vp],
    "corr_ri_build_bpq": [_vp, _i, _i, _vp, _vp, _vp],
    "corr_ri_metric_inv_sqrt": [_vp, _i, _vp, _d, _vp, ctypes.POINTER(_i)],
    "corr_calculate_ri": [_vp, _i, _i, _vp, _vp, _vp],
    "corr_ri_apply_metric": [_vp, _i, _ll, _vp, _vp, _vp],
    "corr_rimp2_energy_from_3index": [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, _i,
                                      ctypes.POINTER(MP2Energy), ctypes.POINTER(_i)],
    "corr_dgemm": [_vp, _i, _i, _i, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i],
    "corr_syev": [_vp, _i, _vp, _vp, _vp],
    "corr_ri_integrals": [_vp, ctypes.POINTER(BasisC), ctypes.POINTER(BasisC), _vp, _vp],
    "corr_ints_so": [_vp, _i, _vp, _vp],
    "corr_cc_fock": [_vp, _i, _i, _vp, _vp, _vp, _vp, _vp],
    "corr_dgemm_tc": [_vp, _i, _i, _i, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i],
    "corr_build_fmat": [_vp, _i, _vp, _vp, _ll, _vp, _vp, _vp, _vp],
    "corr_run_scf": [_vp, _i, _i, _d, _vp, _vp, _ll, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp,
                     _vp],
    "corr_read_system": [ctypes.c_char_p, ctypes.POINTER(SystemInfo), _vp, _vp, _vp, _vp],
    "corr_read_oei": [_vp, ctypes.c_char_p, _i, _vp, _vp, _vp, _vp],
    "corr_read_tei": [_vp, ctypes.c_char_p, _ll, _vp, _vp, _vp],
    "corr_read_wav_hf": [_vp, ctypes.c_char_p, _i, _vp, _vp],
    "corr_write_wav_hf": [ctypes.c_char_p, _i, _vp, _vp],
    "corr_read_rimp2": [_vp, ctypes.c_char_p, _i, _i, _vp],
}
_RESTYPES = {"corr_version": ctypes.c_char_p, "corr_last_error": ctypes.c_char_p}

_LIB = None


def header_symbols():
    """Every function the public header declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(corr_\w+)\(", text, re.M)))


def load():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with corr_gb300.build.build() "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _LIB = L
    return _LIB


def check(status):
    if status != CORR_OK:
        msg = load().corr_last_error()
        raise CorrError(status, msg.decode() if msg else "")
    return status
