"""The allocation-free RI-MP2 entry point, through the C ABI.

Callers that cannot allocate device memory (their device memory is all owned
by their own pool allocator, or they run in a loop where an allocation is not
allowed) call corr_rimp2_energy_noalloc, which keeps its scratch in a fixed
device array inside the library.  Its results must equal those of the
regular entry point, corr_rimp2_energy, on the same inputs -- also on a second
call in a row, when the array still holds the previous call's contents.
This file is collected last so that a failure here does not hide the others.
"""
import ctypes

import numpy as np
import pytest

from corr_gb300 import _lib
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_ABS, FP64_REL = 1e-10, 1e-12  # the FP64-form tolerance of the other tests
PREC = {"fp64": 0, "split_fp16": 1, "split_bf16": 2}


def _regular(L, B, eps, o, v, X, prec):
    h = ctypes.c_void_p()
    assert L.corr_create(ctypes.byref(h), 0, None) == 0, L.corr_last_error()
    try:
        out = _lib.MP2Energy()
        st = L.corr_rimp2_energy(h, o, v, X, ctypes.c_void_p(B.data_ptr()),
                                 ctypes.c_void_p(eps.data_ptr()), prec, ctypes.byref(out))
        assert st == 0, L.corr_last_error()
        return out.as_tuple()
    finally:
        L.corr_destroy(h)


@pytest.mark.parametrize("prec", ["fp64", "split_fp16", "split_bf16"])
def test_noalloc_matches_regular_entry_point_twice(prec):
    import torch

    L = _lib.load()
    o, v, X = 7, 150, 190
    B, eps = O.synth_rimp2(o, v, X, 4242)
    Bd = torch.from_numpy(B).cuda()
    ed = torch.from_numpy(eps).cuda()
    ref = _regular(L, Bd, ed, o, v, X, PREC[prec])
    for _ in range(2):
        out = _lib.MP2Energy()
        st = L.corr_rimp2_energy_noalloc(0, None, o, v, X, ctypes.c_void_p(Bd.data_ptr()),
                                         ctypes.c_void_p(ed.data_ptr()), PREC[prec],
                                         ctypes.byref(out))
        assert st == 0, L.corr_last_error()
        for g, r in zip(out.as_tuple(), ref):
            assert abs(g - r) <= max(FP64_ABS, FP64_REL * abs(r)), (out, ref)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    L = _lib.load()
    o, v, X = 40, 360, 1200  # ~105 MB of slices > 32 MiB
    Bd = torch.zeros(8, dtype=torch.float64, device="cuda")  # never read: rejected first
    ed = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = _lib.MP2Energy()
    st = L.corr_rimp2_energy_noalloc(0, None, o, v, X, ctypes.c_void_p(Bd.data_ptr()),
                                     ctypes.c_void_p(ed.data_ptr()), 2, ctypes.byref(out))
    assert st == 1  # CORR_ERR_BAD_ARG
    assert b"scratch" in L.corr_last_error()


def test_noalloc_fp64_form_at_sizes_beyond_the_precision_limit():
    """The FP64 form keeps one partial per CTA, so its scratch stays a few KB
    at any size: nocc=150, nvir=1500 has 3.4 million 64-wide tile units (54 MB
    of per-unit partials, beyond the 32 MiB array) and must still run and
    equal the regular entry point."""
    import torch

    L = _lib.load()
    o, v, X = 150, 1500, 6
    B, eps = O.synth_rimp2(o, v, X, 4343)
    Bd = torch.from_numpy(B).cuda()
    ed = torch.from_numpy(eps).cuda()
    ref = _regular(L, Bd, ed, o, v, X, PREC["fp64"])
    out = _lib.MP2Energy()
    st = L.corr_rimp2_energy_noalloc(0, None, o, v, X, ctypes.c_void_p(Bd.data_ptr()),
                                     ctypes.c_void_p(ed.data_ptr()), PREC["fp64"],
                                     ctypes.byref(out))
    assert st == 0, L.corr_last_error()
    for g, r in zip(out.as_tuple(), ref):
        assert abs(g - r) <= max(FP64_ABS, FP64_REL * abs(r)), (out, ref)


def test_noalloc_rejects_occupied_counts_beyond_the_pair_index_range():
    """nocc above 46000 overflows the 32-bit occupied-pair count: rejected
    before any device work, as by corr_rimp2_energy."""
    import torch

    L = _lib.load()
    Bd = torch.zeros(8, dtype=torch.float64, device="cuda")  # never read: rejected first
    ed = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = _lib.MP2Energy()
    st = L.corr_rimp2_energy_noalloc(0, None, 46341, 2, 1, ctypes.c_void_p(Bd.data_ptr()),
                                     ctypes.c_void_p(ed.data_ptr()), 0, ctypes.byref(out))
    assert st == 1  # CORR_ERR_BAD_ARG
