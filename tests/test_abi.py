"""C-ABI checks that need no GPU: the library loads, exports every symbol the
public header declares, and reports a missing device as an error status."""
import ctypes

import pytest

from corr_gb300 import _lib


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_header_symbols_exported(lib):
    names = _lib.header_symbols()
    assert "corr_rimp2_energy" in names
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    assert set(_lib.header_symbols()) == set(_lib.SIGNATURES)


def test_version(lib):
    assert b"sm_103a" in lib.corr_version()


def test_no_device_or_bad_args(lib):
    h = ctypes.c_void_p()
    st = lib.corr_create(ctypes.byref(h), 0, None)
    try:
        import torch

        have_gpu = torch.cuda.is_available()
    except Exception:
        have_gpu = False
    if not have_gpu:
        assert st == 6  # CORR_ERR_NO_DEVICE
        assert b"device" in lib.corr_last_error()
    else:
        assert st == 0
        lib.corr_destroy(h)
    assert lib.corr_create(None, 0, None) == 1  # CORR_ERR_BAD_ARG
    out = _lib.MP2Energy()
    assert lib.corr_rimp2_energy(None, 1, 1, 1, None, None, 0, ctypes.byref(out)) == 1


def test_selftest_rejects_bad_limit_without_gpu():
    """Argument checking of the diagnostic happens before any device work."""
    import ctypes

    from corr_gb300 import _lib

    L = _lib.load()
    assert L.corr_selftest_wait_timeout(None, 10) == 1  # CORR_ERR_BAD_ARG


def test_dense_helpers_reject_bad_args_without_gpu():
    """corr_dgemm / corr_syev check their arguments before any device work."""
    import ctypes

    import numpy as np

    from corr_gb300 import _lib

    L = _lib.load()
    a = np.zeros((2, 2))
    p = ctypes.c_void_p(a.ctypes.data)
    assert L.corr_dgemm(None, 0, 0, 2, 2, 2, 1.0, p, 2, p, 2, 0.0, p, 2) == 1
    assert L.corr_syev(None, 2, p, p, p) == 1


def test_energy_estimate_rejects_bad_args_without_gpu():
    import ctypes

    from corr_gb300 import _lib

    L = _lib.load()
    out = _lib.MP2Energy()
    err = ctypes.c_double()
    assert L.corr_rimp2_energy_estimate(None, 1, 1, 1, None, None, 1, ctypes.byref(out),
                                        ctypes.byref(err)) == 1
