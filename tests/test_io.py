"""The hand-off file readers and writer (src/IO/ops_io.cc:63-124, 203-212,
259-299) on their host path, which needs no GPU: byte-exact against the arrays
written in the reference's layouts, against the reference's own readers
(compiled in oracle/_ref where the reference checkout exists), and their error
behaviour."""
import os

import numpy as np
import pytest

import corr_gb300
from corr_gb300 import _lib
from oracle import oracle as O
from oracle import refwrap

import files as F  # tests/files.py (the test directory is on sys.path)


def _ref_available():
    return os.path.exists(refwrap.SO)


def test_read_system(tmp_path):
    r = O.rng(11)
    coord, charges, zeff, mass = F.random_system(r, 7)
    prefix = str(tmp_path / "mol")
    F.write_sys(prefix, 10, 24, 130, 76, 12345, 678, 9012, coord, charges, zeff, mass,
                ["DEF2-SVP", "DEF2-UNIVERSAL-JKFIT", "DEF2-SVP-RI"])
    info, c, q, z, m = corr_gb300.read_system(prefix)
    assert (info.nroe, info.nroa, info.nroao, info.naux_1, info.naux_2) == (10, 7, 24, 130, 76)
    assert (info.nrofint, info.nrofaux, info.nrofaux2) == (12345, 678, 9012)
    assert np.array_equal(c, coord) and np.array_equal(q, charges)
    assert np.array_equal(z, zeff) and np.array_equal(m, mass)
    assert (info.basis_ob, info.basis_jk, info.basis_ri) == (b"DEF2-SVP", b"DEF2-UNIVERSAL-JKFIT",
                                                              b"DEF2-SVP-RI")
    if _ref_available():
        ints, lls, rc, rq, rz, rm, names = refwrap.read_system(prefix)
        assert list(ints) == [10, 7, 24, 130, 76] and list(lls) == [12345, 678, 9012]
        assert np.array_equal(rc, c) and np.array_equal(rm, m)
        assert names == ["DEF2-SVP", "DEF2-UNIVERSAL-JKFIT", "DEF2-SVP-RI"]


def test_read_oei_and_tei_host(tmp_path):
    r = O.rng(12)
    n, nint = 13, 5000
    mats = [r.standard_normal((n, n)) for _ in range(4)]
    sc = np.array([100, 900, 2500, 4000], dtype=np.int64)
    iv = r.standard_normal(nint)
    inum = r.integers(0, 65536, (nint, 4)).astype(np.uint16)
    prefix = str(tmp_path / "mol")
    F.write_oei(prefix, *mats)
    F.write_tei(prefix, sc, iv, inum)
    got_m, (gsc, giv, gin) = corr_gb300.read_files_host(prefix, n, nint)
    for a, b in zip(got_m, mats):
        assert np.array_equal(a, b)
    assert np.array_equal(gsc, sc) and np.array_equal(giv, iv) and np.array_equal(gin, inum)
    if _ref_available():
        for a, b in zip(refwrap.read_oei(prefix, n), got_m):
            assert np.array_equal(a, b)
        rsc, riv, rin = refwrap.read_tei(prefix, nint)
        assert np.array_equal(rsc, gsc) and np.array_equal(riv, giv) and np.array_equal(rin, gin)


def test_wavefunction_round_trip_with_the_reference(tmp_path):
    r = O.rng(13)
    n = 17
    e, c = np.sort(r.standard_normal(n)), r.standard_normal((n, n))
    ours = str(tmp_path / "ours")
    corr_gb300.write_wav_hf(ours + ".ahfw", e, c)
    raw = open(ours + ".ahfw", "rb").read()
    assert raw == np.int32(n).tobytes() + e.tobytes() + c.tobytes()
    if _ref_available():
        re_, rc = refwrap.read_wav_hf(ours, n)
        assert np.array_equal(re_, e) and np.array_equal(rc, c)
        theirs = str(tmp_path / "theirs")
        refwrap.write_wav_hf(theirs + ".ahfw", e, c)
        assert open(theirs + ".ahfw", "rb").read() == raw


def test_reader_errors(tmp_path):
    L = _lib.load()
    prefix = str(tmp_path / "none")
    with pytest.raises(_lib.CorrError) as ex:
        corr_gb300.read_system(prefix)
    assert ex.value.status == 8  # CORR_ERR_IO: missing file
    # a .tei shorter than its count
    F.write_tei(prefix, np.zeros(4, dtype=np.int64), np.zeros(10), np.zeros((10, 4), np.uint16))
    with pytest.raises(_lib.CorrError) as ex:
        corr_gb300.read_files_host(prefix, 2, 11)
    assert ex.value.status == 8
    # a wavefunction of another size: CORR_ERR_BAD_ARG (the reference exits)
    corr_gb300.write_wav_hf(prefix + ".ahfw", np.zeros(3), np.zeros((3, 3)))
    e, c = np.empty(4), np.empty((4, 4))
    st = L.corr_read_wav_hf(None, prefix.encode(), 4, e.ctypes.data, c.ctypes.data)
    assert st == 1 and b"3 orbitals" in L.corr_last_error()
