"""The drop-in C++ layer (corr_gb300/shim) on CPU: it exports the reference's
own mangled C++ symbols and compiles against the reference's util.h."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM_LIB = os.path.join(ROOT, "corr_gb300", "libcorr_shim.so")
REFERENCE_SYMBOLS = [
    "_Z9build_FMoP10systeminfoP6OEintsP3pHF",            # motrans.h:22
    "_Z7MOtransP10systeminfoP6OEintsP6TEintsP3pHF",       # motrans.h:5
    "_Z17run_canonical_mp2P10systeminfoP3pHF",            # can_mp2.h:4
    "_Z12transform_riP10systeminfoP6OEintsP3pHF",         # ri.h:9
    "_Z20run_canonical_mp2_riP10systeminfoP3pHF",         # can_mp2.h:5
]


def _defined(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_shim_exports_reference_symbols():
    from corr_gb300 import build

    build.build_shim()
    syms = _defined(SHIM_LIB)
    for s in REFERENCE_SYMBOLS:
        assert s in syms, s


def test_symbols_equal_the_reference_builds():
    from oracle import refwrap

    if not os.path.exists(refwrap.SO):
        pytest.skip("reference oracle not built here")
    ref = _defined(refwrap.SO)
    for s in REFERENCE_SYMBOLS:
        assert s in ref, s


def test_shim_compiles_against_reference_headers(tmp_path):
    from oracle import refwrap

    src = os.path.join(refwrap.REF, "src")
    if not os.path.isdir(src):
        pytest.skip("reference checkout not present")
    cmd = ["g++", "-std=c++14", "-fsyntax-only", "-DCORR_SHIM_USE_REFERENCE_HEADERS",
           "-include", "cstring", "-include", "memory",
           "-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + src,
           os.path.join(ROOT, "corr_gb300", "shim", "corr_shim.cc")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_driver_compiles(tmp_path):
    from corr_gb300 import build

    build.build_shim()
    exe = tmp_path / "shim_driver"
    cmd = ["g++", "-O1", "-std=c++14", "-o", str(exe), os.path.join(ROOT, "tests", "shim_driver.cc"),
           "-L" + os.path.join(ROOT, "corr_gb300"), "-lcorr_shim", "-lcorr_gb300",
           "-Wl,-rpath," + os.path.join(ROOT, "corr_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
