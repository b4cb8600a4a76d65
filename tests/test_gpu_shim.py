"""The drop-in C++ layer on the GPU: the post-HF sequence of the reference's
main (build_FMo, MOtrans, run_canonical_mp2, calculate_ri, transform_ri,
run_canonical_mp2_ri; src/main.cc:130-166) through the shim, against the
oracle's restatement of the same sequence."""
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _energies(text, block):
    i = text.index(block)
    vals = {}
    for key in ("EMP2_SS:", "EMP2_OS:", "EMP2:"):
        m = re.search(re.escape(key) + r"\s*(\S+)", text[i:])
        vals[key] = float(m.group(1))
    return vals["EMP2_SS:"], vals["EMP2_OS:"], vals["EMP2:"]


@pytest.mark.parametrize("N,nocc,X,precision", [(12, 3, 30, "fp64"), (16, 4, 44, "split_bf16")])
def test_shim_pipeline(tmp_path, N, nocc, X, precision):
    from corr_gb300 import build

    build.build_shim()
    exe = tmp_path / "shim_driver"
    subprocess.run(["g++", "-O1", "-std=c++14", "-o", str(exe),
                    os.path.join(ROOT, "tests", "shim_driver.cc"),
                    "-L" + os.path.join(ROOT, "corr_gb300"), "-lcorr_shim", "-lcorr_gb300",
                    "-Wl,-rpath," + os.path.join(ROOT, "corr_gb300")], check=True)
    eri, _ = O.synth_eri(N, 11 + N)
    pk = O.pack_eri(eri)
    mos = O.synth_orbitals(N, 12 + N)
    r = O.rng(13 + N)
    # Fock matrix whose MO diagonal is ordered (occupied below virtual):
    # F = C^T diag(e) C + small symmetric noise, with mos = C (orthonormal rows)
    e = np.concatenate([np.sort(r.uniform(-1.5, -0.3, nocc)),
                        np.sort(r.uniform(0.05, 3.0, N - nocc))])
    noise = r.standard_normal((N, N)) * 1e-3
    F = mos.T @ np.diag(e) @ mos + noise + noise.T
    L = r.standard_normal((X, X)) / np.sqrt(X)
    J = L @ L.T + 0.5 * np.eye(X)
    P3 = r.standard_normal((X, N, N)) * 0.1
    P3 = 0.5 * (P3 + P3.transpose(0, 2, 1))
    d = tmp_path
    mos.tofile(d / "mos.bin")
    F.tofile(d / "fmat.bin")
    pk.intval.tofile(d / "intval.bin")
    pk.intnums.tofile(d / "intnums.bin")
    pk.sortcount.tofile(d / "sortcount.bin")
    J.tofile(d / "J.bin")
    P3.tofile(d / "Pmn.bin")
    env = dict(os.environ, CORR_RIMP2_PRECISION=precision)
    out = subprocess.run([str(exe), str(d), str(2 * nocc), str(N), str(X), str(pk.nrofint)],
                         capture_output=True, text=True, env=env, check=True).stdout

    fmo = O.build_fmo(mos, F)
    can = O.canonical_mp2(2 * nocc, O.motrans(mos, pk), fmo)
    jm, _ = O.ri_metric_inv_sqrt(J)
    bia = O.transform_ri(2 * nocc, mos, O.ri_build_bpq(jm, P3))
    ri = O.rimp2_energy(bia, np.diag(fmo), nocc, N - nocc)
    got_can = _energies(out, "MP2-Results")
    got_ri = _energies(out, "RI-MP2-Results")
    for g, e in zip(got_can, can):
        assert abs(g - e) <= 1e-12 + 1e-12 * abs(e)
    tol = 1e-12 if precision == "fp64" else 2e-7
    for g, e in zip(got_ri, ri):
        assert abs(g - e) <= 1e-12 + tol * abs(ri[2])
