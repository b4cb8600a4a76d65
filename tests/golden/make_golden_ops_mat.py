"""Golden fixtures of the reference's dense helpers (src/MATH/ops_mat.cc) and
of read_transform_ri (src/POSTHF/ri.cc:109-144), from the reference's own
compiled code (oracle/_ref/libcorr_ref.so, built by oracle/Makefile).

Inputs are regenerated from their seeds by ops_mat_inputs(); ops_mat.npz holds
the reference's outputs.  Usage (where the reference checkout exists):
    python tests/golden/make_golden_ops_mat.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

SIZES = (9, 33)
RI_FILE_CASE = (20, 9, 3, 611)  # (naux, nroao, nocc, seed)


def ops_mat_inputs(n, seed):
    """sym: symmetric; asym: general (diag_mat reads one triangle of it);
    a, b: general square; t: orthogonal-ish transform; v: vector."""
    r = O.rng(seed)
    a = r.standard_normal((n, n))
    b = r.standard_normal((n, n))
    sym = a + a.T
    asym = r.standard_normal((n, n))
    t, _ = np.linalg.qr(r.standard_normal((n, n)))
    t = t + 0.05 * r.standard_normal((n, n))
    v = r.standard_normal(n)
    return {"sym": sym, "asym": asym, "a": a, "b": b, "t": t, "v": v}


def ri_file_inputs(naux, nroao, nocc, seed):
    r = O.rng(seed)
    bpq = r.standard_normal((naux, nroao, nroao)) * 0.1
    bpq = 0.5 * (bpq + bpq.transpose(0, 2, 1))
    return bpq, O.synth_orbitals(nroao, seed + 1)


def main():
    from oracle import refwrap as R

    R.build()
    out = {}
    for n in SIZES:
        x = ops_mat_inputs(n, 500 + n)
        w, V = R.diag_mat(x["sym"])
        out[f"n{n}_diag_vals"], out[f"n{n}_diag_vecs"] = w, V
        w2, V2 = R.diag_mat(x["asym"])
        out[f"n{n}_diag_asym_vals"], out[f"n{n}_diag_asym_vecs"] = w2, V2
        m, dum = R.symmortho_mat(x["sym"], x["t"])
        out[f"n{n}_symmortho_mat"], out[f"n{n}_symmortho_dummat"] = m, dum
        c, tmp = R.transform_MOs(x["a"], x["t"])
        out[f"n{n}_transform_MOs"], out[f"n{n}_transform_MOs_tmpvec"] = c, tmp
        out[f"n{n}_mat_mat_T"] = R.mat_mat_T(x["a"], x["b"])
        out[f"n{n}_mat_T_mat"] = R.mat_T_mat(x["a"], x["b"])
        out[f"n{n}_mat_mat_T_ll"] = R.mat_mat_T(x["a"], x["b"], wide=True)
        out[f"n{n}_mat_T_mat_ll"] = R.mat_T_mat(x["a"], x["b"], wide=True)
        out[f"n{n}_pmv"] = R.pmv(x["a"], x["v"])
    naux, N, nocc, seed = RI_FILE_CASE
    bpq, mos = ri_file_inputs(naux, N, nocc, seed)
    with tempfile.TemporaryDirectory() as d:
        prefix = os.path.join(d, "case")
        bpq.tofile(prefix + ".rimp2")
        out["read_transform_ri_bia"] = R.read_transform_ri(prefix, 2 * nocc, N, naux, mos)
    np.savez_compressed(os.path.join(HERE, "ops_mat.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
