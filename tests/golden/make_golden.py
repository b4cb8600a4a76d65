"""Generate the golden fixtures from the reference's own compiled code.

Runs the reference functions (oracle/_ref/libcorr_ref.so, built from the
reference sources by oracle/Makefile) on seeded synthetic inputs and writes
  golden.json   energies (17 significant digits), packing statistics and
                input checksums
  *.npz         small output arrays (MO tensor, BPQ, Bia, FMo)
next to this script.  Inputs are regenerated from their seeds by
oracle.oracle's generators; the stored checksums make a generator drift show
up as a clear failure instead of a silent parity miss.

Usage (where the reference checkout exists):  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

RIMP2_CASES = [  # (nocc, nvir, naux, seed)
    (1, 1, 1, 101), (1, 3, 2, 102), (2, 2, 5, 103), (3, 5, 7, 12), (5, 19, 60, 13),
    (2, 64, 17, 14), (6, 129, 70, 15), (7, 33, 95, 16), (4, 257, 40, 17), (8, 150, 200, 18),
    (12, 96, 300, 19),
]
MOTRANS_CASES = [  # (N, nocc, eri_seed, mos_seed)
    (6, 2, 201, 202), (10, 3, 203, 204), (13, 4, 205, 206),
]
RI_CASES = [  # (naux, N, nocc, seed)
    (24, 8, 3, 301), (40, 11, 4, 302),
]


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest()[:16]


def checksum(a):
    a = np.asarray(a, dtype=np.float64)
    return [float(a.sum()), float((a * a).sum())]


def eps_for(N, nocc, seed):
    r = O.rng(seed)
    return np.concatenate([np.sort(r.uniform(-1.5, -0.3, nocc)),
                           np.sort(r.uniform(0.05, 3.0, N - nocc))])


def synth_metric(naux, N, seed):
    """(P|Q) positive definite and (P|mn) symmetric in m,n."""
    r = O.rng(seed)
    L = r.standard_normal((naux, naux)) / np.sqrt(naux)
    J = L @ L.T + 0.5 * np.eye(naux)
    P3 = r.standard_normal((naux, N, N)) * 0.1
    P3 = 0.5 * (P3 + P3.transpose(0, 2, 1))
    return J, P3


def motrans_case(N, nocc, es, ms):
    """One reference MOtrans per process (function-static buffers)."""
    from oracle import refwrap as R

    eri, _ = O.synth_eri(N, es)
    mos = O.synth_orbitals(N, ms)
    pk = R.pack_eri(eri)
    prec = R.motrans(2 * nocc, mos, pk)
    eps = eps_for(N, nocc, es + 1000)
    fmo = np.diag(eps)
    e = R.canonical_mp2(2 * nocc, prec, fmo)
    bf = [R.mo2int_bf(i, j, k, l, mos, pk) for (i, j, k, l) in [(0, 1, 2, 3), (1, 1, 0, 0),
                                                               (N - 1, 0, N - 2, 1)]]
    return {
        "N": N, "nocc": nocc, "eri_seed": es, "mos_seed": ms,
        "eri_checksum": checksum(eri), "nrofint": pk.nrofint,
        "sortcount": [int(x) for x in pk.sortcount],
        "intnums_sha": digest(pk.intnums), "intval_sha": digest(pk.intval),
        "mp2": [float(x) for x in e], "mo2int_bf": bf,
    }, prec


def main():
    from oracle import refwrap as R

    R.build()
    out = {"generator": "numpy PCG64 via oracle.oracle", "rimp2": [], "motrans": [], "ri": []}
    for (o, v, X, s) in RIMP2_CASES:
        B, eps = O.synth_rimp2(o, v, X, s)
        e = R.rimp2_energy(B, eps, o, v)
        out["rimp2"].append({"nocc": o, "nvir": v, "naux": X, "seed": s,
                             "B_checksum": checksum(B), "eps_checksum": checksum(eps),
                             "energy": [float(x) for x in e]})
        print("rimp2", o, v, X, e)

    for (N, nocc, es, ms) in MOTRANS_CASES:
        code = (f"import sys; sys.path.insert(0, {ROOT!r}); sys.path.insert(0, {HERE!r});"
                f"import make_golden as M, json, numpy as np;"
                f"d, p = M.motrans_case({N}, {nocc}, {es}, {ms});"
                f"np.save({os.path.join(HERE, f'_tmp_motrans_{N}.npy')!r}, p);"
                f"print(json.dumps(d))")
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                           check=True)
        d = json.loads(r.stdout.strip().splitlines()[-1])
        tmp = os.path.join(HERE, f"_tmp_motrans_{N}.npy")
        prec = np.load(tmp)
        os.remove(tmp)
        np.savez_compressed(os.path.join(HERE, f"motrans_n{N}.npz"), prec=prec)
        out["motrans"].append(d)
        print("motrans", N, d["mp2"])

    for (X, N, nocc, s) in RI_CASES:
        J, P3 = synth_metric(X, N, s)
        mos = O.synth_orbitals(N, s + 7)
        bpq = R.calculate_ri(J, P3)
        bia = R.transform_ri(2 * nocc, mos, bpq)
        eps = eps_for(N, nocc, s + 11)
        e = R.rimp2_energy(bia, eps, nocc, N - nocc)
        F = O.rng(s + 13).standard_normal((N, N))
        F = F + F.T
        fmo = R.build_fmo(mos, F)
        np.savez_compressed(os.path.join(HERE, f"ri_x{X}_n{N}.npz"), bpq=bpq, bia=bia, fmo=fmo)
        out["ri"].append({"naux": X, "N": N, "nocc": nocc, "seed": s,
                          "J_checksum": checksum(J), "P3_checksum": checksum(P3),
                          "rimp2": [float(x) for x in e]})
        print("ri", X, N, e)

    # KAT-1: (mn|ls) = sum_P L_Pmn L_Pls  =>  canonical MP2 == RI-MP2 with J = 1, (P|mn) = L
    N, nocc, P = 12, 3, 30
    eri, L = O.synth_eri(N, 401, rank=P)
    mos = O.synth_orbitals(N, 402)
    eps = eps_for(N, nocc, 403)
    code = (f"import sys; sys.path.insert(0, {ROOT!r});"
            f"import numpy as np; from oracle import oracle as O, refwrap as R;"
            f"eri, L = O.synth_eri({N}, 401, rank={P}); mos = O.synth_orbitals({N}, 402);"
            f"pk = R.pack_eri(eri); p = R.motrans({2 * nocc}, mos, pk);"
            f"import json; eps=np.array({eps.tolist()!r});"
            f"print(json.dumps([float(x) for x in R.canonical_mp2({2 * nocc}, p, np.diag(eps))]))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True)
    can = json.loads(r.stdout.strip().splitlines()[-1])
    bpq = R.calculate_ri(np.eye(P), L)
    bia = R.transform_ri(2 * nocc, mos, bpq)
    ri = R.rimp2_energy(bia, eps, nocc, N - nocc)
    out["kat1"] = {"N": N, "nocc": nocc, "rank": P, "eri_seed": 401, "mos_seed": 402,
                   "eps": eps.tolist(), "canonical": can, "ri": [float(x) for x in ri]}
    print("kat1", can, ri)

    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
