"""Golden fixtures for the molecular workloads, from the reference's own code.

config 1: H2O (O at the origin, O-H 0.9572 A, H-O-H 104.52 deg), def2-SVP /
  def2-SVP-RI.  Integrals from oracle/ints.c; the reference's packing
  (calculate_libint_tei + resort_integrals), RHF (calc_S12, core guess,
  run_scf with DIIS), build_FMo, MOtrans, run_canonical_mp2, calculate_ri,
  transform_ri and run_canonical_mp2_ri (oracle/_ref).  Writes
  config1_h2o.npz (MOs, Fock matrix) and golden_molecules.json.
config 3: 20 H2O in a 9 A cube (min O-O 2.6 A, seed 303), def2-SVP /
  def2-SVP-RI (N = 480, naux = 1520).  The reference's SCF needs the N^4 ERI
  list, so the orbitals come from the oracle's density-fitted RHF; then the
  reference's calculate_ri, transform_ri and run_canonical_mp2_ri.  Writes
  config3_cluster.npz (MOs, orbital energies).

Usage (where the reference checkout exists):
  python tests/golden/make_golden_molecules.py [config1] [config3]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import molecule as M  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "golden_molecules.json")


def checksum(a):
    a = np.asarray(a, dtype=np.float64)
    return [float(a.sum()), float((a * a).sum())]


def _load():
    if os.path.exists(OUT):
        with open(OUT) as f:
            return json.load(f)
    return {}


def _save(d):
    with open(OUT, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
        f.write("\n")


def config1():
    from oracle import refwrap as R

    atoms = M.water()
    I = M.Integrals(atoms, "def2-svp", "def2-svp-ri")
    eri = I.eri()
    J, P3 = I.metric(), I.three_center()
    pk = R.pack_eri(eri)
    mos, F, moens, ehf = R.rhf(10, I.enuc, I.S, I.T, I.V, pk)
    fmo = R.build_fmo(mos, F)
    # MOtrans keeps function-static buffers: run it in its own process
    np.savez(os.path.join(HERE, "_tmp_c1.npz"), mos=mos, eri=eri)
    code = (f"import sys; sys.path.insert(0, {ROOT!r}); import numpy as np, json;"
            f"from oracle import refwrap as R;"
            f"d = np.load({os.path.join(HERE, '_tmp_c1.npz')!r}); pk = R.pack_eri(d['eri']);"
            f"p = R.motrans(10, d['mos'], pk); fmo = np.array({fmo.tolist()!r});"
            f"print(json.dumps([float(x) for x in R.canonical_mp2(10, p, fmo)]))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True)
    os.remove(os.path.join(HERE, "_tmp_c1.npz"))
    can = json.loads(r.stdout.strip().splitlines()[-1])
    bpq = R.calculate_ri(J, P3)
    bia = R.transform_ri(10, mos, bpq)
    ri = R.rimp2_energy(bia, np.diag(fmo), 5, 19)
    np.savez_compressed(os.path.join(HERE, "config1_h2o.npz"), mos=mos, fmat=F)
    d = _load()
    d["config1"] = {
        "atoms": atoms, "N": I.N, "naux": I.aux.nbf, "nocc": 5, "enuc": I.enuc,
        "E_HF_reference_scf": ehf, "nrofint": pk.nrofint, "sortcount": [int(x) for x in pk.sortcount],
        "checksums": {"S": checksum(I.S), "T": checksum(I.T), "V": checksum(I.V),
                      "eri": checksum(eri), "J": checksum(J), "P3": checksum(P3)},
        "canonical_mp2": can, "ri_mp2": [float(x) for x in ri],
    }
    _save(d)
    print("config1", ehf, can, ri)


def config3():
    from oracle import refwrap as R

    t0 = time.time()
    atoms = M.water_cluster(20, box=9.0, min_oo=2.6, seed=303)
    I = M.Integrals(atoms, "def2-svp", "def2-svp-ri")
    J, P3 = I.metric(), I.three_center()
    print("integrals", time.time() - t0, flush=True)
    jm, ncut = O.ri_metric_inv_sqrt(J)
    bq = O.ri_build_bpq(jm, P3)
    ehf, C, e, F = M.rhf(I, 100, bq=bq, conv=1e-10)
    del bq
    print("df-rhf", ehf, time.time() - t0, flush=True)
    mos = np.ascontiguousarray(C.T)
    fmo = R.build_fmo(mos, F)
    eps = np.diag(fmo).copy()
    bpq = R.calculate_ri(J, P3)
    print("calculate_ri", time.time() - t0, flush=True)
    bia = R.transform_ri(200, mos, bpq)
    del bpq
    print("transform_ri", time.time() - t0, flush=True)
    R.set_threads(os.cpu_count() or 1)
    ri = R.rimp2_energy(bia, eps, 100, 380)
    print("rimp2", ri, time.time() - t0, flush=True)
    np.savez_compressed(os.path.join(HERE, "config3_cluster.npz"), mos=mos, eps=eps)
    d = _load()
    d["config3"] = {
        "seed": 303, "box": 9.0, "min_oo": 2.6, "N": I.N, "naux": I.aux.nbf, "nocc": 100,
        "enuc": I.enuc, "E_HF_df": ehf, "ncut": ncut,
        "checksums": {"S": checksum(I.S), "J": checksum(J), "P3": checksum(P3)},
        "ri_mp2": [float(x) for x in ri],
    }
    _save(d)


if __name__ == "__main__":
    which = sys.argv[1:] or ["config1", "config3"]
    if "config1" in which:
        config1()
    if "config3" in which:
        config3()
