"""Writes tests/golden/systems.npz: the molecules of configurations 1 (H2O) and
3 (20-water cluster, seed 303) as the inputs of corr_ri_integrals -- nuclear
charges and positions (bohr) and the def2-SVP / def2-SVP-RI shells with the
contraction coefficients of the reference's basis-set files
(basissets/def2-svp.g94, def2-svp-ri.g94, parsed by oracle/make_basis.py into
oracle/basis_h2o.json).  The geometries come from oracle/molecule.py, the same
code that made config1_h2o.npz and config3_cluster.npz, so the MO coefficients
stored there belong to these bases.

    python tests/golden/make_golden_systems.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import molecule as M  # noqa: E402

ZNUC = {"H": 1.0, "O": 8.0}


def shells(atoms, basis):
    db = json.load(open(os.path.join(ROOT, "oracle", "basis_h2o.json")))["basis"][basis]
    l, nprim, poff, center, exps, coefs = [], [], [], [], [], []
    for el, xyz in atoms:
        for sh in db[el]:
            l.append(sh["l"])
            nprim.append(len(sh["exps"]))
            poff.append(len(exps))
            center.extend(xyz)
            exps.extend(sh["exps"])
            coefs.extend(sh["coefs"])
    return (np.array(l, np.int32), np.array(nprim, np.int32), np.array(poff, np.int32),
            np.array(center, np.float64), np.array(exps, np.float64), np.array(coefs, np.float64))


def main():
    out = {}
    for tag, atoms in (("c1", M.water()), ("c3", M.water_cluster(20, box=9.0, min_oo=2.6,
                                                                     seed=303))):
        out[f"{tag}_Z"] = np.array([ZNUC[a] for a, _ in atoms])
        out[f"{tag}_xyz"] = np.array([c for _, c in atoms], dtype=np.float64)
        for bname, key in (("def2-svp", "obs"), ("def2-svp-ri", "aux")):
            for name, arr in zip(("l", "nprim", "poff", "center", "exps", "coefs"),
                                 shells(atoms, bname)):
                out[f"{tag}_{key}_{name}"] = arr
    np.savez_compressed(os.path.join(HERE, "systems.npz"), **out)


if __name__ == "__main__":
    main()
