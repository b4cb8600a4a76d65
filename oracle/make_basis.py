"""Extract the H and O shells of def2-SVP, def2-SVP-RI and STO-3G (Gaussian-94 files of
the EMSL Basis Set Exchange, shipped as basissets/*.g94 with the reference)
into oracle/basis_h2o.json, the fixture the integral engine reads.

Usage (where the reference checkout exists):  python oracle/make_basis.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: CORR_REFERENCE_DIR, else a sibling of the repository
REF = os.environ.get("CORR_REFERENCE_DIR",
                     os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
L = {"S": 0, "P": 1, "D": 2, "F": 3, "G": 4}


def parse_g94(path, elements):
    out = {}
    lines = open(path).read().splitlines()
    k = 0
    while k < len(lines):
        tok = lines[k].split()
        if len(tok) == 2 and tok[0] in elements and tok[1] == "0":
            el = tok[0]
            shells = []
            k += 1
            while k < len(lines) and not lines[k].startswith("****"):
                t = lines[k].split()
                if t and t[0] in L:
                    n = int(t[1])
                    exps, coefs = [], []
                    for r in range(n):
                        e, c = lines[k + 1 + r].split()[:2]
                        exps.append(float(e.replace("D", "E")))
                        coefs.append(float(c.replace("D", "E")))
                    shells.append({"l": L[t[0]], "exps": exps, "coefs": coefs})
                    k += n
                k += 1
            out[el] = shells
        k += 1
    return out


def main():
    bs = {}
    for name, f in (("def2-svp", "def2-svp.g94"), ("def2-svp-ri", "def2-svp-ri.g94"),
                    ("sto-3g", "sto-3g.g94")):
        bs[name] = parse_g94(os.path.join(REF, "basissets", f), {"H", "O"})
    with open(os.path.join(HERE, "basis_h2o.json"), "w") as fh:
        json.dump({"source": "EMSL Basis Set Exchange def2-SVP / def2-SVP-RI (Weigend, Ahlrichs "
                             "2005; Weigend, Haeser, Patzelt, Ahlrichs 1998)", "basis": bs},
                  fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    sys.exit(main())
