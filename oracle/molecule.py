"""ORACLE -- test infrastructure, not product code.

Molecular inputs for the H2O (def2-SVP) and water-cluster (def2-SVP /
def2-SVP-RI) workloads: basis shells from oracle/basis_h2o.json, geometries,
integrals from the oracle's Gaussian-integral engine (oracle/ints.c, a stand-in
for the absent libint), and an RHF restatement (Roothaan iterations with DIIS;
the reference's own run_scf, src/SCF/scf.cc:145-320, is used where its
compiled oracle exists).  Lengths in bohr.
"""
from __future__ import annotations

import ctypes
import json
import math
import os

import numpy as np

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
BOHR_PER_ANGSTROM = 1.0 / 0.52917721067
ZNUC = {"H": 1, "O": 8}
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _basis_db():
    with open(os.path.join(HERE, "basis_h2o.json")) as f:
        return json.load(f)["basis"]


def _dfact(n):
    return 1.0 if n <= 0 else float(np.prod(np.arange(n, 0, -2)))


class Shells:
    """Flat shell arrays in the layout oracle/ints.c expects."""

    def __init__(self, atoms, basis):
        db = _basis_db()[basis]
        ls, nps, offs, cen, ex, co = [], [], [], [], [], []
        for (el, xyz) in atoms:
            for sh in db[el]:
                l = sh["l"]
                offs.append(len(ex))
                ls.append(l)
                nps.append(len(sh["exps"]))
                cen.extend(xyz)
                for a, c in zip(sh["exps"], sh["coefs"]):
                    # radial normalisation of x^l exp(-a r^2)
                    nrm = (2 * a / math.pi) ** 0.75 * (4 * a) ** (l / 2) / math.sqrt(_dfact(2 * l - 1))
                    ex.append(a)
                    co.append(c * nrm)
        self.l = np.array(ls, dtype=np.int32)
        self.nprim = np.array(nps, dtype=np.int32)
        self.poff = np.array(offs, dtype=np.int32)
        self.center = np.array(cen, dtype=np.float64)
        self.exps = np.array(ex, dtype=np.float64)
        self.coefs = np.array(co, dtype=np.float64)
        self.nsh = len(ls)
        self.nbf = int(sum(2 * l + 1 for l in ls))

    def args(self):
        return (self.nsh, self.l.ctypes.data_as(_ip), self.nprim.ctypes.data_as(_ip),
                self.poff.ctypes.data_as(_ip), self.center.ctypes.data_as(_dp),
                self.exps.ctypes.data_as(_dp), self.coefs.ctypes.data_as(_dp))


def water(o_xyz=(0.0, 0.0, 0.0), rot=None, r_oh=0.9572, angle=104.52):
    """H2O with O at o_xyz (angstrom), O-H r_oh (angstrom), H-O-H angle (deg)."""
    t = math.radians(angle) / 2
    h1 = np.array([r_oh * math.sin(t), 0.0, r_oh * math.cos(t)])
    h2 = np.array([-r_oh * math.sin(t), 0.0, r_oh * math.cos(t)])
    if rot is not None:
        h1, h2 = rot @ h1, rot @ h2
    o = np.array(o_xyz, dtype=np.float64)
    s = BOHR_PER_ANGSTROM
    return [("O", tuple(o * s)), ("H", tuple((o + h1) * s)), ("H", tuple((o + h2) * s))]


def water_cluster(n=20, box=9.0, min_oo=2.6, seed=303):
    """n waters, O positions uniform in a box (angstrom) with every O-O distance
    >= min_oo (rejection sampling), random orientations; seeded."""
    r = O.rng(seed)
    centers = []
    while len(centers) < n:
        c = r.uniform(0.0, box, 3)
        if all(np.linalg.norm(c - d) >= min_oo for d in centers):
            centers.append(c)
    atoms = []
    for c in centers:
        q, rr = np.linalg.qr(r.standard_normal((3, 3)))
        q = q * np.sign(np.diag(rr))
        if np.linalg.det(q) < 0:
            q[:, 0] = -q[:, 0]
        atoms += water(c, q)
    return atoms


def nuclear_repulsion(atoms):
    e = 0.0
    for a in range(len(atoms)):
        for b in range(a + 1, len(atoms)):
            d = np.linalg.norm(np.array(atoms[a][1]) - np.array(atoms[b][1]))
            e += ZNUC[atoms[a][0]] * ZNUC[atoms[b][0]] / d
    return e


class Integrals:
    """Normalised spherical integrals of a molecule in one orbital basis (and
    optionally an auxiliary basis)."""

    def __init__(self, atoms, basis, aux=None):
        self.atoms = atoms
        self.obs = Shells(atoms, basis)
        self.aux = Shells(atoms, aux) if aux else None
        self.N = self.obs.nbf
        L = O.lib()
        N = self.N
        S = np.zeros((N, N))
        L.ints_one(*self.obs.args(), 0, 0, None, None, S.ctypes.data_as(_dp))
        self.norm = 1.0 / np.sqrt(np.diag(S).copy())
        self.S = S * np.outer(self.norm, self.norm)
        Z = np.array([float(ZNUC[a]) for a, _ in atoms])
        xyz = np.array([c for _, c in atoms], dtype=np.float64).ravel()
        T = np.zeros((N, N))
        V = np.zeros((N, N))
        L.ints_one(*self.obs.args(), 1, 0, None, None, T.ctypes.data_as(_dp))
        L.ints_one(*self.obs.args(), 2, len(atoms), Z.ctypes.data_as(_dp), xyz.ctypes.data_as(_dp),
                   V.ctypes.data_as(_dp))
        nn = np.outer(self.norm, self.norm)
        self.T = T * nn
        self.V = V * nn
        self.enuc = nuclear_repulsion(atoms)
        if self.aux is not None:
            X = self.aux.nbf
            Sa = np.zeros((X, X))
            L.ints_one(*self.aux.args(), 0, 0, None, None, Sa.ctypes.data_as(_dp))
            self.anorm = 1.0 / np.sqrt(np.diag(Sa).copy())

    def eri(self):
        N = self.N
        out = np.zeros((N, N, N, N))
        O.lib().ints_eri4(*self.obs.args(), out.ctypes.data_as(_dp))
        n = self.norm
        out *= n[:, None, None, None] * n[None, :, None, None] * n[None, None, :, None] * n
        return out

    def metric(self):
        X = self.aux.nbf
        J = np.zeros((X, X))
        O.lib().ints_2c(*self.aux.args(), J.ctypes.data_as(_dp))
        return J * np.outer(self.anorm, self.anorm)

    def three_center(self, screen=1e-12):
        """(P|mu nu) [X][N][N]; orbital shell pairs below the Schwarz bound
        sqrt|(ab|ab)| max_P sqrt|(P|P)| < screen are left zero."""
        X, N = self.aux.nbf, self.N
        out = np.zeros((X, N, N))
        L = O.lib()
        L.ints_3c.argtypes = None
        L.ints_3c(*self.aux.args(), *self.obs.args(), None, ctypes.c_double(0.0),
                  out.ctypes.data_as(_dp))
        out *= self.anorm[:, None, None]
        out *= np.outer(self.norm, self.norm)[None, :, :]
        return out


def rhf(ints, nocc, eri=None, bq=None, maxiter=200, conv=1e-12):
    """Restricted Hartree-Fock (Roothaan iterations with DIIS on FDS - SDF),
    with exact ERIs (eri[N^4]) or density-fitted ones (bq[Q][mu][nu] =
    J^-1/2 (Q|mu nu)).  Returns (E_HF, C[mu][p] columns, eps, F)."""
    S, H = ints.S, ints.T + ints.V
    w, U = np.linalg.eigh(S)
    Xm = U @ np.diag(w ** -0.5) @ U.T
    F = H.copy()
    e, Cp = np.linalg.eigh(Xm.T @ F @ Xm)
    C = Xm @ Cp
    Eold = 0.0
    focks, errs = [], []
    for it in range(maxiter):
        Co = C[:, :nocc]
        P = 2.0 * Co @ Co.T
        if eri is not None:
            Jm = np.einsum("mnls,ls->mn", eri, P, optimize=True)
            Km = np.einsum("mlns,ls->mn", eri, P, optimize=True)
        else:
            gamma = np.einsum("Qls,ls->Q", bq, P, optimize=True)
            Jm = np.einsum("Q,Qmn->mn", gamma, bq, optimize=True)
            tmp = np.einsum("Qml,li->Qmi", bq, Co, optimize=True)
            Km = 2.0 * np.einsum("Qmi,Qni->mn", tmp, tmp, optimize=True)
        F = H + Jm - 0.5 * Km
        E = 0.5 * np.sum(P * (H + F)) + ints.enuc
        err = F @ P @ S - S @ P @ F
        focks.append(F)
        errs.append(err)
        if len(focks) > 8:
            focks.pop(0)
            errs.pop(0)
        if len(focks) > 1:
            n = len(focks)
            Bm = -np.ones((n + 1, n + 1))
            Bm[n, n] = 0.0
            for a in range(n):
                for b in range(n):
                    Bm[a, b] = np.sum(errs[a] * errs[b])
            rhs = np.zeros(n + 1)
            rhs[n] = -1.0
            c = np.linalg.solve(Bm, rhs)
            F = sum(c[k] * focks[k] for k in range(n))
        e, Cp = np.linalg.eigh(Xm.T @ F @ Xm)
        C = Xm @ Cp
        if abs(E - Eold) < conv and np.abs(err).max() < 1e-9:
            break
        Eold = E
    # final Fock of the converged density, as the reference recomputes it (scf.cc:289-290)
    Co = C[:, :nocc]
    P = 2.0 * Co @ Co.T
    if eri is not None:
        Jm = np.einsum("mnls,ls->mn", eri, P, optimize=True)
        Km = np.einsum("mlns,ls->mn", eri, P, optimize=True)
    else:
        gamma = np.einsum("Qls,ls->Q", bq, P, optimize=True)
        Jm = np.einsum("Q,Qmn->mn", gamma, bq, optimize=True)
        tmp = np.einsum("Qml,li->Qmi", bq, Co, optimize=True)
        Km = 2.0 * np.einsum("Qmi,Qni->mn", tmp, tmp, optimize=True)
    F = H + Jm - 0.5 * Km
    E = 0.5 * np.sum(P * (H + F)) + ints.enuc
    return E, C, e, F
