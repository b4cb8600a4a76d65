"""The oracle's molecular inputs (test infrastructure standing in for libint
and psi4): known answers of the integral engine, consistency of the 2-, 3-
and 4-index integrals, the RHF restatement against the reference's run_scf,
and drift checks against the committed fixtures."""
import json
import os

import numpy as np
import pytest

from oracle import molecule as M
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "golden_molecules.json")) as _f:
    GOLD = json.load(_f)


def test_h2_sto3g_szabo_ostlund():
    """H2, STO-3G, R = 1.4 bohr: Szabo & Ostlund, Modern Quantum Chemistry,
    section 3.5.2 (S12 0.6593, T11 0.7600, T12 0.2365, (11|11) 0.7746,
    (11|22) 0.5697, (21|21) 0.2970, (21|11) 0.4441, E0 -1.1167)."""
    I = M.Integrals([("H", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 1.4))], "sto-3g")
    eri = I.eri()
    assert abs(I.S[0, 1] - 0.6593) < 1e-4
    assert abs(I.T[0, 0] - 0.7600) < 1e-4 and abs(I.T[0, 1] - 0.2365) < 1e-4
    assert abs(eri[0, 0, 0, 0] - 0.7746) < 1e-4 and abs(eri[0, 0, 1, 1] - 0.5697) < 1e-4
    assert abs(eri[1, 0, 1, 0] - 0.2970) < 1e-4 and abs(eri[1, 0, 0, 0] - 0.4441) < 1e-4
    E, _, _, _ = M.rhf(I, 1, eri=eri)
    assert abs(E - (-1.1167)) < 1e-4


def test_config1_integrals_against_fixture():
    g = GOLD["config1"]
    I = M.Integrals(M.water(), "def2-svp", "def2-svp-ri")
    eri = I.eri()
    ref = g["checksums"]
    for name, arr in (("S", I.S), ("T", I.T), ("V", I.V), ("eri", eri), ("J", I.metric()),
                      ("P3", I.three_center())):
        a = np.asarray(arr)
        assert np.allclose([a.sum(), (a * a).sum()], ref[name], rtol=1e-12, atol=1e-12), name
    # 8-fold symmetry, positive metric
    assert np.abs(eri - eri.transpose(1, 0, 2, 3)).max() < 1e-14
    assert np.abs(eri - eri.transpose(2, 3, 0, 1)).max() < 1e-14
    assert np.linalg.eigvalsh(I.metric()).min() > 0


def test_ri_fit_consistent_with_four_index():
    """RI-MP2 with the 2-/3-index integrals is within the usual def2-SVP-RI
    fitting error (~1e-4 Eh) of canonical MP2 with the 4-index ones."""
    g = GOLD["config1"]
    assert abs(g["ri_mp2"][2] - g["canonical_mp2"][2]) < 2e-4
    assert abs(g["ri_mp2"][2] - g["canonical_mp2"][2]) > 1e-6  # it is a fit, not exact


def test_rhf_restatement_matches_reference_scf():
    g = GOLD["config1"]
    I = M.Integrals(M.water(), "def2-svp")
    E, C, e, F = M.rhf(I, 5, eri=I.eri())
    assert abs(E - g["E_HF_reference_scf"]) < 1e-8  # reference converges |dE| < 1e-8


def test_cluster_geometry():
    atoms = M.water_cluster(20, seed=303)
    O_xyz = np.array([c for (el, c) in atoms if el == "O"]) / M.BOHR_PER_ANGSTROM
    assert len(O_xyz) == 20
    d = np.linalg.norm(O_xyz[:, None] - O_xyz[None], axis=-1) + np.eye(20) * 99
    assert d.min() >= 2.6
    assert O_xyz.min() >= 0 and O_xyz.max() <= 9.0
