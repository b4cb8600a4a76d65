"""Pin the oracle (oracle/oracle.py + oracle/corr_oracle.c) to the reference.

* against the committed golden fixtures (outputs of the reference's own
  compiled code, tests/golden/make_golden.py) -- runs everywhere;
* against the live reference build (oracle/_ref) on further seeded cases --
  only where the reference checkout exists.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD_DIR = os.path.join(HERE, "golden")
with open(os.path.join(GOLD_DIR, "golden.json")) as _f:
    GOLD = json.load(_f)


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def _checksum_ok(a, ref):
    a = np.asarray(a, dtype=np.float64)
    return np.allclose([a.sum(), (a * a).sum()], ref, rtol=1e-12, atol=1e-12)


def _eps_for(N, nocc, seed):
    r = O.rng(seed)
    return np.concatenate([np.sort(r.uniform(-1.5, -0.3, nocc)),
                           np.sort(r.uniform(0.05, 3.0, N - nocc))])


@pytest.mark.parametrize("case", GOLD["rimp2"], ids=lambda c: f"o{c['nocc']}v{c['nvir']}x{c['naux']}")
def test_rimp2_energy_vs_golden(case):
    o, v, X = case["nocc"], case["nvir"], case["naux"]
    B, eps = O.synth_rimp2(o, v, X, case["seed"])
    assert _checksum_ok(B, case["B_checksum"]), "input generator drifted"
    assert _checksum_ok(eps, case["eps_checksum"]), "input generator drifted"
    got = O.rimp2_energy(B, eps, o, v)
    for g, r in zip(got, case["energy"]):
        assert abs(g - r) <= 1e-12 * max(1.0, abs(case["energy"][2])), (got, case["energy"])


def test_tiny_closed_form():
    """o=1, v=1: E = -(ia|ia)^2 / (2 e_a - 2 e_i), E_SS = 0."""
    B = np.array([[[0.3]], [[-0.2]]])
    eps = np.array([-0.5, 0.25])
    iaia = 0.3 ** 2 + 0.2 ** 2
    ess, eos, e = O.rimp2_energy(B, eps, 1, 1)
    assert ess == 0.0
    assert abs(eos - (-iaia ** 2 / 1.5)) < 1e-16


@pytest.mark.parametrize("case", GOLD["motrans"], ids=lambda c: f"N{c['N']}")
def test_packing_and_motrans_vs_golden(case):
    N, nocc = case["N"], case["nocc"]
    eri, _ = O.synth_eri(N, case["eri_seed"])
    assert _checksum_ok(eri, case["eri_checksum"])
    pk = O.pack_eri(eri)
    # packing is integer/index work: bit-exact
    assert pk.nrofint == case["nrofint"]
    assert [int(x) for x in pk.sortcount] == case["sortcount"]
    assert _digest(pk.intnums) == case["intnums_sha"]
    assert _digest(pk.intval) == case["intval_sha"]
    # dense unpack restores the full tensor
    assert np.abs(O.unpack_eri(N, pk) - eri).max() < 1e-15
    mos = O.synth_orbitals(N, case["mos_seed"])
    prec = O.motrans(mos, pk)
    ref = np.load(os.path.join(GOLD_DIR, f"motrans_n{N}.npz"))["prec"]
    assert np.abs(prec - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    eps = _eps_for(N, nocc, case["eri_seed"] + 1000)
    e = O.canonical_mp2(2 * nocc, prec, np.diag(eps))
    for g, r in zip(e, case["mp2"]):
        assert abs(g - r) <= 1e-13
    for (idx, r) in zip([(0, 1, 2, 3), (1, 1, 0, 0), (N - 1, 0, N - 2, 1)], case["mo2int_bf"]):
        assert abs(O.mo2int_bf(*idx, mos, pk) - r) <= 1e-14
        assert abs(prec[idx] - r) <= 1e-13


@pytest.mark.parametrize("case", GOLD["ri"], ids=lambda c: f"X{c['naux']}N{c['N']}")
def test_ri_build_transform_vs_golden(case):
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg", os.path.join(GOLD_DIR, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    X, N, nocc, s = case["naux"], case["N"], case["nocc"], case["seed"]
    J, P3 = mg.synth_metric(X, N, s)
    assert _checksum_ok(J, case["J_checksum"]) and _checksum_ok(P3, case["P3_checksum"])
    ref = np.load(os.path.join(GOLD_DIR, f"ri_x{X}_n{N}.npz"))
    jm, ncut = O.ri_metric_inv_sqrt(J)
    assert ncut == 0
    bpq = O.ri_build_bpq(jm, P3)
    assert np.abs(bpq - ref["bpq"]).max() <= 1e-12 * np.abs(ref["bpq"]).max()
    mos = O.synth_orbitals(N, s + 7)
    bia = O.transform_ri(2 * nocc, mos, ref["bpq"])
    assert np.abs(bia - ref["bia"]).max() <= 1e-14
    eps = _eps_for(N, nocc, s + 11)
    e = O.rimp2_energy(bia, eps, nocc, N - nocc)
    for g, r in zip(e, case["rimp2"]):
        assert abs(g - r) <= 1e-13
    F = O.rng(s + 13).standard_normal((N, N))
    F = F + F.T
    assert np.abs(O.build_fmo(mos, F) - ref["fmo"]).max() <= 1e-13


def test_kat1_low_rank_identity():
    """Canonical MP2 on (mn|ls) = sum_P L_Pmn L_Pls equals RI-MP2 with J = 1."""
    k = GOLD["kat1"]
    assert abs(k["canonical"][2] - k["ri"][2]) <= 1e-13
    N, nocc, P = k["N"], k["nocc"], k["rank"]
    eri, L = O.synth_eri(N, k["eri_seed"], rank=P)
    mos = O.synth_orbitals(N, k["mos_seed"])
    eps = np.array(k["eps"])
    can = O.canonical_mp2(2 * nocc, O.motrans(mos, O.pack_eri(eri)), np.diag(eps))
    bia = O.transform_ri(2 * nocc, mos, O.ri_build_bpq(np.eye(P), L))
    ri = O.rimp2_energy(bia, eps, nocc, N - nocc)
    for a, b, r in zip(can, ri, k["canonical"]):
        assert abs(a - r) <= 1e-13 and abs(b - r) <= 1e-13


def test_gradient_restatement_matches_finite_differences():
    o, v, X = 2, 5, 6
    B, eps = O.synth_rimp2(o, v, X, 77)
    E, dB, de = O.rimp2_gradient(B, eps, o, v)
    assert abs(E - O.rimp2_energy(B, eps, o, v)[2]) < 1e-14
    h = 1e-6
    r = O.rng(5)
    for _ in range(6):
        idx = tuple(int(r.integers(0, n)) for n in B.shape)
        Bp, Bm = B.copy(), B.copy()
        Bp[idx] += h
        Bm[idx] -= h
        fd = (O.rimp2_energy(Bp, eps, o, v)[2] - O.rimp2_energy(Bm, eps, o, v)[2]) / (2 * h)
        assert abs(fd - dB[idx]) <= 1e-7 * max(1.0, abs(fd))
    for p in range(o + v):
        ep, em = eps.copy(), eps.copy()
        ep[p] += h
        em[p] -= h
        fd = (O.rimp2_energy(B, ep, o, v)[2] - O.rimp2_energy(B, em, o, v)[2]) / (2 * h)
        assert abs(fd - de[p]) <= 1e-7 * max(1.0, abs(fd))


# ---- live reference (only where the checkout exists) -----------------------
def _ref():
    from oracle import refwrap
    if not refwrap.available():
        pytest.skip("reference checkout not present")
    return refwrap


@pytest.mark.parametrize("o,v,X,seed", [(3, 40, 33, 1), (9, 70, 130, 2), (1, 200, 10, 3)])
def test_rimp2_energy_vs_live_reference(o, v, X, seed):
    R = _ref()
    B, eps = O.synth_rimp2(o, v, X, seed)
    ref = R.rimp2_energy(B, eps, o, v)
    got = O.rimp2_energy(B, eps, o, v)
    for g, r in zip(got, ref):
        assert abs(g - r) <= 1e-12 * max(1.0, abs(ref[2]))


def test_ri_metric_with_cut_eigenvalues_vs_live_reference():
    """Rank-deficient J: the 1e-10 relative cutoff removes eigenvalues."""
    R = _ref()
    X, N = 20, 6
    r = O.rng(9)
    V = r.standard_normal((X, 14))
    J = V @ V.T  # rank 14
    P3 = r.standard_normal((X, N, N))
    P3 = P3 + P3.transpose(0, 2, 1)
    bpq_ref = R.calculate_ri(J, P3)
    jm, ncut = O.ri_metric_inv_sqrt(J)
    assert ncut == X - 14
    bpq = O.ri_build_bpq(jm, P3)
    # the cut subspace is ill-conditioned; compare the metric-weighted product
    G_ref = np.einsum("Pmn,Pls->mnls", bpq_ref, bpq_ref)
    G = np.einsum("Pmn,Pls->mnls", bpq, bpq)
    assert np.abs(G - G_ref).max() <= 1e-8 * np.abs(G_ref).max()


def test_bench_workloads_match_the_oracle_inputs():
    """The benchmark's input generators (corr_gb300.workloads) produce the
    same arrays as the oracle's, so bench lines and parity tests describe the
    same workload."""
    import numpy as np

    from corr_gb300 import workloads as W
    from oracle import oracle as O

    for args in ((3, 20, 40, 7), (40, 360, 64, 2024)):
        b1, e1 = W.synth_rimp2(*args)
        b2, e2 = O.synth_rimp2(*args)
        assert np.array_equal(b1, b2) and np.array_equal(e1, e2)
    assert W.synth_batch_sizes(256, 5005) == O.synth_batch_sizes(256, 5005)


def _ops_mat_fixture():
    import sys

    sys.path.insert(0, GOLD_DIR)
    import make_golden_ops_mat as M

    return M, np.load(os.path.join(GOLD_DIR, "ops_mat.npz"))


@pytest.mark.parametrize("n", [9, 33])
def test_ops_mat_restatements_vs_golden(n):
    """oracle.diag_mat & co. against the reference's ops_mat.cc outputs.  The
    general-matrix case pins the triangle dsyev reads (row-major lower)."""
    M, g = _ops_mat_fixture()
    x = M.ops_mat_inputs(n, 500 + n)
    tol = 1e-13 * n
    for key in ("sym", "asym"):
        w, V = O.diag_mat(x[key])
        pre = f"n{n}_diag_" + ("" if key == "sym" else "asym_")
        assert np.allclose(w, g[pre + "vals"], rtol=0, atol=tol)
        # eigenvector signs are arbitrary: compare |<v_k, v_k^ref>|
        assert np.allclose(np.abs((V * g[pre + "vecs"]).sum(1)), 1.0, atol=1e-10)
    m, d = O.symmortho_mat(x["sym"], x["t"])
    assert np.allclose(m, g[f"n{n}_symmortho_mat"], rtol=0, atol=tol)
    assert np.allclose(d, g[f"n{n}_symmortho_dummat"], rtol=0, atol=tol)
    c, t = O.transform_MOs(x["a"], x["t"])
    assert np.allclose(c, g[f"n{n}_transform_MOs"], rtol=0, atol=tol)
    assert np.allclose(t, g[f"n{n}_transform_MOs_tmpvec"], rtol=0, atol=tol)
    for suf in ("", "_ll"):
        assert np.allclose(O.mat_mat_T(x["a"], x["b"]), g[f"n{n}_mat_mat_T{suf}"], rtol=0, atol=tol)
        assert np.allclose(O.mat_T_mat(x["a"], x["b"]), g[f"n{n}_mat_T_mat{suf}"], rtol=0, atol=tol)
    assert np.allclose(O.pmv(x["a"], x["v"]), g[f"n{n}_pmv"], rtol=0, atol=tol)


def test_read_transform_ri_restatement_vs_golden(tmp_path):
    M, g = _ops_mat_fixture()
    naux, N, nocc, seed = M.RI_FILE_CASE
    bpq, mos = M.ri_file_inputs(naux, N, nocc, seed)
    bpq.tofile(tmp_path / "case.rimp2")
    got = O.read_transform_ri(str(tmp_path / "case.rimp2"), 2 * nocc, N, naux, mos)
    assert np.allclose(got, g["read_transform_ri_bia"], rtol=0, atol=1e-14)


def test_ccsd_spin_orbital_restatements_vs_reference():
    """oracle.ints_so / oracle.cc_fock against the reference's calc_ints_so and
    form_fock (src/POSTHF/ccsd.cc:509, :11) on synthetic MO integrals."""
    from oracle import refwrap

    if not refwrap.available():
        pytest.skip("reference oracle not available")
    N, nroe = 7, 6
    eri, _ = O.synth_eri(N, 81)
    mos = O.synth_orbitals(N, 82)
    prec = O.motrans(mos, O.pack_eri(eri))
    ref = refwrap.ints_so(nroe, prec)
    assert np.array_equal(O.ints_so(prec), ref)
    H = O.rng(83).standard_normal((N, N))
    H = H + H.T
    rh, rf = refwrap.cc_fock(nroe, mos, H, prec)
    h, f = O.cc_fock(nroe, mos, H, prec)
    assert np.abs(h - rh).max() <= 1e-13 * np.abs(rh).max()
    assert np.abs(f - rf).max() <= 1e-13 * np.abs(rf).max()


def _h2o_scf_inputs():
    from oracle import molecule as M

    I = M.Integrals(M.water(), "def2-svp")
    return I, O.pack_eri(I.eri())


def test_scf_restatement_vs_golden():
    """oracle.run_scf (run_scf, scf.cc:145) on H2O / def2-SVP reproduces the
    reference's printed HF energy, and its final Fock matrix the reference's
    (config1_h2o.npz, written by the reference's own run_scf)."""
    import json

    I, pk = _h2o_scf_inputs()
    with open(os.path.join(HERE, "golden", "golden_molecules.json")) as f:
        g = json.load(f)["config1"]
    r = O.run_scf(10, I.S, I.T + I.V, pk, I.enuc)
    assert abs(r["energy"] - g["E_HF_reference_scf"]) < 1e-9
    fx = np.load(os.path.join(HERE, "golden", "config1_h2o.npz"))
    assert np.abs(r["fmat"] - fx["fmat"]).max() < 1e-6
    Co = fx["mos"][:5]
    P = 2.0 * Co.T @ Co
    assert np.abs(O.build_fmat(P, I.T + I.V, pk) - fx["fmat"]).max() < 1e-12


def test_scf_restatements_vs_reference():
    """oracle.build_fmat / oracle.run_scf against the reference's build_Fmat
    (ops_rhf.cc:549) and run_scf (scf.cc:145): same Fock matrices, the same
    energy and the same number of iterations."""
    R = _ref()
    I, pk = _h2o_scf_inputs()
    H = I.T + I.V
    P = O.rng(91).standard_normal((I.N, I.N))
    P = P + P.T
    ref = R.build_fmat(P, H, pk)
    assert np.abs(O.build_fmat(P, H, pk) - ref).max() <= 1e-12 * np.abs(ref).max()
    mos, f, e, E = R.rhf(10, I.enuc, I.S, I.T, I.V, pk)
    r = O.run_scf(10, I.S, H, pk, I.enuc)
    assert r["iterations"] == R.rhf_iterations()
    assert abs(r["energy"] - E) < 1e-9  # E is printed to 10 decimals
    assert np.abs(r["fmat"] - f).max() < 1e-7
    assert np.abs(r["moens"] - e).max() < 1e-7
