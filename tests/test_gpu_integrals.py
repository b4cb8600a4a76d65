"""The RI integrals on the GPU (corr_ri_integrals: the libint part of
calculate_ri, src/POSTHF/ri.cc:25-47, 70-100) for the H2O and 20-water
molecules of configurations 1 and 3: against the oracle's integral engine
elementwise (H2O), the checksums the golden fixtures recorded (sum and sum of
squares of J and (P|mu nu), both molecules), and the reference's RI-MP2
energies computed from the oracle's integrals (golden_molecules.json) -- the
MO coefficients of config1_h2o.npz / config3_cluster.npz belong to exactly
these basis functions, so the energies also pin the function order, signs
and normalisation of the orbital basis."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden_molecules.json")))
SYS = np.load(os.path.join(HERE, "golden", "systems.npz"))


def _basis(tag, key):
    import corr_gb300

    return corr_gb300.Basis(*(SYS[f"{tag}_{key}_{n}"]
                              for n in ("l", "nprim", "poff", "center", "exps", "coefs")))


def _check_sums(name, a, ref):
    a = np.asarray(a, dtype=np.float64)
    got = [float(a.sum()), float((a * a).sum())]
    for g, r in zip(got, ref):
        assert abs(g - r) <= 1e-10 * abs(r), (name, got, ref)


def test_config1_integrals_and_energy(ctx):
    from oracle import molecule as M

    obs, aux = _basis("c1", "obs"), _basis("c1", "aux")
    J, P = ctx.ri_integrals(obs, aux, device="cuda")
    Jh, Ph = J.cpu().numpy(), P.cpu().numpy()
    g = GOLD["config1"]
    _check_sums("J", Jh, g["checksums"]["J"])
    _check_sums("P3", Ph, g["checksums"]["P3"])
    I = M.Integrals(M.water(), "def2-svp", "def2-svp-ri")
    Jo, Po = I.metric(), I.three_center()
    assert np.abs(Jh - Jo).max() <= 1e-12 * np.abs(Jo).max()
    assert np.abs(Ph - Po).max() <= 1e-12 * np.abs(Po).max()
    fx = np.load(os.path.join(HERE, "golden", "config1_h2o.npz"))
    mos, F = fx["mos"], fx["fmat"]
    eps = np.diag(mos @ F @ mos.T).copy()
    e, ncut = ctx.rimp2_energy_from_3index(10, mos, eps, J, P, "fp64")
    assert ncut == 0
    assert abs(e.e_total - g["ri_mp2"][2]) <= 1e-10, (e, g["ri_mp2"])


def test_config3_cluster_from_gpu_integrals(ctx):
    """The 20-water cluster end to end on the GPU: (P|Q) and (P|mu nu)
    (2.8 GB, kept on the device), then the RI-MP2 energy in FP64 (the
    reference's -4.110973802301 Eh) and in the precision forms (within 1 uEh
    of FP64)."""
    import time

    import torch

    obs, aux = _basis("c3", "obs"), _basis("c3", "aux")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J, P = ctx.ri_integrals(obs, aux, device="cuda")
    t_int = time.perf_counter() - t0
    g = GOLD["config3"]
    _check_sums("J", J.cpu().numpy(), g["checksums"]["J"])
    s1 = float(P.sum())
    s2 = float((P * P).sum())
    for got, r in zip((s1, s2), g["checksums"]["P3"]):
        assert abs(got - r) <= 1e-10 * abs(r), (got, g["checksums"]["P3"])
    fx = np.load(os.path.join(HERE, "golden", "config3_cluster.npz"))
    mos, eps = fx["mos"], fx["eps"]
    e64, ncut = ctx.rimp2_energy_from_3index(200, mos, eps, J, P, "fp64")
    assert abs(e64.e_total - g["ri_mp2"][2]) <= 1e-9, (e64, g["ri_mp2"])
    for prec in ("split_fp16", "split_bf16"):
        e, _ = ctx.rimp2_energy_from_3index(200, mos, eps, J, P, prec)
        assert abs(e.e_total - e64.e_total) <= 1e-6, (prec, e, e64)
    print(f"config3 integrals on the GPU: {t_int * 1e3:.0f} ms (X={aux.nbf}, N={obs.nbf})")
