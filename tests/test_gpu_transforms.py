"""FP64 transforms and canonical MP2 on the GPU against the reference's own
outputs (golden fixtures) and the oracle."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD_DIR = os.path.join(HERE, "golden")
with open(os.path.join(GOLD_DIR, "golden.json")) as _f:
    GOLD = json.load(_f)


def _eps_for(N, nocc, seed):
    r = O.rng(seed)
    return np.concatenate([np.sort(r.uniform(-1.5, -0.3, nocc)),
                           np.sort(r.uniform(0.05, 3.0, N - nocc))])


def _metric(X, N, s):
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg", os.path.join(GOLD_DIR, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.synth_metric(X, N, s)


@pytest.mark.parametrize("case", GOLD["motrans"], ids=lambda c: f"N{c['N']}")
def test_motrans_and_canonical_vs_reference(ctx, case):
    N, nocc = case["N"], case["nocc"]
    eri, _ = O.synth_eri(N, case["eri_seed"])
    pk = O.pack_eri(eri)
    mos = O.synth_orbitals(N, case["mos_seed"])
    prec = ctx.motrans(2 * nocc, mos, pk)
    ref = np.load(os.path.join(GOLD_DIR, f"motrans_n{N}.npz"))["prec"]
    assert np.abs(prec - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    eps = _eps_for(N, nocc, case["eri_seed"] + 1000)
    e = ctx.canonical_mp2(2 * nocc, prec, eps)
    for g, r in zip(e.as_tuple(), case["mp2"]):
        assert abs(g - r) <= 1e-12, (e, case["mp2"])
    ov = ctx.motrans_ovov(2 * nocc, mos, pk)
    o, v = nocc, N - nocc
    assert np.abs(ov - ref[:o, o:, :o, o:]).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    e2 = ctx.canonical_mp2_ovov(ov, eps)
    for g, r in zip(e2.as_tuple(), case["mp2"]):
        assert abs(g - r) <= 1e-12


@pytest.mark.parametrize("N,nocc", [(24, 5), (19, 4), (32, 7)])
def test_motrans_config1_sizes_vs_oracle(ctx, N, nocc):
    eri, _ = O.synth_eri(N, 500 + N)
    pk = O.pack_eri(eri)
    mos = O.synth_orbitals(N, 600 + N)
    ref = O.motrans(mos, pk)
    got = ctx.motrans(2 * nocc, mos, pk)
    assert np.abs(got - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    eps = _eps_for(N, nocc, 700 + N)
    r = O.canonical_mp2(2 * nocc, ref, np.diag(eps))
    g = ctx.canonical_mp2(2 * nocc, got, eps)
    assert abs(g.e_total - r[2]) <= 1e-12


@pytest.mark.parametrize("case", GOLD["ri"], ids=lambda c: f"X{c['naux']}N{c['N']}")
def test_ri_build_and_transform_vs_reference(ctx, case):
    X, N, nocc, s = case["naux"], case["N"], case["nocc"], case["seed"]
    J, P3 = _metric(X, N, s)
    ref = np.load(os.path.join(GOLD_DIR, f"ri_x{X}_n{N}.npz"))
    jm, _ = O.ri_metric_inv_sqrt(J)
    bpq = ctx.ri_build_bpq(jm, P3)
    assert np.abs(bpq - ref["bpq"]).max() <= 1e-12 * np.abs(ref["bpq"]).max()
    mos = O.synth_orbitals(N, s + 7)
    bia = ctx.transform_ri(2 * nocc, mos, ref["bpq"])
    assert np.abs(bia - ref["bia"]).max() <= 1e-13 * max(1.0, np.abs(ref["bia"]).max())
    F = O.rng(s + 13).standard_normal((N, N))
    F = F + F.T
    assert np.abs(ctx.build_fmo(mos, F) - ref["fmo"]).max() <= 1e-13 * np.abs(ref["fmo"]).max()
    eps = _eps_for(N, nocc, s + 11)
    e = ctx.rimp2_energy(bia, eps, nocc, N - nocc, X, "fp64")
    for g, r in zip(e.as_tuple(), case["rimp2"]):
        assert abs(g - r) <= 1e-12


@pytest.mark.parametrize("X,N,nocc", [(200, 60, 10), (77, 33, 6), (130, 48, 11)])
def test_transform_ri_larger_vs_oracle(ctx, X, N, nocc):
    r = O.rng(X + N)
    bpq = r.standard_normal((X, N, N))
    mos = O.synth_orbitals(N, X)
    ref = O.transform_ri_np(nocc, mos, bpq)
    got = ctx.transform_ri(2 * nocc, mos, bpq)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_kat1_gpu_canonical_equals_ri(ctx):
    k = GOLD["kat1"]
    N, nocc, P = k["N"], k["nocc"], k["rank"]
    eri, L = O.synth_eri(N, k["eri_seed"], rank=P)
    mos = O.synth_orbitals(N, k["mos_seed"])
    eps = np.array(k["eps"])
    ov = ctx.motrans_ovov(2 * nocc, mos, O.pack_eri(eri))
    can = ctx.canonical_mp2_ovov(ov, eps)
    bia = ctx.transform_ri(2 * nocc, mos, ctx.ri_build_bpq(np.eye(P), L))
    ri = ctx.rimp2_energy(bia, eps, nocc, N - nocc, P, "fp64")
    assert abs(can.e_total - k["canonical"][2]) <= 1e-12
    assert abs(ri.e_total - k["ri"][2]) <= 1e-12


def test_device_resident_transform_chain(ctx):
    import torch

    X, N, nocc = 64, 40, 8
    r = O.rng(3)
    bpq = torch.from_numpy(r.standard_normal((X, N, N))).cuda()
    mos = torch.from_numpy(O.synth_orbitals(N, 4)).cuda()
    bia = ctx.transform_ri(2 * nocc, mos, bpq)
    assert bia.is_cuda
    ref = O.transform_ri_np(nocc, mos.cpu().numpy(), bpq.cpu().numpy())
    assert np.abs(bia.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
