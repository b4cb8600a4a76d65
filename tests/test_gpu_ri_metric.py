"""RI metric J^-1/2 (src/POSTHF/ri.cc:50-69) and calculate_ri (ri.cc:7) on the
GPU against the reference's own BPQ (golden fixtures) and the oracle."""
import json
import os

import numpy as np
import pytest

import corr_gb300
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD_DIR = os.path.join(HERE, "golden")
with open(os.path.join(GOLD_DIR, "golden.json")) as _f:
    GOLD = json.load(_f)


def _metric(X, N, s):
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg", os.path.join(GOLD_DIR, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.synth_metric(X, N, s)


@pytest.mark.parametrize("case", GOLD["ri"], ids=lambda c: f"X{c['naux']}N{c['N']}")
def test_calculate_ri_vs_reference(ctx, case):
    X, N, s = case["naux"], case["N"], case["seed"]
    J, P3 = _metric(X, N, s)
    ref = np.load(os.path.join(GOLD_DIR, f"ri_x{X}_n{N}.npz"))["bpq"]
    bpq = ctx.calculate_ri(J, P3)
    assert np.abs(bpq - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("X", [1, 2, 7, 64, 129, 300])
def test_inv_sqrt_vs_oracle(ctx, X):
    r = O.rng(X)
    L = r.standard_normal((X, X)) / np.sqrt(X)
    J = L @ L.T + 0.3 * np.eye(X)
    ref, ncut_ref = O.ri_metric_inv_sqrt(J)
    got, ncut = ctx.ri_metric_inv_sqrt(J)
    assert ncut == ncut_ref == 0
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    # J^-1/2 J J^-1/2 = 1
    assert np.abs(got @ J @ got - np.eye(X)).max() <= 1e-11


def test_inv_sqrt_with_cut_eigenvalues(ctx):
    """Rank-deficient metric: the 1e-10 relative cutoff removes X - rank
    eigenvalues; compare the metric-weighted product, which is unique."""
    X, rank, N = 40, 29, 7
    r = O.rng(11)
    V = r.standard_normal((X, rank))
    J = V @ V.T
    P3 = r.standard_normal((X, N, N))
    P3 = P3 + P3.transpose(0, 2, 1)
    jm, ncut = ctx.ri_metric_inv_sqrt(J)
    jr, ncut_r = O.ri_metric_inv_sqrt(J)
    assert ncut == ncut_r == X - rank
    # projector onto the kept space is unique
    Pg = jm @ J @ jm
    Pr = jr @ J @ jr
    assert np.abs(Pg - Pr).max() <= 1e-8
    bpq = ctx.calculate_ri(J, P3)
    G = np.einsum("Pmn,Pls->mnls", bpq, bpq)
    Gr = np.einsum("Pmn,Pls->mnls", O.ri_build_bpq(jr, P3), O.ri_build_bpq(jr, P3))
    assert np.abs(G - Gr).max() <= 1e-7 * np.abs(Gr).max()


def test_not_positive_definite_is_an_error(ctx):
    with pytest.raises(corr_gb300.CorrError) as ei:
        ctx.ri_metric_inv_sqrt(-np.eye(5))
    assert ei.value.status == 3  # CORR_ERR_NOT_PD
