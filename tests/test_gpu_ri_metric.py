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


@pytest.mark.parametrize("X,decades", [(257, 6), (700, 7)])
def test_inv_sqrt_ill_conditioned(ctx, X, decades):
    """Orders from 64 on take the FP32 sweeps, the FP64 re-orthogonalisation
    and the FP64 refinement sweeps; the result must still be the FP64
    J^-1/2 (spectrum 1 .. 1e-decades, a degenerate block at the top)."""
    r = O.rng(X + decades)
    Q, _ = np.linalg.qr(r.standard_normal((X, X)))
    lam = np.geomspace(1.0, 10.0 ** -decades, X)
    lam[: X // 10] = lam[X // 10]
    J = (Q * lam) @ Q.T
    J = 0.5 * (J + J.T)
    ref, ncut_ref = O.ri_metric_inv_sqrt(J)
    got, ncut = ctx.ri_metric_inv_sqrt(J)
    assert ncut == ncut_ref == 0
    # LAPACK's own error here is ~ kappa^(1/2) eps relative to max|J^-1/2|
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()
    G = got @ J @ got
    assert np.abs(G - np.eye(X)).max() <= 1e-9


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


def _from_3index_case(X, N, nocc, seed, spectrum=None):
    r = O.rng(seed)
    if spectrum is None:
        L = r.standard_normal((X, X)) / np.sqrt(X)
        J = L @ L.T + 0.5 * np.eye(X)
    else:
        Q, _ = np.linalg.qr(r.standard_normal((X, X)))
        J = (Q * spectrum) @ Q.T
        J = 0.5 * (J + J.T)
    P3 = r.standard_normal((X, N, N)) * 0.1
    P3 = 0.5 * (P3 + P3.transpose(0, 2, 1))
    mos = O.synth_orbitals(N, seed + 1)
    eps = np.concatenate([np.sort(r.uniform(-1.5, -0.3, nocc)),
                          np.sort(r.uniform(0.05, 3.0, N - nocc))])
    return J, P3, mos, eps


def _oracle_from_3index(J, P3, mos, eps, nocc):
    N = mos.shape[0]
    jm, ncut = O.ri_metric_inv_sqrt(J)
    pia = np.einsum("im,Qmn,an->Qia", mos[:nocc], P3, mos[nocc:], optimize=True)
    B = (jm @ pia.reshape(J.shape[0], -1)).reshape(J.shape[0], nocc, N - nocc)
    return O.rimp2_energy(B, eps, nocc, N - nocc), ncut


@pytest.mark.parametrize("prec", ["fp64", "split_fp16"])
@pytest.mark.parametrize("kind", ["certified", "rank_deficient", "near_cutoff"])
def test_from_3index_metric_paths(ctx, kind, prec):
    """Energy from (P|mn) and J: a certified metric takes the Cholesky path
    (chol.cu; for the precision forms W = L^-1 by blocked inversion and the
    tensor-core product), a metric with eigenvalues at or below 10 tol
    lambda_max takes the eigendecomposition with the reference's cutoff.  All
    must give the reference energy (the precision form within its digit
    rounding, 2e-7 relative)."""
    X, N, nocc = 96, 22, 5
    spec = None
    if kind == "rank_deficient":
        spec = np.concatenate([np.geomspace(1.0, 1e-3, 80), np.zeros(16)])
    elif kind == "near_cutoff":
        # smallest eigenvalue 5e-10 lambda_max: kept by the reference's cutoff,
        # below the certificate's 10 tol ||J||_inf
        spec = np.concatenate([np.geomspace(1.0, 1e-4, 95), [5e-10]])
    J, P3, mos, eps = _from_3index_case(X, N, nocc, 71, spec)
    (ess, eos, et), ncut_ref = _oracle_from_3index(J, P3, mos, eps, nocc)
    e, ncut = ctx.rimp2_energy_from_3index(2 * nocc, mos, eps, J, P3, prec)
    assert ncut == ncut_ref
    if kind == "rank_deficient":
        assert ncut == 16
    tol = {"certified": 1e-10, "rank_deficient": 1e-8, "near_cutoff": 1e-6}[kind]
    if prec != "fp64":
        tol = max(tol, 2e-7)
    assert abs(e.e_total - et) <= tol * abs(et), (e, et)
    assert abs(e.e_os - eos) <= tol * abs(eos)


@pytest.mark.parametrize("prec", ["fp64", "split_fp16"])
@pytest.mark.parametrize("X,N,nocc", [(64, 16, 3), (200, 30, 7), (650, 40, 9)])
def test_from_3index_cholesky_sizes(ctx, X, N, nocc, prec):
    """Certified metrics of sizes around the 64-row block edges (for the
    precision forms: the recursive inversion's splits)."""
    J, P3, mos, eps = _from_3index_case(X, N, nocc, X + N)
    (ess, eos, et), ncut_ref = _oracle_from_3index(J, P3, mos, eps, nocc)
    e, ncut = ctx.rimp2_energy_from_3index(2 * nocc, mos, eps, J, P3, prec)
    assert ncut == ncut_ref == 0
    assert abs(e.e_total - et) <= (1e-10 if prec == "fp64" else 2e-7) * abs(et)


def test_fp64_strict_switch(ctx):
    """corr_set_fp64_strict: the eigendecomposition and FP64-pipe products
    give the same J^-1/2 and BPQ as the default (Newton-Schulz, digit GEMM)
    to FP64 accuracy."""
    r = O.rng(77)
    X, N = 300, 12
    L = r.standard_normal((X, X)) / np.sqrt(X)
    J = L @ L.T + 0.3 * np.eye(X)
    P3 = r.standard_normal((X, N, N))
    P3 = P3 + P3.transpose(0, 2, 1)
    jm_fast, _ = ctx.ri_metric_inv_sqrt(J)
    b_fast = ctx.calculate_ri(J, P3)
    ctx.set_fp64_strict(True)
    try:
        jm_strict, _ = ctx.ri_metric_inv_sqrt(J)
        b_strict = ctx.calculate_ri(J, P3)
    finally:
        ctx.set_fp64_strict(False)
    assert np.abs(jm_fast - jm_strict).max() <= 1e-12 * np.abs(jm_strict).max()
    assert np.abs(b_fast - b_strict).max() <= 1e-12 * np.abs(b_strict).max()
