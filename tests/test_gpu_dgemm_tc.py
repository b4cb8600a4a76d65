"""corr_dgemm_tc: the FP64-accurate GEMM on the tensor cores (exact digit
slicing), against an extended-precision product (numpy longdouble, 64-bit
mantissa on x86-64 and 113-bit on aarch64) and against the FP64 GEMM.

Bound per element: 8 * 2^-53 * sqrt(k) * max|row of op(A)| * max|column of
op(B)| (digit truncation at 2^-56 per product, plus one rounding to FP64).
On data without a wide range inside a row the maximum error must not exceed
the FP64 GEMM's by more than a factor of 2.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _exact(A, B, ta=False, tb=False):
    a = (A.T if ta else A).astype(np.longdouble)
    b = (B.T if tb else B).astype(np.longdouble)
    return a @ b


def _bound(A, B, ta=False, tb=False):
    a = A.T if ta else A
    b = B.T if tb else B
    k = a.shape[1]
    return 8.0 * 2.0 ** -53 * np.sqrt(k) * np.outer(np.abs(a).max(axis=1), np.abs(b).max(axis=0))


@pytest.mark.parametrize("m,n,k,seed", [
    (1, 1, 1, 1),
    (128, 64, 32, 2),
    (100, 480, 480, 3),      # the (P|i nu) shape of the 20-water cluster
    (300, 380, 480, 4),      # the (P|ia) shape (rows of several P)
    (129, 65, 33, 5),        # one past every tile and K-block edge
    (257, 200, 1100, 6),     # three K passes of <= 512
    (64, 700, 513, 7),
])
def test_random_matches_extended_precision(ctx, m, n, k, seed):
    r = O.rng(seed)
    A = r.standard_normal((m, k))
    B = r.standard_normal((k, n))
    C = ctx.dgemm(A, B, tensor_cores=True)
    ex = _exact(A, B)
    err = np.abs(C - ex).astype(np.float64)
    assert (err <= _bound(A, B)).all(), err.max()
    f64 = np.abs(A @ B - ex).astype(np.float64).max()
    assert err.max() <= 2.0 * f64 + 1e-300, (err.max(), f64)


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_transposes_alpha_beta(ctx, ta, tb):
    r = O.rng(11 + 2 * ta + tb)
    m, n, k = 150, 90, 260
    A = r.standard_normal((k, m) if ta else (m, k))
    B = r.standard_normal((n, k) if tb else (k, n))
    C0 = r.standard_normal((m, n))
    for alpha, beta in [(1.0, 0.0), (-0.5, 1.0), (2.0, 0.25)]:
        C = ctx.dgemm(A, B, transa=bool(ta), transb=bool(tb), alpha=alpha, beta=beta,
                      out=C0.copy(), tensor_cores=True)
        ex = alpha * _exact(A, B, ta, tb) + beta * C0.astype(np.longdouble)
        bound = abs(alpha) * _bound(A, B, ta, tb) + 2.0 ** -52 * np.abs(ex).astype(np.float64)
        assert (np.abs(C - ex).astype(np.float64) <= bound).all(), (alpha, beta)


def test_wide_range_rows_and_zero_rows(ctx):
    """Rows spanning 40 decades, zero rows and columns, tiny values: the error
    stays inside the row/column-scale bound."""
    r = O.rng(21)
    m, n, k = 140, 70, 300
    A = r.standard_normal((m, k)) * 10.0 ** r.uniform(-20, 20, size=(m, k))
    B = r.standard_normal((k, n)) * 10.0 ** r.uniform(-3, 3, size=(1, n))
    A[5] = 0.0
    B[:, 7] = 0.0
    A[9, 3] = 1e-300
    C = ctx.dgemm(A, B, tensor_cores=True)
    ex = _exact(A, B)
    assert (np.abs(C - ex).astype(np.float64) <= _bound(A, B)).all()
    assert (C[5] == 0.0).all() and (C[:, 7] == 0.0).all()


def test_device_arrays(ctx):
    import torch

    r = O.rng(31)
    A = r.standard_normal((200, 333))
    B = r.standard_normal((333, 77))
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    C = ctx.dgemm(dA, dB, tensor_cores=True)
    assert C.is_cuda
    err = np.abs(C.cpu().numpy() - _exact(A, B)).astype(np.float64)
    assert (err <= _bound(A, B)).all()


def _dot2(A, Bt):
    """sum_k A[m][k] Bt[n][k] in twice FP64's precision (Dekker products,
    Knuth sums, the Dot2 scheme of Ogita, Rump and Oishi): (hi, lo)."""
    def split(x):
        c = 134217729.0 * x
        h = c - (c - x)
        return h, x - h

    s = np.zeros((A.shape[0], Bt.shape[0]))
    c = np.zeros_like(s)
    for k in range(A.shape[1]):
        a, b = A[:, k, None], Bt[None, :, k]
        p = a * b
        ah, al = split(a)
        bh, bl = split(b)
        e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
        t = s + p
        bp = t - s
        c += ((s - (t - bp)) + (p - bp)) + e
        s = t
    return s, c


def test_config3_transform_error_not_above_fp64(ctx):
    """(P|i nu) = sum_mu C_i mu (P|mu nu) on the 20-water cluster's data (its
    RHF occupied orbitals and the (P|mu nu) of the auxiliary functions of one
    water, K = 480): the digit GEMM's largest error is at most the FP64
    GEMM's."""
    import json
    import os

    from oracle import molecule as M

    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "golden_molecules.json")) as f:
        g = json.load(f)["config3"]
    atoms = M.water_cluster(20, box=g["box"], min_oo=g["min_oo"], seed=g["seed"])
    I = M.Integrals(atoms, "def2-svp")
    I.aux = M.Shells(atoms[:3], "def2-svp-ri")
    S = np.zeros((I.aux.nbf, I.aux.nbf))
    O.lib().ints_one(*I.aux.args(), 0, 0, None, None, S.ctypes.data_as(M._dp))
    I.anorm = 1.0 / np.sqrt(np.diag(S))
    P3 = I.three_center()[:8]                 # [P][mu][nu], 8 aux functions
    X, N, _ = P3.shape
    mos = np.load(os.path.join(here, "golden", "config3_cluster.npz"))["mos"]
    Cocc = np.ascontiguousarray(mos[:100])    # [i][mu]
    Bt = np.ascontiguousarray(P3.reshape(X * N, N))  # rows (P, nu) over mu
    got = ctx.dgemm(Bt, Cocc, transb=True, tensor_cores=True)  # [(P, nu)][i]
    hi, lo = _dot2(Bt, Cocc)
    e_tc = np.abs((got - hi) - lo).max()
    e_64 = np.abs(((Bt @ Cocc.T) - hi) - lo).max()
    print(f"config-3 transform: max error digit GEMM {e_tc:.3e}, FP64 GEMM {e_64:.3e}")
    assert e_tc <= e_64, (e_tc, e_64)
