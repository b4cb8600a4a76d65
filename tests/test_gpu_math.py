"""The dense FP64 helpers on the GPU: corr_dgemm and corr_syev through the C
ABI, and the reference-signature wrappers of src/MATH/ops_mat.cc and
read_transform_ri (ri.cc:109-144) in the shim, against the oracle's
restatements and the reference's own outputs (tests/golden/ops_mat.npz)."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD_DIR = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLD_DIR)
import make_golden_ops_mat as M  # noqa: E402

G = np.load(os.path.join(GOLD_DIR, "ops_mat.npz"))


@pytest.fixture(scope="module")
def ctx():
    import corr_gb300

    c = corr_gb300.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def shim():
    from corr_gb300 import build

    path = build.build_shim()
    return ctypes.CDLL(path)


def _gemm_tol(k, a, b):
    return 1e-15 * k * np.abs(a).max() * np.abs(b).max() + 1e-300


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (3, 5, 7), (64, 64, 64), (130, 67, 201),
                                   (257, 1, 300), (1, 300, 129)])
@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_dgemm_host_arrays(ctx, m, n, k, ta, tb):
    r = O.rng(1000 + m + 7 * n + 13 * k + 2 * ta + tb)
    A = r.standard_normal((k, m) if ta else (m, k))
    B = r.standard_normal((n, k) if tb else (k, n))
    C0 = r.standard_normal((m, n))
    ref = 0.7 * (A.T if ta else A) @ (B.T if tb else B) - 1.3 * C0
    out = C0.copy()
    ctx.dgemm(A, B, transa=ta, transb=tb, alpha=0.7, beta=-1.3, out=out)
    assert np.abs(out - ref).max() <= _gemm_tol(k, A, B) + 1e-15 * np.abs(C0).max() * 4


def test_dgemm_device_tensors_and_leading_dimensions(ctx):
    """Device pointers and ld > row length (sub-blocks of wider arrays)."""
    import torch

    from corr_gb300 import _lib

    r = O.rng(77)
    Aw = r.standard_normal((50, 40))
    Bw = r.standard_normal((33, 61))
    Cw = np.zeros((50, 70))
    m, n, k = 45, 29, 33  # A[:45, :33], B[:33, :29] (B stored k x n with ldb 61)
    dA, dB, dC = (torch.from_numpy(x).cuda() for x in (Aw, Bw, Cw))
    L = _lib.load()
    _lib.check(L.corr_dgemm(ctx._h, 0, 0, m, n, k, 1.0, ctypes.c_void_p(dA.data_ptr()), 40,
                            ctypes.c_void_p(dB.data_ptr()), 61, 0.0,
                            ctypes.c_void_p(dC.data_ptr()), 70))
    got = dC.cpu().numpy()
    ref = Aw[:m, :k] @ Bw[:k, :n]
    assert np.abs(got[:m, :n] - ref).max() <= _gemm_tol(k, Aw, Bw)
    assert not got[:m, n:].any() and not got[m:].any()  # nothing outside C touched


def test_dgemm_rejects_short_leading_dimension(ctx):
    from corr_gb300 import CorrError

    with pytest.raises(CorrError):
        from corr_gb300 import _lib

        a = np.zeros((4, 4))
        p = ctypes.c_void_p(a.ctypes.data)
        _lib.check(_lib.load().corr_dgemm(ctx._h, 0, 0, 4, 4, 4, 1.0, p, 3, p, 4, 0.0, p, 4))


def _check_eig(A, w, V, wref, tol_rel=1e-12):
    """Eigenvalues against wref, residual |A v - w v| and orthonormality."""
    scale = max(np.abs(wref).max(), 1e-300)
    n = A.shape[0]
    assert np.all(np.diff(w) >= 0), "eigenvalues not ascending"
    assert np.abs(w - wref).max() <= tol_rel * n * scale
    assert np.abs(A @ V.T - V.T * w).max() <= tol_rel * n * scale
    assert np.abs(V @ V.T - np.eye(n)).max() <= 1e-12 * n


@pytest.mark.parametrize("n", [9, 33])
def test_syev_vs_reference_diag_mat(ctx, n):
    x = M.ops_mat_inputs(n, 500 + n)
    for key, pre in (("sym", f"n{n}_diag_"), ("asym", f"n{n}_diag_asym_")):
        w, V = ctx.syev(x[key])
        Asym = np.tril(x[key]) + np.tril(x[key], -1).T
        _check_eig(Asym, w, V, G[pre + "vals"])
        assert np.allclose(np.abs((V * G[pre + "vecs"]).sum(1)), 1.0, atol=1e-9)


@pytest.mark.parametrize("n", [1, 2, 3, 64, 127, 128, 300, 513])
def test_syev_random_sizes(ctx, n):
    r = O.rng(900 + n)
    a = r.standard_normal((n, n))
    A = a + a.T
    w, V = ctx.syev(A)
    _check_eig(A, w, V, np.linalg.eigvalsh(A))


def test_syev_degenerate_and_device(ctx):
    """Repeated eigenvalues (any orthonormal basis of the eigenspace is
    right) and device tensors in and out."""
    import torch

    r = O.rng(31)
    Q, _ = np.linalg.qr(r.standard_normal((40, 40)))
    lam = np.repeat([-2.0, 0.0, 1.0, 5.0], 10)
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    dA = torch.from_numpy(A).cuda()
    w, V = ctx.syev(dA)
    assert w.is_cuda and V.is_cuda
    _check_eig(A, w.cpu().numpy(), V.cpu().numpy(), np.sort(lam))
    w, V = ctx.syev(np.eye(5) * 3.0)
    assert np.allclose(w, 3.0, atol=0, rtol=1e-15)


def test_syev_clusters_mixed_path(ctx):
    """n >= 64 runs FP32 sweeps first: clustered and exactly repeated
    eigenvalues of both signs, and a matrix of tiny norm (the FP32 stage
    works on A scaled by a power of two)."""
    r = O.rng(77)
    n = 260
    Q, _ = np.linalg.qr(r.standard_normal((n, n)))
    lam = np.concatenate([np.repeat([-3.0, 1.0], 60), 2.0 + 1e-9 * r.standard_normal(40),
                          r.uniform(-1.0, 4.0, n - 160)])
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    for scale in (1.0, 2.0 ** -400, 2.0 ** 300):
        w, V = ctx.syev(A * scale)
        _check_eig(A * scale, w, V, np.sort(lam) * scale)


def _f(fn, *argtypes):
    fn.argtypes = list(argtypes)
    fn.restype = None
    return fn


_dp = ctypes.POINTER(ctypes.c_double)


def _p(a):
    return a.ctypes.data_as(_dp)


@pytest.mark.parametrize("n", [9, 33])
def test_shim_ops_mat_vs_reference(shim, n):
    """The reference-signature wrappers against the reference's outputs."""
    x = {k: np.ascontiguousarray(v) for k, v in M.ops_mat_inputs(n, 500 + n).items()}
    tol = 1e-13 * n
    i, ll = ctypes.c_int, ctypes.c_longlong

    vals, vecs = np.zeros(n), np.zeros((n, n))
    _f(shim._Z8diag_matiPdS_S_, i, _dp, _dp, _dp)(n, _p(x["asym"].copy()), _p(vals), _p(vecs))
    assert np.abs(vals - G[f"n{n}_diag_asym_vals"]).max() <= tol * 10
    assert np.allclose(np.abs((vecs * G[f"n{n}_diag_asym_vecs"]).sum(1)), 1.0, atol=1e-9)

    mat, dum = x["sym"].copy(), np.zeros((n, n))
    _f(shim._Z13symmortho_matiPdS_S_, i, _dp, _dp, _dp)(n, _p(mat), _p(x["t"]), _p(dum))
    assert np.abs(mat - G[f"n{n}_symmortho_mat"]).max() <= tol
    assert np.abs(dum - G[f"n{n}_symmortho_dummat"]).max() <= tol

    mos, tmp = x["a"].copy(), np.zeros(n)
    _f(shim._Z13transform_MOsiPdS_S_, i, _dp, _dp, _dp)(n, _p(mos), _p(x["t"]), _p(tmp))
    assert np.abs(mos - G[f"n{n}_transform_MOs"]).max() <= tol
    assert np.abs(tmp - G[f"n{n}_transform_MOs_tmpvec"]).max() <= tol

    for sym, t, key in (("_Z9mat_mat_TiPdS_S_", i, "mat_mat_T"), ("_Z9mat_mat_TxPdS_S_", ll, "mat_mat_T_ll"),
                        ("_Z9mat_T_matiPdS_S_", i, "mat_T_mat"), ("_Z9mat_T_matxPdS_S_", ll, "mat_T_mat_ll")):
        f = np.zeros((n, n))
        _f(getattr(shim, sym), t, _dp, _dp, _dp)(n, _p(x["a"]), _p(x["b"]), _p(f))
        assert np.abs(f - G[f"n{n}_{key}"]).max() <= tol, sym

    vo = np.zeros(n)
    _f(shim._Z3pmvPdS_S_i, _dp, _dp, _dp, i)(_p(x["a"]), _p(x["v"]), _p(vo), n)
    assert np.abs(vo - G[f"n{n}_pmv"]).max() <= tol

    # declared in ops_mat.h but only defined (commented out) in ops_mat.cc:155-190
    f = np.zeros((n, n))
    _f(shim._Z7mat_matiPdS_S_, i, _dp, _dp, _dp)(n, _p(x["a"]), _p(x["b"]), _p(f))
    assert np.abs(f - x["a"] @ x["b"]).max() <= tol
    for d in (0, 1):
        mat, tmpm = x["sym"].copy(), np.zeros((n, n))
        _f(shim._Z9trans_matiPdS_S_i, i, _dp, _dp, _dp, i)(n, _p(mat), _p(x["t"]), _p(tmpm), d)
        T = x["t"]
        ref = T.T @ x["sym"] @ T if d == 0 else T @ x["sym"] @ T.T
        assert np.abs(mat - ref).max() <= tol


def test_shim_read_transform_ri_vs_reference(shim, tmp_path):
    naux, N, nocc, seed = M.RI_FILE_CASE
    bpq, mos = M.ri_file_inputs(naux, N, nocc, seed)
    prefix = tmp_path / "case"
    bpq.tofile(str(prefix) + ".rimp2")
    np.ascontiguousarray(mos).tofile(str(prefix) + ".mos")
    exe = tmp_path / "drv"
    subprocess.run(["g++", "-O1", "-std=c++14", "-o", str(exe),
                    os.path.join(ROOT, "tests", "shim_ri_file_driver.cc"),
                    "-L" + os.path.join(ROOT, "corr_gb300"), "-lcorr_shim", "-lcorr_gb300",
                    "-Wl,-rpath," + os.path.join(ROOT, "corr_gb300")], check=True)
    subprocess.run([str(exe), str(prefix), str(2 * nocc), str(N), str(naux)], check=True)
    got = np.fromfile(str(prefix) + ".bia").reshape(naux, nocc, N - nocc)
    assert np.abs(got - G["read_transform_ri_bia"]).max() <= 1e-14
    # a missing BPQ file aborts loudly instead of transforming garbage
    np.ascontiguousarray(mos).tofile(str(tmp_path / "missing") + ".mos")
    r = subprocess.run([str(exe), str(tmp_path / "missing"), str(2 * nocc), str(N), str(naux)],
                       capture_output=True, text=True)
    assert r.returncode != 0
