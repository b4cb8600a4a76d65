"""RI-MP2 adjoint (dE/dB, dE/deps) on the GPU: against the FP64 restatement
of the gradient, against central finite differences, and through the
torch.autograd.Function.  Tolerance for the adjoint: 1e-6 relative to FD
(written per test), 1e-11 against the FP64 restatement."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("o,v,X,seed", [(1, 1, 1, 1), (3, 7, 9, 2), (5, 70, 33, 3), (4, 130, 65, 4)])
def test_gradient_vs_fp64_restatement(ctx, o, v, X, seed):
    B, eps = O.synth_rimp2(o, v, X, seed)
    E, dB, de = O.rimp2_gradient(B, eps, o, v)
    Eg, dBg, deg = ctx.rimp2_gradient(B, eps, o, v, X)
    assert abs(Eg - E) <= 1e-12 * max(1.0, abs(E))
    assert np.abs(dBg - dB).max() <= 1e-11 * max(1e-30, np.abs(dB).max())
    assert np.abs(deg - de).max() <= 1e-11 * max(1e-30, np.abs(de).max())


@pytest.mark.parametrize("o,v,X,seed", [(1, 1, 1, 1), (3, 7, 9, 2), (5, 70, 33, 3), (4, 130, 65, 4),
                                        (9, 200, 600, 5)])
def test_gradient_tc_vs_fp64_restatement(ctx, o, v, X, seed):
    """The tensor-core adjoint (digit GEMMs): the FP64 restatement's values to
    the digit GEMM's accuracy (1e-10 of the largest component; X = 600 runs two
    K passes)."""
    B, eps = O.synth_rimp2(o, v, X, seed)
    E, dB, de = O.rimp2_gradient(B, eps, o, v)
    Eg, dBg, deg = ctx.rimp2_gradient(B, eps, o, v, X, tensor_cores=True)
    assert abs(Eg - E) <= 1e-11 * max(1.0, abs(E))
    assert np.abs(dBg - dB).max() <= 1e-10 * max(1e-30, np.abs(dB).max())
    assert np.abs(deg - de).max() <= 1e-10 * max(1e-30, np.abs(de).max())


def test_gradient_vs_central_differences_small(ctx):
    o, v, X = 4, 40, 30
    B, eps = O.synth_rimp2(o, v, X, 9)
    _, dB, de = ctx.rimp2_gradient(B, eps, o, v, X)
    r = O.rng(10)
    h = 1e-5
    for _ in range(40):
        q, i, a = int(r.integers(X)), int(r.integers(o)), int(r.integers(v))
        Bp, Bm = B.copy(), B.copy()
        Bp[q, i, a] += h
        Bm[q, i, a] -= h
        fd = (O.rimp2_energy_local(Bp, eps, o, v, i, a) -
              O.rimp2_energy_local(Bm, eps, o, v, i, a)) / (2 * h)
        assert abs(fd - dB[q, i, a]) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(dB).max())
    for p in range(o + v):
        ep, em = eps.copy(), eps.copy()
        ep[p] += h
        em[p] -= h
        fd = (O.rimp2_energy(B, ep, o, v)[2] - O.rimp2_energy(B, em, o, v)[2]) / (2 * h)
        assert abs(fd - de[p]) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(de).max())


@pytest.fixture(scope="module")
def config4():
    o, v, X = 64, 512, 2048
    B32, eps = O.synth_rimp2(o, v, X, 4004, dtype=np.float32)
    return o, v, X, B32.astype(np.float64), eps  # the stored values, exactly


@pytest.fixture(scope="module")
def config4_fp64(ctx, config4):
    import time

    import torch

    o, v, X, B, eps = config4
    Bd, ed = torch.from_numpy(B).cuda(), torch.from_numpy(eps).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E, dB, de = ctx.rimp2_gradient(Bd, ed, o, v, X)
    torch.cuda.synchronize()
    print(f"config-4 adjoint, FP64 form: {1e3 * (time.perf_counter() - t0):.1f} ms")
    return E, dB.cpu().numpy(), de.cpu().numpy()


def test_gradient_tc_config4_vs_fp64(ctx, config4, config4_fp64):
    """Config 4 through the tensor-core adjoint (device arrays): the FP64 form's
    gradient to 1e-10 of its largest component, and its time beside it."""
    import time

    import torch

    o, v, X, B, eps = config4
    Bd, ed = torch.from_numpy(B).cuda(), torch.from_numpy(eps).cuda()
    ctx.rimp2_gradient(Bd, ed, o, v, X, tensor_cores=True)  # warm (workspace)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E, dB, de = ctx.rimp2_gradient(Bd, ed, o, v, X, tensor_cores=True)
    torch.cuda.synchronize()
    print(f"config-4 adjoint, tensor-core form: {1e3 * (time.perf_counter() - t0):.1f} ms")
    E64, dB64, de64 = config4_fp64
    dB = dB.cpu().numpy()
    de = de.cpu().numpy()
    assert abs(E - E64) <= 1e-11 * abs(E64)
    assert np.abs(dB - dB64).max() <= 1e-10 * np.abs(dB64).max()
    assert np.abs(de - de64).max() <= 1e-10 * np.abs(de64).max()


@pytest.mark.parametrize("tc", [False, True])
def test_gradient_config4_finite_differences(ctx, config4, config4_fp64, tc):
    """nocc=64, nvir=512, naux=2048 (config-2 distributions, FP32 storage):
    central differences (h=1e-4) on 200 seeded entries of B, and sampled
    rows of the FP64 restatement; both adjoint forms."""
    o, v, X, B, eps = config4
    B = B.copy()
    if tc:
        E, dB, de = ctx.rimp2_gradient(B, eps, o, v, X, tensor_cores=True)
    else:
        E, dB, de = config4_fp64
    r = O.rng(4005)
    h = 1e-4
    scale = np.abs(dB).max()
    worst = 0.0
    for _ in range(200):
        q, i, a = int(r.integers(X)), int(r.integers(o)), int(r.integers(v))
        old = B[q, i, a]
        B[q, i, a] = old + h
        ep = O.rimp2_energy_local(B, eps, o, v, i, a)
        B[q, i, a] = old - h
        em = O.rimp2_energy_local(B, eps, o, v, i, a)
        B[q, i, a] = old
        fd = (ep - em) / (2 * h)
        err = abs(fd - dB[q, i, a]) / max(abs(fd), 1e-3 * scale)
        worst = max(worst, err)
    assert worst <= 1e-6, worst
    # dE/deps against central differences of the FP64 GPU energy
    for p in (0, o - 1, o, o + v // 2, o + v - 1):
        e1, e2 = eps.copy(), eps.copy()
        e1[p] += 1e-4
        e2[p] -= 1e-4
        fd = (ctx.rimp2_energy(B, e1, o, v, X, "fp64").e_total -
              ctx.rimp2_energy(B, e2, o, v, X, "fp64").e_total) / 2e-4
        assert abs(fd - de[p]) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(de).max())


def test_autograd_function(ctx):
    import torch

    from corr_gb300.autograd import rimp2_energy

    o, v, X = 5, 60, 40
    B, eps = O.synth_rimp2(o, v, X, 21)
    Bt = torch.tensor(B, device="cuda", requires_grad=True)
    et = torch.tensor(eps, device="cuda", requires_grad=True)
    E = rimp2_energy(Bt, et, o, v, "fp64", ctx)
    E.backward()
    Eo, dB, de = O.rimp2_gradient(B, eps, o, v)
    assert abs(E.item() - Eo) <= 1e-12 * abs(Eo)
    assert np.abs(Bt.grad.cpu().numpy() - dB).max() <= 1e-11 * np.abs(dB).max()
    assert np.abs(et.grad.cpu().numpy() - de).max() <= 1e-11 * np.abs(de).max()
    # FP32 storage, precision-form forward
    B32 = torch.tensor(B.astype(np.float32), device="cuda", requires_grad=True)
    E32 = rimp2_energy(B32, et.detach(), o, v, "split_bf16", ctx)
    (g,) = torch.autograd.grad(E32, B32)
    assert g.dtype == torch.float32
    # the precision-form forward's backward is the tensor-core adjoint
    _, dB32, _ = O.rimp2_gradient(B.astype(np.float32).astype(np.float64), eps, o, v)
    assert np.abs(g.cpu().numpy() - dB32).max() <= 1e-6 * np.abs(dB32).max()
    assert abs(E32.item() - O.rimp2_energy(B.astype(np.float32).astype(np.float64), eps, o, v)[2]) \
        <= 2e-7 * abs(Eo)
