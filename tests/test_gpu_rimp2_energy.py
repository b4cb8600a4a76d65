"""RI-MP2 energy (src/POSTHF/can_mp2.cc:53) on the GPU against the oracle.

FP64 form: |dE| <= 1e-10 Eh or 1e-12 relative (the synthetic configs have
|E| up to ~6e4 Eh, where a different FP64 summation order alone moves the last
~4 digits).  Split forms: relative error bounds written per test.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_ABS, FP64_REL = 1e-10, 1e-12

SHAPES = [
    (1, 1, 1, 11),      # smallest: E = -(ia|ia)^2/D
    (3, 5, 7, 12),
    (5, 19, 60, 13),     # config-1 orbital sizes
    (2, 64, 17, 14),     # exactly one FP64 tile
    (6, 129, 70, 15),    # crosses the 128 tcgen05 tile by one
    (7, 33, 95, 16),     # naux not a multiple of the 32-wide K block
    (4, 257, 40, 17),
]


def _close(e, ref, abs_tol, rel_tol):
    return abs(e - ref) <= max(abs_tol, rel_tol * abs(ref))


@pytest.mark.parametrize("o,v,X,seed", SHAPES)
def test_fp64_matches_oracle(ctx, o, v, X, seed):
    B, eps = O.synth_rimp2(o, v, X, seed)
    ref = O.rimp2_energy(B, eps, o, v)
    got = ctx.rimp2_energy(B, eps, o, v, X, "fp64")
    for g, r in zip(got.as_tuple(), ref):
        assert _close(g, r, FP64_ABS, FP64_REL), (got, ref)
    assert abs(got.e_scs - (ref[0] / 3 + ref[1] * 6 / 5)) <= 1e-10 + 1e-12 * abs(ref[2])


@pytest.mark.parametrize("o,v,X,seed", SHAPES)
# split_fp16 carries two FP16 digits (about 21 bits of each row's scale), so
# shapes with a handful of terms see up to ~3e-7 relative; split_bf16 carries
# three BF16 digits (21-27 bits), up to ~4e-9.  Bounds: about 3x the largest
# deviation measured over these shapes (E, E_OS; E_SS relative to E).
@pytest.mark.parametrize("prec,rel,rel_ss", [("split_fp16", 9e-7, 2e-7),
                                             ("split_bf16", 1.3e-8, 8e-9)])
def test_split_matches_oracle(ctx, o, v, X, seed, prec, rel, rel_ss):
    B, eps = O.synth_rimp2(o, v, X, seed)
    ref = O.rimp2_energy(B, eps, o, v)
    got = ctx.rimp2_energy(B, eps, o, v, X, prec)
    print(f"REL split_matches {prec} o={o} v={v} X={X}: "
          f"{abs(got.e_total - ref[2]) / abs(ref[2]):.3e} {abs(got.e_os - ref[1]) / abs(ref[1]):.3e} "
          f"{abs(got.e_ss - ref[0]) / abs(ref[2]):.3e}")
    assert abs(got.e_total - ref[2]) <= rel * abs(ref[2]), (prec, got, ref)
    assert abs(got.e_os - ref[1]) <= rel * abs(ref[1]), (prec, got, ref)
    # E_SS is a difference; bound it relative to the total
    assert abs(got.e_ss - ref[0]) <= rel_ss * abs(ref[2]), (prec, got, ref)


@pytest.mark.parametrize("o,v,X,seed", [
    (5, 7, 1600, 21),   # row statistics staged in shared memory, 8 rows per block (limit)
    (3, 41, 3200, 22),  # staged, 4 rows per block, at its size limit
    (2, 30, 3300, 23),  # beyond the staged form: two-pass global form
])
def test_split_fp16_row_statistics_forms(ctx, o, v, X, seed):
    B, eps = O.synth_rimp2(o, v, X, seed)
    ref = O.rimp2_energy(B, eps, o, v)
    got = ctx.rimp2_energy(B, eps, o, v, X, "split_fp16")
    print(f"REL rowstat o={o} v={v} X={X}: {abs(got.e_total - ref[2]) / abs(ref[2]):.3e} "
          f"{abs(got.e_ss - ref[0]) / abs(ref[2]):.3e}")
    assert abs(got.e_total - ref[2]) <= 1e-6 * abs(ref[2]), (got, ref)
    assert abs(got.e_ss - ref[0]) <= 1e-6 * abs(ref[2]), (got, ref)


def test_config2_full_size(ctx):
    """nocc=40, nvir=360, naux=1200 (decaying aux spectrum)."""
    o, v, X = 40, 360, 1200
    B, eps = O.synth_rimp2(o, v, X, 2024)
    ref = O.rimp2_energy(B, eps, o, v)
    f64 = ctx.rimp2_energy(B, eps, o, v, X, "fp64")
    assert _close(f64.e_total, ref[2], FP64_ABS, FP64_REL), (f64, ref)
    assert _close(f64.e_ss, ref[0], FP64_ABS, FP64_REL), (f64, ref)
    h16 = ctx.rimp2_energy(B, eps, o, v, X, "split_fp16")
    print(f"REL config2 {abs(h16.e_total - ref[2]) / abs(ref[2]):.3e}")
    assert abs(h16.e_total - ref[2]) <= 1e-7 * abs(ref[2]), (h16, ref)  # measured 3.1e-8


def test_device_resident_inputs(ctx):
    import torch

    o, v, X = 5, 40, 50
    B, eps = O.synth_rimp2(o, v, X, 99)
    ref = ctx.rimp2_energy(B, eps, o, v, X, "fp64")
    Bd = torch.from_numpy(B).cuda()
    ed = torch.from_numpy(eps).cuda()
    got = ctx.rimp2_energy(Bd, ed, o, v, X, "fp64")
    assert got.as_tuple() == ref.as_tuple()


@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_unaligned_device_input(ctx, prec):
    """B starting 8 bytes into an allocation (not 16-byte aligned): the
    pre-pass takes its 8-byte copy path and gives the same energy."""
    import torch

    o, v, X = 6, 140, 300
    B, eps = O.synth_rimp2(o, v, X, 123)
    ed = torch.from_numpy(eps).cuda()
    aligned = torch.from_numpy(B).cuda()
    buf = torch.empty(B.size + 1, dtype=torch.float64, device="cuda")
    shifted = buf[1:].view(B.shape)
    shifted.copy_(aligned)
    assert shifted.data_ptr() % 16 == 8
    a = ctx.rimp2_energy(aligned, ed, o, v, X, prec)
    b = ctx.rimp2_energy(shifted, ed, o, v, X, prec)
    assert a.as_tuple() == b.as_tuple()


def test_repeat_is_deterministic(ctx):
    o, v, X = 6, 150, 90
    B, eps = O.synth_rimp2(o, v, X, 5)
    for prec in ("fp64", "split_fp16"):
        a = ctx.rimp2_energy(B, eps, o, v, X, prec)
        b = ctx.rimp2_energy(B, eps, o, v, X, prec)
        assert a.as_tuple() == b.as_tuple()


@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_split_wide_dynamic_range(ctx, prec):
    """B with per-Q scales spread log-uniformly over six decades and a few
    spiky rows (one dominant Q): most products are of elements far below the
    row scale, the regime where dropping the lowest-digit products biases
    the energy."""
    o, v, X = 6, 140, 300
    r = O.rng(404)
    B = r.standard_normal((X, o, v)) * (10.0 ** (-6.0 * r.uniform(size=X)))[:, None, None]
    B[r.integers(0, X, 20), r.integers(0, o, 20), r.integers(0, v, 20)] *= 1e4
    eps = np.concatenate([np.sort(r.uniform(-1.5, -0.3, o)), np.sort(r.uniform(0.05, 3.0, v))])
    ref = O.rimp2_energy(B, eps, o, v)
    got = ctx.rimp2_energy(B, eps, o, v, X, prec)
    print(f"REL wide {prec}: {abs(got.e_total - ref[2]) / abs(ref[2]):.3e} "
          f"{abs(got.e_os - ref[1]) / abs(ref[1]):.3e}")
    rel = {"split_fp16": 3e-9, "split_bf16": 6e-11}[prec]  # measured 8.4e-10, 1.7e-11
    assert abs(got.e_total - ref[2]) <= rel * abs(ref[2]), (prec, got, ref)
    assert abs(got.e_os - ref[1]) <= rel * abs(ref[1]), (prec, got, ref)


@pytest.mark.parametrize("o,v,X", [(3, 64, 40), (5, 150, 70), (7, 300, 90), (4, 192, 50),
                                   (9, 257, 100)])
@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_padded_last_tile(ctx, o, v, X, prec):
    """Last virtual tiles of 64, 22, 44, 64 and 1 columns padded to 128 (the
    padded columns are zeros with column scale 0) against the oracle; the
    tile setting is accepted and changes nothing."""
    B, eps = O.synth_rimp2(o, v, X, 61 + v)
    e1 = ctx.rimp2_energy(B, eps, o, v, X, prec)
    ctx.set_energy_tiles(0)
    try:
        e0 = ctx.rimp2_energy(B, eps, o, v, X, prec)
    finally:
        ctx.set_energy_tiles(1)
    assert e1.as_tuple() == e0.as_tuple()
    ref = O.rimp2_energy(B, eps, o, v)
    assert abs(e1.e_total - ref[2]) <= 2e-7 * abs(ref[2]), (prec, e1, ref)


def _exact_digit_inputs(o, v, X, seed):
    """B whose rows are small integers times 2^-10 (|k| <= 20, one element of
    each row at +-20): every row scaled by its power of two is an integer of at
    most 11 bits, so both precision forms represent B exactly in their leading
    digit and every tensor-core sum, hence every (ia|jb) value the epilogue
    receives, is exact in FP32."""
    r = O.rng(seed)
    k = r.integers(-20, 21, size=(X, o, v)).astype(np.float64)
    k[0] = np.where(r.uniform(size=(o, v)) < 0.5, -20.0, 20.0)
    B = np.ascontiguousarray(k * 2.0 ** -10)
    eps = np.concatenate([np.sort(r.uniform(-1.5, -0.3, o)), np.sort(r.uniform(0.05, 3.0, v))])
    return B, eps


@pytest.mark.parametrize("o,v,X,seed", [(1, 1, 1, 71), (3, 5, 7, 72), (6, 129, 70, 73),
                                        (4, 257, 40, 74), (8, 300, 256, 75), (12, 200, 600, 76)])
@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_epilogue_accuracy_on_exact_digits(ctx, o, v, X, seed, prec):
    """The energy arithmetic of the precision forms in isolation: on inputs
    whose digit representation is exact, every (ia|jb) reaches the epilogue
    without error, so the difference from the FP64 energy of the same B is the
    epilogue's own (denominators from FP64 orbital energies, 1/D, squares,
    products and the compensated per-unit sums).  Bound: 1e-12 relative."""
    B, eps = _exact_digit_inputs(o, v, X, seed)
    ref = O.rimp2_energy(B, eps, o, v)
    got = ctx.rimp2_energy(B, eps, o, v, X, prec)
    rel = [abs(g - r) / abs(ref[2]) for g, r in zip(got.as_tuple(), ref)]
    print(f"{prec} o={o} v={v} X={X}: relative deviation E_SS/E_OS/E {rel}")
    assert max(rel) <= 1e-12, (prec, got, ref, rel)


@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_error_estimate(ctx, prec):
    """corr_rimp2_energy_estimate: the energy equals corr_rimp2_energy's, and
    the estimate (one standard deviation of the digit rounding's effect) is of
    the size of the actual deviation from the FP64 energy: over several
    workloads the geometric mean of deviation / estimate lies within a factor
    of 4 of 1 (single cases may be a few sigma out)."""
    import math

    ratios = []
    for (o, v, X, seed) in [(8, 128, 300, 31), (12, 200, 400, 32), (16, 256, 512, 33),
                            (24, 300, 800, 34), (40, 360, 1200, 2024)]:
        B, eps = O.synth_rimp2(o, v, X, seed)
        e64 = ctx.rimp2_energy(B, eps, o, v, X, "fp64").e_total
        e1 = ctx.rimp2_energy(B, eps, o, v, X, prec)
        e2, est = ctx.rimp2_energy_estimate(B, eps, o, v, X, prec)
        assert e2.as_tuple() == e1.as_tuple()
        assert est > 0.0
        ratios.append(abs(e1.e_total - e64) / est)
    gm = math.exp(sum(math.log(max(r, 1e-3)) for r in ratios) / len(ratios))
    print(f"{prec}: deviation / estimate per workload {[round(r, 2) for r in ratios]}, "
          f"geometric mean {gm:.2f}")
    assert 0.25 <= gm <= 4.0, ratios
    e, est = ctx.rimp2_energy_estimate(*O.synth_rimp2(3, 20, 30, 35), 3, 20, 30, "fp64")
    assert est == 0.0
