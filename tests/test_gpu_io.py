"""The hand-off file readers on their device path: arrays of several pinned
chunks streamed from PREFIX.oei/.tei/.ahfw/.rimp2 into GPU memory, bit-exact,
and the packed ERI list of a .tei file fed from device memory into the MO
transform (the reference's read_tei -> MOtrans hand-off, main.cc:93-132)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

import files as F  # tests/files.py (the test directory is on sys.path)

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_device_destinations_span_several_chunks(ctx, tmp_path):
    import torch

    r = O.rng(21)
    prefix = str(tmp_path / "big")
    nint = 3_000_001  # 24 MB of values and 24 MB of indices: three 8 MB chunks each
    sc = np.array([7, 70, 700, 7000], dtype=np.int64)
    iv = r.standard_normal(nint)
    inum = r.integers(0, 65536, (nint, 4)).astype(np.uint16)
    F.write_tei(prefix, sc, iv, inum)
    gsc, giv, gin = ctx.read_tei(prefix, nint, device="cuda")
    assert giv.is_cuda and gin.is_cuda
    assert np.array_equal(gsc, sc)
    assert np.array_equal(giv.cpu().numpy(), iv)
    assert np.array_equal(gin.cpu().numpy().view(np.uint16), inum)
    n = 1100  # four 9.7 MB matrices
    mats = [r.standard_normal((n, n)) for _ in range(4)]
    F.write_oei(prefix, *mats)
    for a, b in zip(ctx.read_oei(prefix, n, device="cuda"), mats):
        assert torch.equal(a.cpu(), torch.from_numpy(b))
    e, c = np.sort(r.standard_normal(n)), r.standard_normal((n, n))
    import corr_gb300

    corr_gb300.write_wav_hf(prefix + ".ahfw", e, c)
    ge, gc = ctx.read_wav_hf(prefix, n, device="cuda")
    assert np.array_equal(ge.cpu().numpy(), e) and np.array_equal(gc.cpu().numpy(), c)
    bpq = r.standard_normal((9, 40, 40))
    F.write_rimp2(prefix, bpq)
    assert np.array_equal(ctx.read_rimp2(prefix, 9, 40, device="cuda").cpu().numpy(), bpq)


def test_tei_file_to_device_motrans(ctx, tmp_path):
    """Packed ERIs written in the reference's .tei layout, read into device
    memory and transformed there: the same (ij|kl) as from host arrays."""
    N, nocc = 13, 3
    eri, _ = O.synth_eri(N, 31)
    pk = O.pack_eri(eri)
    mos = O.synth_orbitals(N, 32)
    prefix = str(tmp_path / "h2o")
    F.write_tei(prefix, pk.sortcount, pk.intval, pk.intnums.reshape(-1, 4))
    sc, iv, inum = ctx.read_tei(prefix, pk.nrofint, device="cuda")

    class Dev:
        nrofint = pk.nrofint
        sortcount = np.ascontiguousarray(sc)
        intval = iv
        intnums = inum

    got = ctx.motrans(2 * nocc, mos, Dev)
    ref = ctx.motrans(2 * nocc, mos, pk)
    assert np.array_equal(got, ref)
