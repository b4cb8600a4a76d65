"""The CCSD consumer of the MO integrals (src/POSTHF/ccsd.cc:6-48, 509-535) on
the GPU: the spin-orbital integrals <ij||kl> and the spin-orbital core
Hamiltonian and Fock matrix, from a prec_ints tensor that corr_motrans leaves
in device memory, against the oracle's restatements (pinned to the reference's
calc_ints_so and form_fock in test_oracle_pin.py)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,nroe", [(2, 2), (7, 6), (13, 10), (24, 10)])
def test_ints_so_and_fock_from_device_integrals(ctx, N, nroe):
    import torch

    eri, _ = O.synth_eri(N, 90 + N)
    pk = O.pack_eri(eri)
    mos = O.synth_orbitals(N, 91 + N)
    prec_d = torch.empty((N, N, N, N), dtype=torch.float64, device="cuda")
    ctx.motrans(nroe, mos, pk, out=prec_d)  # stays on the device
    prec = prec_d.cpu().numpy()
    so = ctx.ints_so(prec_d)
    assert so.is_cuda
    assert np.array_equal(so.cpu().numpy(), O.ints_so(prec))  # a gather: bit-exact
    H = O.rng(92 + N).standard_normal((N, N))
    H = H + H.T
    h, f = ctx.cc_fock(nroe, mos, H, prec_d)
    rh, rf = O.cc_fock(nroe, mos, H, prec)
    scale = max(1.0, np.abs(rf).max())
    assert np.abs(h.cpu().numpy() - rh).max() <= 1e-13 * scale
    assert np.abs(f.cpu().numpy() - rf).max() <= 1e-13 * scale


def test_ints_so_host_and_unaligned_outputs(ctx):
    import torch

    N = 6
    eri, _ = O.synth_eri(N, 95)
    prec = O.motrans(O.synth_orbitals(N, 96), O.pack_eri(eri))
    ref = O.ints_so(prec)
    assert np.array_equal(ctx.ints_so(prec), ref)  # host in, host out
    M = 2 * N
    buf = torch.empty(M ** 4 + 1, dtype=torch.float64, device="cuda")
    out = buf[1:].view(M, M, M, M)  # 8 bytes off a 16-byte boundary
    assert out.data_ptr() % 16 == 8
    ctx.ints_so(prec, out=out)
    assert np.array_equal(out.cpu().numpy(), ref)
