"""Seeded synthetic workloads of the benchmark (the RI-MP2 shapes and
distributions the configurations name).  Inputs only: nothing here computes
an energy.

* rimp2: B^Q_ia = G_Qia s_Q with G ~ N(0,1), s_Q = 0.05 exp(-Q/400);
  eps_occ ~ U[-1.5,-0.3] sorted, eps_vir ~ U[0.05,3.0] sorted (PCG64 seed).
* batch_sizes: nocc ~ U{5..60}, nvir = nocc U{4..8}, naux = round(3.5 nvir).
* ri_pipeline: the inputs of the RI pipeline downstream of the integral code
  (a positive definite metric J, symmetric (P|mn), orthonormal MO
  coefficients and orbital energies) at the water-cluster sizes, generated on
  the GPU from a seeded torch generator.
"""
from __future__ import annotations

import numpy as np


def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def synth_rimp2(nocc, nvir, naux, seed, dtype=np.float64):
    """Returns (B[Q][i][a], eps[nocc+nvir])."""
    r = rng(seed)
    B = r.standard_normal((naux, nocc, nvir))
    B *= (0.05 * np.exp(-np.arange(naux) / 400.0))[:, None, None]
    eo = np.sort(r.uniform(-1.5, -0.3, nocc))
    ev = np.sort(r.uniform(0.05, 3.0, nvir))
    return np.ascontiguousarray(B, dtype=dtype), np.concatenate([eo, ev])


def synth_batch_sizes(count, seed):
    r = rng(seed)
    out = []
    for _ in range(count):
        o = int(r.integers(5, 61))
        v = o * int(r.integers(4, 9))
        out.append((o, v, int(round(3.5 * v))))
    return out


def synth_ri_pipeline(nbf, nocc, naux, seed, device="cuda"):
    """(mos[p][mu], eps, J[P][Q], Pmn[P][mu][nu]) as float64 torch tensors on
    `device`.  J = L L^T / naux + 0.5 I (condition number ~10), (P|mn)
    symmetric in m, n with a decaying auxiliary spectrum, mos orthonormal.
    The (P|mn) amplitude 0.0035 exp(-P/600) puts the RI-MP2 energy at the
    water-cluster sizes near -4 Eh, the magnitude of the molecule's."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    f64 = torch.float64
    L = torch.randn((naux, naux), generator=g, device=device, dtype=f64)
    J = L @ L.T / naux + 0.5 * torch.eye(naux, device=device, dtype=f64)
    s = 0.0035 * torch.exp(-torch.arange(naux, device=device, dtype=f64) / 600.0)
    P = torch.randn((naux, nbf, nbf), generator=g, device=device, dtype=f64) * s[:, None, None]
    P = 0.5 * (P + P.transpose(1, 2))
    # orthonormalised on the host: torch's lazily loaded GPU linear-algebra
    # library is not always loadable (e.g. under a profiler)
    R = torch.randn((nbf, nbf), generator=g, device=device, dtype=f64).cpu().numpy()
    Q, _ = np.linalg.qr(R)
    mos = torch.from_numpy(np.ascontiguousarray(Q.T)).to(device)
    eo = torch.sort(torch.rand(nocc, generator=g, device=device, dtype=f64) * 1.2 - 1.5)[0]
    ev = torch.sort(torch.rand(nbf - nocc, generator=g, device=device, dtype=f64) * 2.95 + 0.05)[0]
    return mos, torch.cat([eo, ev]).contiguous(), J.contiguous(), P.contiguous()
