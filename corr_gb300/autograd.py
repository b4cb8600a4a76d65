"""torch.autograd.Function over the GPU RI-MP2 energy and its adjoint.

Forward runs corr_rimp2_energy (FP64 or the tcgen05 precision form); backward
runs the adjoint of the same form: corr_rimp2_gradient (FP64 panels) after an
FP64 forward, corr_rimp2_gradient_tc (FP64-accurate digit GEMMs on the tensor
cores) after a precision-form forward; both recompute the (ia|jb) tiles per
block of occupied orbitals instead of storing amplitudes.  This module does not import
psi4, so it can sit next to the syshfwplug plugin without pulling it in.
"""
from __future__ import annotations

import torch

from . import default_context


class RIMP2Energy(torch.autograd.Function):
    """E = E_OS + E_SS of the RI-MP2 energy for B[Q][i][a] (CUDA, float64 or
    float32) and eps[nocc+nvir]; differentiable in both."""

    @staticmethod
    def forward(ctx, B, eps, nocc, nvir, precision="split_bf16", context=None):
        c = context or default_context()
        Bd = B.detach().to(torch.float64).contiguous()
        ed = eps.detach().to(torch.float64).contiguous()
        naux = Bd.shape[0]
        e = c.rimp2_energy(Bd, ed, nocc, nvir, naux, precision)
        ctx.save_for_backward(Bd, ed)
        ctx.dims = (nocc, nvir, naux)
        ctx.context = c
        ctx.in_dtypes = (B.dtype, eps.dtype)
        ctx.precision = precision
        return torch.tensor(e.e_total, dtype=torch.float64, device=B.device)

    @staticmethod
    def backward(ctx, gE):
        Bd, ed = ctx.saved_tensors
        nocc, nvir, naux = ctx.dims
        # the adjoint follows the forward: FP64 panels for the FP64 form, the
        # tensor-core (digit-GEMM) adjoint for the precision forms
        _, dB, de = ctx.context.rimp2_gradient(Bd, ed, nocc, nvir, naux,
                                               tensor_cores=ctx.precision != "fp64")
        g = gE.to(torch.float64)
        dB = (dB * g).to(ctx.in_dtypes[0])
        de = (de * g).to(ctx.in_dtypes[1])
        return dB, de, None, None, None, None


def rimp2_energy(B, eps, nocc, nvir, precision="split_bf16", context=None):
    return RIMP2Energy.apply(B, eps, nocc, nvir, precision, context)
