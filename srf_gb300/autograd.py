"""Differentiable Siddon projector (not in the reference).

``project(image, lors, center, size, tof=None, tof_nsigma=0.0)`` is a ``torch.autograd.Function``
whose forward is the sm_103a projector (srf_projection / srf_projection_tof: the reference's
projector rules) and whose backward is ``srf_projection_adjoint``, the exact adjoint of that
projector (projector skip rules and 1/L^2 weights). The reference's backprojector is *not* this
adjoint (no endpoint/steep skips, no 1/L^2), so it cannot serve as a gradient.

``image`` is (nx, ny, nz) or a batch (B, nx, ny, nz) of float32 CUDA tensors; the result is (N,)
or (B, N). A batch runs through srf_projection_batch / srf_projection_adjoint_batch, which set up
and traverse each LOR once for up to 8 images. ``poisson_nll(p, y)`` is the list-mode/binned Poisson negative log-likelihood
sum(p - y log p) used as the training loss.
"""
from __future__ import annotations

from typing import Optional, Sequence, Tuple

import torch

from . import kernels


class _Project(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image: torch.Tensor, lors: torch.Tensor, center, size, tof, tof_nsigma):
        ctx.save_for_backward(lors)
        ctx.meta = (list(image.shape[-3:]), list(center), list(size), tof, tof_nsigma, image.dim())
        if image.dim() == 3:
            return kernels.project(lors, image.detach(), center, size, tof=tof, tof_nsigma=tof_nsigma)
        B = kernels.MAX_BATCH
        return torch.cat([kernels.project_batch(lors, image[k:k + B].detach(), center, size, tof=tof,
                                                tof_nsigma=tof_nsigma) for k in range(0, image.shape[0], B)])

    @staticmethod
    def backward(ctx, grad_p: torch.Tensor):
        (lors,) = ctx.saved_tensors
        shape, center, size, tof, tof_nsigma, dim = ctx.meta
        g = grad_p.detach().to(torch.float32)

        if dim == 3:
            grad = kernels.backproject(lors, g.contiguous(), shape, center, size, tof=tof,
                                       tof_nsigma=tof_nsigma, adjoint=True)
        else:
            B = kernels.MAX_BATCH
            grad = torch.cat([kernels.adjoint_batch(lors, g[k:k + B], shape, center, size, tof=tof,
                                                    tof_nsigma=tof_nsigma) for k in range(0, g.shape[0], B)])
        return grad, None, None, None, None, None


def project(image: torch.Tensor, lors: torch.Tensor, center: Sequence[float], size: Sequence[float],
            tof: Optional[Tuple[float, float]] = None, tof_nsigma: float = 0.0) -> torch.Tensor:
    return _Project.apply(image, lors, list(center), list(size), tof, tof_nsigma)


def poisson_nll(p: torch.Tensor, y: torch.Tensor, eps: float = 0.0) -> torch.Tensor:
    return (p - y * torch.log(p + eps)).sum()
