"""Image warping on the GPU: deformation by a displacement field, its inverse, rigid shifts and
in-plane rotation (srfnef/ops/deform_mixins.py:18-89 over the TF ops of srfnef/cc/deform/).

Images and displacement fields are (nx, ny, nz) device tensors, displacements in voxels. The
functions default to the rules of the texture op library, which is the one srfnef's
``DeformMixin`` calls (clamped linear texture reads at position + 0.5); ``texture=False``
selects the plain library's rules (deform.cu.cc: neighbourhoods leaving the image give 0). See
csrc/deform.cu for both rules and for the FP32 interpolation weights.

``DeformMixin`` keeps the reference's method names (``_deform_tf`` ... ``_rotate_tf``) for code
written against srfnef.
"""
from __future__ import annotations

import math
from typing import Tuple

import torch

from ._lib import call, f32, i32, i32x3, ptr, stream_ptr
from .kernels import _require_cuda


def _xfast(t: torch.Tensor, name: str) -> torch.Tensor:
    _require_cuda(t, name)
    if t.dim() != 3:
        raise ValueError(f"{name} must be (nx, ny, nz)")
    return t.permute(2, 1, 0).contiguous()  # (nz, ny, nx) memory: x fastest


def _out_like(x: torch.Tensor) -> torch.Tensor:
    return torch.empty_like(x)


def deform(image: torch.Tensor, mx: torch.Tensor, my: torch.Tensor, mz: torch.Tensor, *,
           texture: bool = True) -> torch.Tensor:
    """image sampled at (i + m(i)) for every voxel i."""
    shape = list(image.shape)
    img = _xfast(image, "image")
    f = [_xfast(m, n) for m, n in ((mx, "mx"), (my, "my"), (mz, "mz"))]
    if any(list(m.shape) != list(img.shape) for m in f):
        raise ValueError("displacement fields must have the image's shape")
    out = _out_like(img)
    call("srf_deform", ptr(img), ptr(f[0]), ptr(f[1]), ptr(f[2]), i32x3(shape), i32(int(texture)),
         ptr(out), stream_ptr(img.device))
    return out.permute(2, 1, 0)


def deform_invert(mx: torch.Tensor, my: torch.Tensor, mz: torch.Tensor,
                  iterations: int = 30) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """The inverse displacement field by fixed-point iteration (30 steps, as the reference)."""
    shape = list(mx.shape)
    f = [_xfast(m, n) for m, n in ((mx, "mx"), (my, "my"), (mz, "mz"))]
    if any(m.shape != f[0].shape for m in f):
        raise ValueError("displacement fields must have one shape")
    o = [_out_like(f[0]) for _ in range(3)]
    call("srf_deform_invert", ptr(f[0]), ptr(f[1]), ptr(f[2]), i32x3(shape), i32(iterations), ptr(o[0]),
         ptr(o[1]), ptr(o[2]), stream_ptr(f[0].device))
    return tuple(t.permute(2, 1, 0) for t in o)


def shift(image: torch.Tensor, mx: float, my: float, mz: float, *, texture: bool = True) -> torch.Tensor:
    shape = list(image.shape)
    img = _xfast(image, "image")
    out = _out_like(img)
    call("srf_shift", ptr(img), f32(mx), f32(my), f32(mz), i32x3(shape), i32(int(texture)), ptr(out),
         stream_ptr(img.device))
    return out.permute(2, 1, 0)


def shift_z(image: torch.Tensor, mz: float, *, texture: bool = True) -> torch.Tensor:
    shape = list(image.shape)
    img = _xfast(image, "image")
    out = _out_like(img)
    call("srf_shift_z", ptr(img), f32(mz), i32x3(shape), i32(int(texture)), ptr(out), stream_ptr(img.device))
    return out.permute(2, 1, 0)


def rotate(image: torch.Tensor, angle: float, *, texture: bool = True) -> torch.Tensor:
    """In-plane rotation by ``angle`` (radians) about the grid centre, slice by slice."""
    shape = list(image.shape)
    img = _xfast(image, "image")
    out = _out_like(img)
    call("srf_rotate", ptr(img), f32(math.cos(angle)), f32(math.sin(angle)), i32x3(shape),
         i32(int(texture)), ptr(out), stream_ptr(img.device))
    return out.permute(2, 1, 0)


class DeformMixin:
    """srfnef's DeformMixin methods (deform_mixins.py:18-89) on device tensors."""

    def _deform_tf(self, image_data, mx, my, mz):
        return deform(image_data, mx, my, mz)

    def _deform_invert_tf(self, image_data, mx, my, mz):
        # the reference's op inverts the field and deforms the image by the inverse
        ix, iy, iz = deform_invert(mx, my, mz)
        return deform(image_data, ix, iy, iz)

    def _shift_tf(self, image_data, mx: float, my: float, mz: float):
        return shift(image_data, mx, my, mz)

    def _shift_z_tf(self, image_data, mz: float):
        return shift_z(image_data, mz)

    def _rotate_tf(self, image_data, angle: float):
        return rotate(image_data, angle)
