"""Tensor-level entry points over the C ABI (device tensors in, device tensors out).

Layouts: images are handled as (nx, ny, nz) tensors of any strides. For speed the projector is
given an x-fastest view (memory order z, y, x; strides (1, nx, nx*ny)) for x-dominant LORs and a
y-fastest copy (memory order z, x, y) for y-dominant ones, so that the lanes of a LOR group touch
consecutive addresses; backprojections accumulate into the same two layouts and are folded once.
LORs are (N, >= 6) float32 rows with unit column stride; TOF values come from column 6.
"""
from __future__ import annotations

from typing import Optional, Sequence, Tuple

import torch

from . import _lib
from ._lib import call, f32, f32x3, i32, i32x3, i64, i64x3, ptr, stream_ptr

F32 = torch.float32


def _require_cuda(t: torch.Tensor, name: str) -> None:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (srf_gb300 has no CPU path)")
    if t.dtype != F32:
        raise ValueError(f"{name} must be float32")


def check_lors(lors: torch.Tensor, tof: bool) -> Tuple[int, int]:
    _require_cuda(lors, "lors")
    if lors.dim() != 2 or lors.shape[1] < (7 if tof else 6):
        raise ValueError(f"lors must be (N, {'>=7' if tof else '>=6'}), got {tuple(lors.shape)}")
    if lors.stride(1) != 1 or lors.stride(0) < lors.shape[1]:
        raise ValueError("lors rows must be contiguous")
    return lors.shape[0], lors.stride(0)


def _tof_ptr(lors: torch.Tensor):
    return _lib.ctypes.c_void_p(lors.data_ptr() + 6 * 4)


def xfast(img: torch.Tensor) -> torch.Tensor:
    """(nx, ny, nz) view whose memory is x-fastest (a copy unless it already is)."""
    return img.permute(2, 1, 0).contiguous().permute(2, 1, 0)


def yfast(img: torch.Tensor) -> torch.Tensor:
    """(nx, ny, nz) view whose memory is y-fastest."""
    return img.permute(2, 0, 1).contiguous().permute(1, 2, 0)


def new_xfast(shape: Sequence[int], device) -> torch.Tensor:
    nx, ny, nz = shape
    return torch.zeros((nz, ny, nx), dtype=F32, device=device).permute(2, 1, 0)


def new_yfast(shape: Sequence[int], device) -> torch.Tensor:
    nx, ny, nz = shape
    return torch.zeros((nz, nx, ny), dtype=F32, device=device).permute(1, 2, 0)


def _tof_args(tof_bin, tof_sigma2, nsigma):
    return f32(tof_bin), f32(tof_sigma2), f32(nsigma)


def project(lors: torch.Tensor, image: torch.Tensor, center, size, *, tof: Optional[Tuple[float, float]] = None,
            tof_nsigma: float = 0.0, image_t: Optional[torch.Tensor] = None,
            out: Optional[torch.Tensor] = None, make_t: bool = True) -> torch.Tensor:
    """p = A image for every LOR; tof = (tof_bin, tof_sigma2) selects the TOF projector."""
    n, stride = check_lors(lors, tof is not None)
    _require_cuda(image, "image")
    shape = list(image.shape)
    if image.stride(0) != 1:
        image = xfast(image)
    if image_t is None and make_t:
        image_t = yfast(image)
    if out is None:
        out = torch.empty(n, dtype=F32, device=lors.device)
    st = i64x3(image.stride())
    t_args = (ptr(image_t), i64x3(image_t.stride())) if image_t is not None else (None, None)
    s = stream_ptr(lors.device)
    if tof is None:
        call("srf_projection", ptr(lors), i64(n), i32(stride), ptr(image), st, *t_args,
             i32x3(shape), f32x3(center), f32x3(size), ptr(out), s)
    else:
        call("srf_projection_tof", ptr(lors), i64(n), i32(stride), _tof_ptr(lors), i32(stride),
             *_tof_args(tof[0], tof[1], tof_nsigma), ptr(image), st, *t_args,
             i32x3(shape), f32x3(center), f32x3(size), ptr(out), s)
    return out


def backproject(lors: torch.Tensor, values: torch.Tensor, shape, center, size, *,
                tof: Optional[Tuple[float, float]] = None, tof_nsigma: float = 0.0,
                adjoint: bool = False, use_t: bool = True) -> torch.Tensor:
    """A_bp^T values as an x-fastest (nx, ny, nz) tensor (adjoint=True: exact adjoint of
    ``project``)."""
    n, stride = check_lors(lors, tof is not None)
    _require_cuda(values, "values")
    values = values.contiguous()
    if values.numel() != n:
        raise ValueError("values must have one entry per LOR")
    acc = new_xfast(shape, lors.device)
    acc_t = new_yfast(shape, lors.device) if use_t else None
    st = i64x3(acc.stride())
    t_args = (ptr(acc_t), i64x3(acc_t.stride())) if acc_t is not None else (None, None)
    s = stream_ptr(lors.device)
    if adjoint:
        tof_p = _tof_ptr(lors) if tof is not None else None
        tb, ts = tof if tof is not None else (0.0, 0.0)
        call("srf_projection_adjoint", ptr(lors), i64(n), i32(stride), tof_p, i32(stride),
             *_tof_args(tb, ts, tof_nsigma), ptr(values), ptr(acc), st, *t_args,
             i32x3(shape), f32x3(center), f32x3(size), s)
    elif tof is None:
        call("srf_backprojection", ptr(lors), i64(n), i32(stride), ptr(values), ptr(acc), st,
             *t_args, i32x3(shape), f32x3(center), f32x3(size), s)
    else:
        call("srf_backprojection_tof", ptr(lors), i64(n), i32(stride), _tof_ptr(lors), i32(stride),
             *_tof_args(tof[0], tof[1], tof_nsigma), ptr(values), ptr(acc), st, *t_args,
             i32x3(shape), f32x3(center), f32x3(size), s)
    if acc_t is not None:
        fold(acc, acc_t)
    return acc


MAX_BATCH = 8


def project_batch(lors: torch.Tensor, images: torch.Tensor, center, size, *,
                  tof: Optional[Tuple[float, float]] = None, tof_nsigma: float = 0.0) -> torch.Tensor:
    """(B, N) projections of a batch of (nx, ny, nz) images (B <= 8), one traversal per LOR."""
    n, stride = check_lors(lors, tof is not None)
    _require_cuda(images, "images")
    if images.dim() != 4 or not 1 <= images.shape[0] <= MAX_BATCH:
        raise ValueError(f"images must be (B <= {MAX_BATCH}, nx, ny, nz)")
    B, nx, ny, nz = images.shape
    xb = images.permute(0, 3, 2, 1).contiguous()             # (B, nz, ny, nx): x fastest
    yb = images.permute(0, 3, 1, 2).contiguous()             # (B, nz, nx, ny): y fastest
    out = torch.empty((B, n), dtype=F32, device=lors.device)
    tof_p = _tof_ptr(lors) if tof is not None else None
    tb, tsg = tof if tof is not None else (0.0, 0.0)
    call("srf_projection_batch", ptr(lors), i64(n), i32(stride), tof_p, i32(stride),
         *_tof_args(tb, tsg, tof_nsigma), i32(B), i64(nx * ny * nz), ptr(xb), i64x3((1, nx, nx * ny)),
         ptr(yb), i64x3((ny, 1, nx * ny)), i32x3((nx, ny, nz)), f32x3(center), f32x3(size), ptr(out),
         i64(n), stream_ptr(lors.device))
    return out


def adjoint_batch(lors: torch.Tensor, values: torch.Tensor, shape, center, size, *,
                  tof: Optional[Tuple[float, float]] = None, tof_nsigma: float = 0.0) -> torch.Tensor:
    """(B, nx, ny, nz) exact adjoint of ``project_batch`` for (B, N) LOR values."""
    n, stride = check_lors(lors, tof is not None)
    _require_cuda(values, "values")
    values = values.contiguous()
    if values.dim() != 2 or values.shape[1] != n or not 1 <= values.shape[0] <= MAX_BATCH:
        raise ValueError(f"values must be (B <= {MAX_BATCH}, N)")
    B = values.shape[0]
    nx, ny, nz = shape
    acc = torch.zeros((B, nz, ny, nx), dtype=F32, device=lors.device)
    acc_t = torch.zeros((B, nz, nx, ny), dtype=F32, device=lors.device)
    tof_p = _tof_ptr(lors) if tof is not None else None
    tb, tsg = tof if tof is not None else (0.0, 0.0)
    call("srf_projection_adjoint_batch", ptr(lors), i64(n), i32(stride), tof_p, i32(stride),
         *_tof_args(tb, tsg, tof_nsigma), i32(B), ptr(values), i64(n), ptr(acc), i64(nx * ny * nz),
         i64x3((1, nx, nx * ny)), ptr(acc_t), i64x3((ny, 1, nx * ny)), i32x3(shape), f32x3(center),
         f32x3(size), stream_ptr(lors.device))
    out = acc.permute(0, 3, 2, 1)                             # (B, nx, ny, nz) views, x fastest
    for b in range(B):
        fold(out[b], acc_t[b].permute(1, 2, 0))
    return out


def count_pairs(lors: torch.Tensor, shape, center, size, *, rules: int,
                tof: Optional[Tuple[float, float]] = None, tof_nsigma: float = 0.0) -> int:
    """Exact number of (LOR, voxel) visits of the projector (rules=0) or backprojector (1)."""
    n, stride = check_lors(lors, tof is not None)
    cnt = torch.zeros(1, dtype=torch.int64, device=lors.device)
    tof_p = _tof_ptr(lors) if tof is not None else None
    tb, ts = tof if tof is not None else (0.0, 0.0)
    call("srf_count_pairs", ptr(lors), i64(n), i32(stride), tof_p, i32(stride),
         *_tof_args(tb, ts, tof_nsigma), i32(rules), i32x3(shape), f32x3(center), f32x3(size),
         ptr(cnt), stream_ptr(lors.device))
    return int(cnt.item())


def fold(dst: torch.Tensor, src: torch.Tensor) -> None:
    call("srf_fold_views", ptr(dst), i64x3(dst.stride()), ptr(src), i64x3(src.stride()),
         i32x3(dst.shape), stream_ptr(dst.device))


def copy_view(dst: torch.Tensor, src: torch.Tensor) -> None:
    call("srf_copy_view", ptr(dst), i64x3(dst.stride()), ptr(src), i64x3(src.stride()),
         i32x3(dst.shape), stream_ptr(dst.device))


class SubsetState:
    """Device state of a list-mode MLEM/OSEM reconstruction: x (x-fastest) and its y-fastest copy,
    two backprojection accumulators and an FP64 log-likelihood accumulator."""

    def __init__(self, shape, center, size, device, x0: Optional[torch.Tensor] = None):
        self.shape, self.center, self.size = list(shape), list(center), list(size)
        self.x = new_xfast(shape, device)
        if x0 is None:
            self.x.fill_(1.0)
        else:
            self.x.copy_(x0)
        self.x_t = yfast(self.x)
        # both backprojection accumulators in one flat buffer (one collective sums both)
        nx, ny, nz = self.shape
        v = nx * ny * nz
        self._acc = torch.zeros(2 * v, dtype=F32, device=device)
        self.bp = self._acc[:v].view(nz, ny, nx).permute(2, 1, 0)
        self.bp_t = self._acc[v:].view(nz, nx, ny).permute(1, 2, 0)
        self.loglik = torch.zeros(1, dtype=torch.float64, device=device)

    def accumulators(self) -> torch.Tensor:
        """The flat buffer holding both backprojection accumulators (what an event-sharded
        reconstruction sums over its ranks before the update)."""
        return self._acc

    def subset(self, lors: torch.Tensor, y: Optional[torch.Tensor], *, rule: int, eps: float,
               tof: Optional[Tuple[float, float]] = None, tof_nsigma: float = 0.0,
               track_loglik: bool = False, add: Optional[torch.Tensor] = None) -> None:
        n, stride = check_lors(lors, tof is not None)
        if y is not None:
            _require_cuda(y, "y")
        tof_p = _tof_ptr(lors) if tof is not None else None
        tb, ts = tof if tof is not None else (0.0, 0.0)
        call("srf_osem_subset", ptr(lors), i64(n), i32(stride), tof_p, i32(stride),
             *_tof_args(tb, ts, tof_nsigma), ptr(y), ptr(add), i32(rule), f32(eps), ptr(self.x),
             ptr(self.x_t), ptr(self.bp), ptr(self.bp_t), i32x3(self.shape),
             f32x3(self.center), f32x3(self.size), ptr(self.loglik) if track_loglik else None,
             stream_ptr(lors.device))

    def update(self, emap_xfast: torch.Tensor, guard_zero: bool) -> None:
        call("srf_osem_update", ptr(self.x), ptr(self.x_t), ptr(self.bp), ptr(self.bp_t),
             ptr(emap_xfast), i32(1 if guard_zero else 0), i32x3(self.shape),
             stream_ptr(self.x.device))


def emap_block_full(table: torch.Tensor, n_blocks: int, shape, center, size) -> torch.Tensor:
    _require_cuda(table, "crystal table")
    m = table.shape[0] // n_blocks
    acc = new_xfast(shape, table.device)
    acc_t = new_yfast(shape, table.device)
    call("srf_emap_block_full", ptr(table), i32(n_blocks), i32(m), ptr(acc), i64x3(acc.stride()),
         ptr(acc_t), i64x3(acc_t.stride()), i32x3(shape), f32x3(center), f32x3(size),
         stream_ptr(table.device))
    fold(acc, acc_t)
    return acc


def sss(pairs: torch.Tensor, crystal_pos: torch.Tensor, scatter_pos: torch.Tensor,
        sumup_emission: torch.Tensor, atten: torch.Tensor, umap: torch.Tensor, umap_size,
        nb_crystals_per_ring: int, nb_blocks_per_ring: int, grid_block, low_energy: int,
        high_energy: int, resolution: float) -> Tuple[torch.Tensor, torch.Tensor]:
    dev = pairs.device
    n = pairs.shape[0]
    scatter = torch.empty(n, dtype=F32, device=dev)
    scale = torch.empty(n, dtype=F32, device=dev)
    umap = umap.contiguous()
    call("srf_sss", ptr(pairs.contiguous()), i64(n), ptr(crystal_pos.contiguous()),
         i32(crystal_pos.shape[0]), ptr(scatter_pos.contiguous()), i32(scatter_pos.shape[0]),
         ptr(sumup_emission.contiguous()), ptr(atten.contiguous()), ptr(umap),
         i32x3(umap.shape), f32x3(umap_size), i32(nb_crystals_per_ring), i32(nb_blocks_per_ring),
         i32x3(grid_block), i32(low_energy), i32(high_energy), f32(resolution), ptr(scatter),
         ptr(scale), stream_ptr(dev))
    return scatter, scale


# ---------------------------------------------------------------- list-mode ingestion

def scanner_args(scanner):
    """(double[8], int64[4]) description of a PetEcatScanner for the list-mode kernels."""
    import ctypes
    b = scanner.blocks
    d = (ctypes.c_double * 8)(scanner.average_radius, scanner.angle_per_block, scanner.axial_length,
                              scanner.gap, b.size[1], b.size[2], b.unit_size[1], b.unit_size[2])
    s = (ctypes.c_int64 * 4)(int(b.shape[1]), int(b.shape[2]), int(scanner.nb_blocks_per_ring),
                             int(scanner.nb_rings))
    return d, s


def snap(lors: torch.Tensor, scanner, want_ids: bool = False, out: Optional[torch.Tensor] = None):
    """Endpoints snapped to crystal centres (columns 6 .. out's width - 1 kept); optionally the
    crystal ids. ``out`` (N, >= 6) float32 rows with unit column stride, default like ``lors``."""
    _require_cuda(lors, "lors")
    n, stride = lors.shape[0], lors.stride(0)
    if lors.dim() != 2 or lors.shape[1] < 6 or lors.stride(1) != 1:
        raise ValueError("lors must be (N, >= 6) rows with unit column stride")
    if out is None:
        out = torch.empty_like(lors)
    else:
        _require_cuda(out, "out")
        if out.dim() != 2 or out.shape[0] != n or out.shape[1] < 6 or out.stride(1) != 1 \
                or out.stride(0) < out.shape[1] or out.device != lors.device:
            raise ValueError("out must be (N, >= 6) rows with unit column stride on the LORs' device")
    ids = torch.empty((n, 2), dtype=torch.int64, device=lors.device) if want_ids else None
    d, s = scanner_args(scanner)
    call("srf_listmode_snap", ptr(lors), i64(n), i32(stride), d, s, ptr(out), i32(out.stride(0)),
         ptr(ids), stream_ptr(lors.device))
    return (out, ids) if want_ids else out


def lm2sino(lors: torch.Tensor, values: Optional[torch.Tensor], scanner) -> Tuple[torch.Tensor, int]:
    """Triangular crystal-pair sinogram (float64, n(n-1)/2 bins) and the number of dropped events."""
    _require_cuda(lors, "lors")
    nc = scanner.nb_crystals
    sino = torch.zeros(nc * (nc - 1) // 2, dtype=torch.float64, device=lors.device)
    dropped = torch.zeros(1, dtype=torch.int64, device=lors.device)
    d, s = scanner_args(scanner)
    call("srf_lm2sino", ptr(lors), i64(lors.shape[0]), i32(lors.stride(0)),
         ptr(values.contiguous() if values is not None else None), d, s, ptr(sino), i64(sino.numel()),
         ptr(dropped), stream_ptr(lors.device))
    return sino, int(dropped.item())


def attenuation(lors: torch.Tensor, umap: torch.Tensor, center, size,
                values: Optional[torch.Tensor] = None) -> torch.Tensor:
    """exp(-(P mu) L^2 / unit) per LOR, or values / that (AttenuationCorrect) when values given."""
    n, stride = check_lors(lors, False)
    _require_cuda(umap, "umap")
    if umap.stride(0) != 1:
        umap = xfast(umap)
    out = torch.empty(n, dtype=F32, device=lors.device)
    call("srf_attenuation", ptr(lors), i64(n), i32(stride), ptr(umap), i64x3(umap.stride()),
         i32x3(umap.shape), f32x3(center), f32x3(size),
         ptr(values.contiguous() if values is not None else None), ptr(out), stream_ptr(lors.device))
    return out
