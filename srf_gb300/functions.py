"""srfnef's projector function classes over the sm_103a kernels.

* ``Project(mode)(image, lors) -> Listmode``            srfnef/functions/project.py:21-40
* ``BackProject(mode)(listmode, image) -> Image``        srfnef/functions/back_project.py:22-49
* ``ProjectTof(mode, tof)(image, lors) -> Listmode``     srfnef/functions/project_tof.py:22-47
* ``BackProjectTof(mode, tof)(listmode, image) -> Image`` srfnef/functions/back_project_tof.py:21-52

``mode`` is 'tf-eager' (results come back as the caller's array type: numpy in, numpy out) or 'tf'
(results stay on the GPU as torch tensors), as in the reference; other modes raise
``NotImplementedError``. Images are (nx, ny, nz) as srfnef's ``Image.data``; the reference's
device-side transposes are replaced by strided views. The backprojection output has the shape
of the given image and is zero-initialised (the op's memset), ignoring the image's values.

``tof_nsigma`` (default 0 = the reference's untruncated Gaussian) is an optional extra field of
the TOF classes.
"""
from __future__ import annotations

import dataclasses
from typing import Any, Optional

import numpy as np
import torch

from . import kernels
from .data import Image, Listmode, Lors, _NefLike
from .geometry import TofConfig

_MODES = ("tf", "tf-eager")


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("srf_gb300 needs a CUDA device (there is no CPU path)")
    return torch.device("cuda", torch.cuda.current_device())


def to_dev(a, dtype=torch.float32) -> torch.Tensor:
    """The array on the current CUDA device. A pinned host tensor is copied asynchronously in
    stream order (the caller keeps it unchanged until the stream has passed the copy)."""
    if isinstance(a, torch.Tensor):
        pinned = a.device.type == "cpu" and a.is_pinned()
        return a.to(device=device(), dtype=dtype, non_blocking=pinned)
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).to(device())


_COPY_STREAMS: "dict" = {}


def to_dev_overlapped(a, dtype=torch.float32) -> torch.Tensor:
    """Like ``to_dev``, but a pinned host tensor travels on a side stream of its own: the current
    stream waits for the copy only, so the copy overlaps device work already queued (a previous
    reconstruction's kernels) instead of queueing behind it."""
    if not (isinstance(a, torch.Tensor) and a.device.type == "cpu" and a.is_pinned()):
        return to_dev(a, dtype)
    dev = device()
    side = _COPY_STREAMS.get(dev.index)
    if side is None:
        side = _COPY_STREAMS[dev.index] = torch.cuda.Stream(dev)
    main = torch.cuda.current_stream(dev)
    with torch.cuda.stream(side):
        t = a.to(device=dev, dtype=dtype, non_blocking=True)
    done = torch.cuda.Event()
    done.record(side)
    main.wait_event(done)
    t.record_stream(main)  # the allocator keeps the block until main is past its uses
    return t


def like_input(t: torch.Tensor, ref, mode: str):
    """'tf-eager' returns the caller's array type; 'tf' keeps device tensors."""
    if mode == "tf-eager" and not isinstance(ref, torch.Tensor):
        return t.detach().cpu().numpy()
    return t


def _mode_ok(mode: str) -> None:
    if mode not in _MODES:
        raise NotImplementedError(f"mode {mode!r} (supported: {_MODES})")


def _lors_dev(lors: Lors, need_tof: bool) -> torch.Tensor:
    t = to_dev(lors.data)
    if t.dim() != 2 or t.shape[1] < (7 if need_tof else 6):
        raise ValueError(f"Lors.data must be (N, {'7' if need_tof else '6 or 7'})")
    return t.contiguous()


def _geom(image):
    return list(image.shape), [float(c) for c in image.center], [float(s) for s in image.size]


@dataclasses.dataclass(frozen=True)
class Project(_NefLike):
    mode: Optional[str] = None

    def __call__(self, image: Image, lors: Lors) -> Listmode:
        _mode_ok(self.mode)
        shape, center, size = _geom(image)
        p = kernels.project(_lors_dev(lors, False), to_dev(image.data), center, size)
        return Listmode(like_input(p, image.data, self.mode), lors)


@dataclasses.dataclass(frozen=True)
class BackProject(_NefLike):
    mode: Optional[str] = None

    def __call__(self, listmode: Listmode, image: Image) -> Image:
        _mode_ok(self.mode)
        shape, center, size = _geom(image)
        bp = kernels.backproject(_lors_dev(listmode.lors, False), to_dev(listmode.data), shape,
                                 center, size)
        return image.update(data=like_input(bp.contiguous(), image.data, self.mode))


@dataclasses.dataclass(frozen=True)
class ProjectTof(_NefLike):
    mode: Optional[str] = None
    tof: Optional[TofConfig] = None
    tof_nsigma: float = 0.0

    def __call__(self, image: Image, lors: Lors) -> Listmode:
        _mode_ok(self.mode)
        shape, center, size = _geom(image)
        p = kernels.project(_lors_dev(lors, True), to_dev(image.data), center, size,
                            tof=(self.tof.tof_bin, self.tof.tof_sigma2), tof_nsigma=self.tof_nsigma)
        return Listmode(like_input(p, image.data, self.mode), lors)


@dataclasses.dataclass(frozen=True)
class BackProjectTof(_NefLike):
    mode: Optional[str] = None
    tof: Optional[TofConfig] = None
    tof_nsigma: float = 0.0

    def __call__(self, listmode: Listmode, image: Image) -> Image:
        _mode_ok(self.mode)
        shape, center, size = _geom(image)
        bp = kernels.backproject(_lors_dev(listmode.lors, True), to_dev(listmode.data), shape,
                                 center, size, tof=(self.tof.tof_bin, self.tof.tof_sigma2),
                                 tof_nsigma=self.tof_nsigma)
        return image.update(data=like_input(bp.contiguous(), image.data, self.mode))
