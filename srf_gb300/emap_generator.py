"""Sensitivity image ("emap") generation on the GPU.

``EmapGenerator(mode, scanner)(image)`` follows srfnef/functions/emap_generator.py:246-257 and
``EcatEmapGenerator`` (:25-117):

* 'block-full' / 'rsector-full' (:77-111, :114-115): sum over all ordered crystal pairs, self
  pairs included, of the non-TOF backprojection of 1. Crystal positions are built in the
  reference's order and rounding (``geometry.block_full_crystal_table``) and the pairs are
  generated on the device by ``srf_emap_block_full``: one launch instead of nb^2 host-built LOR
  arrays.
* 'full' (:32-41) is shape-broken in the reference (np.kron of an (N, 3) array with a 3N list);
  here it means the same all-pairs sum over ``EcatIndexToCrystalPos(scanner)`` positions.
* 'block' / 'rsector' rotate partial images with the deform ops (out of scope) and 'ring' is not
  implemented for ECAT scanners in the reference either: both raise NotImplementedError.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np
import torch

from . import kernels
from .data import Emap
from .functions import device, like_input
from .geometry import EcatIndexToCrystalPos, PetEcatScanner, block_full_crystal_table
from .data import _NefLike


@dataclasses.dataclass(frozen=True)
class EcatEmapGenerator(_NefLike):
    mode: Optional[str] = None
    scanner: Optional[PetEcatScanner] = None

    def __call__(self, image) -> Emap:
        shape = list(image.shape)
        center = [float(c) for c in image.center]
        size = [float(s) for s in image.size]
        if self.mode in ("block-full", "rsector-full"):
            table = block_full_crystal_table(self.scanner)
            nb = self.scanner.nb_blocks_per_ring
        elif self.mode == "full":
            table = EcatIndexToCrystalPos(self.scanner)(np.arange(self.scanner.nb_crystals))
            nb = 1
        else:
            raise NotImplementedError(f"emap mode {self.mode!r}")
        t = torch.as_tensor(table, dtype=torch.float32).to(device())
        acc = kernels.emap_block_full(t, nb, shape, center, size).contiguous()
        ref = getattr(image, "data", None)
        return Emap(like_input(acc, ref if ref is not None else np.zeros(0), "tf-eager"),
                    center, size)


@dataclasses.dataclass(frozen=True)
class EmapGenerator(_NefLike):
    mode: Optional[str] = None
    scanner: Optional[PetEcatScanner] = None

    def __call__(self, *args, **kwargs) -> Emap:
        if isinstance(self.scanner, PetEcatScanner):
            return EcatEmapGenerator(self.mode, self.scanner)(*args, **kwargs)
        raise NotImplementedError("only PetEcatScanner geometries are supported")
