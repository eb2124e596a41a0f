"""Scanner geometry with srfnef's fields, index conventions and rounding.

* ``Block``, ``TofConfig``, ``ImageConfig``, ``PetEcatScanner``: srfnef/geometry/block.py:14-22,
  tof_config.py:14-17, image_config.py:14-22, pet_ecat_scanner.py:17-25; derived properties from
  srfnef/ops/geometry/pet_ecat_scanner.py:13-45.
* ``EcatCrystalPosToIndex`` / ``EcatIndexToCrystalPos``: srfnef/functions/geometry/
  pet_ecat_scanner.py:15-89. Crystal index = iy + iz*shape[1] + iblock*per_block + iring*per_ring.
* ``PetEcatListmodeTrans``: snap LOR endpoints to crystal centres, keeping the TOF column
  (srfnef/functions/data_transform/pet_ecat.py:43-60).
* ``LorsToListmode``: unit values (srfnef/functions/lors_to_listmode.py:15-19).

These run on the host in numpy (float64 arithmetic, float32 results), as the reference does.
"""
from __future__ import annotations

import dataclasses
from math import pi
from typing import List, Optional

import numpy as np

from .data import Listmode, Lors, _NefLike


@dataclasses.dataclass(frozen=True)
class Block(_NefLike):
    size: Optional[List[float]] = None
    shape: Optional[List[int]] = None
    interval: Optional[List[float]] = None

    def __post_init__(self):
        if self.interval is None:
            object.__setattr__(self, "interval", [0, 0, 0])

    @property
    def unit_size(self) -> List[float]:
        return [s1 / s2 for s1, s2 in zip(self.size, self.shape)]


@dataclasses.dataclass(frozen=True)
class TofConfig(_NefLike):
    tof_bin: float = 3.66
    tof_sigma2: float = 1000


@dataclasses.dataclass(frozen=True)
class ImageConfig(_NefLike):
    shape: Optional[List[int]] = None
    center: Optional[List[float]] = None
    size: Optional[List[float]] = None

    @property
    def unit_size(self) -> List[float]:
        return [s1 / s2 for s1, s2 in zip(self.size, self.shape)]


@dataclasses.dataclass(frozen=True)
class PetEcatScanner(_NefLike):
    inner_radius: Optional[float] = None
    outer_radius: Optional[float] = None
    nb_rings: Optional[int] = None
    nb_blocks_per_ring: Optional[int] = None
    gap: Optional[float] = None
    blocks: Optional[Block] = None
    tof: Optional[TofConfig] = None

    @property
    def average_radius(self) -> float:
        return (self.inner_radius + self.outer_radius) / 2

    @property
    def axial_length(self) -> float:
        return self.blocks.size[2] * self.nb_rings + self.gap * (self.nb_rings - 1)

    @property
    def nb_crystals_per_block(self) -> int:
        return self.blocks.shape[1] * self.blocks.shape[2]

    @property
    def nb_crystals_per_ring(self) -> int:
        return self.nb_crystals_per_block * self.nb_blocks_per_ring

    @property
    def nb_crystals(self) -> int:
        return self.nb_crystals_per_ring * self.nb_rings

    @property
    def angle_per_block(self) -> float:
        return 2 * pi / self.nb_blocks_per_ring


@dataclasses.dataclass(frozen=True)
class EcatCrystalPosToIndex(_NefLike):
    scanner: Optional[PetEcatScanner] = None

    def __call__(self, pos: np.ndarray, verbose: bool = False):
        if len(pos.shape) == 1:
            pos = pos.reshape((1, pos.size))
        s = self.scanner
        xc, yc, zc = pos[:, 0], pos[:, 1], pos[:, 2]
        iblock = np.round(np.arctan2(yc, xc) / s.angle_per_block).astype(int) % s.nb_blocks_per_ring
        iring = np.floor((zc + s.axial_length / 2) / (s.gap + s.blocks.size[2])).astype(int)
        angle = iblock * s.angle_per_block
        y_corr = -xc * np.sin(angle) + yc * np.cos(angle) + s.blocks.size[1] / 2
        iy = np.round(y_corr / s.blocks.unit_size[1] - 0.5).astype(int)
        z_corr = zc + s.axial_length / 2 - iring * (s.blocks.size[2] + s.gap)
        iz = np.round(z_corr / s.blocks.unit_size[2] - 0.5).astype(int)
        if verbose:
            return iy, iz, iblock, iring
        return iy + iz * s.blocks.shape[1] + iblock * s.nb_crystals_per_block \
            + iring * s.nb_crystals_per_ring


@dataclasses.dataclass(frozen=True)
class EcatIndexToCrystalPos(_NefLike):
    scanner: Optional[PetEcatScanner] = None

    def __call__(self, ind, verbose: bool = False) -> np.ndarray:
        s = self.scanner
        if verbose:
            iy, iz, iblock, iring = ind
        else:
            ind = np.asarray(ind)
            iy = ind % s.blocks.shape[1]
            iz = (ind // s.blocks.shape[1]) % s.blocks.shape[2]
            iblock = (ind // s.blocks.shape[1] // s.blocks.shape[2]) % s.nb_blocks_per_ring
            iring = ind // s.blocks.shape[1] // s.blocks.shape[2] // s.nb_blocks_per_ring
        pos = np.zeros((np.asarray(iy).size, 3), dtype=np.float32)
        x0 = s.average_radius
        y0 = (iy + 0.5) * s.blocks.unit_size[1] - s.blocks.size[1] / 2
        theta = s.angle_per_block * iblock
        pos[:, 0] = x0 * np.cos(theta) - y0 * np.sin(theta)
        pos[:, 1] = x0 * np.sin(theta) + y0 * np.cos(theta)
        pos[:, 2] = (iz + 0.5) * s.blocks.unit_size[2] + iring * (s.gap + s.blocks.size[2]) \
            - s.axial_length / 2
        return pos


@dataclasses.dataclass(frozen=True)
class PetEcatListmodeTrans(_NefLike):
    scanner: Optional[PetEcatScanner] = None

    def __call__(self, listmode: Listmode) -> Listmode:
        try:
            import torch
            on_gpu = isinstance(listmode.lors.data, torch.Tensor) and listmode.lors.data.is_cuda
        except ImportError:  # pragma: no cover
            on_gpu = False
        if on_gpu:  # one GPU pass (srf_listmode_snap)
            from . import kernels
            return listmode.update(lors=Lors(kernels.snap(listmode.lors.data.contiguous(), self.scanner)))
        lors = np.asarray(listmode.lors.data)
        ind1 = EcatCrystalPosToIndex(self.scanner)(lors[:, :3])
        ind2 = EcatCrystalPosToIndex(self.scanner)(lors[:, 3:6])
        pos1 = EcatIndexToCrystalPos(self.scanner)(ind1)
        pos2 = EcatIndexToCrystalPos(self.scanner)(ind2)
        if lors.shape[1] == 6:
            new = np.hstack((pos1, pos2)).astype(np.float32)
        else:
            new = np.hstack((pos1, pos2, lors[:, -1].reshape(-1, 1))).astype(np.float32)
        return listmode.update(lors=Lors(new))


@dataclasses.dataclass(frozen=True)
class LorsToListmode(_NefLike):
    def __call__(self, lors: Lors) -> Listmode:
        return Listmode(np.ones((lors.shape[0],), dtype=np.float32), lors)


def block_full_crystal_table(scanner: PetEcatScanner) -> np.ndarray:
    """Crystal centres in the order and rounding of srfnef's 'block-full' sensitivity generator.

    ``EcatEmapGenerator('block-full')`` (srfnef/functions/emap_generator.py:77-111) takes the
    crystals of block 0 over all rings from a one-block scanner as float32, then rotates them by
    ``i * angle_per_block`` in float64 and rounds the LOR array to float32. Row
    ``i * M + m`` of the returned (nb_blocks * M, 3) float32 table is crystal ``m`` of block column
    ``i``, M = crystals per block * rings; endpoint pairs (row r, row s) over all r, s are exactly
    the LORs the reference backprojects.
    """
    single = scanner.update(nb_blocks_per_ring=1)
    m = scanner.nb_crystals_per_block * scanner.nb_rings
    pos = EcatIndexToCrystalPos(single)(np.arange(m))
    out = np.empty((scanner.nb_blocks_per_ring * m, 3), dtype=np.float32)
    px = pos[:, 0].astype(np.float64)
    py = pos[:, 1].astype(np.float64)
    for i in range(scanner.nb_blocks_per_ring):
        a = i * scanner.angle_per_block
        out[i * m:(i + 1) * m, 0] = (px * np.cos(a) - py * np.sin(a)).astype(np.float32)
        out[i * m:(i + 1) * m, 1] = (px * np.sin(a) + py * np.cos(a)).astype(np.float32)
        out[i * m:(i + 1) * m, 2] = pos[:, 2]
    return out
