"""Attenuation and single-scatter correction around the GPU kernels.

Mirrors srfnef's corrections:

* ``UmapProject()(u_map, lors) -> Listmode``  exp(-(P mu) L^2 / unit_size[0])
  (srfnef/corrections/attenuation/attenuation_correct.py:31-40); the projection is the non-TOF
  Siddon projector, whose weights carry 1/L^2, hence the L^2.
* ``AttenuationCorrect(u_map)(listmode)``      listmode / exp(-...)   (attenuation_correct.py:16-28)
* sinogram formats (srfnef/corrections/scattering/listmode2sinogram.py:17-99):
  ``get_all_lors_id`` (all pairs i > j, row-major), ``lm2sino`` (triangular bin i(i-1)/2 + j
  after ordering each pair so that i > j, float64 weights), ``sino2lm`` (bins with
  0 < value < 1e8 back to LORs).
* ``scatter_preprocess`` (srfnef/corrections/scattering/scatter.py:57-73, preprocess.py:6-75):
  scatter points every floor(50 mm / voxel) voxels, crystal positions, emission and attenuation
  line integrals crystal -> scatter point through the GPU projector, attenuation of the measured
  pairs with mu x 1.3. Returns the eight arrays the reference saves with np.save (and saves them
  too when ``outdir`` is given).
* ``ScatterCorrect(low_energy, high_energy, resolution, scatter_fraction)``
  (srfnef/corrections/scattering/scatter.py:18-55): raw SSS sums and scales from ``srf_sss``,
  the host scaling of scatter_fraction.py:27-36 and the corrected sinogram
  (sino - f/sum(f) * sum(sino) * SF) * scale / (atten_lors + DBL_MIN), returned as list mode.

The per-pair SSS arithmetic runs on the GPU (srf_gb300/csrc/sss.cu); host steps are float64
numpy as in the reference.
"""
from __future__ import annotations

import dataclasses
import math
import os
import sys
from typing import Any, Optional

import numpy as np
import torch

from . import kernels
from .data import Image, Listmode, Lors, Umap, _NefLike
from .functions import Project, device, to_dev
from .geometry import EcatCrystalPosToIndex, EcatIndexToCrystalPos, PetEcatScanner


# ------------------------------------------------------------------ attenuation

def _lor_lengths(lors: np.ndarray) -> np.ndarray:
    dx = lors[:, 0] - lors[:, 3]
    dy = lors[:, 1] - lors[:, 4]
    dz = lors[:, 2] - lors[:, 5]
    return np.sqrt(dx ** 2 + dy ** 2 + dz ** 2)


def _back(t: torch.Tensor, like):
    return t if isinstance(like, torch.Tensor) else t.cpu().numpy()


@dataclasses.dataclass(frozen=True)
class UmapProject(_NefLike):
    """One fused GPU pass (srf_attenuation): projection of mu and exp(-p L^2 / unit)."""

    def __call__(self, u_map: Image, lors: Lors) -> Listmode:
        lt = to_dev(lors.data).contiguous()
        a = kernels.attenuation(lt, to_dev(u_map.data), list(u_map.center), list(u_map.size))
        return Listmode(_back(a, lors.data), lors)


@dataclasses.dataclass(frozen=True)
class AttenuationCorrect(_NefLike):
    u_map: Optional[Umap] = None

    def __call__(self, listmode: Listmode) -> Listmode:
        lt = to_dev(listmode.lors.data).contiguous()
        y = kernels.attenuation(lt, to_dev(self.u_map.data), list(self.u_map.center),
                                list(self.u_map.size), values=to_dev(listmode.data))
        return listmode.update(data=_back(y, listmode.data))


# ------------------------------------------------------------------ sinogram formats

def get_all_lors_id(total_num_crystal: int) -> np.ndarray:
    """All crystal pairs (i, j) with i > j, ordered by i then j (listmode2sinogram.py:26-35)."""
    n = int(total_num_crystal)
    i = np.repeat(np.arange(n, dtype=np.int64), np.arange(n, dtype=np.int64))
    start = i * (i - 1) // 2
    j = np.arange(i.size, dtype=np.int64) - start
    return np.stack([i, j], 1).astype(np.int32)


def lm2sino(listmode: Listmode, scanner: PetEcatScanner) -> np.ndarray:
    """Histogram list mode into the triangular pair sinogram (listmode2sinogram.py:76-85, :17-23)."""
    lors = np.asarray(listmode.lors.data)
    id1 = EcatCrystalPosToIndex(scanner)(lors[:, :3]).astype(np.int64)
    id2 = EcatCrystalPosToIndex(scanner)(lors[:, 3:6]).astype(np.int64)
    hi = np.maximum(id1, id2)
    lo = np.minimum(id1, id2)
    pos = (hi - 1) * hi // 2 + lo
    n = scanner.nb_crystals
    w = np.zeros((n * (n - 1) // 2, 1))
    np.add.at(w[:, 0], pos, np.asarray(listmode.data, dtype=np.float64))
    return w


def sino2lm(scanner: PetEcatScanner, sinogram: np.ndarray, lors: np.ndarray) -> np.ndarray:
    """Bins with 0 < value < 1e8 as (x1 y1 z1 x2 y2 z2 value) rows (listmode2sinogram.py:88-99)."""
    s = np.asarray(sinogram).reshape(-1)
    index = np.where((s > 0) & (s < 1e8))[0]
    out = np.zeros((len(index), 6))
    out[:, :3] = EcatIndexToCrystalPos(scanner)(lors[index, 0])
    out[:, 3:6] = EcatIndexToCrystalPos(scanner)(lors[index, 1])
    return np.hstack((out, s[index].reshape(-1, 1)))


# ------------------------------------------------------------------ preprocess

def pre_all_scatter_position(emission_image: Image) -> np.ndarray:
    """Scatter points every floor(50 mm / voxel) voxels, at block centres (preprocess.py:6-18, 57-61)."""
    size_voxel = np.array(emission_image.unit_size)
    step = np.floor(50 / size_voxel)
    time = np.floor(np.array(emission_image.shape) / step)
    size_img = np.array(emission_image.size)
    xs, ys, zs = (np.arange(int(t)) for t in time)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    pos = np.stack([step[0] * (X.ravel() + 0.5) * size_voxel[0],
                    step[1] * (Y.ravel() + 0.5) * size_voxel[1],
                    step[2] * (Z.ravel() + 0.5) * size_voxel[2]], 1) - size_img / 2
    return pos.astype(np.float32)


def get_all_crystal_position(scanner: PetEcatScanner) -> np.ndarray:
    return EcatIndexToCrystalPos(scanner)(np.arange(scanner.nb_crystals)).astype(np.float32)


def get_lors(P1: np.ndarray, P2: np.ndarray) -> Lors:
    """Every P1 row paired with every P2 row, P1-major, 7 columns of ones (preprocess.py:49-57)."""
    lors = np.ones((P1.shape[0] * P2.shape[0], 7), dtype=np.float32)
    lors[:, 0:3] = np.repeat(P1, P2.shape[0], axis=0)
    lors[:, 3:6] = np.tile(P2, (P1.shape[0], 1))
    return Lors(lors)


def pre_sumup_of_emission(emission_image: Image, p1: np.ndarray, p2: np.ndarray) -> np.ndarray:
    lors = get_lors(p1, p2)
    value = Project("tf-eager")(emission_image, lors).data
    d = lors.data
    len2 = (d[:, 3] - d[:, 0]) ** 2 + (d[:, 4] - d[:, 1]) ** 2 + (d[:, 5] - d[:, 2]) ** 2
    return value * len2


def pre_atten(transmission_image: Image, p1: np.ndarray, p2: np.ndarray) -> np.ndarray:
    return UmapProject()(transmission_image, get_lors(p1, p2)).data


def pre_lors_atten(transmission_image: Image, p1: np.ndarray, p2: np.ndarray) -> np.ndarray:
    lors = np.hstack((np.hstack((p1, p2)), np.ones((p1.shape[0], 1), dtype=np.float32)))
    return UmapProject()(transmission_image * 1.3, Lors(lors)).data


def scatter_preprocess(scanner: PetEcatScanner, listmode: Listmode, emission_image: Image,
                       umap: Image, outdir: Optional[str] = None, out_append: Optional[str] = None):
    lors = get_all_lors_id(scanner.nb_crystals)
    sinogram = lm2sino(listmode, scanner)
    index = np.where(sinogram > 0)[0].astype(np.int32)
    scatter_position = pre_all_scatter_position(emission_image)
    crystal_position = get_all_crystal_position(scanner)
    sumup_emission = pre_sumup_of_emission(emission_image, crystal_position, scatter_position)
    atten = pre_atten(umap, crystal_position, scatter_position)
    atten_lors = pre_lors_atten(umap, crystal_position[lors[index, 0]],
                                crystal_position[lors[index, 1]]).reshape(-1, 1)
    out = dict(lors=lors, sinogram=sinogram, index=index, scatter_position=scatter_position,
               crystal_position=crystal_position, sumup_emission=sumup_emission, atten=atten,
               atten_lors=atten_lors)
    if outdir is not None:
        app = out_append or ""
        for k, v in out.items():
            np.save(os.path.join(outdir, f"{k}{app}.npy"), v)
    return out


# ------------------------------------------------------------------ SSS

def eff_without_scatter(low: int, high: int, energy_resolution: float) -> float:
    """scatter_fraction.py:94-100."""
    eff = 0.0
    for i in range(int(low), int(high), 5):
        eff += math.exp(-(float(i) - 511) ** 2 / 2 / energy_resolution ** 2)
    return eff


def scatter_scaling(scatter: np.ndarray, scale: np.ndarray, low: int, high: int, resolution: float,
                    grid_block, size_block):
    """Host post-scaling of scatter_fraction.py:27-36 (float64)."""
    e0 = eff_without_scatter(low, high, math.sqrt(511) * resolution) * 5 / (1022 * math.pi) ** 0.5 / resolution
    area = size_block[1] * size_block[2] / grid_block[1] / grid_block[2]
    sc = scatter * e0 * area ** 2 * 5 / (1022 * math.pi) ** 0.5 / resolution / 4 / math.pi
    sl = scale * 4 * math.pi / e0 ** 2 / area ** 2
    return sc, sl


def scatter_fraction(emission_image: Image, u_map: Image, index: np.ndarray, lors: np.ndarray,
                     nb_blocks_per_ring: int, nb_crystals_per_ring: int, grid_block, size_block,
                     low_energy: int, high_energy: int, resolution: float,
                     scatter_position: np.ndarray, crystal_position: np.ndarray,
                     sumup_emission: np.ndarray, atten: np.ndarray):
    """GPU SSS for the LOR pairs ``lors[index]`` (scatter_fraction.py:12-37)."""
    dev = device()
    pairs = torch.as_tensor(np.ascontiguousarray(lors[index, :2]), dtype=torch.int32).to(dev)
    umap = to_dev(np.asarray(u_map.data, np.float32))
    sc, sl = kernels.sss(pairs, to_dev(crystal_position), to_dev(scatter_position),
                         to_dev(np.asarray(sumup_emission, np.float32).reshape(crystal_position.shape[0], -1)),
                         to_dev(np.asarray(atten, np.float32).reshape(crystal_position.shape[0], -1)),
                         umap, list(u_map.size), nb_crystals_per_ring, nb_blocks_per_ring,
                         list(grid_block), int(low_energy), int(high_energy), float(resolution))
    sc = sc.cpu().numpy().astype(np.float64).reshape(-1, 1)
    sl = sl.cpu().numpy().astype(np.float64).reshape(-1, 1)
    return scatter_scaling(sc, sl, low_energy, high_energy, resolution, grid_block, size_block)


@dataclasses.dataclass(frozen=True)
class ScatterCorrect(_NefLike):
    low_energy: Optional[float] = None
    high_energy: Optional[float] = None
    resolution: Optional[float] = None
    scatter_fraction: Optional[float] = None

    def __call__(self, emission_image: Image, u_map: Image, scanner: PetEcatScanner, outdir,
                 out_append: Optional[str] = None) -> Listmode:
        """``outdir``: a directory holding scatter_preprocess's .npy files (the reference's
        form), the dict scatter_preprocess returns, or a Listmode (preprocessed here)."""
        if isinstance(outdir, Listmode):
            pre = scatter_preprocess(scanner, outdir, emission_image, u_map)
        elif isinstance(outdir, dict):
            pre = outdir
        else:
            app = out_append or ""
            keys = ("lors", "sinogram", "index", "scatter_position", "crystal_position",
                    "sumup_emission", "atten", "atten_lors")
            pre = {k: np.load(os.path.join(outdir, f"{k}{app}.npy")) for k in keys}
        nb_blocks_per_ring = scanner.nb_blocks_per_ring
        nb_crystals_per_ring = scanner.nb_blocks_per_ring * scanner.blocks.shape[1]
        grid_block = np.array(scanner.blocks.shape, dtype=np.int32)
        size_block = np.array(scanner.blocks.size, dtype=np.float32)
        sinogram, index = pre["sinogram"], pre["index"]
        fraction, scale = scatter_fraction(
            emission_image, u_map, index, pre["lors"], nb_blocks_per_ring, nb_crystals_per_ring,
            grid_block, size_block, int(self.low_energy), int(self.high_energy),
            float(self.resolution), pre["scatter_position"], pre["crystal_position"],
            pre["sumup_emission"], pre["atten"])
        corrected = np.zeros_like(sinogram)
        corrected[index] = (sinogram[index] - fraction / np.sum(fraction) * np.sum(sinogram[index])
                            * self.scatter_fraction) * scale / (pre["atten_lors"] + sys.float_info.min)
        data = sino2lm(scanner, corrected, pre["lors"])
        return Listmode(data[:, 6].astype(np.float32), Lors(data.astype(np.float32)))
