"""srf_gb300 -- GB300-native (sm_103a) list-mode PET reconstruction hot path with srfnef's API.

The projector/backprojector (non-TOF and TOF), the MLEM/OSEM update with its sensitivity image
and the single-scatter simulation run as hand-written CUDA kernels in ``libsrf_gb300.so``
(C ABI: include/srf_gb300.h), called through ctypes. There is no CPU fallback: on a machine
without a CUDA device, or without the built library, the compute entry points raise.
"""
from .data import Emap, Image, Listmode, Lors, Umap
from .geometry import (Block, EcatCrystalPosToIndex, EcatIndexToCrystalPos, ImageConfig,
                       LorsToListmode, PetEcatListmodeTrans, PetEcatScanner, TofConfig)
from .functions import BackProject, BackProjectTof, Project, ProjectTof
from .emap_generator import EcatEmapGenerator, EmapGenerator
from .recon import Mlem, MlemFull, MlemFullTof, OsemFull, OsemFullTof
from .scatter import AttenuationCorrect, ScatterCorrect, UmapProject

__all__ = [
    "Emap", "Image", "Listmode", "Lors", "Umap", "Block", "EcatCrystalPosToIndex",
    "EcatIndexToCrystalPos", "ImageConfig", "LorsToListmode", "PetEcatListmodeTrans",
    "PetEcatScanner", "TofConfig", "BackProject", "BackProjectTof", "Project", "ProjectTof",
    "EcatEmapGenerator", "EmapGenerator", "Mlem", "MlemFull", "MlemFullTof", "OsemFull",
    "OsemFullTof", "AttenuationCorrect", "ScatterCorrect", "UmapProject",
]
