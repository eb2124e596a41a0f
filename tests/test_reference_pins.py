"""Host restatements against output of the reference's own code (CPU).

tests/golden/geometry.npz and loops.npz were made by tests/golden/make_golden.py, which imports
the reference's modules from its tree under stub modules (no TensorFlow here: the op libraries
are served by the reference's own Siddon device functions compiled for the host):

* geometry.npz: EcatIndexToCrystalPos / EcatCrystalPosToIndex
  (srfnef/functions/geometry/pet_ecat_scanner.py:15-89) and PetEcatListmodeTrans
  (srfnef/functions/data_transform/pet_ecat.py:43-60) on the small and the clinical scanner, at
  crystal centres and jittered hits, plus the scanner's derived properties
  (srfnef/ops/geometry/pet_ecat_scanner.py:13-45);
* loops.npz: the images of Mlem, MlemFull, MlemFullTof and OsemFull (srfnef/functions/mlem.py,
  mlem_full.py, mlem_full_tof.py, osem_full.py) and the four projector wrappers' outputs.

srf_gb300.geometry must reproduce the geometry bit for bit; the oracle's numpy loops and its
projector must reproduce the reference's loops and wrappers bit for bit.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def geo():
    return dict(np.load(os.path.join(GOLD, "geometry.npz")))


@pytest.fixture(scope="module")
def loops():
    return dict(np.load(os.path.join(GOLD, "loops.npz")))


def _scanner(name):
    from srf_gb300 import synth
    return synth.scanner_small() if name == "small" else synth.scanner_clinical()


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.int32)


@pytest.mark.parametrize("name", ["small", "clinical"])
def test_crystal_geometry_matches_reference(geo, name):
    from srf_gb300.geometry import EcatCrystalPosToIndex, EcatIndexToCrystalPos
    sc = _scanner(name)
    props = np.array([sc.average_radius, sc.axial_length, sc.angle_per_block, sc.nb_crystals_per_block,
                      sc.nb_crystals_per_ring, sc.nb_crystals], np.float64)
    assert np.array_equal(props, geo[f"{name}_props"])
    pos = EcatIndexToCrystalPos(sc)(geo[f"{name}_ind"])
    assert np.array_equal(_bits(pos), _bits(geo[f"{name}_pos"]))
    assert np.array_equal(EcatCrystalPosToIndex(sc)(geo[f"{name}_jit"]), geo[f"{name}_ids"])
    assert np.array_equal(EcatCrystalPosToIndex(sc)(geo[f"{name}_pos"]), geo[f"{name}_ids_centres"])


@pytest.mark.parametrize("name", ["small", "clinical"])
def test_listmode_snapping_matches_reference(geo, name):
    from srf_gb300.data import Listmode, Lors
    from srf_gb300.geometry import PetEcatListmodeTrans
    sc = _scanner(name)
    l7 = geo[f"{name}_lors7"]
    y = np.ones(len(l7), np.float32)
    s7 = PetEcatListmodeTrans(sc)(Listmode(y, Lors(l7))).lors.data
    s6 = PetEcatListmodeTrans(sc)(Listmode(y, Lors(np.ascontiguousarray(l7[:, :6])))).lors.data
    assert np.array_equal(_bits(s7), _bits(geo[f"{name}_snapped7"]))
    assert np.array_equal(_bits(s6), _bits(geo[f"{name}_snapped6"]))


def _case(loops):
    from srf_gb300 import synth
    sc = synth.scanner_small()
    sh, c, s = list(loops["shape"]), list(loops["center"]), list(loops["size"])
    tof = dict(tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2)
    return loops["lors"], np.ascontiguousarray(loops["lors"][:, :6]), sh, c, s, tof


def test_oracle_loops_match_reference_loops(oracle, loops):
    lors, l6, sh, c, s, tof = _case(loops)
    ones = np.ones(len(lors), np.float32)
    em = loops["emap"]
    got = oracle.mlem(lors, ones, em, sh, c, s, 3, rule="full_tof", **tof)
    assert np.array_equal(_bits(got), _bits(loops["mlem_full_tof"]))
    got = oracle.mlem(l6, ones, em, sh, c, s, 3, rule="full")
    assert np.array_equal(_bits(got), _bits(loops["mlem_full"]))
    got = oracle.mlem(l6, loops["counts"], em, sh, c, s, 3, rule="mlem")
    assert np.array_equal(_bits(got), _bits(loops["mlem"]))
    got = oracle.osem(l6, ones, loops["osem_emap"], sh, c, s, 4, 2, loops["osem_perm"], rule="osem",
                      guard=False, subset_index="reference")
    assert np.array_equal(_bits(got), _bits(loops["osem_full"]))


def test_oracle_projector_matches_reference_wrappers(oracle, loops):
    lors, l6, sh, c, s, tof = _case(loops)
    img, vals = loops["wrap_image"], loops["wrap_values"]
    n = len(vals)
    assert np.array_equal(_bits(oracle.projection(img, l6[:n], sh, c, s)), _bits(loops["wrap_proj"]))
    assert np.array_equal(_bits(oracle.projection(img, lors[:n], sh, c, s, **tof)), _bits(loops["wrap_proj_tof"]))
    assert np.array_equal(_bits(oracle.backprojection(vals, l6[:n], sh, c, s)), _bits(loops["wrap_bp"]))
    assert np.array_equal(_bits(oracle.backprojection(vals, lors[:n], sh, c, s, **tof)),
                          _bits(loops["wrap_bp_tof"]))
