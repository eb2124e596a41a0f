"""The drop-in classes on the GPU against output of the reference's own code.

tests/golden/loops.npz holds images of the reference's Mlem, MlemFull, MlemFullTof and OsemFull
loops and its four projector wrappers (run by tests/golden/make_golden.py with the op libraries
served by the reference's Siddon device functions compiled for the host); geometry.npz holds the
reference's list-mode snapping. Tolerance: 1e-5 relative L2 for FP32 results (sums in another
order, FP32 TOF exponential), bit-exact for snapped endpoints.
"""
import os

import numpy as np
import pytest

from conftest import rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def loops():
    return dict(np.load(os.path.join(GOLD, "loops.npz")))


def _setup(loops):
    import srf_gb300 as nef
    from srf_gb300 import synth
    sc = synth.scanner_small()
    ic = nef.ImageConfig(list(map(int, loops["shape"])), list(map(float, loops["center"])),
                         list(map(float, loops["size"])))
    return nef, sc, ic


def test_mlem_classes_match_reference_loops(cuda_lib, loops):
    nef, sc, ic = _setup(loops)
    lors = loops["lors"]
    l6 = np.ascontiguousarray(lors[:, :6])
    ones = np.ones(len(lors), np.float32)
    em = nef.Emap(loops["emap"], ic.center, ic.size)
    got = nef.MlemFullTof(3, ic, sc, nef.Listmode(ones, nef.Lors(lors)), None, None, None, em)()
    assert rel_l2(got.data, loops["mlem_full_tof"]) <= TOL
    got = nef.MlemFull(3, ic, sc, nef.Listmode(ones, nef.Lors(l6)), None, None, None, em)()
    assert rel_l2(got.data, loops["mlem_full"]) <= TOL
    got = nef.Mlem(3, em)(nef.Listmode(loops["counts"], nef.Lors(l6)))
    assert rel_l2(got.data, loops["mlem"]) <= TOL


def test_osem_full_matches_reference_loop(cuda_lib, loops):
    """OsemFull with the reference's own shuffle (numpy's global generator, seeded as the
    reference run was) and its literal subset index i // n_sub."""
    nef, sc, ic = _setup(loops)
    l6 = np.ascontiguousarray(loops["lors"][:, :6])
    em = nef.Emap(loops["osem_emap"], ic.center, ic.size)
    np.random.seed(608)
    got = nef.OsemFull(4, 2, ic, sc, nef.Listmode(np.ones(len(l6), np.float32), nef.Lors(l6)), None, None,
                       None, None, em, None)()
    assert rel_l2(got.data, loops["osem_full"]) <= TOL


def test_projector_wrappers_match_reference(cuda_lib, loops):
    nef, sc, ic = _setup(loops)
    lors, img, vals = loops["lors"], loops["wrap_image"], loops["wrap_values"]
    n = len(vals)
    l6 = np.ascontiguousarray(lors[:n, :6])
    l7 = np.ascontiguousarray(lors[:n])
    image = nef.Image(img, ic.center, ic.size)
    assert rel_l2(nef.Project("tf-eager")(image, nef.Lors(l6)).data, loops["wrap_proj"]) <= TOL
    assert rel_l2(nef.ProjectTof("tf-eager", sc.tof)(image, nef.Lors(l7)).data, loops["wrap_proj_tof"]) <= TOL
    assert rel_l2(nef.BackProject("tf-eager")(nef.Listmode(vals, nef.Lors(l6)), image).data,
                  loops["wrap_bp"]) <= TOL
    assert rel_l2(nef.BackProjectTof("tf-eager", sc.tof)(nef.Listmode(vals, nef.Lors(l7)), image).data,
                  loops["wrap_bp_tof"]) <= TOL


@pytest.mark.parametrize("name", ["small", "clinical"])
def test_gpu_snapping_matches_reference(cuda_lib, name):
    import torch
    from srf_gb300 import kernels, synth
    g = dict(np.load(os.path.join(GOLD, "geometry.npz")))
    sc = synth.scanner_small() if name == "small" else synth.scanner_clinical()
    l7 = torch.as_tensor(g[f"{name}_lors7"], device="cuda")
    out = kernels.snap(l7, sc).cpu().numpy()
    assert np.array_equal(out.view(np.int32), g[f"{name}_snapped7"].view(np.int32))
