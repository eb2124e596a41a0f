"""GPU list-mode ingestion (snapping, crystal ids, sinogram histogram) and the fused attenuation
pass, against the numpy host code (itself checked against the reference's own code on the CPU)
and the CPU oracle projector."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _jittered(sc, n, seed, tof=True):
    from srf_gb300.geometry import EcatIndexToCrystalPos
    rng = np.random.default_rng(seed)
    pos = EcatIndexToCrystalPos(sc)(np.arange(sc.nb_crystals))
    a, b = rng.integers(0, sc.nb_crystals, n), rng.integers(0, sc.nb_crystals, n)
    unit = min(sc.blocks.unit_size[1], sc.blocks.unit_size[2])
    jit = rng.uniform(-0.35 * unit, 0.35 * unit, (n, 6))
    cols = [np.hstack([pos[a], pos[b]]) + jit]
    if tof:
        cols.append(rng.normal(0, 40, (n, 1)))
    return np.hstack(cols).astype(np.float32), a, b


@pytest.mark.parametrize("which", ["small", "clinical"])
def test_snap_and_ids_match_host(cuda_lib, which):
    from srf_gb300 import kernels, synth
    from srf_gb300.data import Listmode, Lors
    from srf_gb300.geometry import EcatCrystalPosToIndex, PetEcatListmodeTrans
    sc = synth.scanner_small() if which == "small" else synth.scanner_clinical()
    lors, a, b = _jittered(sc, 20000, 1)
    host = PetEcatListmodeTrans(sc)(Listmode(np.ones(len(lors), np.float32), Lors(lors))).lors.data
    dev = torch.as_tensor(lors).cuda()
    out, ids = kernels.snap(dev, sc, want_ids=True)
    ids = ids.cpu().numpy()
    assert np.array_equal(ids[:, 0], EcatCrystalPosToIndex(sc)(lors[:, :3]))
    assert np.array_equal(ids[:, 1], EcatCrystalPosToIndex(sc)(lors[:, 3:6]))
    assert np.array_equal(ids[:, 0], a) and np.array_equal(ids[:, 1], b)
    got = out.cpu().numpy()
    assert np.abs(got[:, :6] - host[:, :6]).max() <= 1e-4
    assert np.array_equal(got[:, 6], lors[:, 6])
    # the drop-in class takes the GPU path for CUDA tensors
    lm = PetEcatListmodeTrans(sc)(Listmode(torch.ones(len(lors)).cuda(), Lors(dev)))
    assert torch.equal(lm.lors.data, out)


def test_lm2sino_matches_host(cuda_lib):
    from srf_gb300 import kernels, synth
    from srf_gb300.data import Listmode, Lors
    from srf_gb300.scatter import lm2sino
    sc = synth.scanner_small()
    lors, a, b = _jittered(sc, 50000, 2, tof=False)
    keep = a != b
    lors = lors[keep]
    w = np.random.default_rng(3).random(len(lors)).astype(np.float32)
    host = lm2sino(Listmode(w, Lors(lors)), sc)[:, 0]
    got, dropped = kernels.lm2sino(torch.as_tensor(lors).cuda(), torch.as_tensor(w).cuda(), sc)
    assert dropped == 0
    np.testing.assert_allclose(got.cpu().numpy(), host, rtol=1e-12, atol=1e-12)


def test_attenuation_fused_matches_oracle(cuda_lib, oracle, small_case):
    import srf_gb300 as nef
    from srf_gb300.scatter import AttenuationCorrect, UmapProject
    ic = small_case["ic"]
    lors = np.ascontiguousarray(small_case["lors"][:, :6])
    mu = (np.random.default_rng(4).random(ic.shape) * 0.01).astype(np.float32)
    p = oracle.projection(mu, lors, ic.shape, ic.center, ic.size)
    L = np.sqrt((lors[:, 0] - lors[:, 3]) ** 2 + (lors[:, 1] - lors[:, 4]) ** 2 + (lors[:, 2] - lors[:, 5]) ** 2)
    want = np.exp(-(p * L * L / ic.unit_size[0]))
    um = nef.Umap(mu, ic.center, ic.size)
    got = UmapProject()(um, nef.Lors(lors)).data
    assert isinstance(got, np.ndarray)
    assert rel_l2(got, want) <= 1e-5
    y = np.random.default_rng(5).random(len(lors)).astype(np.float32)
    corr = AttenuationCorrect(um)(nef.Listmode(y, nef.Lors(lors))).data
    assert rel_l2(corr, y / want) <= 1e-5
