"""GPU: many studies per launch (persistent batch kernel), CUDA-graph replay and the autotuner.

The batch kernels must reproduce, study by study, the single-study subset step (same LOR
batches, different atomic order: 1e-5 relative L2), and one study must match the CPU oracle.
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def studies_setup(cuda_lib):
    import srf_gb300 as nef
    from srf_gb300 import kernels, synth
    from srf_gb300.geometry import ImageConfig
    sc = synth.scanner_small()
    dev = torch.device("cuda", 0)
    specs = [([64, 64, 16], 2.0, 3000), ([48, 48, 16], 2.5, 8000), ([32, 32, 8], 4.0, 1000),
             ([40, 40, 12], 3.0, 5000)]
    out = []
    for j, (shape, vox, n) in enumerate(specs):
        ic = ImageConfig(shape, [0.0, 0.0, 0.0], [s * vox for s in shape])
        act = synth.phantom_cylinder(ic)
        lors = synth.sample_events(sc, ic, act, n, seed=100 + j, tof_fwhm_ps=530.0, device=dev)
        em = nef.EmapGenerator("block-full", sc)(ic).data
        out.append((ic, lors, em))
    return sc, out


def _single(lors, ic, em_x, perm, n_sub, tof, n_iter):
    from srf_gb300 import kernels
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    st = kernels.SubsetState(ic.shape, ic.center, ic.size, lors.device)
    lp = lors.index_select(0, perm).contiguous()
    per = lp.shape[0] // n_sub
    for _ in range(n_iter):
        for k in range(n_sub):
            st.subset(lp[k * per:(k + 1) * per], None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=tof,
                      tof_nsigma=3.0)
            st.update(em_x, guard_zero=True)
    return st.x.contiguous().cpu().numpy()


def test_batch_matches_single_and_graph(studies_setup, oracle):
    from srf_gb300 import kernels
    from srf_gb300.studies import Study, StudyBatch
    sc, specs = studies_setup
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    n_sub, seed = 3, 7
    dev = torch.device("cuda", 0)
    studies = []
    for ic, lors, em in specs:
        emx = kernels.xfast(torch.as_tensor(em, device=dev) / n_sub)
        studies.append(Study(lors.clone(), ic.shape, ic.center, ic.size, emx))
    batch = StudyBatch(studies, n_sub, tof, tof_nsigma=3.0, seed=seed)
    for _ in range(2):
        batch.iteration()
    eager = [x.cpu().numpy() for x in batch.images()]
    rng = np.random.default_rng(seed)
    perms = [torch.as_tensor(rng.permutation(l.shape[0]), device=dev) for _, l, _ in specs]
    for (ic, lors, em), perm, got in zip(specs, perms, eager):
        emx = kernels.xfast(torch.as_tensor(em, device=dev) / n_sub)
        want = _single(lors, ic, emx, perm, n_sub, tof, 2)
        assert rel_l2(got, want) <= TOL
    # one study against the CPU oracle
    ic, lors, em = specs[2]
    ref = oracle.osem(lors.cpu().numpy(), np.ones(lors.shape[0], np.float32), em, ic.shape,
                      ic.center, ic.size, 2 * n_sub, n_sub, perms[2].cpu().numpy(),
                      rule="full_tof", emap_scale=1.0 / n_sub, guard=True, subset_index="mod",
                      tof=True, tof_bin=tof[0], tof_sigma2=tof[1], tof_nsigma=3.0)
    assert rel_l2(eager[2], ref) <= TOL
    # the same two iterations replayed from a captured graph
    batch.reset()
    batch.capture()          # capture runs one eager warm-up iteration first
    batch.reset()
    for _ in range(2):
        batch.replay()
    torch.cuda.synchronize()
    for got, want in zip([x.cpu().numpy() for x in batch.images()], eager):
        assert rel_l2(got, want) <= TOL
    # and as concurrent per-study chains: eager, then replayed from a graph with parallel branches
    batch.reset()
    for _ in range(2):
        batch.iteration_concurrent(n_streams=3)
    torch.cuda.synchronize()
    for got, want in zip([x.cpu().numpy() for x in batch.images()], eager):
        assert rel_l2(got, want) <= TOL
    batch.reset()
    batch.capture(concurrent=True, n_streams=3)
    batch.reset()
    for _ in range(2):
        batch.replay()
    torch.cuda.synchronize()
    for got, want in zip([x.cpu().numpy() for x in batch.images()], eager):
        assert rel_l2(got, want) <= TOL


def test_autotune_picks_and_caches(studies_setup, tmp_path):
    from srf_gb300 import _lib, autotune
    sc, specs = studies_setup
    ic, lors, _ = specs[1]
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    cache = str(tmp_path / "tuning.json")
    try:
        best = autotune.tune(lors, ic.shape, ic.center, ic.size, tof, 3.0, reps=1, cache=cache)
        assert (best["lanes"], best["slabs_per_lane"]) in autotune.CANDIDATES
        assert best["tried"] == 2 * len(autotune.CANDIDATES) and best["ms"] > 0
        again = autotune.tune(lors, ic.shape, ic.center, ic.size, tof, 3.0, reps=1, cache=cache)
        assert again["lanes"] == best["lanes"] and again["slabs_per_lane"] == best["slabs_per_lane"]
        perm = autotune.direction_order(lors, 64)
        assert torch.equal(torch.sort(perm).values, torch.arange(lors.shape[0], device=lors.device))
    finally:
        _lib.set_tuning(32, 4)
