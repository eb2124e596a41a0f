"""GPU parity at the clinical configuration of the headline benchmark.

Scanner: 32,448 crystals (424/444 mm radii, 48 blocks of 13 x 13 crystals, 4 block rings). Image:
200 x 200 x 109 at 2.04 x 2.04 x 2.03 mm. Events: 2e5 seeded TOF events of the body phantom
(530 ps FWHM), a sample of the benchmark's 2e7. The oracle runs on all host threads.

At this size an exact (untruncated) TOF LOR spans up to 200 slabs. The fused kernel's default
variant (32 lanes x 4 slabs per chunk) therefore walks many LORs in several chunks and recomputes
their candidates for the backprojection. At 3 sigma every LOR fits one chunk, so the
backprojection reuses the projection's candidates. Both paths are compared here. At 4 sigma a
LOR spans up to about 133 slabs, so LORs that fit one chunk and LORs that take two meet in the
same batch of 32.

Tolerance: 1e-5 relative L2 (FP32), as the small-scanner parity tests.
"""
import os

import numpy as np
import pytest

from conftest import rel_l2

TOL = 1e-5
N_EVENTS = 200_000
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clinical(oracle):
    import torch
    from srf_gb300 import synth
    sc, ic = synth.scanner_clinical(), synth.image_clinical()
    dev = torch.device("cuda", 0)
    act = synth.phantom_body(ic, seed=404, device=dev)
    lors = synth.sample_events(sc, ic, act, N_EVENTS, seed=405, tof_fwhm_ps=530.0, device=dev)
    rng = np.random.default_rng(406)
    img = (act.cpu().numpy() + 0.05 + 0.02 * rng.random(ic.shape)).astype(np.float32)
    emap = (0.5 + rng.random(ic.shape)).astype(np.float32)
    prev = oracle.set_threads(os.cpu_count() or 1)
    try:
        yield dict(scanner=sc, ic=ic, lors=lors.cpu().numpy(), img=img, emap=emap,
                   tof=(sc.tof.tof_bin, sc.tof.tof_sigma2))
    finally:
        oracle.set_threads(prev)


def _dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _slab_spans(lors, ic):
    """Slabs of the dominant axis over which each LOR's other two coordinates stay within the
    image box (plus a voxel): the untruncated slab range of the traversal, in whole slabs."""
    vox = np.asarray(ic.size, np.float64) / np.asarray(ic.shape, np.float64)
    half = np.asarray(ic.size, np.float64) / 2
    p1, p2 = lors[:, 0:3].astype(np.float64), lors[:, 3:6].astype(np.float64)
    d = p2 - p1
    xdom = np.abs(d[:, 0]) > np.abs(d[:, 1])
    a = np.where(xdom, 0, 1)
    b = np.where(xdom, 1, 0)
    idx = np.arange(len(lors))
    pd = d[idx, a]
    lo_t = np.full(len(lors), -np.inf)
    hi_t = np.full(len(lors), np.inf)
    for ax in (b, np.full(len(lors), 2)):
        k = d[idx, ax]
        lim = half[ax] + vox[ax]
        with np.errstate(divide="ignore", invalid="ignore"):
            t1 = (-lim - p1[idx, ax]) / k
            t2 = (lim - p1[idx, ax]) / k
        tl, th = np.minimum(t1, t2), np.maximum(t1, t2)
        flat = k == 0
        tl[flat], th[flat] = -np.inf, np.inf
        lo_t, hi_t = np.maximum(lo_t, tl), np.minimum(hi_t, th)
    pa, pb = p1[idx, a] + lo_t * pd, p1[idx, a] + hi_t * pd
    pa = np.clip(pa, -half[a], half[a])
    pb = np.clip(pb, -half[a], half[a])
    return np.abs(pb - pa) / vox[a]


def test_clinical_lors_need_several_chunks(clinical):
    """The sample holds LORs longer than one default chunk (32 lanes x 4 slabs = 128 slabs)."""
    spans = _slab_spans(clinical["lors"], clinical["ic"])
    assert (spans > 130).mean() > 0.1


@pytest.mark.parametrize("nsigma", [0.0, 3.0])
def test_clinical_tof_projection_and_backprojection(cuda_lib, oracle, clinical, nsigma):
    from srf_gb300 import kernels
    ic, lors, img, t = clinical["ic"], clinical["lors"], clinical["img"], clinical["tof"]
    kw = dict(tof=True, tof_bin=t[0], tof_sigma2=t[1], tof_nsigma=nsigma)
    ref = oracle.projection(img, lors, ic.shape, ic.center, ic.size, **kw)
    got = kernels.project(_dev(lors), _dev(img), ic.center, ic.size, tof=t, tof_nsigma=nsigma).cpu().numpy()
    print(f"clinical TOF projection nsigma={nsigma}: rel L2 {rel_l2(got, ref):.3e}")
    assert rel_l2(got, ref) <= TOL
    assert np.array_equal(got == 0, ref == 0)
    vals = np.random.default_rng(407).random(len(lors)).astype(np.float32)
    ref_b = oracle.backprojection(vals, lors, ic.shape, ic.center, ic.size, **kw)
    got_b = kernels.backproject(_dev(lors), _dev(vals), ic.shape, ic.center, ic.size, tof=t,
                                tof_nsigma=nsigma).cpu().numpy()
    assert rel_l2(got_b, ref_b) <= TOL


def test_clinical_nontof_projection_and_backprojection(cuda_lib, oracle, clinical):
    from srf_gb300 import kernels
    ic, img = clinical["ic"], clinical["img"]
    lors6 = np.ascontiguousarray(clinical["lors"][:, :6])
    ref = oracle.projection(img, lors6, ic.shape, ic.center, ic.size)
    got = kernels.project(_dev(lors6), _dev(img), ic.center, ic.size).cpu().numpy()
    assert rel_l2(got, ref) <= TOL
    vals = np.random.default_rng(408).random(len(lors6)).astype(np.float32)
    ref_b = oracle.backprojection(vals, lors6, ic.shape, ic.center, ic.size)
    got_b = kernels.backproject(_dev(lors6), _dev(vals), ic.shape, ic.center, ic.size).cpu().numpy()
    assert rel_l2(got_b, ref_b) <= TOL


@pytest.mark.parametrize("nsigma", [0.0, 3.0, 4.0])
def test_clinical_osem_subset_step(cuda_lib, oracle, clinical, nsigma):
    """One fused subset step (projection, MlemFullTof's ratio, backprojection) and the update,
    under the default tuning, with the FP64 log-likelihood sum y log(p + eps)."""
    import torch
    from srf_gb300 import _lib, kernels
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    ic, lors, img, emap, t = (clinical[k] for k in ("ic", "lors", "img", "emap", "tof"))
    _lib.set_tuning(32, 4)
    dev = torch.device("cuda", 0)
    st = kernels.SubsetState(ic.shape, ic.center, ic.size, dev, x0=torch.as_tensor(img, device=dev))
    st.subset(_dev(lors), None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=t, tof_nsigma=nsigma,
              track_loglik=True)
    st.update(kernels.xfast(_dev(emap)), guard_zero=True)
    got = st.x.contiguous().cpu().numpy()
    kw = dict(tof=True, tof_bin=t[0], tof_sigma2=t[1], tof_nsigma=nsigma)
    p = oracle.projection(img, lors, ic.shape, ic.center, ic.size, **kw)
    r = oracle.ratio(np.ones(len(lors), np.float32), p, "full_tof")
    bp = oracle.backprojection(r, lors, ic.shape, ic.center, ic.size, **kw)
    want = (img * bp / oracle.guard_emap(emap)).astype(np.float32)
    print(f"clinical subset step nsigma={nsigma}: rel L2 {rel_l2(got, want):.3e}")
    assert rel_l2(got, want) <= TOL
    den = (p + np.float32(1e-5)).astype(np.float64)
    terms = np.log(den[den > 0])
    ll = float(st.loglik.item())
    assert abs(ll - terms.sum()) <= 1e-5 * np.abs(terms).sum()


def test_clinical_osem_tof_two_subsets(cuda_lib, oracle, clinical):
    """One iteration of OsemFullTof with two subsets (3 sigma) from x = 1 against the oracle's
    loop, on 2e6 events: a tenth of the benchmark's (at 1e5 events per subset most voxels of the
    4.4e6 see a handful of LORs, and the ratio y / p of LORs through such voxels amplifies FP32
    rounding beyond any fixed bound)."""
    import torch
    import srf_gb300 as nef
    from srf_gb300 import synth
    sc, ic, emap = clinical["scanner"], clinical["ic"], clinical["emap"]
    dev = torch.device("cuda", 0)
    act = synth.phantom_body(ic, seed=404, device=dev)
    lors = synth.sample_events(sc, ic, act, 10 * N_EVENTS, seed=410, tof_fwhm_ps=530.0,
                               device=dev).cpu().numpy()
    lm = nef.Listmode(np.ones(len(lors), np.float32), nef.Lors(lors))
    em = nef.Emap(emap, ic.center, ic.size)
    out = nef.OsemFullTof(1, 2, ic, sc, lm, em, tof_nsigma=3.0, seed=409)()
    perm = np.random.default_rng(409).permutation(len(lors))
    ref = oracle.osem(lors, lm.data, emap, ic.shape, ic.center, ic.size, 2, 2, perm,
                      rule="full_tof", emap_scale=0.5, guard=True, subset_index="mod", tof=True,
                      tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2, tof_nsigma=3.0)
    err = rel_l2(out.data, ref)
    print(f"clinical OSEM 2 subsets: rel L2 {err:.3e}")
    assert err <= TOL


def test_clinical_emap_block_columns(cuda_lib, oracle, clinical):
    """The block-full sensitivity kernel on the clinical geometry over six block columns spread
    around the ring (36 block pairs, 1.6e7 crystal pairs) against the oracle's generator."""
    import torch
    from srf_gb300 import kernels
    from srf_gb300.geometry import block_full_crystal_table
    sc, ic = clinical["scanner"], clinical["ic"]
    table = block_full_crystal_table(sc)
    m = table.shape[0] // sc.nb_blocks_per_ring
    cols = [0, 8, 16, 24, 32, 40]
    sub = np.ascontiguousarray(np.concatenate([table[c * m:(c + 1) * m] for c in cols]))
    ref = oracle.emap_block_full(sub, len(cols), ic.shape, ic.center, ic.size)
    got = kernels.emap_block_full(torch.as_tensor(sub, device="cuda"), len(cols), ic.shape,
                                  ic.center, ic.size).contiguous().cpu().numpy()
    assert rel_l2(got, ref) <= TOL
    assert (got > 0).sum() == (ref > 0).sum()
