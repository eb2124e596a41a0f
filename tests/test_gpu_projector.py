"""GPU parity of the four Siddon kernels and the exact adjoint against the CPU oracle.

Tolerance: 1e-5 relative L2 (FP32 results; the oracle follows the reference operand by operand,
the GPU sums a LOR's slabs in a different order and evaluates the TOF exponential in FP32).
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.as_tensor(a).cuda()


def _geom(case):
    ic = case["ic"]
    return ic.shape, ic.center, ic.size


@pytest.mark.parametrize("tof", [False, True])
@pytest.mark.parametrize("use_t", [False, True])
def test_projection_matches_oracle(cuda_lib, oracle, small_case, tof, use_t):
    from srf_gb300 import kernels
    sh, c, s = _geom(small_case)
    lors, img, sc = small_case["lors"], small_case["img"], small_case["scanner"]
    kw = dict(tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2) if tof else {}
    ref = oracle.projection(img, lors if tof else lors[:, :6], sh, c, s, **kw)
    got = kernels.project(_dev(lors if tof else np.ascontiguousarray(lors[:, :6])), _dev(img), c, s,
                          tof=(sc.tof.tof_bin, sc.tof.tof_sigma2) if tof else None,
                          make_t=use_t).cpu().numpy()
    assert rel_l2(got, ref) <= TOL
    # the same LORs are skipped
    assert np.array_equal(got == 0, ref == 0)


@pytest.mark.parametrize("tof", [False, True])
@pytest.mark.parametrize("use_t", [False, True])
def test_backprojection_matches_oracle(cuda_lib, oracle, small_case, tof, use_t):
    from srf_gb300 import kernels
    sh, c, s = _geom(small_case)
    lors, sc = small_case["lors"], small_case["scanner"]
    vals = np.random.default_rng(3).random(len(lors)).astype(np.float32)
    kw = dict(tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2) if tof else {}
    ref = oracle.backprojection(vals, lors, sh, c, s, **kw)
    got = kernels.backproject(_dev(lors), _dev(vals), sh, c, s,
                              tof=(sc.tof.tof_bin, sc.tof.tof_sigma2) if tof else None,
                              use_t=use_t).cpu().numpy()
    assert rel_l2(got, ref) <= TOL


@pytest.mark.parametrize("nsigma", [3.0, 1.5])
def test_truncated_tof_matches_oracle(cuda_lib, oracle, small_case, nsigma):
    from srf_gb300 import kernels
    sh, c, s = _geom(small_case)
    lors, img, sc = small_case["lors"], small_case["img"], small_case["scanner"]
    t = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    ref = oracle.projection(img, lors, sh, c, s, tof=True, tof_bin=t[0], tof_sigma2=t[1], tof_nsigma=nsigma)
    got = kernels.project(_dev(lors), _dev(img), c, s, tof=t, tof_nsigma=nsigma).cpu().numpy()
    assert rel_l2(got, ref) <= TOL
    vals = np.random.default_rng(4).random(len(lors)).astype(np.float32)
    ref_b = oracle.backprojection(vals, lors, sh, c, s, tof=True, tof_bin=t[0], tof_sigma2=t[1], tof_nsigma=nsigma)
    got_b = kernels.backproject(_dev(lors), _dev(vals), sh, c, s, tof=t, tof_nsigma=nsigma).cpu().numpy()
    assert rel_l2(got_b, ref_b) <= TOL


@pytest.mark.parametrize("tof", [False, True])
def test_adjoint_matches_oracle_and_dot_product(cuda_lib, oracle, small_case, tof):
    from srf_gb300 import kernels
    sh, c, s = _geom(small_case)
    lors, img, sc = small_case["lors"], small_case["img"], small_case["scanner"]
    t = (sc.tof.tof_bin, sc.tof.tof_sigma2) if tof else None
    vals = np.random.default_rng(5).random(len(lors)).astype(np.float32)
    kw = dict(tof=True, tof_bin=t[0], tof_sigma2=t[1]) if tof else {}
    ref = oracle.projection_adjoint(vals, lors, sh, c, s, **kw)
    got = kernels.backproject(_dev(lors), _dev(vals), sh, c, s, tof=t, adjoint=True).cpu().numpy()
    assert rel_l2(got, ref) <= TOL
    p = kernels.project(_dev(lors), _dev(img), c, s, tof=t).cpu().numpy()
    lhs = float(np.dot(p.astype(np.float64), vals.astype(np.float64)))
    rhs = float(np.sum(img.astype(np.float64) * got.astype(np.float64)))
    assert abs(lhs - rhs) / abs(lhs) <= 1e-6


def test_edge_cases(cuda_lib, oracle):
    """Empty input, short and steep LORs, endpoints inside the image, axis ties, NaN rows,
    non-square voxels and an 8-float row stride."""
    from srf_gb300 import kernels
    rng = np.random.default_rng(7)
    sh, c, s = [40, 32, 12], [1.5, -2.0, 0.5], [80.0, 72.0, 30.0]  # dy != dx
    img = rng.random(sh).astype(np.float32)
    rows = [
        [-100, 0, 0, 100, 0, 0],          # axis-aligned
        [-100, -100, -10, 100, 100, 10],  # |xd| == |yd| tie
        [-3, 0, 0, 4, 1, 0],              # transaxial length < 10 voxels: skipped
        [-50, 0, -200, 50, 0, 200],       # steeper than 45 deg (non-TOF projector skips)
        [-120, 30, 5, 10, -5, 2],         # endpoint 2 inside the image
        [15, 5, -3, 130, -60, 8],         # endpoint 1 inside the image
        [np.nan, 0, 0, 100, 0, 0],        # non-finite: contributes nothing
        [-100, 36, 0, 100, 36, 0],        # along the image boundary
    ]
    rand = rng.uniform(-150, 150, size=(500, 6))
    lors6 = np.vstack([np.array(rows, dtype=np.float64), rand]).astype(np.float32)
    tofcol = rng.normal(0, 40, size=(len(lors6), 1)).astype(np.float32)
    lors8 = np.hstack([lors6, tofcol, np.zeros_like(tofcol)]).astype(np.float32)
    finite = np.isfinite(lors6).all(1)
    for tof in (False, True):
        t = (3.66, 1138.0) if tof else None
        kw = dict(tof=True, tof_bin=3.66, tof_sigma2=1138.0) if tof else {}
        ref = oracle.projection(img, lors8[finite], sh, c, s, **kw)
        got = kernels.project(_dev(lors8), _dev(img), c, s, tof=t).cpu().numpy()
        assert got[~finite].tolist() == [0.0]
        assert rel_l2(got[finite], ref) <= TOL
        vals = rng.random(len(lors8)).astype(np.float32)
        ref_b = oracle.backprojection(vals[finite], lors8[finite], sh, c, s, **kw)
        got_b = kernels.backproject(_dev(lors8), _dev(vals), sh, c, s, tof=t).cpu().numpy()
        assert rel_l2(got_b, ref_b) <= TOL
    empty = torch.zeros((0, 7), dtype=torch.float32, device="cuda")
    assert kernels.project(empty, _dev(img), c, s).numel() == 0
    assert float(kernels.backproject(empty, torch.zeros(0, device="cuda"), sh, c, s).abs().sum()) == 0.0


def test_dropin_classes(cuda_lib, oracle, small_case):
    import srf_gb300 as nef
    sh, c, s = _geom(small_case)
    lors, img, sc = small_case["lors"], small_case["img"], small_case["scanner"]
    image = nef.Image(img, c, s)
    lm = nef.Project("tf-eager")(image, nef.Lors(lors[:, :6]))
    assert isinstance(lm.data, np.ndarray) and lm.data.shape == (len(lors),)
    assert rel_l2(lm.data, oracle.projection(img, lors[:, :6], sh, c, s)) <= TOL
    bp = nef.BackProject("tf-eager")(lm, image)
    assert bp.data.shape == tuple(sh) and bp.center == c
    assert rel_l2(bp.data, oracle.backprojection(lm.data, lors[:, :6], sh, c, s)) <= TOL
    lmt = nef.ProjectTof("tf-eager", sc.tof)(image, nef.Lors(lors))
    ref = oracle.projection(img, lors, sh, c, s, tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2)
    assert rel_l2(lmt.data, ref) <= TOL
    bpt = nef.BackProjectTof("tf-eager", sc.tof)(lmt, image)
    ref_b = oracle.backprojection(lmt.data, lors, sh, c, s, tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2)
    assert rel_l2(bpt.data, ref_b) <= TOL
    with pytest.raises(NotImplementedError):
        nef.Project("numba")(image, nef.Lors(lors[:, :6]))


@pytest.mark.parametrize("lanes", [8, 16, 32])
def test_group_lanes_agree(cuda_lib, oracle, small_case, lanes):
    from srf_gb300 import _lib, kernels
    sh, c, s = _geom(small_case)
    lors, img, sc = small_case["lors"], small_case["img"], small_case["scanner"]
    t = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    ref = oracle.projection(img, lors, sh, c, s, tof=True, tof_bin=t[0], tof_sigma2=t[1])
    _lib.set_group_lanes(lanes)
    try:
        got = kernels.project(_dev(lors), _dev(img), c, s, tof=t).cpu().numpy()
    finally:
        _lib.set_group_lanes(32)
    assert rel_l2(got, ref) <= TOL
