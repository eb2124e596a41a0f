"""GPU: differentiable projector (finite differences in FP64, adjoint identity) and the
single-scatter simulation (kernel and full correction pipeline) against the CPU oracle."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tof", [False, True])
def test_projector_gradient_finite_differences(cuda_lib, small_case, tof):
    """d/dx_v of sum(p - y log p) against central differences in FP64 on 64 voxels.
    A is linear, so p(x +- h e_v) = p(x) +- h A e_v with A e_v the projection of a one-hot image."""
    from srf_gb300 import autograd, kernels
    ic, sc = small_case["ic"], small_case["scanner"]
    t = (sc.tof.tof_bin, sc.tof.tof_sigma2) if tof else None
    dev = torch.device("cuda", 0)
    lors = torch.as_tensor(small_case["lors"], device=dev)
    x0 = torch.as_tensor(small_case["act"] + 0.5, device=dev)
    x = x0.clone().requires_grad_(True)
    p = autograd.project(x, lors, ic.center, ic.size, tof=t)
    y = torch.poisson(p.detach().clamp(min=0) * 50 + 1)
    loss = autograd.poisson_nll(p, y, eps=1e-3)
    loss.backward()
    grad = x.grad.cpu().numpy().astype(np.float64)
    p64 = p.detach().cpu().numpy().astype(np.float64)
    y64 = y.cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(0)
    flat = np.flatnonzero(np.abs(grad) > 1e-3 * np.abs(grad).max())
    vox = rng.choice(flat, 64, replace=False)
    h = 1e-3

    def L(pp):
        return float(np.sum(pp - y64 * np.log(pp + 1e-3)))
    for v in vox:
        e = torch.zeros(ic.shape, device=dev)
        e.view(-1)[v] = 1.0
        a = kernels.project(lors, e, ic.center, ic.size, tof=t).cpu().numpy().astype(np.float64)
        fd = (L(p64 + h * a) - L(p64 - h * a)) / (2 * h)
        g = grad.reshape(-1)[v]
        assert abs(fd - g) <= 1e-4 * max(abs(fd), 1e-6 * np.abs(grad).max()), (v, fd, g)


def test_batched_projector_adjoint_identity(cuda_lib, small_case):
    from srf_gb300 import autograd
    ic, sc = small_case["ic"], small_case["scanner"]
    dev = torch.device("cuda", 0)
    lors = torch.as_tensor(small_case["lors"], device=dev)
    rng = np.random.default_rng(1)
    xb = torch.as_tensor(rng.random((3, *ic.shape)).astype(np.float32), device=dev).requires_grad_(True)
    t = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    p = autograd.project(xb, lors, ic.center, ic.size, tof=t)
    assert p.shape == (3, lors.shape[0])
    yv = torch.as_tensor(rng.random((3, lors.shape[0])).astype(np.float32), device=dev)
    (p * yv).sum().backward()
    lhs = float((p.detach().double() * yv.double()).sum())
    rhs = float((xb.detach().double() * xb.grad.double()).sum())
    assert abs(lhs - rhs) / abs(lhs) <= 1e-6


@pytest.mark.parametrize("tof", [False, True])
def test_batched_projector_matches_single_image_kernels(cuda_lib, small_case, tof):
    """srf_projection_batch / srf_projection_adjoint_batch against the single-image kernels, for
    a batch of 8 and a batch of 11 (split 8 + 3) through the autograd path."""
    from srf_gb300 import autograd, kernels
    ic, sc = small_case["ic"], small_case["scanner"]
    dev = torch.device("cuda", 0)
    lors = torch.as_tensor(small_case["lors"], device=dev)
    t = (sc.tof.tof_bin, sc.tof.tof_sigma2) if tof else None
    rng = np.random.default_rng(3)
    xb = torch.as_tensor(rng.random((8, *ic.shape)).astype(np.float32), device=dev)
    pb = kernels.project_batch(lors, xb, ic.center, ic.size, tof=t)
    for b in range(8):
        ps = kernels.project(lors, xb[b], ic.center, ic.size, tof=t)
        assert rel_l2(pb[b].cpu().numpy(), ps.cpu().numpy()) <= 1e-6
    vb = torch.as_tensor(rng.random((8, lors.shape[0])).astype(np.float32), device=dev)
    gb = kernels.adjoint_batch(lors, vb, ic.shape, ic.center, ic.size, tof=t)
    for b in range(8):
        gs = kernels.backproject(lors, vb[b], ic.shape, ic.center, ic.size, tof=t, adjoint=True)
        assert rel_l2(gb[b].cpu().numpy(), gs.cpu().numpy()) <= 1e-5
    x11 = torch.as_tensor(rng.random((11, *ic.shape)).astype(np.float32), device=dev).requires_grad_(True)
    p11 = autograd.project(x11, lors, ic.center, ic.size, tof=t)
    y11 = torch.as_tensor(rng.random(p11.shape).astype(np.float32), device=dev)
    (p11 * y11).sum().backward()
    lhs = float((p11.detach().double() * y11.double()).sum())
    rhs = float((x11.detach().double() * x11.grad.double()).sum())
    assert abs(lhs - rhs) / abs(lhs) <= 1e-6


def test_sss_kernel_matches_oracle(cuda_lib, oracle):
    import os
    from srf_gb300 import kernels
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "sss.npz")))
    rng = np.random.default_rng(3)
    n_c = g["crystal"].shape[0]
    pairs = np.vstack([g["pairs"], rng.integers(0, n_c, size=(3000, 2))]).astype(np.int32)
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    ref_s, ref_c = oracle.sss(pairs, g["crystal"], g["scatter"], g["sumup"], g["atten"], g["umap"],
                              g["usize"], int(g["ncpr"]), int(g["nbpr"]), g["grid_block"],
                              int(g["low"]), int(g["high"]), float(g["res"]))
    dev = torch.device("cuda", 0)
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to(dev)
    sc, sl = kernels.sss(d(pairs), d(g["crystal"]), d(g["scatter"]), d(g["sumup"]), d(g["atten"]),
                         d(g["umap"]), list(g["usize"]), int(g["ncpr"]), int(g["nbpr"]),
                         list(g["grid_block"]), int(g["low"]), int(g["high"]), float(g["res"]))
    sc, sl = sc.cpu().numpy(), sl.cpu().numpy()
    assert rel_l2(sc, ref_s) <= 1e-5
    np.testing.assert_allclose(sc, ref_s, rtol=2e-5, atol=1e-6 * np.abs(ref_s).max())
    ok = np.isfinite(ref_c) & (ref_c < 1e6)
    np.testing.assert_allclose(sl[ok], ref_c[ok], rtol=1e-5)


def test_sss_kernel_many_undecided_angles(cuda_lib, oracle):
    """Scatter points on the segment between two crystals (scattering angle 0, cosine 1) put 80
    points of one pair on the double-precision angle path, so that pair's queued evaluations are
    drained while it is still being summed; other pairs queue a few each."""
    import os
    from srf_gb300 import kernels
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "sss.npz")))
    c = g["crystal"]
    a0 = int(np.argmin(np.abs(c[:, 2])))
    u = c[:, :2] / np.linalg.norm(c[:, :2], axis=1, keepdims=True)
    score = u @ u[a0] + 0.01 * np.abs(c[:, 2] - c[a0, 2])
    b0 = int(np.argmin(score))  # about opposite a0, at a similar z
    t = np.linspace(0.25, 0.75, 80, dtype=np.float64)[:, None]
    line = (c[a0] + t * (c[b0].astype(np.float64) - c[a0])).astype(np.float32)
    rng = np.random.default_rng(11)
    spos = np.vstack([g["scatter"], line, rng.uniform([-60, -60, -14], [60, 60, 14], (8, 3))]).astype(np.float32)
    n_s = len(spos)
    sumup = rng.uniform(0.5, 2.0, (len(c), n_s)).astype(np.float32)
    atten = rng.uniform(0.2, 1.0, (len(c), n_s)).astype(np.float32)
    pairs = np.vstack([[[a0, b0]] * 3, [[b0, a0]], g["pairs"], rng.integers(0, len(c), (500, 2))]).astype(np.int32)
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    args = (g["umap"], g["usize"], int(g["ncpr"]), int(g["nbpr"]), g["grid_block"], int(g["low"]),
            int(g["high"]), float(g["res"]))
    ref_s, _ = oracle.sss(pairs, c, spos, sumup, atten, *args)
    dev = torch.device("cuda", 0)
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to(dev)
    sc, _ = kernels.sss(d(pairs), d(c), d(spos), d(sumup), d(atten), d(g["umap"]), list(g["usize"]),
                        int(g["ncpr"]), int(g["nbpr"]), list(g["grid_block"]), int(g["low"]),
                        int(g["high"]), float(g["res"]))
    sc = sc.cpu().numpy()
    assert ref_s[0] > 0
    np.testing.assert_allclose(sc[:4], ref_s[:4], rtol=2e-5)  # the collinear pair, both orders
    np.testing.assert_allclose(sc, ref_s, rtol=2e-5, atol=1e-6 * np.abs(ref_s).max())


def test_scatter_correct_pipeline_matches_oracle(cuda_lib, oracle, small_case):
    import srf_gb300 as nef
    from srf_gb300 import scatter as S
    sc = small_case["scanner"]
    rng = np.random.default_rng(4)
    shape, size = [32, 32, 16], [128.0, 128.0, 128.0]
    emission = nef.Image(rng.random(shape).astype(np.float32), [0.0, 0.0, 0.0], size)
    umap = nef.Umap((rng.random(shape) * 0.01).astype(np.float32), [0.0, 0.0, 0.0], size)
    lors = small_case["lors"][:4000, :6]
    lm = nef.Listmode(np.ones(len(lors), np.float32), nef.Lors(lors))
    corr = S.ScatterCorrect(350, 650, 0.15, 0.3)
    pre = S.scatter_preprocess(sc, lm, emission, umap)
    ref_pre = oracle.scatter_preprocess(sc, lm, emission, umap)
    for k in ("sumup_emission", "atten", "atten_lors"):
        assert rel_l2(pre[k], ref_pre[k]) <= 1e-5, k
    for k in ("lors", "sinogram", "index", "scatter_position", "crystal_position"):
        assert np.array_equal(pre[k], ref_pre[k]), k
    out = corr(emission, umap, sc, pre)
    ref = oracle.scatter_correct(corr, emission, umap, sc, ref_pre)
    assert out.lors.data.shape == ref.lors.data.shape
    assert np.array_equal(out.lors.data[:, :6], ref.lors.data[:, :6])
    assert rel_l2(out.data, ref.data) <= 1e-5
