"""Image warping (srf_gb300.deform; srfnef/cc/deform/deform.cu.cc, deform_tex.cu.cc).

CPU: properties of the oracle's restatement (integer shifts translate exactly, a zero rotation
and a zero field are identities inside the image, the inverse of a constant field is its
negative). GPU: every op under both rules against the oracle, 1e-6 relative L2 (FP32 sums in
another order), and the plain rules' zero-filled voxels exactly where the oracle's are.
"""
import numpy as np
import pytest

from conftest import rel_l2


@pytest.fixture(scope="module")
def D():
    import deform_oracle
    return deform_oracle


def _case(seed=0, shape=(40, 36, 12)):
    rng = np.random.default_rng(seed)
    img = rng.random(shape).astype(np.float32)
    m = [(rng.standard_normal(shape) * 1.7).astype(np.float32) for _ in range(3)]
    return img, m


def test_oracle_warp_properties(D):
    img, m = _case(1)
    sh = D.shift(img, 2.0, -3.0, 1.0, texture=False)
    assert np.array_equal(sh[1:-3, 3:-1, 0:-2], img[3:-1, 0:-4, 1:-1])
    tsh = D.shift(img, 2.0, -3.0, 1.0, texture=True)
    assert np.array_equal(tsh[2:, :-3, 1:], img[:-2, 3:, :-1])
    assert np.allclose(D.rotate(img, 1.0, 0.0, texture=True), img, atol=1e-7)
    z = np.zeros_like(img)
    assert np.array_equal(D.deform(img, z, z, z, texture=True), img)
    assert np.array_equal(D.deform(img, z, z, z, texture=False)[1:-1, 1:-1, 1:-1], img[1:-1, 1:-1, 1:-1])
    c = [np.full(img.shape, v, np.float32) for v in (0.25, -0.5, 0.75)]
    inv = D.deform_invert(*c)
    for a, b in zip(inv, c):
        assert np.allclose(a, -b, atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("texture", [True, False])
def test_gpu_warps_match_oracle(cuda_lib, D, texture):
    import torch
    from srf_gb300 import deform
    img, m = _case(2)
    d = lambda a: torch.as_tensor(a, device="cuda")
    cases = [
        (deform.deform(d(img), d(m[0]), d(m[1]), d(m[2]), texture=texture), D.deform(img, *m, texture=texture)),
        (deform.shift(d(img), 1.3, -2.6, 0.4, texture=texture), D.shift(img, 1.3, -2.6, 0.4, texture=texture)),
        (deform.shift_z(d(img), -1.7, texture=texture), D.shift_z(img, -1.7, texture=texture)),
        (deform.shift_z(d(img), 0.6, texture=texture), D.shift_z(img, 0.6, texture=texture)),
        (deform.rotate(d(img), 0.3, texture=texture),
         D.rotate(img, np.float32(np.cos(0.3)), np.float32(np.sin(0.3)), texture=texture)),
    ]
    for got, want in cases:
        got = got.cpu().numpy()
        assert got.shape == want.shape
        assert rel_l2(got, want) <= 1e-6
        if not texture:
            assert np.array_equal(got == 0, want == 0)


def _smooth_field(shape, amp=1.2, seed=5):
    """A smooth displacement field (long-wavelength sinusoids): the 30-step inversion is a
    contraction for it, so rounding differences do not grow."""
    rng = np.random.default_rng(seed)
    x, y, z = np.meshgrid(*[np.arange(n, dtype=np.float64) / n for n in shape], indexing="ij")
    out = []
    for _ in range(3):
        a, b, c = rng.uniform(0, 2 * np.pi, 3)
        out.append((amp * np.sin(2 * np.pi * x + a) * np.cos(2 * np.pi * y + b) * np.cos(np.pi * z + c)).astype(np.float32))
    return out


@pytest.mark.gpu
def test_gpu_deform_invert_matches_oracle(cuda_lib, D):
    import torch
    from srf_gb300 import deform
    m = _smooth_field((40, 36, 12))
    d = lambda a: torch.as_tensor(a, device="cuda")
    got = deform.deform_invert(d(m[0]), d(m[1]), d(m[2]))
    want = D.deform_invert(*m)
    for g, w in zip(got, want):
        assert rel_l2(g.cpu().numpy(), w) <= 1e-5
    img, _ = _case(4)
    mix = deform.DeformMixin()
    back = mix._deform_invert_tf(d(img), d(m[0]), d(m[1]), d(m[2])).cpu().numpy()
    assert rel_l2(back, D.deform(img, *want, texture=True)) <= 1e-5
