"""GPU: the surrogate network's BF16 kernels against the float64 CPU oracle (oracle/cnn_oracle.py).

Inputs and weights are drawn as bfloat16 values, so the oracle sees exactly what the tensor cores
see; the FP32-accumulated results must match to 1e-5 relative, BF16-stored results to BF16
rounding (4e-3).
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _bf(a):
    return torch.as_tensor(a, dtype=torch.float32).to(torch.bfloat16)


def _np(t):
    return t.to(torch.float32).cpu().numpy().astype(np.float64)


@pytest.fixture(scope="module")
def cnn():
    import cnn_oracle
    from srf_gb300 import _lib
    _lib.load()
    return cnn_oracle


def test_conv_forward_dgrad_wgrad(cuda_lib, cnn):
    from srf_gb300._lib import call, i32, ptr, stream_ptr
    from srf_gb300.surrogate import act
    rng = np.random.default_rng(0)
    dev = torch.device("cuda", 0)
    n, d, h, w, cin, cout = 2, 5, 6, 7, 32, 48
    # x lives in a wider buffer at a channel offset (as a U-Net skip slice)
    xbuf = _bf(rng.standard_normal((n, d, h, w, cin + 16))).to(dev)
    wt = _bf(rng.standard_normal((cout, 27, cin)) * 0.1).to(dev)
    bias = torch.as_tensor(rng.standard_normal(cout).astype(np.float32)).to(dev)
    ybuf = torch.zeros((n, d, h, w, cout + 32), dtype=torch.bfloat16, device=dev)
    yf = torch.zeros((n, d, h, w, cout + 32), dtype=torch.float32, device=dev)
    s = stream_ptr(dev)
    call("srf_conv3d_fwd", ptr(xbuf), act(xbuf, 16), i32(cin), ptr(wt), ptr(bias), i32(cout), i32(1),
         ptr(ybuf), act(ybuf, 32), ptr(yf), s)
    x64 = _np(xbuf)[..., 16:]
    ref = cnn.conv3d(x64, _np(wt), bias.cpu().numpy(), relu=True)
    got = yf.cpu().numpy()[..., 32:]
    assert rel_l2(got, ref) <= 1e-5
    assert rel_l2(_np(ybuf)[..., 32:], ref) <= 4e-3
    assert np.all(_np(ybuf)[..., :32] == 0)  # nothing written outside the slice
    # data gradient: the forward kernel on flipped weights
    dy = _bf(rng.standard_normal((n, d, h, w, cout))).to(dev)
    wf = torch.empty((cin, 27, cout), dtype=torch.bfloat16, device=dev)
    call("srf_conv3d_flip_weights", ptr(wt), i32(cout), i32(cin), ptr(wf), s)
    dxf = torch.zeros((n, d, h, w, cin), dtype=torch.float32, device=dev)
    dxb = torch.zeros((n, d, h, w, cin), dtype=torch.bfloat16, device=dev)
    call("srf_conv3d_fwd", ptr(dy), act(dy), i32(cout), ptr(wf), None, i32(cin), i32(0), ptr(dxb),
         act(dxb), ptr(dxf), s)
    assert rel_l2(dxf.cpu().numpy(), cnn.conv3d_dgrad(_np(dy), _np(wt))) <= 1e-5
    # weight gradient (FP32 accumulation, split over voxels)
    dw = torch.zeros((cout, 27, cin), dtype=torch.float32, device=dev)
    call("srf_conv3d_wgrad", ptr(xbuf), act(xbuf, 16), i32(cin), ptr(dy), act(dy), i32(cout), ptr(dw), s)
    assert rel_l2(dw.cpu().numpy(), cnn.conv3d_wgrad(x64, _np(dy))) <= 1e-5


def test_conv_forward_tile_shapes(cuda_lib, cnn):
    """srf_conv3d_fwd picks its tile from the grid it is given: grids large enough for 64 x 64
    tiles (Cout = 64) and for 128 x 32 tiles (Cout = 32) against the oracle (the small grid of the
    test above takes the split-K tile)."""
    from srf_gb300._lib import call, i32, ptr, stream_ptr
    from srf_gb300.surrogate import act
    rng = np.random.default_rng(5)
    dev = torch.device("cuda", 0)
    s = stream_ptr(dev)
    for shape, cin, cout in (((1, 13, 40, 40), 32, 64), ((1, 25, 40, 40), 16, 32)):
        x = _bf(rng.standard_normal(shape + (cin,))).to(dev)
        wt = _bf(rng.standard_normal((cout, 27, cin)) * 0.1).to(dev)
        bias = torch.as_tensor(rng.standard_normal(cout).astype(np.float32)).to(dev)
        y = torch.zeros(shape + (cout,), dtype=torch.bfloat16, device=dev)
        yf = torch.zeros(shape + (cout,), dtype=torch.float32, device=dev)
        call("srf_conv3d_fwd", ptr(x), act(x), i32(cin), ptr(wt), ptr(bias), i32(cout), i32(1), ptr(y),
             act(y), ptr(yf), s)
        ref = cnn.conv3d(_np(x), _np(wt), bias.cpu().numpy(), relu=True)
        assert rel_l2(yf.cpu().numpy(), ref) <= 1e-5, (shape, cin, cout)
        assert rel_l2(_np(y), ref) <= 4e-3


def test_conv_forward_tcgen05_tile(cuda_lib, cnn):
    """The tcgen05 kernels (accumulator in tensor memory) against the oracle and against the
    mma.sync kernels (mode 0): the 128-voxel x 32-channel K-step kernel (path 2, mode 1) and, for
    batch-1 layers with W >= 96 and Cout = 32, the halo-tile kernel with cp.async halos (path 5,
    mode 2) and with TMA halos (path 3, mode 3): one W-row tile of 128 voxels plus a partial one,
    a single partial tile at W = 100; input and output channel slices of wider buffers; a small
    batch-2 layer keeps the split-K kernel (path 4), a larger one takes the K-step kernel with
    the batch index in the grid (as in training)."""
    from srf_gb300._lib import call, i32, ptr, stream_ptr
    from srf_gb300.surrogate import act
    rng = np.random.default_rng(9)
    dev = torch.device("cuda", 0)
    s = stream_ptr(dev)
    cases = (((1, 25, 40, 40), 16, 32, 0, 0, 2), ((1, 25, 40, 40), 96, 32, 16, 32, 2),
             ((1, 25, 40, 41), 32, 96, 0, 32, 2), ((1, 6, 5, 160), 32, 32, 0, 0, 3),
             ((1, 4, 3, 130), 96, 32, 16, 32, 3), ((1, 3, 4, 100), 16, 32, 0, 0, 3),
             ((2, 3, 4, 100), 16, 32, 0, 0, 4), ((2, 13, 40, 40), 32, 32, 16, 32, 2))
    # mode 1 (the default) takes the K-step tcgen05 kernel, modes 2 and 3 also the halo kernels
    try:
        for shape, cin, cout, xoff, yoff, path in cases:
            xbuf = _bf(rng.standard_normal(shape + (cin + xoff,))).to(dev)
            wt = _bf(rng.standard_normal((cout, 27, cin)) * 0.1).to(dev)
            bias = torch.as_tensor(rng.standard_normal(cout).astype(np.float32)).to(dev)
            ref = cnn.conv3d(_np(xbuf)[..., xoff:], _np(wt), bias.cpu().numpy(), relu=True)
            modes = {0: None, 1: path} if path != 3 else {0: None, 2: 5, 3: 3}
            f0 = None
            for tc, want in modes.items():
                call("srf_set_conv_tc", i32(tc))
                y = torch.zeros(shape + (cout + yoff,), dtype=torch.bfloat16, device=dev)
                yf = torch.zeros(shape + (cout + yoff,), dtype=torch.float32, device=dev)
                call("srf_conv3d_fwd", ptr(xbuf), act(xbuf, xoff), i32(cin), ptr(wt), ptr(bias), i32(cout),
                     i32(1), ptr(y), act(y, yoff), ptr(yf), s)
                got = yf.cpu().numpy()[..., yoff:]
                if want is None:  # mma.sync
                    f0 = got
                    continue
                used = ctypes.c_int32(-1)
                call("srf_conv_last_path", ctypes.byref(used))
                assert used.value == want, (shape, cin, cout, tc, used.value)
                status = ctypes.c_int32(0)
                call("srf_conv_tc_status", ctypes.byref(status))
                assert status.value == 0
                assert rel_l2(got, ref) <= 1e-5, (shape, cin, cout, tc)
                assert rel_l2(got, f0) <= 1e-5  # FP32 sums in another order
                assert rel_l2(_np(y)[..., yoff:], ref) <= 4e-3
                assert np.all(_np(y)[..., :yoff] == 0)
    finally:
        call("srf_set_conv_tc", i32(1))


def test_pool_upsample_and_adjoints(cuda_lib, cnn):
    """Pooling, upsampling and their adjoints against the oracle, on whole 16-channel buffers (the
    8-channel vector path) and on a 12-channel slice at channel offset 4 (the scalar path); the
    channels outside the slice stay untouched."""
    from srf_gb300._lib import call, i32, ptr, stream_ptr
    from srf_gb300.surrogate import act
    rng = np.random.default_rng(1)
    dev = torch.device("cuda", 0)
    fine = (2, 5, 6, 7, 16)
    coarse = (2, 3, 3, 4, 16)
    s = stream_ptr(dev)
    for c, off in ((16, 0), (12, 4)):
        sl = slice(off, off + c)
        # multiples of 1/8 with small numerators are exact in bfloat16 and in the sums below
        x = _bf(rng.integers(-8, 8, fine) / 8.0).to(dev)
        cb = torch.zeros(coarse, dtype=torch.bfloat16, device=dev)
        call("srf_cnn_pool2", ptr(x), act(x, off), ptr(cb), act(cb, off), i32(c), i32(0), s)
        got = _np(cb)
        assert np.allclose(got[..., sl], cnn.pool2(_np(x)[..., sl]), atol=1e-2)
        assert not got[..., :off].any()
        g = _bf(rng.integers(-8, 8, coarse)).to(dev)
        gx = torch.zeros(fine, dtype=torch.bfloat16, device=dev)
        call("srf_cnn_pool2", ptr(gx), act(gx, off), ptr(g), act(g, off), i32(c), i32(1), s)
        got = _np(gx)
        assert np.array_equal(got[..., sl], cnn.pool2_adjoint(_np(g)[..., sl], fine[:4] + (c,)))
        assert not got[..., :off].any()
        u = torch.zeros(fine, dtype=torch.bfloat16, device=dev)
        call("srf_cnn_upsample2", ptr(g), act(g, off), ptr(u), act(u, off), i32(c), i32(0), s)
        got = _np(u)
        assert np.array_equal(got[..., sl], cnn.upsample2(_np(g)[..., sl], fine[:4] + (c,)))
        assert not got[..., :off].any()
        gc = torch.zeros(coarse, dtype=torch.bfloat16, device=dev)
        call("srf_cnn_upsample2", ptr(gc), act(gc, off), ptr(x), act(x, off), i32(c), i32(1), s)
        got = _np(gc)
        assert np.allclose(got[..., sl], cnn.upsample2_adjoint(_np(x)[..., sl], coarse[:4] + (c,)), atol=1e-2)
        assert not got[..., :off].any()


def test_head8_forward_and_gradients(cuda_lib, cnn):
    from srf_gb300._lib import call, i32, ptr, stream_ptr
    from srf_gb300.surrogate import act
    import ctypes
    rng = np.random.default_rng(4)
    dev = torch.device("cuda", 0)
    n, d, h, w, c = 2, 3, 4, 5, 32
    fine = (6, 7, 10)  # cropped in y
    x = _bf(rng.standard_normal((n, d, h, w, c + 8))).to(dev)
    wt = torch.as_tensor(rng.standard_normal((8, c)).astype(np.float32)).to(dev)
    b = torch.as_tensor(rng.standard_normal(8).astype(np.float32)).to(dev)
    out = torch.zeros((n, *fine), dtype=torch.float32, device=dev)
    f3 = (ctypes.c_int32 * 3)(*fine)
    s = stream_ptr(dev)
    call("srf_cnn_head8", ptr(x), act(x, 8), i32(c), ptr(wt), ptr(b), ptr(out), f3, None, None, None,
         None, None, s)
    x64 = _np(x)[..., 8:]
    ref = cnn.head8(x64, wt.cpu().numpy(), b.cpu().numpy(), fine)
    assert rel_l2(out.cpu().numpy(), ref) <= 1e-5
    gout = torch.as_tensor(rng.standard_normal((n, *fine)).astype(np.float32)).to(dev)
    gx = torch.zeros((n, d, h, w, c), dtype=torch.bfloat16, device=dev)
    gw = torch.zeros((8, c), dtype=torch.float32, device=dev)
    gb = torch.zeros(8, dtype=torch.float32, device=dev)
    call("srf_cnn_head8", ptr(x), act(x, 8), i32(c), ptr(wt), ptr(b), None, f3, ptr(gout), ptr(gx),
         act(gx), ptr(gw), ptr(gb), s)
    rgx, rgw, rgb = cnn.head8_grads(x64, wt.cpu().numpy(), gout.cpu().numpy().astype(np.float64))
    assert rel_l2(gw.cpu().numpy(), rgw) <= 1e-5
    assert rel_l2(gb.cpu().numpy(), rgb) <= 1e-5
    assert rel_l2(_np(gx), rgx) <= 4e-3


def test_unet_gradient_matches_finite_differences_and_trains(cuda_lib):
    """Backpropagated gradients of the whole network against central differences of its own
    forward pass (FP32 head output), and a few Adam steps lowering the loss."""
    from srf_gb300.surrogate import UNet3D
    dev = torch.device("cuda", 0)
    net = UNet3D(channels=(16, 32, 48), seed=3, device=dev)
    rng = np.random.default_rng(2)
    n, g = 2, (6, 8, 12)
    inp = np.zeros((n, *g, 16), np.float32)
    inp[..., :2] = rng.random((n, *g, 2))
    inp = _bf(inp).to(dev)
    target = torch.as_tensor(rng.random((n, *(2 * v for v in g))).astype(np.float32), device=dev)
    inv_den = (1.0 / (target ** 2).sum(dim=(1, 2, 3))).contiguous()

    def loss_only():
        out = net.forward(inp)
        return float(net.loss(out, target, None, inv_den, None).item())

    out = net.forward(inp)
    grad = torch.empty_like(out)
    l0 = float(net.loss(out, target, None, inv_den, grad).item())
    net.zero_grad()
    net.backward(grad)
    # the head biases: exact linear response, gradient = sum of the output gradient
    gb = float(net.ghb.sum().item())
    h = 1e-2
    net.hb += h
    lp = loss_only()
    net.hb -= 2 * h
    lm = loss_only()
    net.hb += h
    fd = (lp - lm) / (2 * h)
    assert abs(fd - gb) <= 1e-3 * max(abs(fd), 1e-6)
    # a conv bias deep in the network: BF16 activations make FD noisy, so compare direction and size
    c = net.e2a
    k = int(torch.argmax(c.gb.abs()))
    gk = float(c.gb[k])
    h = 5e-2
    c.b[k] += h
    lp = loss_only()
    c.b[k] -= 2 * h
    lm = loss_only()
    c.b[k] += h
    fd = (lp - lm) / (2 * h)
    assert np.sign(fd) == np.sign(gk) and abs(fd - gk) <= 0.25 * abs(gk) + 1e-6
    # training reduces the loss
    for _ in range(30):
        out = net.forward(inp)
        net.loss(out, target, None, inv_den, grad)
        net.zero_grad()
        net.backward(grad)
        net.step(3e-3)
    assert loss_only() < 0.5 * l0


def test_spot_fit_and_scale_by_basis_match_the_oracle(cuda_lib, cnn):
    """The surrogate's spot-check correction kernels against the oracle: srf_spot_fit (FP64
    normal equations and Cholesky in one block) on a noisy prediction with a planted smooth
    correction, with repeated and out-of-range sample bins; srf_scale_by_basis applying it; and a
    prediction that is zero everywhere, which gets the identity correction."""
    from srf_gb300.surrogate import correction_basis, scale_by_basis, spot_fit
    dev = torch.device("cuda", 0)
    basis = correction_basis(dev)
    phi = basis.double().cpu().numpy()
    k, nb = phi.shape
    rng = np.random.default_rng(11)
    ref_full = rng.uniform(0.5, 2.0, nb)
    beta_true = np.array([0.9, -0.04, 0.03, 0.02, -0.05, 0.01, 0.02, -0.03, 0.01])
    pred = (ref_full / (beta_true @ phi) * (1.0 + 0.05 * rng.standard_normal(nb))).astype(np.float32)
    bins = rng.integers(0, nb, 2048)
    bins[7] = bins[9]
    bins[5], bins[8] = nb + 3, -1                  # left out by the kernel and the oracle
    ref = ref_full[np.clip(bins, 0, nb - 1)].astype(np.float32)
    pred_d = torch.as_tensor(pred, device=dev)
    bins_d = torch.as_tensor(bins, device=dev)
    ref_d = torch.as_tensor(ref, device=dev)
    out = torch.zeros(k + 2, device=dev)
    spot_fit(pred_d, bins_d, ref_d, basis, out)
    beta, judged, raw = cnn.spot_fit(pred, bins, ref, phi)
    got = out.cpu().numpy().astype(np.float64)
    assert np.allclose(got[:k], beta, rtol=1e-5, atol=1e-6)
    assert np.allclose(beta, beta_true, atol=0.01)
    assert abs(got[k] - judged) <= 1e-5 * judged and abs(got[k + 1] - raw) <= 1e-5 * raw
    assert 0.03 < judged < 0.07 < raw
    x = pred_d.clone()
    scale_by_basis(x, basis, out)
    want = pred.astype(np.float64) * (got[:k] @ phi)
    assert rel_l2(x.cpu().numpy(), want) <= 1e-6
    spot_fit(torch.zeros_like(pred_d), bins_d, ref_d, basis, out)
    got = out.cpu().numpy()
    assert np.array_equal(got[:k], np.eye(k)[0]) and abs(got[k] - 1.0) < 1e-6 and abs(got[k + 1] - 1.0) < 1e-6
