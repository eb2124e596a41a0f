"""Learned single-scatter surrogate (not in the reference).

A 3-D U-Net of about 1.1M parameters maps sinogram-domain features of a study (emission line
integrals and attenuation factors along each bin's LOR) to the single-scatter-simulation
sinogram. Every layer runs on hand-written kernels (srf_gb300/csrc/cnn.cu): BF16 activations
and weights, FP32 accumulation on the tensor cores for the 3x3x3 convolutions (forward, data
gradient through flipped weights, split-K weight gradient), FP32 master weights under Adam.

Architecture on a (D, H, W) grid (the half-resolution sinogram), channels (32, 64, 96):
    e1a, e1b: 3x3x3 16->32->32            (input: 2 feature channels padded to 16)
    pool -> e2a, e2b: 32->64->64
    pool -> e3a, e3b: 64->96->96
    up + skip(e2b) -> d2a, d2b: 160->64->64
    up + skip(e1b) -> d1a, d1b: 96->32->32
    sub-voxel 1x1x1 head: 32->8 FP32 outputs per voxel, one per voxel of the 2x finer grid
ReLU after every 3x3x3 convolution. Skip concatenation is free: e1b/e2b write straight into the
channel slices the decoder reads. The network runs on the 2x-pooled sinogram and its head writes
the full-resolution sinogram directly (no interpolation floor).

``ScatterSurrogate`` wraps the network with SSS as the judge: ``estimate`` predicts the scatter
sinogram, runs SSS on a random subset of bins, fits a smooth multiplicative correction of the
prediction on half of those bins and judges the corrected prediction on the other half; when the
judged relative L2 difference exceeds ``fallback_tol`` it returns the full SSS instead.
"""
from __future__ import annotations

import ctypes
import math
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from ._lib import call, f32, f64, i32, i64, ptr, stream_ptr

BF16 = torch.bfloat16
F32 = torch.float32


def act(t: torch.Tensor, coff: int = 0):
    """int32[6] NDHWC descriptor of a (N, D, H, W, C) tensor (a channel slice from coff)."""
    n, d, h, w, c = t.shape
    return (ctypes.c_int32 * 6)(n, d, h, w, c, coff)


def half(shape):
    return tuple((s + 1) // 2 for s in shape)


class Conv3:
    """3x3x3 convolution parameters: FP32 master weights [Cout][27][Cin], BF16 copies."""

    def __init__(self, cin: int, cout: int, gen: torch.Generator, device):
        std = math.sqrt(2.0 / (27 * cin))
        self.cin, self.cout = cin, cout
        self.w = (torch.randn(cout, 27, cin, generator=gen) * std).to(device)
        self.b = torch.zeros(cout, device=device)
        self.gw = torch.zeros_like(self.w)
        self.gb = torch.zeros_like(self.b)
        self.wb = self.w.to(BF16)
        self.wf = torch.empty(cin, 27, cout, dtype=BF16, device=device)

    def params(self):
        return [(self.w, self.gw, self.wb), (self.b, self.gb, None)]

    def refresh(self, stream):
        call("srf_conv3d_flip_weights", ptr(self.wb), i32(self.cout), i32(self.cin), ptr(self.wf), stream)


class UNet3D:
    IN_CH = 16

    def __init__(self, channels=(32, 64, 96), seed: int = 0, device="cuda"):
        g = torch.Generator().manual_seed(seed)
        self.device = torch.device(device)
        c1, c2, c3 = channels
        self.c = channels
        self.e1a, self.e1b = Conv3(self.IN_CH, c1, g, self.device), Conv3(c1, c1, g, self.device)
        self.e2a, self.e2b = Conv3(c1, c2, g, self.device), Conv3(c2, c2, g, self.device)
        self.e3a, self.e3b = Conv3(c2, c3, g, self.device), Conv3(c3, c3, g, self.device)
        self.d2a, self.d2b = Conv3(c3 + c2, c2, g, self.device), Conv3(c2, c2, g, self.device)
        self.d1a, self.d1b = Conv3(c2 + c1, c1, g, self.device), Conv3(c1, c1, g, self.device)
        self.hw = (torch.randn(8, c1, generator=g) * math.sqrt(1.0 / c1)).to(self.device)
        self.hb = torch.zeros(8, device=self.device)
        self.ghw = torch.zeros_like(self.hw)
        self.ghb = torch.zeros_like(self.hb)
        self.convs = [self.e1a, self.e1b, self.e2a, self.e2b, self.e3a, self.e3b, self.d2a,
                      self.d2b, self.d1a, self.d1b]
        self.adam: Dict[int, Tuple[torch.Tensor, torch.Tensor]] = {}
        self.step_count = 0
        self.buf: Dict[str, torch.Tensor] = {}
        self.shape = None
        s = stream_ptr(self.device)
        for c in self.convs:
            c.refresh(s)

    def n_params(self) -> int:
        return sum(c.w.numel() + c.b.numel() for c in self.convs) + self.hw.numel() + self.hb.numel()

    def _alloc(self, n: int, g1):
        if self.shape == (n, tuple(g1)):
            return
        c1, c2, c3 = self.c
        g2 = half(g1)
        g3 = half(g2)
        dev = self.device

        def z(g, c):
            return torch.zeros((n, *g, c), dtype=BF16, device=dev)
        b = {}
        b["e1a"], b["cat1"], b["l2in"] = z(g1, c1), z(g1, c2 + c1), z(g2, c1)
        b["e2a"], b["cat2"], b["l3in"] = z(g2, c2), z(g2, c3 + c2), z(g3, c2)
        b["e3a"], b["e3b"] = z(g3, c3), z(g3, c3)
        b["d2a"], b["d2b"] = z(g2, c2), z(g2, c2)
        b["d1a"], b["d1b"] = z(g1, c1), z(g1, c1)
        b["out"] = torch.zeros((n, *(2 * s for s in g1)), dtype=F32, device=dev)
        for k in ("d1b", "d1a", "cat1", "d2b", "d2a", "cat2", "e3b", "e3a", "l3in", "e2a", "l2in", "e1a"):
            b["g_" + k] = torch.zeros_like(b[k])
        b["g_pool2"] = z(g2, c2)
        b["g_pool1"] = z(g1, c1)
        self.buf = b
        self.shape = (n, tuple(g1))

    # ---------------------------------------------------------------- forward
    def _conv(self, layer: Conv3, x, xoff, y, yoff, relu=True, s=None):
        call("srf_conv3d_fwd", ptr(x), act(x, xoff), i32(layer.cin), ptr(layer.wb), ptr(layer.b),
             i32(layer.cout), i32(1 if relu else 0), ptr(y), act(y, yoff), None, s)

    def _fine(self):
        return (ctypes.c_int32 * 3)(*self.buf["out"].shape[1:])

    def forward(self, inp: torch.Tensor) -> torch.Tensor:
        """inp: (N, D, H, W, 16) bfloat16 -> (N, 2D, 2H, 2W) float32."""
        if inp.dim() != 5 or inp.shape[-1] != self.IN_CH or inp.dtype != BF16:
            raise ValueError(f"expected (N, D, H, W, {self.IN_CH}) bfloat16, got {tuple(inp.shape)} {inp.dtype}")
        dv = self.device
        if inp.device.type != dv.type or (dv.index is not None and inp.device.index != dv.index) \
                or not inp.is_contiguous():
            raise ValueError(f"input must be a contiguous tensor on {self.device}")
        n, d, h, w, c = inp.shape
        self._alloc(n, (d, h, w))
        self._inp = inp
        b, s = self.buf, stream_ptr(self.device)
        c1, c2, c3 = self.c
        self._conv(self.e1a, inp, 0, b["e1a"], 0, s=s)
        self._conv(self.e1b, b["e1a"], 0, b["cat1"], c2, s=s)
        call("srf_cnn_pool2", ptr(b["cat1"]), act(b["cat1"], c2), ptr(b["l2in"]), act(b["l2in"]), i32(c1), i32(0), s)
        self._conv(self.e2a, b["l2in"], 0, b["e2a"], 0, s=s)
        self._conv(self.e2b, b["e2a"], 0, b["cat2"], c3, s=s)
        call("srf_cnn_pool2", ptr(b["cat2"]), act(b["cat2"], c3), ptr(b["l3in"]), act(b["l3in"]), i32(c2), i32(0), s)
        self._conv(self.e3a, b["l3in"], 0, b["e3a"], 0, s=s)
        self._conv(self.e3b, b["e3a"], 0, b["e3b"], 0, s=s)
        call("srf_cnn_upsample2", ptr(b["e3b"]), act(b["e3b"]), ptr(b["cat2"]), act(b["cat2"], 0), i32(c3), i32(0), s)
        self._conv(self.d2a, b["cat2"], 0, b["d2a"], 0, s=s)
        self._conv(self.d2b, b["d2a"], 0, b["d2b"], 0, s=s)
        call("srf_cnn_upsample2", ptr(b["d2b"]), act(b["d2b"]), ptr(b["cat1"]), act(b["cat1"], 0), i32(c2), i32(0), s)
        self._conv(self.d1a, b["cat1"], 0, b["d1a"], 0, s=s)
        self._conv(self.d1b, b["d1a"], 0, b["d1b"], 0, s=s)
        call("srf_cnn_head8", ptr(b["d1b"]), act(b["d1b"]), i32(c1), ptr(self.hw), ptr(self.hb),
             ptr(b["out"]), self._fine(), None, None, None, None, None, s)
        return b["out"]

    # ---------------------------------------------------------------- backward
    def _conv_bwd(self, layer: Conv3, x, xoff, y, yoff, gy, gyoff, gx, gxoff, s):
        """gy: gradient at the layer output (post-ReLU values y); writes gx unless None."""
        call("srf_cnn_relu_bwd", ptr(gy), act(gy, gyoff), ptr(y), act(y, yoff), i32(layer.cout), s)
        call("srf_cnn_bias_grad", ptr(gy), act(gy, gyoff), i32(layer.cout), ptr(layer.gb), s)
        call("srf_conv3d_wgrad", ptr(x), act(x, xoff), i32(layer.cin), ptr(gy), act(gy, gyoff),
             i32(layer.cout), ptr(layer.gw), s)
        if gx is not None:
            call("srf_conv3d_fwd", ptr(gy), act(gy, gyoff), i32(layer.cout), ptr(layer.wf), None,
                 i32(layer.cin), i32(0), ptr(gx), act(gx, gxoff), None, s)

    def backward(self, gout: torch.Tensor) -> None:
        """Accumulate parameter gradients for d(loss)/d(out) = gout (N, 2D, 2H, 2W) float32."""
        b, s = self.buf, stream_ptr(self.device)
        c1, c2, c3 = self.c
        call("srf_cnn_head8", ptr(b["d1b"]), act(b["d1b"]), i32(c1), ptr(self.hw), ptr(self.hb), None,
             self._fine(), ptr(gout.contiguous()), ptr(b["g_d1b"]), act(b["g_d1b"]), ptr(self.ghw),
             ptr(self.ghb), s)
        self._conv_bwd(self.d1b, b["d1a"], 0, b["d1b"], 0, b["g_d1b"], 0, b["g_d1a"], 0, s)
        self._conv_bwd(self.d1a, b["cat1"], 0, b["d1a"], 0, b["g_d1a"], 0, b["g_cat1"], 0, s)
        call("srf_cnn_upsample2", ptr(b["g_d2b"]), act(b["g_d2b"]), ptr(b["g_cat1"]), act(b["g_cat1"], 0), i32(c2), i32(1), s)
        self._conv_bwd(self.d2b, b["d2a"], 0, b["d2b"], 0, b["g_d2b"], 0, b["g_d2a"], 0, s)
        self._conv_bwd(self.d2a, b["cat2"], 0, b["d2a"], 0, b["g_d2a"], 0, b["g_cat2"], 0, s)
        call("srf_cnn_upsample2", ptr(b["g_e3b"]), act(b["g_e3b"]), ptr(b["g_cat2"]), act(b["g_cat2"], 0), i32(c3), i32(1), s)
        self._conv_bwd(self.e3b, b["e3a"], 0, b["e3b"], 0, b["g_e3b"], 0, b["g_e3a"], 0, s)
        self._conv_bwd(self.e3a, b["l3in"], 0, b["e3a"], 0, b["g_e3a"], 0, b["g_l3in"], 0, s)
        # e2b feeds the pool and the skip: gradient = skip slice + pool adjoint
        call("srf_cnn_pool2", ptr(b["g_pool2"]), act(b["g_pool2"]), ptr(b["g_l3in"]), act(b["g_l3in"]), i32(c2), i32(1), s)
        call("srf_cnn_add", ptr(b["g_cat2"]), act(b["g_cat2"], c3), ptr(b["g_pool2"]), act(b["g_pool2"]), i32(c2), s)
        self._conv_bwd(self.e2b, b["e2a"], 0, b["cat2"], c3, b["g_cat2"], c3, b["g_e2a"], 0, s)
        self._conv_bwd(self.e2a, b["l2in"], 0, b["e2a"], 0, b["g_e2a"], 0, b["g_l2in"], 0, s)
        call("srf_cnn_pool2", ptr(b["g_pool1"]), act(b["g_pool1"]), ptr(b["g_l2in"]), act(b["g_l2in"]), i32(c1), i32(1), s)
        call("srf_cnn_add", ptr(b["g_cat1"]), act(b["g_cat1"], c2), ptr(b["g_pool1"]), act(b["g_pool1"]), i32(c1), s)
        self._conv_bwd(self.e1b, b["e1a"], 0, b["cat1"], c2, b["g_cat1"], c2, b["g_e1a"], 0, s)
        self._conv_bwd(self.e1a, self._inp, 0, b["e1a"], 0, b["g_e1a"], 0, None, 0, s)

    # ---------------------------------------------------------------- optimiser
    def zero_grad(self) -> None:
        for c in self.convs:
            c.gw.zero_()
            c.gb.zero_()
        self.ghw.zero_()
        self.ghb.zero_()

    def all_params(self) -> List[Tuple[torch.Tensor, torch.Tensor, Optional[torch.Tensor]]]:
        ps = []
        for c in self.convs:
            ps += c.params()
        ps += [(self.hw, self.ghw, None), (self.hb, self.ghb, None)]
        return ps

    def step(self, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
        self.step_count += 1
        s = stream_ptr(self.device)
        for k, (w, g, bf) in enumerate(self.all_params()):
            if k not in self.adam:
                self.adam[k] = (torch.zeros_like(w), torch.zeros_like(w))
            m, v = self.adam[k]
            call("srf_cnn_adam", ptr(w), ptr(m), ptr(v), ptr(g), ptr(bf), i64(w.numel()), f32(lr),
                 f32(b1), f32(b2), f32(eps), i32(self.step_count), s)
        for c in self.convs:
            c.refresh(s)

    def loss(self, pred: torch.Tensor, target: torch.Tensor, mask: Optional[torch.Tensor],
             inv_den: torch.Tensor, grad: Optional[torch.Tensor]) -> torch.Tensor:
        """Relative squared error averaged over samples (FP64 device scalar); fills its gradient."""
        out = torch.zeros(1, dtype=torch.float64, device=pred.device)
        n = pred.shape[0]
        call("srf_cnn_rel_mse", ptr(pred.contiguous()), ptr(target.contiguous()),
             ptr(mask.contiguous() if mask is not None else None), ptr(inv_den.contiguous()),
             i64(pred[0].numel()), i32(n), ptr(grad), ptr(out), stream_ptr(pred.device))
        return out


# ---------------------------------------------------------------- weights
def save_weights(net: UNet3D, path: str, meta: Dict[str, float]) -> None:
    """FP32 master weights and metadata (numpy .npz, no pickled objects)."""
    import numpy as np
    arrs = {}
    for name in ("e1a", "e1b", "e2a", "e2b", "e3a", "e3b", "d2a", "d2b", "d1a", "d1b"):
        c = getattr(net, name)
        arrs[name + ".w"] = c.w.cpu().numpy()
        arrs[name + ".b"] = c.b.cpu().numpy()
    arrs["head.w"] = net.hw.cpu().numpy()
    arrs["head.b"] = net.hb.cpu().numpy()
    arrs["channels"] = np.asarray(net.c, np.int64)
    for k, v in meta.items():
        arrs["meta." + k] = np.asarray(v, np.float64)
    np.savez(path, **arrs)


def load_weights(path: str, device="cuda") -> Tuple[UNet3D, Dict[str, float]]:
    import numpy as np
    z = np.load(path, allow_pickle=False)
    net = UNet3D(channels=tuple(int(c) for c in z["channels"]), device=device)
    for name in ("e1a", "e1b", "e2a", "e2b", "e3a", "e3b", "d2a", "d2b", "d1a", "d1b"):
        c = getattr(net, name)
        c.w.copy_(torch.as_tensor(z[name + ".w"]))
        c.b.copy_(torch.as_tensor(z[name + ".b"]))
        c.wb.copy_(c.w.to(BF16))
    net.hw.copy_(torch.as_tensor(z["head.w"]))
    net.hb.copy_(torch.as_tensor(z["head.b"]))
    s = stream_ptr(net.device)
    for c in net.convs:
        c.refresh(s)
    meta = {k[5:]: float(z[k]) for k in z.files if k.startswith("meta.")}
    return net, meta


DEFAULT_WEIGHTS = __file__.rsplit("/", 1)[0] + "/weights/scatter_unet.npz"
DEFAULT_GUARD = __file__.rsplit("/", 1)[0] + "/weights/scatter_guard.json"


# ---------------------------------------------------------------- surrogate with SSS as the judge
def correction_basis(device) -> torch.Tensor:
    """(9, 51 * 52 * 312) FP32 smooth functions of a bin's position in the coarse sinogram, the
    basis of the spot-check correction: 1, the radial offset and the plane (each to second order,
    normalised to [-1, 1]), and the first and second harmonics of the LOR's mid-point angle
    psi = 2 pi (view + 39 + 1.5 radial) / 312, the crystals of a bin sitting at views v and
    v + 78 + 3 radial (bins are (plane, radial, view), view fastest)."""
    from .scatter_sinogram import PLANES, RADIAL, RADIAL_OFF, RADIAL_STEP, VIEWS
    P, R, V = PLANES - 1, RADIAL, VIEWS
    shape = (P, R, V)
    p = torch.arange(P, dtype=torch.float64, device=device).view(P, 1, 1).expand(shape).reshape(-1)
    r = torch.arange(R, dtype=torch.float64, device=device).view(1, R, 1).expand(shape).reshape(-1)
    v = torch.arange(V, dtype=torch.float64, device=device).view(1, 1, V).expand(shape).reshape(-1)
    pn = (p - 0.5 * (P - 1)) / (0.5 * (P - 1))
    rn = (r - 0.5 * (R - 1)) / (0.5 * (R - 1))
    psi = (2.0 * math.pi / V) * (v + 0.5 * (V // 2 - RADIAL_OFF) + 0.5 * RADIAL_STEP * r)
    rows = [torch.ones_like(p), rn, rn * rn, pn, pn * pn, torch.cos(psi), torch.sin(psi),
            torch.cos(2 * psi), torch.sin(2 * psi)]
    return torch.stack(rows, 0).to(F32).contiguous()


def _check_device_tensors(what: str, like: torch.Tensor, tensors) -> None:
    """Raise ValueError unless every tensor is a contiguous CUDA tensor of its dtype on the device
    of ``like`` (the kernels take raw pointers: a wrong one would reach the GPU unchecked)."""
    for name, (t, dtype) in tensors.items():
        if not t.is_cuda or t.device != like.device:
            raise ValueError(f"{what}: {name} must be a CUDA tensor on {like.device}")
        if not t.is_contiguous():
            raise ValueError(f"{what}: {name} must be contiguous")
        if t.dtype != dtype:
            raise ValueError(f"{what}: {name} must be {dtype}, got {t.dtype}")


def spot_fit(pred: torch.Tensor, bins: torch.Tensor, ref: torch.Tensor, basis: torch.Tensor,
             out: torch.Tensor, ridge: float = 1e-6) -> None:
    """srf_spot_fit: out[:k] = coefficients of the correction pred * (beta . basis) fitted to the
    even spot samples (bins, ref), out[k] / out[k + 1] = relative L2 difference of the corrected /
    uncorrected prediction on the odd samples. Asynchronous on the current stream."""
    k, nb = basis.shape
    _check_device_tensors("spot_fit", pred, {"pred": (pred, F32), "bins": (bins, torch.int64),
                                             "ref": (ref, F32), "basis": (basis, F32), "out": (out, F32)})
    if pred.numel() != nb or out.numel() < k + 2 or bins.numel() != ref.numel():
        raise ValueError("spot_fit: pred must have one entry per basis column, out at least k + 2 "
                         "entries, and bins one entry per ref sample")
    call("srf_spot_fit", ptr(pred), i64(nb), ptr(bins), ptr(ref), i32(bins.numel()), ptr(basis), i32(k),
         f64(ridge), ptr(out), stream_ptr(pred.device))


def scale_by_basis(x: torch.Tensor, basis: torch.Tensor, beta: torch.Tensor) -> None:
    """srf_scale_by_basis: x *= beta . basis, in place (beta on the device)."""
    k, nb = basis.shape
    _check_device_tensors("scale_by_basis", x, {"x": (x, F32), "basis": (basis, F32), "beta": (beta, F32)})
    if x.numel() != nb or beta.numel() < k:
        raise ValueError("scale_by_basis: x must have one entry per basis column and beta at least k")
    call("srf_scale_by_basis", ptr(x), i64(nb), ptr(basis), i32(k), ptr(beta), stream_ptr(x.device))


class ScatterSurrogate:
    """Coarse-sinogram scatter estimate from the network, checked against SSS on a few bins.

    ``estimate(emission, mu)`` returns the flat (51 * 52 * 312) scatter sinogram in SSS units and
    a record of what happened. A fresh SSS on ``spot_bins`` random bins serves twice: on the even
    samples it fits a smooth multiplicative correction (``correction_basis``: global scale,
    radial and plane trends, first and second view harmonics), and on the odd samples, which the
    fit has not seen, it judges the corrected prediction. The record holds that judged relative
    L2 difference, the uncorrected one, the coefficients, and whether the judged difference
    exceeded ``fallback_tol`` so that the full SSS was returned instead. The spot-check SSS runs
    on a side stream while the network runs on the caller's stream; the only host
    synchronisation is one read of the spot samples."""

    N_POOLS = 8
    POOL_POSITIONS = 48

    def __init__(self, geo, net: UNet3D, target_scale: float, fallback_tol: float = 0.05,
                 spot_bins: int = 2048, seed: int = 0):
        self.geo, self.net, self.k = geo, net, float(target_scale)
        self.fallback_tol, self.spot_bins = fallback_tol, spot_bins
        self.gen = torch.Generator(device=geo.device).manual_seed(seed)
        self.side = torch.cuda.Stream(geo.device)
        self.pools = self._make_pools(seed)
        self.calls = 0
        self._graph = self._graph_out = self._em_in = self._mu_in = None
        self._spot_graphs = [None] * self.N_POOLS
        self._pick = torch.zeros(spot_bins, dtype=torch.int64, device=geo.device)
        self.basis = correction_basis(geo.device)
        k = self.basis.shape[0]
        self._fit = torch.zeros(k + 2, dtype=F32, device=geo.device)      # beta, judged, uncorrected
        self._fit_host = torch.zeros(k + 2, dtype=F32).pin_memory()

    def _make_pools(self, seed: int):
        """Spot-check pools, built once: each is a random set of 48 of the 312 transaxial
        positions (all rings), its 1,248 virtual crystals and every bin whose two crystals lie in
        it (as indices into those crystals). A spot check samples bins of one pool, so its SSS
        preprocesses 1,248 crystals instead of 8,112 while the bins still cover every plane,
        radius and 48 views."""
        geo = self.geo
        rng = np.random.default_rng(seed)
        pools = []
        pairs = geo.pairs.astype(np.int64)
        for _ in range(self.N_POOLS):
            pos = np.sort(rng.choice(geo.vt, self.POOL_POSITIONS, replace=False))
            crystals = (np.arange(geo.vr)[:, None] * geo.vt + pos[None, :]).reshape(-1)
            local = np.full(geo.vt * geo.vr, -1, np.int64)
            local[crystals] = np.arange(crystals.size)
            la, lb = local[pairs[:, 0]], local[pairs[:, 1]]
            cand = np.flatnonzero((la >= 0) & (lb >= 0))
            dev = geo.device
            pools.append((torch.as_tensor(cand, device=dev),
                          torch.as_tensor(np.stack([la[cand], lb[cand]], 1).astype(np.int32), device=dev),
                          geo.vpos_dev.index_select(0, torch.as_tensor(crystals, device=dev))))
        return pools

    @classmethod
    def load(cls, geo, path: str = DEFAULT_WEIGHTS, guard: Optional[str] = DEFAULT_GUARD,
             **kw) -> "ScatterSurrogate":
        """The network from ``path``; the fallback threshold from the guard calibration file
        ``guard`` (see calibrate_guard) unless ``fallback_tol`` is given."""
        import json
        import os
        net, meta = load_weights(path, geo.device)
        if "fallback_tol" not in kw and guard is not None and os.path.exists(guard):
            with open(guard) as f:
                kw["fallback_tol"] = float(json.load(f)["fallback_tol"])
        return cls(geo, net, meta["target_scale"], **kw)

    def _predict_eager(self, emission: torch.Tensor, mu: torch.Tensor) -> torch.Tensor:
        from .scatter_sinogram import crop_sino, network_input
        inp, scale = network_input(self.geo, emission, mu)
        out = self.net.forward(inp)                                     # (1, 56, 56, 320)
        return crop_sino(out)[0] * (self.k * scale)

    def predict(self, emission: torch.Tensor, mu: torch.Tensor) -> torch.Tensor:
        """The network's sinogram for these volumes. The whole chain (input projections, the
        U-Net, the output scaling: ~60 launches) is captured into a CUDA graph at the first call
        and replayed, because at batch 1 issuing it costs more than running it."""
        self._ensure_graph(emission, mu)
        self._em_in.copy_(emission)
        self._mu_in.copy_(mu)
        self._graph.replay()
        return self._graph_out.clone()

    def _ensure_graph(self, emission: torch.Tensor, mu: torch.Tensor) -> None:
        if self._graph is None or self._em_in.shape != emission.shape or self._mu_in.shape != mu.shape:
            self._spot_graphs = [None] * self.N_POOLS  # they read the input buffers made here
            self._em_in, self._mu_in = emission.clone(), mu.clone()
            dev = emission.device
            side = torch.cuda.Stream(dev)
            side.wait_stream(torch.cuda.current_stream(dev))
            with torch.cuda.stream(side):
                self._predict_eager(self._em_in, self._mu_in)  # builds caches and activation buffers
            torch.cuda.current_stream(dev).wait_stream(side)
            self._graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self._graph):
                self._graph_out = self._predict_eager(self._em_in, self._mu_in)
            # the graph writes into these activation buffers: keep them alive even if the network
            # later reallocates its buffers for another batch shape
            self._graph_bufs = dict(self.net.buf)

    def _spot_sss(self, emission: torch.Tensor, mu: torch.Tensor):
        """(bins, SSS of those bins) for ``spot_bins`` bins of the next pool; asynchronous."""
        from .scatter_sinogram import sss_pairs
        cand, local, cpos = self.pools[self.calls % self.N_POOLS]
        self.calls += 1
        pick = torch.randint(0, cand.numel(), (self.spot_bins,), generator=self.gen, device=cand.device)
        return cand.index_select(0, pick), sss_pairs(self.geo, emission, mu, cpos, local.index_select(0, pick))

    @staticmethod
    def _rel(p: torch.Tensor, ref: torch.Tensor) -> torch.Tensor:
        return torch.linalg.vector_norm(p - ref) / torch.linalg.vector_norm(ref).clamp_min(1e-30)

    def spot_check(self, emission: torch.Tensor, mu: torch.Tensor, pred: torch.Tensor) -> float:
        bins, ref = self._spot_sss(emission, mu)
        return float(self._rel(pred.index_select(0, bins), ref).item())

    def _spot_graph(self, j: int):
        """Spot-check SSS of pool j on the bins self._pick selects, for the volumes in the
        prediction graph's input buffers, captured into a CUDA graph at first use (its ~25
        launches would otherwise be issued one by one). Returns (graph, bins, sss)."""
        if self._spot_graphs[j] is None:
            from .scatter_sinogram import sss_pairs
            cand, local, cpos = self.pools[j]

            def run():
                return (cand.index_select(0, self._pick),
                        sss_pairs(self.geo, self._em_in, self._mu_in, cpos, local.index_select(0, self._pick)))
            self._pick.zero_()
            side = torch.cuda.Stream(self.geo.device)
            side.wait_stream(torch.cuda.current_stream(self.geo.device))
            with torch.cuda.stream(side):
                run()
            torch.cuda.current_stream(self.geo.device).wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                bins, ref = run()
            self._spot_graphs[j] = (g, bins, ref)
        return self._spot_graphs[j]

    def estimate(self, emission: torch.Tensor, mu: torch.Tensor, fallback: bool = True):
        """(sinogram, record). With ``fallback=False`` the corrected prediction is returned even
        when its spot check failed (the record still says so). The prediction and the spot-check
        SSS are two graph launches on two streams, so they run side by side."""
        from .scatter_sinogram import sss_sinogram
        dev = self.geo.device
        main = torch.cuda.current_stream(dev)
        self._ensure_graph(emission, mu)
        j = self.calls % self.N_POOLS
        self.calls += 1
        g, bins, ref = self._spot_graph(j)
        self._em_in.copy_(emission)
        self._mu_in.copy_(mu)
        ready = torch.cuda.Event()
        ready.record(main)
        self._graph.replay()
        pred = self._graph_out.clone()
        with torch.cuda.stream(self.side):
            self.side.wait_event(ready)
            n_c = self.pools[j][0].numel()
            self._pick.copy_(torch.randint(0, n_c, (self.spot_bins,), generator=self.gen, device=dev))
            g.replay()
        main.wait_stream(self.side)
        # fit and judge the correction, apply it (discarded if the judge fails), read k + 2 numbers
        k = self.basis.shape[0]
        spot_fit(pred, bins, ref, self.basis, self._fit)
        scale_by_basis(pred, self.basis, self._fit)
        self._fit_host.copy_(self._fit, non_blocking=True)
        done = torch.cuda.Event()
        done.record(main)
        done.synchronize()
        h = self._fit_host.tolist()
        err = h[k]
        info = {"spot_rel_l2": err, "spot_rel_l2_uncorrected": h[k + 1], "correction": h[:k],
                "fallback": False}
        if not (err <= self.fallback_tol):
            if fallback:
                info["fallback"] = True
                return sss_sinogram(self.geo, emission, mu), info
            info["spot_failed"] = True
        return pred, info


# ---------------------------------------------------------------- training
def build_dataset(geo, seeds, log=None):
    """Network inputs (N, 28, 28, 160, 16) bf16, targets (N, 56, 56, 320) FP32 in units of each
    study's emission scale, and the scales."""
    from .scatter_sinogram import HALF_GRID, PAD_GRID, network_input, random_phantom, sss_sinogram, target_full
    n = len(seeds)
    dev = geo.device
    X = torch.empty((n, *HALF_GRID, UNet3D.IN_CH), dtype=BF16, device=dev)
    T = torch.empty((n, *PAD_GRID), dtype=F32, device=dev)
    scales = torch.empty(n, dtype=torch.float64)
    for i, sd in enumerate(seeds):
        em, mu = random_phantom(int(sd), device=dev)
        sc = sss_sinogram(geo, em, mu)
        inp, scale = network_input(geo, em, mu)
        X[i] = inp[0]
        T[i] = target_full(sc, scale)
        scales[i] = float(scale)
        if log and (i + 1) % 200 == 0:
            log(f"dataset {i + 1}/{n}")
    return X, T, scales


def corrected_targets(net: UNet3D, X: torch.Tensor, T0: torch.Tensor, batch: int = 4) -> torch.Tensor:
    """Targets for training towards the spot-corrected estimate: per sample T0 / c, where
    c = B beta is the smooth factor of the spot-check correction basis B (normalised to mean 1
    over the bins, floored at 0.2) that maps the network's current prediction closest to T0 by
    least squares over the real bins. The network then spends its capacity on what the
    correction cannot supply."""
    from .scatter_sinogram import PLANES, RADIAL, VIEWS, crop_sino, pad_sino
    B = correction_basis(X.device).double()
    out = torch.empty_like(T0)
    n = X.shape[0]
    for j in range(0, n, batch):
        k = min(batch, n - j)
        p = crop_sino(net.forward(X[j:j + k].contiguous())).double()
        t = crop_sino(T0[j:j + k]).double()
        A = torch.einsum("kb,sb,lb->skl", B, p * p, B)
        r = torch.einsum("kb,sb->sk", B, p * t)
        beta = torch.linalg.solve(A + 1e-12 * torch.eye(B.shape[0], dtype=A.dtype, device=A.device), r)
        c = beta @ B
        c = (c / c.mean(dim=1, keepdim=True)).clamp_min(0.2)
        out[j:j + k] = pad_sino((t / c).reshape(k, PLANES - 1, RADIAL, VIEWS).float())
    return out


def train(net: UNet3D, X: torch.Tensor, T: torch.Tensor, mask: torch.Tensor, epochs: int,
          batch: int = 4, lr: float = 2e-3, seed: int = 0, log=None, every=None,
          retarget=None) -> List[float]:
    """Adam on the masked relative squared error, cosine-decayed learning rate; ``every(epoch)``
    runs after each epoch (monitoring); ``retarget(epoch)`` may return new targets for the
    following epochs."""
    n = X.shape[0]
    g = torch.Generator().manual_seed(seed)
    inv_den = 1.0 / (T * T * mask).sum(dim=(1, 2, 3)).clamp_min(1e-30)
    steps = epochs * (n // batch)
    grad = torch.empty((batch, *T.shape[1:]), dtype=F32, device=X.device)
    hist, run, k = [], 0.0, 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).to(X.device)
        for j in range(n // batch):
            idx = perm[j * batch:(j + 1) * batch]
            frac = k / max(steps - 1, 1)
            cur = lr * min(1.0, (k + 1) / 100) * 0.5 * (1 + math.cos(math.pi * frac))
            out = net.forward(X.index_select(0, idx).contiguous())
            l = net.loss(out, T.index_select(0, idx).contiguous(), mask, inv_den.index_select(0, idx).contiguous(), grad)
            net.zero_grad()
            net.backward(grad)
            net.step(cur)
            run += float(l.item()) if (k % 50 == 0) else 0.0
            k += 1
        hist.append(float(net.loss(net.forward(X[:batch].contiguous()), T[:batch].contiguous(), mask,
                                   inv_den[:batch].contiguous(), None).item()))
        if log:
            log(f"epoch {ep + 1}/{epochs} loss(first batch) {hist[-1]:.5f}")
        if every:
            every(ep + 1)
        if retarget is not None and ep + 1 < epochs:
            nt = retarget(ep + 1)
            if nt is not None:
                T = nt
                inv_den = 1.0 / (T * T * mask).sum(dim=(1, 2, 3)).clamp_min(1e-30)
    return hist


def evaluate_corrected(sur: "ScatterSurrogate", seeds) -> List[float]:
    """Full-resolution relative L2 of the spot-corrected estimate against the full SSS."""
    from .scatter_sinogram import random_phantom, sss_sinogram
    errs = []
    for sd in seeds:
        em, mu = random_phantom(int(sd), device=sur.geo.device)
        ref = sss_sinogram(sur.geo, em, mu)
        p, _ = sur.estimate(em, mu, fallback=False)
        errs.append(float((torch.linalg.vector_norm(p - ref) / torch.linalg.vector_norm(ref)).item()))
    return errs


def evaluate(sur: "ScatterSurrogate", seeds) -> List[float]:
    """Full-resolution relative L2 of the prediction against the full SSS, per held-out seed."""
    from .scatter_sinogram import random_phantom, sss_sinogram
    errs = []
    for sd in seeds:
        em, mu = random_phantom(int(sd), device=sur.geo.device)
        ref = sss_sinogram(sur.geo, em, mu)
        p = sur.predict(em, mu)
        errs.append(float((torch.linalg.vector_norm(p - ref) / torch.linalg.vector_norm(ref)).item()))
    return errs


def guard_threshold(records, image_target: float, margin: float) -> float:
    """The largest spot-check difference s such that every calibration study whose judged spot
    difference is at most s kept its OSEM image within margin * image_target of the SSS-corrected
    image (records: (spot_rel_l2, image_rel_l2) pairs). Never above the largest difference seen;
    below the smallest when even that study missed the bound (then everything falls back)."""
    bound = margin * image_target
    tol = None
    for spot, img in sorted(records):
        if img > bound:
            break
        tol = spot
    if tol is None:
        return 0.0
    return float(tol)


def calibrate_guard(sur: "ScatterSurrogate", seeds, image_target: float = 0.01, margin: float = 0.75,
                    n_trues: int = 2_000_000, log=None) -> Dict:
    """Calibrate the fallback threshold on the OSEM image, the quantity the surrogate must keep
    within ``image_target`` of SSS: for each calibration phantom (seeds apart from the training and
    held-out ones) a ScatterStudy is reconstructed with SSS scatter and with the corrected network
    estimate, and the image difference is paired with the spot check's judged difference."""
    from .scatter_sinogram import ScatterStudy
    recs = []
    for sd in seeds:
        study = ScatterStudy(sur.geo, int(sd), n_trues=n_trues)
        est, info = sur.estimate(study.emission, study.mu, fallback=False)
        img_sss = study.reconstruct(study.sss)
        img_sur = study.reconstruct(est)
        err = float((torch.linalg.vector_norm(img_sur - img_sss) / torch.linalg.vector_norm(img_sss)).item())
        recs.append({"seed": int(sd), "spot_rel_l2": float(info["spot_rel_l2"]), "image_rel_l2": err})
        if log:
            log(f"seed {sd}: spot {info['spot_rel_l2']:.4f} image {err:.5f}")
    tol = guard_threshold([(r["spot_rel_l2"], r["image_rel_l2"]) for r in recs], image_target, margin)
    return {"fallback_tol": tol, "image_target": image_target, "margin": margin, "n_trues": n_trues,
            "studies": recs}


def main(argv=None) -> None:
    """python -m srf_gb300.surrogate --out weights.npz [--train 2000 --held-out 200 --epochs N]
    python -m srf_gb300.surrogate --calibrate guard.json [--studies 40]"""
    import argparse
    import json
    import time
    from . import synth
    from .scatter_sinogram import CoarseGeometry, full_mask
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--train", type=int, default=2000)
    ap.add_argument("--held-out", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--channels", default="32,64,96")
    ap.add_argument("--corrected", type=int, default=0,
                    help="after this many epochs, train towards the spot-corrected estimate "
                         "(targets refreshed every 5 epochs); 0: plain targets")
    ap.add_argument("--calibrate", default=None, help="write the guard calibration to this file")
    ap.add_argument("--studies", type=int, default=40, help="calibration phantoms")
    a = ap.parse_args(argv)
    log = lambda m: print(f"[{time.strftime('%H:%M:%S')}] {m}", flush=True)
    dev = torch.device("cuda", 0)
    geo = CoarseGeometry(synth.scanner_clinical(), device=dev)
    if a.calibrate:
        # calibration phantoms: seeds 3,000,000 + i (training uses 0.., held-out 1,000,000 + i)
        sur = ScatterSurrogate.load(geo, a.out, guard=None)
        rec = calibrate_guard(sur, range(3_000_000, 3_000_000 + a.studies), log=log)
        with open(a.calibrate, "w") as f:
            json.dump(rec, f, indent=1)
        log(f"fallback_tol {rec['fallback_tol']:.4f}")
        return
    t0 = time.time()
    X, T, scales = build_dataset(geo, range(a.train), log)
    torch.cuda.synchronize()
    log(f"dataset built in {time.time() - t0:.1f} s")
    mask = full_mask(dev)
    k = float(((T * mask).sum() / (mask.sum() * T.shape[0])).item())
    T /= k
    net = UNet3D(channels=tuple(int(c) for c in a.channels.split(",")), seed=1, device=dev)
    log(f"parameters {net.n_params()}")
    sur = ScatterSurrogate(geo, net, k)
    mon = range(1_000_000, 1_000_000 + 10)

    def every(ep):
        if ep % 5 == 0 or ep == a.epochs:
            e = evaluate(sur, mon)
            c = evaluate_corrected(sur, mon)
            log(f"epoch {ep}: held-out rel L2 mean {sum(e) / len(e):.4f} max {max(e):.4f}; "
                f"corrected mean {sum(c) / len(c):.4f} max {max(c):.4f}")

    T0 = T

    def retarget(ep):
        if a.corrected and ep >= a.corrected and (ep - a.corrected) % 5 == 0:
            log(f"epoch {ep}: targets towards the corrected estimate")
            return corrected_targets(net, X, T0, a.batch)
        return None

    t0 = time.time()
    hist = train(net, X, T, mask, a.epochs, a.batch, a.lr, log=log, every=every, retarget=retarget)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    del X, T, T0
    errs = evaluate(sur, range(1_000_000, 1_000_000 + a.held_out))
    cerrs = evaluate_corrected(sur, range(1_000_000, 1_000_000 + min(a.held_out, 100)))
    meta = {"target_scale": k, "train_studies": a.train, "epochs": a.epochs, "train_s": t_train,
            "corrected_from_epoch": a.corrected,
            "held_out_mean_rel_l2": sum(errs) / len(errs), "held_out_max_rel_l2": max(errs),
            "held_out_corrected_mean_rel_l2": sum(cerrs) / len(cerrs)}
    save_weights(net, a.out, meta)
    print(json.dumps({**meta, "loss_history": hist}))


if __name__ == "__main__":
    main()
