"""CPU oracle for the scatter-surrogate network kernels. TEST INFRASTRUCTURE ONLY.

float64 numpy restatements of 3x3x3 'same' convolution (NDHWC activations, [Cout][27][Cin]
weights, tap t <-> offsets (t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1)), its data and weight
gradients, 2x2x2 average pooling and nearest 2x upsampling with their adjoints. The reference
(srfnef) has no network; these define the arithmetic the GPU kernels must reproduce.
"""
from __future__ import annotations

import numpy as np

TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def _shifted(x, dz, dy, dx):
    """x shifted so that out[v] = x[v + (dz, dy, dx)], zero outside."""
    n, d, h, w, c = x.shape
    xp = np.zeros((n, d + 2, h + 2, w + 2, c), dtype=np.float64)
    xp[:, 1:-1, 1:-1, 1:-1] = x
    return xp[:, 1 + dz:1 + dz + d, 1 + dy:1 + dy + h, 1 + dx:1 + dx + w]


def conv3d(x, w, b=None, relu=False):
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    y = np.zeros(x.shape[:4] + (w.shape[0],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        y += _shifted(x, dz, dy, dx) @ w[:, t, :].T
    if b is not None:
        y += np.asarray(b, np.float64)
    return np.maximum(y, 0.0) if relu else y


def conv3d_wgrad(x, dy):
    x = np.asarray(x, np.float64)
    dy = np.asarray(dy, np.float64)
    co, ci = dy.shape[-1], x.shape[-1]
    dw = np.zeros((co, 27, ci))
    for t, (dz, dyo, dx) in enumerate(TAPS):
        xs = _shifted(x, dz, dyo, dx).reshape(-1, ci)
        dw[:, t, :] = dy.reshape(-1, co).T @ xs
    return dw


def conv3d_dgrad(dy, w):
    """Gradient w.r.t. the input of conv3d (no bias/activation)."""
    dy = np.asarray(dy, np.float64)
    w = np.asarray(w, np.float64)
    dx_ = np.zeros(dy.shape[:4] + (w.shape[2],))
    for t, (dz, dyo, dx) in enumerate(TAPS):
        dx_ += _shifted(dy, -dz, -dyo, -dx) @ w[:, t, :]
    return dx_


def pool2(x):
    n, d, h, w, c = x.shape
    D, H, W = (d + 1) // 2, (h + 1) // 2, (w + 1) // 2
    xp = np.zeros((n, 2 * D, 2 * H, 2 * W, c))
    xp[:, :d, :h, :w] = x
    return xp.reshape(n, D, 2, H, 2, W, 2, c).sum(axis=(2, 4, 6)) / 8.0


def pool2_adjoint(g, fine_shape):
    n, d, h, w, c = fine_shape
    up = np.repeat(np.repeat(np.repeat(g, 2, 1), 2, 2), 2, 3) / 8.0
    return up[:, :d, :h, :w]


def upsample2(x, fine_shape):
    n, d, h, w, c = fine_shape
    return np.repeat(np.repeat(np.repeat(x, 2, 1), 2, 2), 2, 3)[:, :d, :h, :w]


def upsample2_adjoint(g, coarse_shape):
    n, D, H, W, c = coarse_shape
    gp = np.zeros((n, 2 * D, 2 * H, 2 * W, c))
    gp[:, :g.shape[1], :g.shape[2], :g.shape[3]] = g
    return gp.reshape(n, D, 2, H, 2, W, 2, c).sum(axis=(2, 4, 6))


def head8(x, w, b, fine):
    """Sub-voxel head: out[n, 2z+i, 2y+j, 2x+k] = b[q] + x[n, z, y, x] . w[q], q = 4i + 2j + k,
    cropped to the fine grid."""
    x = np.asarray(x, np.float64)
    n, d, h, ww, c = x.shape
    o = np.einsum("ndhwc,qc->ndhwq", x, np.asarray(w, np.float64)) + np.asarray(b, np.float64)
    full = o.reshape(n, d, h, ww, 2, 2, 2).transpose(0, 1, 4, 2, 5, 3, 6).reshape(n, 2 * d, 2 * h, 2 * ww)
    D, H, W = fine
    return full[:, :D, :H, :W]


def head8_grads(x, w, gout):
    """(gx, gw, gb) of head8 for the fine-grid gradient gout."""
    x = np.asarray(x, np.float64)
    n, d, h, ww, c = x.shape
    D, H, W = gout.shape[1:]
    gp = np.zeros((n, 2 * d, 2 * h, 2 * ww))
    gp[:, :D, :H, :W] = gout
    gq = gp.reshape(n, d, 2, h, 2, ww, 2).transpose(0, 1, 3, 5, 2, 4, 6).reshape(n, d, h, ww, 8)
    gx = gq @ np.asarray(w, np.float64)
    gw = np.einsum("ndhwq,ndhwc->qc", gq, x)
    gb = gq.sum(axis=(0, 1, 2, 3))
    return gx, gw, gb


def spot_fit(pred, bins, ref, phi, ridge=1e-6):
    """The surrogate's spot-check correction (srf_spot_fit): beta minimising, over the even
    samples s, (ref[s] - pred[b] * beta . phi[:, b])^2 with b = bins[s], plus ridge * (trace / k)
    * |beta|^2 of the normal matrix; e0 when that matrix is zero. Samples with a bin outside
    [0, len(pred)) are left out. Returns (beta, judged, uncorrected): the relative L2 differences
    of the corrected and uncorrected prediction from ref over the odd samples."""
    pred = np.asarray(pred, np.float64)
    phi = np.asarray(phi, np.float64)
    bins = np.asarray(bins, np.int64)
    ref = np.asarray(ref, np.float64)
    k, nb = phi.shape
    keep = (bins >= 0) & (bins < nb)
    even = np.zeros(bins.size, bool)
    even[0::2] = True
    fi, ju = np.flatnonzero(even & keep), np.flatnonzero(~even & keep)
    a = pred[bins[fi]][None, :] * phi[:, bins[fi]]
    ata = a @ a.T
    tr = float(np.trace(ata))
    if tr > 0.0 and np.isfinite(tr):
        beta = np.linalg.solve(ata + (ridge * tr / k) * np.eye(k), a @ ref[fi])
    else:
        beta = np.eye(k)[0]
    p, y = pred[bins[ju]], ref[ju]
    den = max(float(np.linalg.norm(y)), 1e-30)
    judged = float(np.linalg.norm(p * (beta @ phi[:, bins[ju]]) - y)) / den
    return beta, judged, float(np.linalg.norm(p - y)) / den
