"""CPU oracle of the image-warping ops. TEST INFRASTRUCTURE ONLY (never imported by srf_gb300).

numpy float32 restatements, vectorised over voxels, of srfnef/cc/deform/deform.cu.cc:13-174
(plain rules: Deform, Shift, ShiftZ, Rotate) and deform_tex.cu.cc:15-100, 228-240, 290-370
(texture rules: a clamped, linearly filtered read at position + 0.5, with FP32 weights where the
texture unit uses 8-bit fractions; DeformInvert's 30-step fixed-point iteration). Images are
(nx, ny, nz) arrays; every function returns a new (nx, ny, nz) float32 array.
"""
from __future__ import annotations

import numpy as np

F = np.float32


def _grid(shape):
    """Voxel indices as float32 arrays (the kernels' int -> float conversions are exact)."""
    nx, ny, nz = shape
    ix, iy, iz = np.meshgrid(np.arange(nx, dtype=F), np.arange(ny, dtype=F), np.arange(nz, dtype=F),
                             indexing="ij")
    return ix, iy, iz


def _trilinear(img, xi, yi, zi, wx2, wy2, wz2):
    wx, wy, wz = F(1) - wx2, F(1) - wy2, F(1) - wz2
    g = lambda a, b, c: img[a, b, c]
    return (g(xi, yi, zi) * wx * wy * wz + g(xi, yi, zi + 1) * wx * wy * wz2 +
            g(xi, yi + 1, zi) * wx * wy2 * wz + g(xi, yi + 1, zi + 1) * wx * wy2 * wz2 +
            g(xi + 1, yi, zi) * wx2 * wy * wz + g(xi + 1, yi, zi + 1) * wx2 * wy * wz2 +
            g(xi + 1, yi + 1, zi) * wx2 * wy2 * wz + g(xi + 1, yi + 1, zi + 1) * wx2 * wy2 * wz2).astype(F)


def _plain(img, px, py, pz, lo, rotate=False, iz=None):
    nx, ny, nz = img.shape
    out = np.zeros(img.shape, F)
    xi = np.floor(px).astype(np.int64)
    yi = np.floor(py).astype(np.int64)
    zi = np.floor(pz).astype(np.int64)
    ok = (xi >= lo) & (xi + 1 < nx) & (yi >= lo) & (yi + 1 < ny)
    if not rotate:
        ok &= (zi >= lo) & (zi + 1 < nz)
    a, b, c = xi[ok], yi[ok], zi[ok]
    wx2 = (px[ok] - a).astype(F)
    wy2 = (py[ok] - b).astype(F)
    if rotate:
        z = iz[ok].astype(np.int64)
        wx, wy = F(1) - wx2, F(1) - wy2
        out[ok] = (img[a, b, z] * wx * wy + img[a, b + 1, z] * wx * wy2 + img[a + 1, b, z] * wx2 * wy +
                   img[a + 1, b + 1, z] * wx2 * wy2).astype(F)
    else:
        wz2 = (pz[ok] - c).astype(F)
        out[ok] = _trilinear(img, a, b, c, wx2, wy2, wz2)
    return out


def tex_sample(img, u, s, t):
    """Clamped linear texture read at unnormalised (u, s, t), FP32 weights."""
    nx, ny, nz = img.shape
    xb, yb, zb = (u - F(0.5)).astype(F), (s - F(0.5)).astype(F), (t - F(0.5)).astype(F)
    fx, fy, fz = np.floor(xb), np.floor(yb), np.floor(zb)
    a, b, c = (xb - fx).astype(F), (yb - fy).astype(F), (zb - fz).astype(F)
    cl = lambda v, n: np.clip(v, 0, n - 1).astype(np.int64)
    x0, x1 = cl(fx, nx), cl(fx + 1, nx)
    y0, y1 = cl(fy, ny), cl(fy + 1, ny)
    z0, z1 = cl(fz, nz), cl(fz + 1, nz)
    g = lambda i, j, k: img[i, j, k]
    c00 = g(x0, y0, z0) * (F(1) - a) + g(x1, y0, z0) * a
    c10 = g(x0, y1, z0) * (F(1) - a) + g(x1, y1, z0) * a
    c01 = g(x0, y0, z1) * (F(1) - a) + g(x1, y0, z1) * a
    c11 = g(x0, y1, z1) * (F(1) - a) + g(x1, y1, z1) * a
    c0 = c00 * (F(1) - b) + c10 * b
    c1 = c01 * (F(1) - b) + c11 * b
    return (c0 * (F(1) - c) + c1 * c).astype(F)


def _rot(shape, cos_phi, sin_phi):
    nx, ny, _ = shape
    ix, iy, iz = _grid(shape)
    cx, cy = F(nx // 2), F(ny // 2)
    u = ((ix + F(0.5)) - cx).astype(F)
    v = ((iy + F(0.5)) - cy).astype(F)
    px = (u * F(cos_phi) - v * F(sin_phi) + cx).astype(F)
    py = (u * F(sin_phi) + v * F(cos_phi) + cy).astype(F)
    return px, py, iz


def deform(img, mx, my, mz, texture=True):
    ix, iy, iz = _grid(img.shape)
    if texture:
        return tex_sample(img, (ix + mx + F(0.5)).astype(F), (iy + my + F(0.5)).astype(F),
                          (iz + mz + F(0.5)).astype(F))
    return _plain(img, (ix + mx).astype(F), (iy + my).astype(F), (iz + mz).astype(F), lo=1)


def shift(img, mx, my, mz, texture=True):
    ix, iy, iz = _grid(img.shape)
    if texture:
        return tex_sample(img, (ix - F(mx) + F(0.5)).astype(F), (iy - F(my) + F(0.5)).astype(F),
                          (iz - F(mz) + F(0.5)).astype(F))
    return _plain(img, (ix + F(mx)).astype(F), (iy + F(my)).astype(F), (iz + F(mz)).astype(F), lo=0)


def shift_z(img, mz, texture=True):
    ix, iy, iz = _grid(img.shape)
    nz = img.shape[2]
    if texture:
        return tex_sample(img, (ix + F(0.5)).astype(F), (iy + F(0.5)).astype(F), (iz - F(mz) + F(0.5)).astype(F))
    pz = (iz + F(mz)).astype(F)
    zi = np.floor(pz).astype(np.int64)
    wz2 = (pz - zi).astype(F)
    wz = F(1) - wz2
    out = np.zeros(img.shape, F)
    zc = np.clip(zi, 0, nz - 1)
    zc2 = np.clip(zi + 1, 0, nz - 1)
    first = zi + 1 == 0
    last = (zi == nz - 1) & ~first
    mid = (zi >= 0) & (zi + 1 < nz) & ~first & ~last
    jx, jy = ix.astype(np.int64), iy.astype(np.int64)
    out[first] = img[jx[first], jy[first], zc2[first]] * wz2[first]
    out[last] = img[jx[last], jy[last], zc[last]] * wz[last]
    out[mid] = img[jx[mid], jy[mid], zc[mid]] * wz[mid] + img[jx[mid], jy[mid], zc2[mid]] * wz2[mid]
    return out.astype(F)


def rotate(img, cos_phi, sin_phi, texture=True):
    px, py, iz = _rot(img.shape, cos_phi, sin_phi)
    if texture:
        return tex_sample(img, px, py, (iz + F(0.5)).astype(F))
    return _plain(img, px, py, iz.astype(F), lo=1, rotate=True, iz=iz)


def deform_invert(mx, my, mz, iterations=30):
    ix, iy, iz = _grid(mx.shape)
    x = np.zeros(mx.shape, F)
    y = np.zeros(mx.shape, F)
    z = np.zeros(mx.shape, F)
    for _ in range(iterations):
        x = -tex_sample(mx, (x + ix + F(0.5)).astype(F), (y + iy + F(0.5)).astype(F), (z + iz + F(0.5)).astype(F))
        y = -tex_sample(my, (x + ix + F(0.5)).astype(F), (y + iy + F(0.5)).astype(F), (z + iz + F(0.5)).astype(F))
        z = -tex_sample(mz, (x + ix + F(0.5)).astype(F), (y + iy + F(0.5)).astype(F), (z + iz + F(0.5)).astype(F))
    return x, y, z
