"""Seeded synthetic list-mode workloads (scanners, phantoms, events).

No public dataset is involved; every input of the tests and of bench.py comes from here.

* ``scanner_small`` -- 99/119 mm radii, 16 blocks/ring of 10 x 4 crystals (3.2 mm), 4 block
  rings: 640 crystals. Image 64 x 64 x 16 at 2 mm.
* ``scanner_clinical`` -- 424/444 mm radii, 48 blocks/ring of 13 x 13 crystals (4 mm), 4 block
  rings: 624 crystals/ring, 52 crystal rings, 32,448 crystals. Image 200 x 200 x 109 at
  2.04 x 2.04 x 2.03 mm. TOF: 530 ps FWHM coincidence timing, i.e. a Gaussian along the LOR with
  sigma = c * sigma_t / 2 = 33.7 mm (tof_sigma2 = 1138 mm^2).

Events: emission points drawn from the activity image, isotropic directions, intersected with the
crystal cylinder (average radius), kept when both hits lie inside the axial extent, snapped to
crystal centres with the reference's index arithmetic (EcatCrystalPosToIndex followed by
EcatIndexToCrystalPos; hits in the gaps between blocks are dropped). TOF column = d2 - d1 + noise in
mm, the reference convention (the kernel centres the Gaussian at (L - tof) / 2 from endpoint 1).

Generation runs in torch float64 on the device given, so the 2e7-event clinical workload is built
on the GPU in a second; results are deterministic per (seed, device).
"""
from __future__ import annotations

import math
from typing import Optional, Tuple

import torch

from .data import Image
from .geometry import Block, ImageConfig, PetEcatScanner, TofConfig

C_MM_PER_PS = 0.299792458
FWHM_TO_SIGMA = 1.0 / (2.0 * math.sqrt(2.0 * math.log(2.0)))


def tof_sigma2_from_fwhm_ps(fwhm_ps: float) -> float:
    """Positional variance (mm^2) along the LOR for a coincidence timing FWHM in ps."""
    sigma_pos = C_MM_PER_PS * fwhm_ps * FWHM_TO_SIGMA / 2.0
    return sigma_pos * sigma_pos


def scanner_small() -> PetEcatScanner:
    return PetEcatScanner(99.0, 119.0, 4, 16, 0.0, Block([20.0, 32.0, 12.8], [1, 10, 4]),
                          TofConfig(3.66, tof_sigma2_from_fwhm_ps(530.0)))


def image_small() -> ImageConfig:
    return ImageConfig([64, 64, 16], [0.0, 0.0, 0.0], [128.0, 128.0, 32.0])


def scanner_clinical() -> PetEcatScanner:
    return PetEcatScanner(424.0, 444.0, 4, 48, 0.0, Block([20.0, 52.0, 52.0], [1, 13, 13]),
                          TofConfig(3.66, tof_sigma2_from_fwhm_ps(530.0)))


def image_clinical() -> ImageConfig:
    return ImageConfig([200, 200, 109], [0.0, 0.0, 0.0], [200 * 2.04, 200 * 2.04, 109 * 2.03])


def _voxel_centres(cfg: ImageConfig, device) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    nx, ny, nz = cfg.shape
    ux, uy, uz = cfg.unit_size
    xs = (torch.arange(nx, device=device, dtype=torch.float64) + 0.5) * ux - cfg.size[0] / 2 + cfg.center[0]
    ys = (torch.arange(ny, device=device, dtype=torch.float64) + 0.5) * uy - cfg.size[1] / 2 + cfg.center[1]
    zs = (torch.arange(nz, device=device, dtype=torch.float64) + 0.5) * uz - cfg.size[2] / 2 + cfg.center[2]
    return torch.meshgrid(xs, ys, zs, indexing="ij")


def phantom_cylinder(cfg: ImageConfig, device="cpu") -> torch.Tensor:
    """Water cylinder r = 40 mm (activity 1) with six hot spheres r = 3..8 mm at 4:1."""
    x, y, z = _voxel_centres(cfg, device)
    act = ((x * x + y * y) <= 40.0 ** 2).to(torch.float64)
    for k, r in enumerate((3.0, 4.0, 5.0, 6.0, 7.0, 8.0)):
        ang = k * math.pi / 3.0
        cx, cy = 22.0 * math.cos(ang), 22.0 * math.sin(ang)
        inside = ((x - cx) ** 2 + (y - cy) ** 2 + z ** 2) <= r * r
        act = torch.where(inside, torch.full_like(act, 4.0), act)
    return act.to(torch.float32)


def phantom_body(cfg: ImageConfig, seed: int = 0, device="cpu", max_lesions: int = 40) -> torch.Tensor:
    """Water ellipsoid body (axes 30 x 20 x 100 cm) plus 0..max_lesions random hot/cold ellipsoids
    with contrast 0.2..8 (activity multiplier), all inside the body."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    x, y, z = _voxel_centres(cfg, device)
    body = (x / 150.0) ** 2 + (y / 100.0) ** 2 + (z / 500.0) ** 2 <= 1.0
    act = body.to(torch.float64)
    n_les = int(torch.randint(0, max_lesions + 1, (1,), generator=g))
    zr = min(cfg.size[2] / 2, 500.0) * 0.8
    for _ in range(n_les):
        r = torch.rand(8, generator=g, dtype=torch.float64).tolist()
        cx, cy, cz = (r[0] - 0.5) * 200.0, (r[1] - 0.5) * 120.0, (r[2] - 0.5) * 2 * zr
        ax, ay, az = 5.0 + 25.0 * r[3], 5.0 + 25.0 * r[4], 5.0 + 25.0 * r[5]
        contrast = 0.2 * (40.0 ** r[6])  # log-uniform in [0.2, 8]
        inside = ((x - cx) / ax) ** 2 + ((y - cy) / ay) ** 2 + ((z - cz) / az) ** 2 <= 1.0
        act = torch.where(inside & body, act * 0 + contrast, act)
    return act.to(torch.float32)


def _snap(scanner: PetEcatScanner, p: torch.Tensor):
    """pos -> (crystal index, snapped pos, valid) with EcatCrystalPosToIndex/EcatIndexToCrystalPos
    arithmetic (srfnef/functions/geometry/pet_ecat_scanner.py:36-89)."""
    s = scanner
    apb = s.angle_per_block
    xc, yc, zc = p[:, 0], p[:, 1], p[:, 2]
    iblock = torch.remainder(torch.round(torch.atan2(yc, xc) / apb).long(), s.nb_blocks_per_ring)
    iring = torch.floor((zc + s.axial_length / 2) / (s.gap + s.blocks.size[2])).long()
    ang = iblock.to(torch.float64) * apb
    y_corr = -xc * torch.sin(ang) + yc * torch.cos(ang) + s.blocks.size[1] / 2
    iy = torch.round(y_corr / s.blocks.unit_size[1] - 0.5).long()
    z_corr = zc + s.axial_length / 2 - iring.to(torch.float64) * (s.blocks.size[2] + s.gap)
    iz = torch.round(z_corr / s.blocks.unit_size[2] - 0.5).long()
    valid = (iy >= 0) & (iy < s.blocks.shape[1]) & (iz >= 0) & (iz < s.blocks.shape[2]) \
        & (iring >= 0) & (iring < s.nb_rings)
    idx = iy + iz * s.blocks.shape[1] + iblock * s.nb_crystals_per_block + iring * s.nb_crystals_per_ring
    x0 = s.average_radius
    y0 = (iy.to(torch.float64) + 0.5) * s.blocks.unit_size[1] - s.blocks.size[1] / 2
    th = apb * iblock.to(torch.float64)
    q = torch.empty_like(p)
    q[:, 0] = x0 * torch.cos(th) - y0 * torch.sin(th)
    q[:, 1] = x0 * torch.sin(th) + y0 * torch.cos(th)
    q[:, 2] = (iz.to(torch.float64) + 0.5) * s.blocks.unit_size[2] \
        + iring.to(torch.float64) * (s.gap + s.blocks.size[2]) - s.axial_length / 2
    return idx, q.to(torch.float32).to(torch.float64), valid


def sample_events(scanner: PetEcatScanner, cfg: ImageConfig, activity: torch.Tensor, n: int,
                  seed: int = 0, tof_fwhm_ps: Optional[float] = None, device="cpu",
                  chunk: int = 1 << 22) -> torch.Tensor:
    """Return an (n, 6) float32 LOR tensor, or (n, 7) with a TOF column in mm when
    ``tof_fwhm_ps`` is given, on ``device``."""
    device = torch.device(device)
    g = torch.Generator(device=device).manual_seed(seed)
    act = activity.to(device=device, dtype=torch.float64).reshape(-1)
    cdf = torch.cumsum(act, 0)
    cdf = cdf / cdf[-1]
    nx, ny, nz = cfg.shape
    ux, uy, uz = cfg.unit_size
    R = scanner.average_radius
    half_ax = scanner.axial_length / 2
    sig_tof = None if tof_fwhm_ps is None else C_MM_PER_PS * tof_fwhm_ps * FWHM_TO_SIGMA
    out = []
    have = 0
    while have < n:
        m = chunk
        u = torch.rand(m, generator=g, device=device, dtype=torch.float64)
        vox = torch.searchsorted(cdf, u).clamp_(max=act.numel() - 1)
        ix = vox // (ny * nz)
        iy = (vox // nz) % ny
        iz = vox % nz
        jit = torch.rand(m, 3, generator=g, device=device, dtype=torch.float64)
        P = torch.stack([(ix + jit[:, 0]) * ux - cfg.size[0] / 2 + cfg.center[0],
                         (iy + jit[:, 1]) * uy - cfg.size[1] / 2 + cfg.center[1],
                         (iz + jit[:, 2]) * uz - cfg.size[2] / 2 + cfg.center[2]], 1)
        w = torch.rand(m, generator=g, device=device, dtype=torch.float64) * 2 - 1
        phi = torch.rand(m, generator=g, device=device, dtype=torch.float64) * (2 * math.pi)
        st = torch.sqrt(torch.clamp(1 - w * w, min=0))
        d = torch.stack([st * torch.cos(phi), st * torch.sin(phi), w], 1)
        a = d[:, 0] ** 2 + d[:, 1] ** 2
        b = 2 * (P[:, 0] * d[:, 0] + P[:, 1] * d[:, 1])
        c = P[:, 0] ** 2 + P[:, 1] ** 2 - R * R
        disc = torch.sqrt(torch.clamp(b * b - 4 * a * c, min=0))
        a_safe = torch.clamp(a, min=1e-12)
        t1 = (-b - disc) / (2 * a_safe)
        t2 = (-b + disc) / (2 * a_safe)
        H1 = P + t1[:, None] * d
        H2 = P + t2[:, None] * d
        ok = (a > 1e-9) & (H1[:, 2].abs() < half_ax) & (H2[:, 2].abs() < half_ax)
        _, E1, v1 = _snap(scanner, H1)
        _, E2, v2 = _snap(scanner, H2)
        ok &= v1 & v2
        cols = [E1, E2]
        if sig_tof is not None:
            d1 = torch.linalg.norm(P - E1, dim=1)
            d2 = torch.linalg.norm(P - E2, dim=1)
            tof = d2 - d1 + sig_tof * torch.randn(m, generator=g, device=device, dtype=torch.float64)
            cols.append(tof[:, None])
        lor = torch.cat(cols, 1)[ok].to(torch.float32)
        out.append(lor)
        have += lor.shape[0]
    return torch.cat(out, 0)[:n].contiguous()


def activity_image(cfg: ImageConfig, act: torch.Tensor) -> Image:
    return Image(act, list(cfg.center), list(cfg.size))
