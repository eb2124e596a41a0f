"""Coarse scatter sinogram on the clinical scanner and its training data (not in the reference).

The reference's SSS (srfnef/corrections/scattering) runs over its flat triangular crystal-pair
index. For the learned surrogate a 2x-downsampled, regular sinogram is defined here:

* virtual crystals: pairs of adjacent crystals in the ring (624 -> 312 per ring) and pairs of
  adjacent crystal rings (52 -> 26), placed at the mean of their four crystal centres;
* bins (plane p, radial r, view v), 52 x 52 x 312: view v is virtual crystal v of ring p // 2,
  its partner is crystal (v + 156 + 3 r - 78) mod 312 of ring (p + 1) // 2, so planes alternate
  direct (same ring) and cross (adjacent rings) pairs; plane 51 is padding and stays empty.
  Radial bins step by 3 virtual crystals (3.5 degrees of ring angle) over +-45 degrees from the
  opposite crystal, i.e. LORs up to 300 mm from the axis: the whole 600 mm transaxial FOV.

``sss_sinogram`` fills it with the repository's own single-scatter simulation (srf_sss, with
the preprocessing projections on the GPU projector); ``network_input`` holds the inputs of the
learned surrogate: emission line integrals and attenuation factors along the bins' LORs.
"""
from __future__ import annotations

import math
from typing import Dict, Tuple

import numpy as np
import torch

from . import _lib, kernels
from .geometry import EcatIndexToCrystalPos, ImageConfig, PetEcatScanner

VIEWS, RADIAL, PLANES = 312, 52, 52
RADIAL_STEP = 3                     # virtual crystals between radial bins
RADIAL_OFF = RADIAL_STEP * RADIAL // 2
FOV_MM = (600.0, 600.0, 208.0)
VOL_SHAPE = (64, 64, 32)
# mu values of the synthetic maps (1/mm at 511 keV)
MU_WATER, MU_BONE, MU_LUNG = 0.0096, 0.017, 0.003


class CoarseGeometry:
    def __init__(self, scanner: PetEcatScanner, device="cuda"):
        self.scanner = scanner
        s = scanner
        n_t = s.nb_blocks_per_ring * s.blocks.shape[1]       # crystals per ring (transaxial)
        n_r = s.nb_rings * s.blocks.shape[2]                 # crystal rings
        self.vt, self.vr = n_t // 2, n_r // 2
        assert self.vt == VIEWS and self.vr == PLANES // 2, "geometry of the clinical scanner expected"
        pos = EcatIndexToCrystalPos(s)(np.arange(s.nb_crystals)).astype(np.float64)
        ids = np.arange(s.nb_crystals)
        iy = ids % s.blocks.shape[1]
        iz = (ids // s.blocks.shape[1]) % s.blocks.shape[2]
        ib = (ids // s.nb_crystals_per_block) % s.nb_blocks_per_ring
        ir = ids // s.nb_crystals_per_ring
        t = ib * s.blocks.shape[1] + iy
        r = ir * s.blocks.shape[2] + iz
        vidx = (r // 2) * self.vt + (t // 2)
        vpos = np.zeros((self.vr * self.vt, 3))
        np.add.at(vpos, vidx, pos)
        self.vpos = (vpos / 4.0).astype(np.float32)                     # (8112, 3)
        self.full_to_virtual = vidx.astype(np.int64)
        p = np.arange(PLANES - 1)
        ra, rb = p // 2, (p + 1) // 2
        rr = np.arange(RADIAL)
        vv = np.arange(VIEWS)
        P, Rr, V = np.meshgrid(p, rr, vv, indexing="ij")
        a = ra[P] * self.vt + V
        b = rb[P] * self.vt + (V + VIEWS // 2 + RADIAL_STEP * Rr - RADIAL_OFF) % VIEWS
        self.pairs = np.stack([a.ravel(), b.ravel()], 1).astype(np.int32)  # (51*52*312, 2)
        self.device = torch.device(device)
        self.pairs_dev = torch.as_tensor(self.pairs, device=self.device)
        self.vpos_dev = torch.as_tensor(self.vpos, device=self.device)
        lors = np.concatenate([self.vpos[self.pairs[:, 0]], self.vpos[self.pairs[:, 1]]], 1)
        self.bin_lors = torch.as_tensor(lors.astype(np.float32), device=self.device)
        self.ic = ImageConfig(list(VOL_SHAPE), [0.0, 0.0, 0.0], list(FOV_MM))
        self.scatter_points = self._scatter_points()
        self.scatter_points_dev = torch.as_tensor(self.scatter_points, dtype=torch.float32, device=self.device)

    def _scatter_points(self) -> np.ndarray:
        """Every floor(50 mm / voxel) voxels, as preprocess.py:6-18 places them."""
        from .scatter import pre_all_scatter_position
        from .data import Image
        img = Image(np.zeros(VOL_SHAPE, np.float32), self.ic.center, self.ic.size)
        return pre_all_scatter_position(img)

    def n_bins(self) -> int:
        return self.pairs.shape[0]

    def to_grid(self, flat: torch.Tensor) -> torch.Tensor:
        """(51*52*312,) bin values -> (52, 52, 312) with the empty padding plane."""
        g = torch.zeros((PLANES, RADIAL, VIEWS), dtype=flat.dtype, device=flat.device)
        g[: PLANES - 1] = flat.reshape(PLANES - 1, RADIAL, VIEWS)
        return g

    def event_bins(self, crystal_ids: torch.Tensor) -> torch.Tensor:
        """Flat bin (or -1) of events given their full-resolution crystal ids (n, 2): the pair is
        ordered lower ring first, the plane is p = ra + rb (clamped to the sampled planes), the
        radial bin is the nearest sampled partner offset, and view/radial come from the pair in
        that order or, in a direct plane, in either order. (312 views span the whole ring, so a
        direct-plane LOR has two equivalent bins.)"""
        f2v = torch.as_tensor(self.full_to_virtual, device=crystal_ids.device)
        va, vb = f2v[crystal_ids[:, 0]], f2v[crystal_ids[:, 1]]
        swap = (va // self.vt) > (vb // self.vt)
        va, vb = torch.where(swap, vb, va), torch.where(swap, va, vb)
        ra, ta = va // self.vt, va % self.vt
        rb, tb = vb // self.vt, vb % self.vt
        p = torch.clamp(ra + rb, 0, PLANES - 2)
        off = VIEWS // 2 - RADIAL_OFF - RADIAL_STEP // 2
        r1 = torch.div((tb - ta - off) % VIEWS, RADIAL_STEP, rounding_mode="floor")
        r2 = torch.div((ta - tb - off) % VIEWS, RADIAL_STEP, rounding_mode="floor")
        direct = ra == rb
        use1 = r1 < RADIAL
        v = torch.where(use1, ta, tb)
        r = torch.where(use1, r1, r2)
        ok = use1 | (direct & (r2 < RADIAL))
        return torch.where(ok, (p * RADIAL + r) * VIEWS + v, torch.full_like(p, -1))


def random_phantom(seed: int, device="cuda") -> Tuple[torch.Tensor, torch.Tensor]:
    """Emission and mu volumes (64 x 64 x 32 over 600 x 600 x 208 mm): a water body ellipse with
    lungs and a spine, and random hot/cold ellipsoids in the emission."""
    g = torch.Generator().manual_seed(seed)
    r = lambda *s: torch.rand(*s, generator=g).tolist()
    nx, ny, nz = VOL_SHAPE
    xs = (torch.arange(nx) + 0.5) * FOV_MM[0] / nx - FOV_MM[0] / 2
    ys = (torch.arange(ny) + 0.5) * FOV_MM[1] / ny - FOV_MM[1] / 2
    zs = (torch.arange(nz) + 0.5) * FOV_MM[2] / nz - FOV_MM[2] / 2
    X, Y, Z = torch.meshgrid(xs, ys, zs, indexing="ij")
    a = r(8)
    bx, by = 120 + 60 * a[0], 80 + 50 * a[1]
    cx, cy = (a[2] - 0.5) * 40, (a[3] - 0.5) * 30
    body = ((X - cx) / bx) ** 2 + ((Y - cy) / by) ** 2 <= 1
    mu = torch.where(body, MU_WATER, 0.0)
    act = body.float() * (0.5 + a[4])
    for side in (-1, 1):  # lungs
        lx, ly = cx + side * bx * 0.45, cy + by * 0.1
        lung = ((X - lx) / (bx * 0.3)) ** 2 + ((Y - ly) / (by * 0.5)) ** 2 + (Z / 80.0) ** 2 <= 1
        mu = torch.where(lung & body, MU_LUNG, mu)
        act = torch.where(lung & body, act * 0.3, act)
    spine = ((X - cx) / 18.0) ** 2 + ((Y - (cy - by * 0.7)) / 18.0) ** 2 <= 1
    mu = torch.where(spine & body, MU_BONE, mu)
    for _ in range(int(r(1)[0] * 8)):
        e = r(7)
        ex, ey, ez = cx + (e[0] - 0.5) * bx, cy + (e[1] - 0.5) * by, (e[2] - 0.5) * 150
        sz = 10 + 30 * e[3]
        les = ((X - ex) / sz) ** 2 + ((Y - ey) / (sz * (0.6 + e[4]))) ** 2 + ((Z - ez) / sz) ** 2 <= 1
        act = torch.where(les & body, act * (0.2 + 7.8 * e[5]), act)
    dx_ = FOV_MM[0] / nx
    # UmapProject multiplies the line integral by the voxel size once more
    # (attenuation_correct.py:34-39); mu is stored per voxel unit so that exp(-...) is physical
    return act.float().to(device), (mu / dx_).float().to(device)


def sss_sinogram(geo: CoarseGeometry, emission: torch.Tensor, mu: torch.Tensor,
                 low: int = 350, high: int = 650, resolution: float = 0.15,
                 bins: torch.Tensor = None) -> torch.Tensor:
    """Raw SSS sums of every bin (or of the bins listed) as a flat FP32 tensor.

    The preprocessing of preprocess.py (emission line integrals x L^2 and attenuation factors
    from every detector to every scatter point, detector-major) runs on the GPU projector; with
    ``bins`` only the virtual crystals those bins touch are preprocessed."""
    if bins is None:
        return sss_pairs(geo, emission, mu, geo.vpos_dev, geo.pairs_dev, low, high, resolution)
    pairs = geo.pairs_dev.index_select(0, bins)
    uniq, inv = torch.unique(pairs.reshape(-1), return_inverse=True)
    return sss_pairs(geo, emission, mu, geo.vpos_dev.index_select(0, uniq),
                     inv.reshape(-1, 2).to(torch.int32), low, high, resolution)


def sss_tables(geo: CoarseGeometry, emission: torch.Tensor, mu: torch.Tensor, cpos: torch.Tensor):
    """The SSS preprocessing (preprocess.py:21-43) of crystals ``cpos`` (m, 3): per crystal and
    scatter point the emission line integral x |LOR|^2 and the attenuation factor, (m, n_points)
    each, on the GPU projector."""
    sp = geo.scatter_points_dev
    ic = geo.ic
    m, k = cpos.shape[0], sp.shape[0]
    Ld = torch.cat([cpos[:, None, :].expand(m, k, 3), sp[None, :, :].expand(m, k, 3)], 2).reshape(-1, 6)
    Ld = Ld.contiguous()
    # detector -> scatter point LORs cross at most 64 slabs of the 64 x 64 x 32 grid: 8 lanes per
    # LOR beat the default 32 (measured 6.5 -> 5.1 ms for the whole coarse sinogram)
    with _lib.tuning(8, 2):
        p = kernels.project(Ld, kernels.xfast(emission), ic.center, ic.size)
        atten = kernels.attenuation(Ld, kernels.xfast(mu), ic.center, ic.size).reshape(m, k)
    len2 = ((Ld[:, 3] - Ld[:, 0]) ** 2 + (Ld[:, 4] - Ld[:, 1]) ** 2 + (Ld[:, 5] - Ld[:, 2]) ** 2)
    sumup = (p * len2).reshape(m, k)
    return sumup.contiguous(), atten.contiguous()


def sss_args(geo: CoarseGeometry, low: int = 350, high: int = 650, resolution: float = 0.15):
    """The scanner and energy arguments of srf_sss for the coarse geometry (after umap, umap_size)."""
    s = geo.scanner
    return (s.nb_blocks_per_ring * s.blocks.shape[1], s.nb_blocks_per_ring, list(s.blocks.shape), low, high,
            resolution)


def sss_pairs(geo: CoarseGeometry, emission: torch.Tensor, mu: torch.Tensor, cpos: torch.Tensor,
              pairs: torch.Tensor, low: int = 350, high: int = 650, resolution: float = 0.15) -> torch.Tensor:
    """SSS of crystal pairs given as int32 indices into the crystal positions ``cpos`` (m, 3):
    preprocessing of those m crystals, then srf_sss. No host synchronisation."""
    sumup, atten = sss_tables(geo, emission, mu, cpos)
    sc, _ = kernels.sss(pairs.contiguous(), cpos.contiguous(), geo.scatter_points_dev, sumup, atten,
                        mu.contiguous(), list(geo.ic.size), *sss_args(geo, low, high, resolution))
    return sc


# ---------------------------------------------------------------- network grid
# The network predicts the sinogram on a padded (planes, radial, views) = (56, 56, 320) grid: views
# wrap around (4 copies each side), planes and radial bins repeat their last row. It runs on the
# 2x coarser (28, 28, 160) grid (three U-Net levels without remainders), whose sub-voxel head
# writes the full grid.
PAD_GRID = (56, 56, 320)
VIEW_PAD = 4
HALF_GRID = (28, 28, 160)
N_FEATURES = 16   # 9 measured + 7 geometry channels


def pad_sino(g: torch.Tensor) -> torch.Tensor:
    """(..., 51, 52, 312) -> (..., 56, 56, 320)."""
    lead = tuple(g.shape[:-3])
    v = torch.cat([g[..., -VIEW_PAD:], g, g[..., :VIEW_PAD]], -1)
    r = torch.cat([v, v[..., -1:, :].expand(*lead, PLANES - 1, PAD_GRID[1] - RADIAL, PAD_GRID[2])], -2)
    return torch.cat([r, r[..., -1:, :, :].expand(*lead, PAD_GRID[0] - PLANES + 1, PAD_GRID[1], PAD_GRID[2])], -3)


def crop_sino(t: torch.Tensor) -> torch.Tensor:
    """(..., 56, 56, 320) -> (..., 51 * 52 * 312) flat bins."""
    c = t[..., : PLANES - 1, :RADIAL, VIEW_PAD: VIEW_PAD + VIEWS]
    return c.reshape(*t.shape[:-3], -1)


def full_mask(device) -> torch.Tensor:
    """(56, 56, 320) FP32: 1 on real bins, 0 on padding."""
    m = torch.zeros(PAD_GRID, dtype=torch.float32, device=device)
    m[: PLANES - 1, :RADIAL, VIEW_PAD: VIEW_PAD + VIEWS] = 1.0
    return m


def _half_cells(geo: CoarseGeometry):
    """Per half-resolution cell (28 x 28 x 160, flattened): the bin it samples (plane 2z, radial
    2y, view 2x - 4, clamped/wrapped like the padding), that bin's LOR, the constant input
    channels (LOR midpoint, direction harmonics, plane coordinate) and the cell's virtual
    crystals."""
    if getattr(geo, "_half", None) is None:
        dev = geo.device
        pz = torch.clamp(torch.arange(HALF_GRID[0], device=dev) * 2, max=PLANES - 2)
        ry = torch.clamp(torch.arange(HALF_GRID[1], device=dev) * 2, max=RADIAL - 1)
        vx = (torch.arange(HALF_GRID[2], device=dev) * 2 - VIEW_PAD) % VIEWS
        idx = ((pz[:, None, None] * RADIAL + ry[None, :, None]) * VIEWS + vx[None, None, :]).reshape(-1)
        L = geo.bin_lors.index_select(0, idx).contiguous()
        pc = ((pz.float() - (PLANES - 2) / 2) / ((PLANES - 2) / 2))[:, None, None].expand(HALF_GRID).reshape(-1)
        xm, ym = (L[:, 0] + L[:, 3]) / 600.0, (L[:, 1] + L[:, 4]) / 600.0
        th = torch.atan2(L[:, 4] - L[:, 1], L[:, 3] - L[:, 0])
        const = torch.stack([xm, ym, torch.cos(2 * th), torch.sin(2 * th), torch.cos(4 * th),
                             torch.sin(4 * th), pc], -1)
        pr = geo.pairs_dev.index_select(0, idx).long()
        len2 = ((L[:, 3] - L[:, 0]) ** 2 + (L[:, 4] - L[:, 1]) ** 2 + (L[:, 5] - L[:, 2]) ** 2)
        geo._half = (idx, L, const, pr[:, 0].contiguous(), pr[:, 1].contiguous(), len2)
    return geo._half


def network_input(geo: CoarseGeometry, emission: torch.Tensor, mu: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
    """(1, 28, 28, 160, 16) bfloat16 network input and the emission scale (a device scalar, so
    that nothing waits for the GPU).

    Each half-resolution cell samples one bin's LOR (virtual crystals A, B). Local channels:
    emission line integral / its mean over the cells (e), attenuation factor (a), e * a, the mu
    line integral / 4 (m). Detector channels: single scatter into a bin sums, over scatter points,
    emission along lines from A and from B, so for each virtual crystal the sums of e and e * a
    over every cell it belongs to (what that detector sees of the object) are given at A and at B,
    each / its mean over crystals. Context: e averaged over the views of the cell's (plane,
    radial) row. Geometry: the scatter points sit on a Cartesian grid, so the target is not
    rotation-equivariant in the views; the LOR's midpoint (x, y) / 300 mm, the 2nd and 4th
    harmonics of its direction and the plane coordinate locate each cell absolutely. Targets and
    predictions are in units of the emission scale, so the network is scale-free."""
    idx, L, const, ca, cb, len2 = _half_cells(geo)
    ic = geo.ic
    # bin LORs cross at most ~90 slabs of the 64 x 64 x 32 grid: 8 lanes per LOR
    # (measured 0.23 -> 0.18 ms for this function in the prediction graph)
    with _lib.tuning(8, 4):
        p = kernels.project(L, kernels.xfast(emission), ic.center, ic.size)
        a = kernels.attenuation(L, kernels.xfast(mu), ic.center, ic.size)
    e = p * len2
    scale = e.mean().clamp_min(1e-30)
    en = e / scale
    ea = en * a
    m = -torch.log(torch.clamp(a, min=1e-30)) * 0.25
    n_c = geo.vpos.shape[0]

    def per_detector(v):
        t = torch.zeros(n_c, dtype=torch.float32, device=v.device)
        t.index_add_(0, ca, v)
        t.index_add_(0, cb, v)
        t = t / t.mean().clamp_min(1e-30)
        return t.index_select(0, ca), t.index_select(0, cb)

    fa, fb = per_detector(en)
    ga, gb = per_detector(ea)
    H = HALF_GRID
    row = lambda t: t.reshape(H).mean(dim=2, keepdim=True).expand(H).reshape(-1)
    feats = [en, a, ea, m, fa, fb, ga, gb, row(en)]
    x = torch.empty((L.shape[0], 16), dtype=torch.bfloat16, device=L.device)
    x[:, :len(feats)] = torch.stack(feats, 1).to(torch.bfloat16)
    x[:, len(feats):] = const.to(torch.bfloat16)
    return x.reshape(1, *H, 16), scale


def target_full(sino_flat: torch.Tensor, scale: float) -> torch.Tensor:
    """(56, 56, 320) FP32 training target: the scatter sinogram / scale on the padded grid."""
    return pad_sino((sino_flat / scale).reshape(PLANES - 1, RADIAL, VIEWS)).contiguous()


# ---------------------------------------------------------------- synthetic scatter events
def crystal_grid(geo: CoarseGeometry) -> torch.Tensor:
    """(52 rings, 624 transaxial) full-resolution crystal ids of the clinical scanner."""
    s = geo.scanner
    nt, nzb = s.blocks.shape[1], s.blocks.shape[2]
    r = torch.arange(s.nb_rings * nzb)[:, None]
    t = torch.arange(s.nb_blocks_per_ring * nt)[None, :]
    ids = (t % nt) + (r % nzb) * nt + (t // nt) * s.nb_crystals_per_block + (r // nzb) * s.nb_crystals_per_ring
    return ids.to(geo.device)


def sample_scatter_events(geo: CoarseGeometry, sino_flat: torch.Tensor, n: int, seed: int,
                          tof_sigma: float = 33.7) -> Tuple[torch.Tensor, torch.Tensor]:
    """(n, 7) float32 scatter LORs and their (n, 2) crystal ids, drawn from a bin sinogram: bin ~ sinogram, the partner moved
    uniformly within the bin's radial step, each virtual crystal resolved to one of its 2 x 2
    crystals uniformly, TOF = uniform over +-300 mm plus noise."""
    from .geometry import EcatIndexToCrystalPos
    dev = geo.device
    g = torch.Generator(device=dev).manual_seed(seed)
    p = torch.clamp(sino_flat.double(), min=0)
    b = torch.multinomial(p / p.sum(), n, replacement=True, generator=g)
    pairs = geo.pairs_dev.index_select(0, b).long()
    grid = crystal_grid(geo)
    pos = torch.as_tensor(EcatIndexToCrystalPos(geo.scanner)(np.arange(geo.scanner.nb_crystals)),
                          dtype=torch.float32, device=dev)
    out, ids = [], []
    va, vb = pairs[:, 0], pairs[:, 1]
    dv = torch.randint(0, RADIAL_STEP, (n,), generator=g, device=dev) - RADIAL_STEP // 2
    vb = (vb // geo.vt) * geo.vt + (vb % geo.vt + dv) % geo.vt
    for v in (va, vb):
        ring = (v // geo.vt) * 2 + torch.randint(0, 2, (n,), generator=g, device=dev)
        t = (v % geo.vt) * 2 + torch.randint(0, 2, (n,), generator=g, device=dev)
        ids.append(grid[ring, t])
        out.append(pos.index_select(0, ids[-1]))
    tof = (torch.rand(n, generator=g, device=dev) * 2 - 1) * 300.0 \
        + torch.randn(n, generator=g, device=dev) * tof_sigma
    return torch.cat([out[0], out[1], tof[:, None]], 1).contiguous(), torch.stack(ids, 1)


# ---------------------------------------------------------------- scatter-corrected OSEM
SCATTER_FRACTION = 0.35
_EMAPS: Dict[int, object] = {}


class ScatterStudy:
    """A study on the clinical scanner built from one synthetic phantom: attenuated trues drawn
    from the emission volume (kept with probability exp(-int mu)), scatters drawn from the SSS
    sinogram of the same phantom (``sf`` of all events), both with 530 ps TOF.

    Reconstruction (64 x 64 x 32 over 600 x 600 x 208 mm, TOF OSEM): events carry their
    attenuation correction factor 1 / a_i as value, and a scatter estimate S enters as the
    per-event additive term b_i = kappa S[bin_i] / a_i, the fixed point of the weighted update
    for an expected density a_i p_i + s_i. kappa scales the estimate to the scatter fraction, as
    the reference's ScatterCorrect does (corrections/scattering/scatter.py: the fraction is
    normalised to ``scatter_fraction`` of the counts): kappa * mean_i S[bin_i] = sf * mean_i a_i
    p_i(x0), x0 the reconstruction without scatter correction. Only the estimate S differs
    between an SSS-corrected and a surrogate-corrected reconstruction."""

    def __init__(self, geo: CoarseGeometry, seed: int, n_trues: int = 2_000_000,
                 sf: float = SCATTER_FRACTION, n_iter: int = 2, n_sub: int = 4):
        from . import synth
        from .data import Listmode, Lors
        self.geo, self.sf, self.n_iter, self.n_sub, self.seed = geo, sf, n_iter, n_sub, seed
        dev, ic, sc = geo.device, geo.ic, geo.scanner
        self.emission, self.mu = random_phantom(seed, device=dev)
        self.sss = sss_sinogram(geo, self.emission, self.mu)
        mu_x = kernels.xfast(self.mu)
        g = torch.Generator(device=dev).manual_seed(seed + 7)
        trues = []
        have, k = 0, 0
        while have < n_trues:
            raw = synth.sample_events(sc, ic, self.emission, 4 * n_trues, seed=seed * 131 + k,
                                      tof_fwhm_ps=530.0, device=dev)
            a = kernels.attenuation(raw, mu_x, ic.center, ic.size)
            t = raw[torch.rand(raw.shape[0], generator=g, device=dev) < a]
            trues.append(t)
            have += t.shape[0]
            k += 1
        trues = torch.cat(trues)[:n_trues]
        n_s = int(round(sf / (1.0 - sf) * n_trues))
        scat, _ = sample_scatter_events(geo, self.sss, n_s, seed + 11)
        ev = torch.cat([trues, scat])
        ev = ev.index_select(0, torch.randperm(ev.shape[0], generator=g, device=dev)).contiguous()
        _, ids = kernels.snap(ev, sc, want_ids=True)
        self.events = ev
        self.bins = geo.event_bins(ids)
        self.a = kernels.attenuation(ev, mu_x, ic.center, ic.size)
        self.lm = Listmode(1.0 / self.a, Lors(ev))
        key = id(geo)
        if key not in _EMAPS:
            from .emap_generator import EmapGenerator
            _EMAPS[key] = EmapGenerator("block-full", sc)(ic)
        self.emap = _EMAPS[key]
        self.x0 = self.reconstruct(None)
        tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
        p0 = kernels.project(ev, self.x0, ic.center, ic.size, tof=tof, tof_nsigma=3.0)
        self.model_mean = float((self.a * p0).mean().item())

    def additive(self, sino: torch.Tensor) -> torch.Tensor:
        s = torch.where(self.bins >= 0, sino.index_select(0, self.bins.clamp_min(0)), torch.zeros_like(self.a))
        kappa = self.sf * self.model_mean / max(float(s.mean().item()), 1e-30)
        return (kappa * s / self.a).contiguous()

    def reconstruct(self, sino=None) -> torch.Tensor:
        from .recon import OsemFullTof
        add = None if sino is None else self.additive(sino)
        r = OsemFullTof(self.n_iter, self.n_sub, self.geo.ic, self.geo.scanner, self.lm, self.emap,
                        tof_nsigma=3.0, seed=self.seed, add=add)()
        return r.data
