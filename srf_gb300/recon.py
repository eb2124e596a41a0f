"""List-mode MLEM / OSEM with srfnef's call signatures, each iteration a fused GPU subset step.

* ``Mlem(n_iter, emap)(listmode)``                          srfnef/functions/mlem.py:23-45
* ``MlemFull(n_iter, image_config, scanner, listmode, atten_corr, scatter_corr, psf_corr, emap)()``
                                                             srfnef/functions/mlem_full.py:28-99
* ``MlemFullTof(...)()``                                     srfnef/functions/mlem_full_tof.py:28-99
* ``OsemFull(n_iter, n_sub, image_config, scanner, listmode, atten_corr, scatter_corr, norm_corr,
  psf_corr, emap, image)()``                                 srfnef/functions/osem_full.py:30-87
* ``OsemFullTof`` -- not in the reference (it has no TOF OSEM): OsemFull's subset loop with
  MlemFullTof's update rule and an emap scaled per subset; cyclic subsets of a seeded
  permutation (``subsets='random'``), or interleaved subsets (``subsets='interleaved'``: event i
  in subset i mod n_sub), which need no reordering of the list-mode data on the device.

Update rules, as the reference (float32 throughout):
  Mlem        r = y / (p + mean(y)*1e-8)       emap zeros -> 1e8
  MlemFull    r = div_no_nan(y, p)             emap zeros -> 1e8
  MlemFullTof r = div_no_nan(y, p + 1e-5)      emap zeros -> 1e8
  OsemFull    r = y / (p + 1e-8)               emap as given; subset i_iter // n_sub
  x <- x * bp / emap
``OsemFull.subset_rule='reference'`` keeps the reference's ``i_iter // n_sub`` (osem_full.py:68);
'cyclic' uses ``i_iter % n_sub``. ``OsemFull.seed=None`` shuffles with numpy's global generator
like the reference (osem_full.py:63-64); an int seeds a private generator.

Each subset step is one ``srf_osem_subset`` launch (projection, ratio and backprojection per LOR)
followed by one ``srf_osem_update`` launch.
"""
from __future__ import annotations

import dataclasses
from typing import Any, Callable, Optional

import numpy as np
import torch

from . import distributed, kernels
from ._lib import SRF_RATIO_DIV_NO_NAN, SRF_RATIO_PLAIN
from .data import Emap, Image, Listmode, _NefLike
from .emap_generator import EmapGenerator
from .functions import device, to_dev, to_dev_overlapped
from .geometry import ImageConfig, PetEcatListmodeTrans, PetEcatScanner


_PERMS: "dict" = {}


def _device_permutation(seed: int, n: int, dev) -> torch.Tensor:
    """numpy's default_rng(seed).permutation(n) on the device, kept for repeated calls with the
    same seed and event count (the permutation depends on nothing else)."""
    key = (int(seed), int(n), str(dev))
    perm = _PERMS.get(key)
    if perm is None:
        if len(_PERMS) >= 4:
            _PERMS.clear()
        perm = torch.as_tensor(np.random.default_rng(seed).permutation(n), device=dev)
        _PERMS[key] = perm
    return perm


def _by_subset(v: torch.Tensor, n_sub: int) -> torch.Tensor:
    """(n_sub, n // n_sub): row k holds events k, k + n_sub, ... of a per-event vector (the
    remainder events are left out, as the subset loop does)."""
    n_per = v.shape[0] // n_sub
    return v[:n_per * n_sub].reshape(n_per, n_sub).t().contiguous()


def _emap_dev(emap) -> torch.Tensor:
    return kernels.xfast(to_dev(emap.data))


def _result(state: kernels.SubsetState, like, center, size) -> Image:
    x = state.x.contiguous()
    if not isinstance(like, torch.Tensor):
        x = x.cpu().numpy()
    return Image(x, list(center), list(size))


def _run_mlem(n_iter, lors_np_or_t, y, emap, shape, center, size, *, tof, rule, eps, guard,
              tof_nsigma=0.0) -> kernels.SubsetState:
    dev = device()
    lors = to_dev(lors_np_or_t).contiguous()
    yd = to_dev(y).contiguous()
    em = _emap_dev(emap)
    st = kernels.SubsetState(shape, center, size, dev)
    for _ in range(n_iter):
        st.subset(lors, yd, rule=rule, eps=eps, tof=tof, tof_nsigma=tof_nsigma)
        st.update(em, guard_zero=guard)
    return st


@dataclasses.dataclass(frozen=True)
class Mlem(_NefLike):
    n_iter: Optional[int] = None
    emap: Optional[Emap] = None

    def __call__(self, listmode: Listmode) -> Image:
        y = np.asarray(listmode.data.cpu() if isinstance(listmode.data, torch.Tensor) else listmode.data,
                       dtype=np.float32)
        eps = float(np.float32(np.mean(y) * 1e-8))
        st = _run_mlem(self.n_iter, listmode.lors.data, listmode.data, self.emap, self.emap.shape,
                       self.emap.center, self.emap.size, tof=None, rule=SRF_RATIO_PLAIN, eps=eps,
                       guard=True)
        return _result(st, self.emap.data, self.emap.center, self.emap.size)


@dataclasses.dataclass(frozen=True)
class MlemFull(_NefLike):
    n_iter: Optional[int] = None
    image_config: Optional[ImageConfig] = None
    scanner: Optional[PetEcatScanner] = None
    listmode: Optional[Listmode] = None
    atten_corr: Any = None
    scatter_corr: Any = None
    psf_corr: Optional[Callable] = None
    emap: Optional[Emap] = None

    _tof = False
    _eps = 0.0

    def generate_emap(self) -> None:
        object.__setattr__(self, "emap", EmapGenerator("block-full", self.scanner)(self.image_config))

    def _tof_args(self):
        return None

    def _recon(self, listmode_) -> Image:
        ic = self.image_config
        st = _run_mlem(self.n_iter, self.listmode.lors.data, listmode_.data, self.emap, ic.shape,
                       ic.center, ic.size, tof=self._tof_args(), rule=SRF_RATIO_DIV_NO_NAN,
                       eps=self._eps, guard=True)
        return _result(st, self.listmode.data, ic.center, ic.size)

    def __call__(self) -> Image:
        if self.emap is None:
            self.generate_emap()
        listmode_ = self.atten_corr(self.listmode) if self.atten_corr is not None else self.listmode
        x = self._recon(listmode_)
        x = self._after(x)
        return self.psf_corr(x) if self.psf_corr is not None else x

    def _after(self, x: Image) -> Image:
        return x


@dataclasses.dataclass(frozen=True)
class MlemFullTof(MlemFull):
    _tof = True
    _eps = 1e-5

    def _tof_args(self):
        return (self.scanner.tof.tof_bin, self.scanner.tof.tof_sigma2)

    def _after(self, x: Image) -> Image:
        # mlem_full_tof.py:71-92: with a scatter correction, rerun on the corrected list mode
        if self.scatter_corr is None:
            return x
        if self.atten_corr is None:
            raise ValueError("MlemFullTof: a scatter correction needs atten_corr (its u_map)")
        listmode_ = self.scatter_corr(x, self.atten_corr.u_map, self.scanner, self.listmode)
        return self._recon(listmode_)


@dataclasses.dataclass(frozen=True)
class OsemFull(_NefLike):
    n_iter: Optional[int] = None
    n_sub: Optional[int] = None
    image_config: Optional[ImageConfig] = None
    scanner: Optional[PetEcatScanner] = None
    listmode: Optional[Listmode] = None
    atten_corr: Any = None
    scatter_corr: Any = None
    norm_corr: Optional[bool] = None
    psf_corr: Optional[Callable] = None
    emap: Optional[Emap] = None
    image: Optional[Image] = None
    subset_rule: str = "reference"
    seed: Optional[int] = None

    def generate_emap(self) -> None:
        # osem_full.py:45-47 asks for mode 'ring', which EcatEmapGenerator does not implement
        object.__setattr__(self, "emap", EmapGenerator("ring", self.scanner)(self.image_config))

    def __call__(self) -> Image:
        if self.emap is None:
            self.generate_emap()
        listmode_ = PetEcatListmodeTrans(self.scanner)(self.listmode)
        if self.atten_corr is not None:
            listmode_ = self.atten_corr(listmode_)
        ic = self.image_config
        n = len(self.listmode)
        rand_inds = np.arange(n)
        if self.seed is None:
            np.random.shuffle(rand_inds)
        else:
            rand_inds = np.random.default_rng(self.seed).permutation(n)
        n_per_sub = n // self.n_sub
        dev = device()
        lors_all = to_dev(np.asarray(self.listmode.lors.data)[rand_inds]).contiguous()
        y_all = to_dev(np.asarray(listmode_.data)[rand_inds]).contiguous()
        em = _emap_dev(self.emap)
        st = kernels.SubsetState(ic.shape, ic.center, ic.size, dev)
        for i_iter in range(self.n_iter):
            ind = i_iter // self.n_sub if self.subset_rule == "reference" else i_iter % self.n_sub
            lo, hi = min(ind * n_per_sub, n), min((ind + 1) * n_per_sub, n)
            st.subset(lors_all[lo:hi], y_all[lo:hi], rule=SRF_RATIO_PLAIN, eps=1e-8)
            st.update(em, guard_zero=False)
        x = _result(st, self.listmode.data, ic.center, ic.size)
        return self.psf_corr(x) if self.psf_corr is not None else x


@dataclasses.dataclass(frozen=True)
class OsemFullTof(_NefLike):
    """TOF list-mode OSEM: ``n_iter`` full passes of ``n_sub`` subsets each."""
    n_iter: Optional[int] = None
    n_sub: Optional[int] = None
    image_config: Optional[ImageConfig] = None
    scanner: Optional[PetEcatScanner] = None
    listmode: Optional[Listmode] = None
    emap: Optional[Emap] = None
    tof_nsigma: float = 0.0
    emap_scale: Optional[float] = None   # default 1 / n_sub
    seed: int = 0
    snap: bool = False
    add: Any = None                      # per-event additive expected counts (e.g. scatter)
    sharded: bool = False                # split each subset's events over the process group's ranks
    group: Any = None                    # torch.distributed group (None: the default group)
    subsets: str = "random"              # 'random' (seeded permutation) or 'interleaved'

    def prepare(self):
        """Device-resident inputs in subset order. Host tensors in pinned memory are copied on a
        side stream, overlapping the device work already queued (with repeated calls, the previous
        reconstruction); the caller keeps them unchanged until the call's result is read.
        'random': LORs and values permuted on the device. 'interleaved': the LORs stay in event
        order (subset k is the strided view of events k, k + n_sub, ...) and only the values and
        the additive term, one float per event, are regrouped by subset."""
        if self.subsets not in ("random", "interleaved"):
            raise ValueError(f"subsets must be 'random' or 'interleaved', got {self.subsets!r}")
        lm = PetEcatListmodeTrans(self.scanner)(self.listmode) if self.snap else self.listmode
        dev = device()
        n = len(lm)
        lors = to_dev_overlapped(lm.lors.data)
        y = to_dev_overlapped(lm.data)
        add = None if self.add is None else to_dev(self.add)
        if self.subsets == "random":
            perm = _device_permutation(self.seed, n, dev)
            lors = lors.index_select(0, perm)
            y = y.index_select(0, perm)
            add = None if add is None else add.index_select(0, perm).contiguous()
        else:
            y = _by_subset(y, self.n_sub)
            add = None if add is None else _by_subset(add, self.n_sub)
        # a frozen record: the reordered additive term is cached beside the fields
        object.__setattr__(self, "_add", add)
        scale = (1.0 / self.n_sub) if self.emap_scale is None else self.emap_scale
        em = (_emap_dev(self.emap) * scale)
        return lors, y, em

    def run(self, lors: torch.Tensor, y: Optional[torch.Tensor], em: torch.Tensor,
            state: Optional[kernels.SubsetState] = None, n_iter: Optional[int] = None,
            track_loglik: bool = False) -> kernels.SubsetState:
        """``n_iter`` passes over the subsets of the events as ``prepare`` returns them. With
        ``sharded``, this rank processes its contiguous share of every subset and the ranks'
        backprojections are summed before each update (every rank ends with the same image)."""
        ic = self.image_config
        st = state or kernels.SubsetState(ic.shape, ic.center, ic.size, lors.device)
        n = lors.shape[0]
        rank, world = distributed.world_of(self.group) if self.sharded else (0, 1)
        driver = distributed.ShardedOsem(st, self.group) if self.sharded else None
        tof = (self.scanner.tof.tof_bin, self.scanner.tof.tof_sigma2)
        add = getattr(self, "_add", None)
        steps = []  # (LORs, values, additive term) of this rank's shard of each subset
        if self.subsets == "interleaved":
            n_per = n // self.n_sub
            lo, hi = distributed.shard_range(n_per, rank, world)
            for k in range(self.n_sub):
                view = lors[k:n_per * self.n_sub:self.n_sub]  # events k, k + n_sub, ...
                steps.append((view[lo:hi], None if y is None else y[k, lo:hi],
                              None if add is None else add[k, lo:hi]))
        else:
            for lo, hi in distributed.subset_shards(n, self.n_sub, rank, world):
                steps.append((lors[lo:hi], None if y is None else y[lo:hi],
                              None if add is None else add[lo:hi]))
        for _ in range(self.n_iter if n_iter is None else n_iter):
            for l_k, y_k, a_k in steps:
                st.subset(l_k, y_k, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=tof,
                          tof_nsigma=self.tof_nsigma, track_loglik=track_loglik, add=a_k)
                if driver is not None:
                    driver.reduce()
                st.update(em, guard_zero=True)
        return st

    def __call__(self) -> Image:
        lors, y, em = self.prepare()
        st = self.run(lors, y, em)
        ic = self.image_config
        return _result(st, self.listmode.data, ic.center, ic.size)
