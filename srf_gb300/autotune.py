"""Autotuner for the fused OSEM subset kernel (not in the reference).

For a workload sample it times ``srf_osem_subset`` over the kernel's launch choices (lanes per
LOR 8/16/32 x slabs per lane 2/4) and over LOR orders (as given, or sorted by transaxial
direction bin and axial position at a chosen granularity), applies the fastest with
``srf_set_tuning`` and caches the choice in a JSON file keyed by device, image shape and TOF
truncation, so later runs with the same key skip the search.
"""
from __future__ import annotations

import json
import math
import os
from typing import Dict, Optional, Sequence, Tuple

import torch

from . import _lib, kernels
from ._lib import SRF_RATIO_DIV_NO_NAN

CANDIDATES: Tuple[Tuple[int, int], ...] = ((32, 4), (32, 2), (16, 4), (16, 2), (8, 4), (8, 2))
DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "srf_gb300", "tuning.json")


def direction_order(lors: torch.Tensor, bins: int) -> torch.Tensor:
    """Permutation that groups LORs by transaxial direction (``bins`` bins over [0, pi)) and,
    within a bin, by axial mid-point, so that LORs processed together touch nearby voxels."""
    phi = torch.atan2(lors[:, 4] - lors[:, 1], lors[:, 3] - lors[:, 0]) % math.pi
    b = torch.clamp((phi / math.pi * bins).long(), max=bins - 1)
    zmid = 0.5 * (lors[:, 2] + lors[:, 5])
    key = b.to(torch.float64) * 1e7 + (zmid.to(torch.float64) - zmid.min().to(torch.float64))
    return torch.argsort(key)


def _key(shape: Sequence[int], tof_nsigma: float) -> str:
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return f"{name}|{'x'.join(str(int(s)) for s in shape)}|nsigma={tof_nsigma:g}"


def _time(fn, reps: int) -> float:
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def tune(lors: torch.Tensor, shape, center, size, tof: Tuple[float, float], tof_nsigma: float = 3.0,
         reps: int = 3, sort_bins: Sequence[int] = (0, 256), cache: Optional[str] = DEFAULT_CACHE,
         force: bool = False) -> Dict:
    """Pick (lanes, slabs_per_lane, sort_bins) for this workload; apply it and return it."""
    key = _key(shape, tof_nsigma)
    table = {}
    if cache and os.path.exists(cache):
        with open(cache) as f:
            table = json.load(f)
        if key in table and not force:
            best = table[key]
            _lib.set_tuning(best["lanes"], best["slabs_per_lane"])
            return best
    st = kernels.SubsetState(shape, center, size, lors.device)
    results = []
    for bins in sort_bins:
        sample = lors if bins == 0 else lors.index_select(0, direction_order(lors, bins)).contiguous()
        for lanes, spl in CANDIDATES:
            _lib.set_tuning(lanes, spl)
            ms = _time(lambda: st.subset(sample, None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=tof,
                                         tof_nsigma=tof_nsigma), reps)
            results.append({"lanes": lanes, "slabs_per_lane": spl, "sort_bins": bins, "ms": ms})
    best = min(results, key=lambda r: r["ms"])
    best = dict(best, key=key, tried=len(results))
    _lib.set_tuning(best["lanes"], best["slabs_per_lane"])
    if cache:
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        table[key] = best
        with open(cache, "w") as f:
            json.dump(table, f, indent=1)
    return best
