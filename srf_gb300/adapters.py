"""GATE list-mode ingestion: sub-run files to crystal-snapped LORs on the GPU.

The reference reads the GATE coincidence output of ``nb_sub`` sub-runs (``path`` with '?'
replaced by 0 .. nb_sub-1, each an (N_i, >= 7) float array saved by numpy: endpoints x1 y1 z1
x2 y2 z2, the TOF value, optionally a bed id in the last column), stacks them and snaps both
endpoints to crystal centres through the ECAT index round trip
(srfnef/adapters/listmode_from_gate_out.py:36-124).

Here each sub-run is copied into pinned host memory and sent to the device on a copy stream
while the previous one is snapped (``srf_listmode_snap``, the kernel of ``PetEcatListmodeTrans``
on the GPU), straight into the output LOR array. Results stay on the device as (N, 6) or (N, 7)
float32 LORs with unit values.

* ``listmode_from_gate_out``: snapped endpoints, 6 columns (listmode_from_gate_out.py:36-59;
  the reference returns the bare array as the LORs, here it is wrapped in ``Lors``).
* ``listmode_tof_from_gate_out``: snapped endpoints plus the TOF column, times ``tof_scale``
  (listmode_from_gate_out.py:84-100; the reference's body calls ListmodeToId / IdToListmode,
  which that module never defines, so it cannot run. What it does is the snap above with column
  7 appended, which is what is done here).
* ``listmode_from_gate_out_multi_bed``: one list mode per bed id (the last column of each file;
  listmode_from_gate_out.py:103-124, which has the same undefined names), each snapped.

Only ``PetEcatScanner`` geometries are supported (cylindrical scanners raise
``NotImplementedError``, as the reference does for unknown scanners).
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import kernels
from .data import Listmode, Lors
from .functions import device
from .geometry import PetEcatScanner


def gate_paths(path: str, nb_sub: int) -> List[str]:
    """The sub-run files: '?' in ``path`` replaced by 0 .. nb_sub-1."""
    if nb_sub < 1:
        raise ValueError("nb_sub must be >= 1")
    return [path.replace("?", str(i)) for i in range(nb_sub)]


def read_gate_rows(path: str, nb_sub: int) -> List[np.ndarray]:
    """Each sub-run's rows as a read-only memory map (no copy), checked for shape and dtype."""
    out = []
    for p in gate_paths(path, nb_sub):
        a = np.load(p, mmap_mode="r")
        if a.ndim != 2 or a.shape[1] < 7:
            raise ValueError(f"{p}: expected an (N, >= 7) array, got {a.shape}")
        if a.dtype.kind != "f":
            raise ValueError(f"{p}: expected floating-point rows, got {a.dtype}")
        out.append(a)
    return out


def _snap_rows(parts: Sequence[np.ndarray], scanner: PetEcatScanner, cols: int, tof_scale: float,
               dev) -> torch.Tensor:
    """Stack the parts' first 7 columns on the device and snap them: (N, cols) float32 LORs."""
    if not isinstance(scanner, PetEcatScanner):
        raise NotImplementedError("only PetEcatScanner geometries are supported")
    n = sum(int(p.shape[0]) for p in parts)
    out = torch.empty((n, cols), dtype=torch.float32, device=dev)
    if n == 0:
        return out
    biggest = max(int(p.shape[0]) for p in parts)
    stage = [torch.empty((biggest, 7), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    raw = [torch.empty((biggest, 7), dtype=torch.float32, device=dev) for _ in range(2)]
    copied = [torch.cuda.Event(), torch.cuda.Event()]   # stage[b] -> raw[b] has landed
    snapped = [torch.cuda.Event(), torch.cuda.Event()]  # the kernel has read raw[b]
    copy = torch.cuda.Stream(dev)
    main = torch.cuda.current_stream(dev)
    off = 0
    for j, part in enumerate(parts):
        b, m = j % 2, int(part.shape[0])
        if m == 0:
            continue
        copied[b].synchronize()  # stage[b]'s previous contents have left for the device
        np.copyto(stage[b][:m].numpy(), part[:, :7], casting="same_kind")
        copy.wait_event(snapped[b])  # raw[b]'s previous part has been snapped
        with torch.cuda.stream(copy):
            raw[b][:m].copy_(stage[b][:m], non_blocking=True)
        copied[b].record(copy)
        main.wait_event(copied[b])
        kernels.snap(raw[b][:m], scanner, out=out[off:off + m])
        snapped[b].record(main)
        off += m
    if cols == 7 and tof_scale != 1.0:
        out[:, 6] *= tof_scale
    return out


def listmode_from_gate_out(path: str, scanner: PetEcatScanner, nb_sub: int) -> Listmode:
    dev = device()
    lors = _snap_rows(read_gate_rows(path, nb_sub), scanner, 6, 1.0, dev)
    return Listmode(torch.ones(lors.shape[0], dtype=torch.float32, device=dev), Lors(lors))


def listmode_tof_from_gate_out(path: str, scanner: PetEcatScanner, nb_sub: int,
                               tof_scale: float = 1.0) -> Listmode:
    dev = device()
    lors = _snap_rows(read_gate_rows(path, nb_sub), scanner, 7, float(tof_scale), dev)
    return Listmode(torch.ones(lors.shape[0], dtype=torch.float32, device=dev), Lors(lors))


def split_by_bed(parts: Sequence[np.ndarray]) -> Dict[float, List[np.ndarray]]:
    """Each part's rows grouped by bed id (last column), in file order within a bed."""
    beds: Dict[float, List[np.ndarray]] = {}
    for p in parts:
        ids = np.asarray(p[:, -1])
        for b in np.unique(ids):
            beds.setdefault(float(b), []).append(np.asarray(p[ids == b]))
    return beds


def listmode_from_gate_out_multi_bed(path: str, scanner: PetEcatScanner,
                                     nb_sub: int) -> Dict[float, Listmode]:
    dev = device()
    out = {}
    for bed, parts in split_by_bed(read_gate_rows(path, nb_sub)).items():
        lors = _snap_rows(parts, scanner, 6, 1.0, dev)
        out[bed] = Listmode(torch.ones(lors.shape[0], dtype=torch.float32, device=dev), Lors(lors))
    return out
