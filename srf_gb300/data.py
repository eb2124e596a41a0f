"""Boundary data types with srfnef's field names and semantics.

srfnef's containers are frozen, slotted attrs classes whose fields all default to ``None`` and that
are copied with ``update(**changes)`` (srfnef/base/base.py:154-177). The hot path only needs the
four containers it passes around:

* ``Image`` / ``Emap`` / ``Umap`` -- ``data`` (nx, ny, nz) float32, ``center`` [3] and ``size`` [3]
  in mm (srfnef/data/image.py:20-37, data/emap.py:20-37, data/umap.py); ``shape`` and
  ``unit_size`` as in srfnef/ops/common/property_mixins.py:13-67;
* ``Lors`` -- ``data`` (N, 6) or (N, 7) float32, column 6 is the TOF value in mm
  (srfnef/data/lors.py:6-26);
* ``Listmode`` -- ``data`` (N,) float32 values plus their ``lors`` (srfnef/data/listmode.py:17-28).

``data`` may be a numpy array or a torch tensor (on the CPU or a CUDA device); the function classes
accept both and return the same kind they were given.
"""
from __future__ import annotations

import dataclasses
from typing import Any, List, Optional

import numpy as np


def _shape_of(data) -> List[int]:
    return [int(x) for x in data.shape]


class _NefLike:
    """Frozen-record behaviour shared by the containers (``update``, ``asdict``)."""

    def update(self, **kwargs):
        return dataclasses.replace(self, **kwargs)

    def asdict(self) -> dict:
        return {f.name: getattr(self, f.name) for f in dataclasses.fields(self)}


class _Arith:
    """Elementwise arithmetic on ``.data`` (srfnef/ops/common/arithmetic_mixins.py:12-87)."""

    def _other(self, other):
        return other.data if hasattr(other, "data") else other

    def __neg__(self):
        return self.update(data=-self.data)

    def __add__(self, other):
        return self.update(data=self.data + self._other(other))

    def __sub__(self, other):
        return self.update(data=self.data - self._other(other))

    def __mul__(self, other):
        return self.update(data=self.data * self._other(other))

    def __truediv__(self, other):
        return self.update(data=self.data / self._other(other))

    def abs(self):
        return self.update(data=abs(self.data))


@dataclasses.dataclass(frozen=True)
class Image(_NefLike, _Arith):
    data: Any = None
    center: Optional[List[float]] = None
    size: Optional[List[float]] = None

    @property
    def shape(self) -> List[int]:
        return _shape_of(self.data)

    @property
    def unit_size(self) -> List[float]:
        return [s1 / s2 for s1, s2 in zip(self.size, self.shape)]


@dataclasses.dataclass(frozen=True)
class Emap(Image):
    pass


@dataclasses.dataclass(frozen=True)
class Umap(Image):
    pass


@dataclasses.dataclass(frozen=True)
class Lors(_NefLike):
    data: Any = None

    @property
    def shape(self) -> List[int]:
        return _shape_of(self.data)

    def __len__(self) -> int:
        return int(self.data.shape[0])

    @property
    def length(self) -> int:
        return len(self)

    @property
    def fst(self):
        return self.data[:, :3]

    @property
    def snd(self):
        return self.data[:, 3:6]

    @property
    def tof_values(self):
        return self.data[:, 6]

    def append(self, lors: "Lors") -> "Lors":
        return self.update(data=np.vstack((self.data, lors.data)))


@dataclasses.dataclass(frozen=True)
class Listmode(_NefLike, _Arith):
    data: Any = None
    lors: Optional[Lors] = None

    @property
    def shape(self) -> List[int]:
        return _shape_of(self.data)

    def __len__(self) -> int:
        return int(self.data.shape[0])

    @property
    def length(self) -> int:
        return len(self)

    def append(self, listmode: "Listmode") -> "Listmode":
        return self.update(data=np.hstack((self.data, listmode.data)),
                           lors=self.lors.append(listmode.lors))
