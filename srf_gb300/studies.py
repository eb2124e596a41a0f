"""Many independent list-mode studies reconstructed together (not in the reference).

``StudyBatch`` holds every study's LORs (permuted once into subset order), its images and its
sensitivity on the device, and runs each OSEM subset step for *all* studies with two launches:
``srf_osem_subset_batch`` (a persistent kernel that walks every study's 32-LOR batches) and
``srf_osem_update_batch``. One full iteration (n_sub subsets) can be captured once into a CUDA
graph and replayed, so an iteration over 64 studies costs 2 * n_sub kernel nodes and no host work.
Alternatively (``capture(concurrent=True)``) the graph holds every study's own chain of subset and
update kernels as independent branches over a pool of streams, which the GPU runs side by side.

The per-study descriptors (``srf_study`` in include/srf_gb300.h) are built on the host from
validated tensors and copied to the device once per subset.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import kernels
from ._lib import SRF_RATIO_DIV_NO_NAN, call, f32, i32, i64, ptr, stream_ptr


class SrfStudy(ctypes.Structure):
    """Host mirror of ``srf_study`` (same field order, natural C alignment)."""
    _fields_ = [
        ("lors", ctypes.c_void_p), ("n", ctypes.c_int64), ("lor_stride", ctypes.c_int32),
        ("tof_stride", ctypes.c_int32), ("tof", ctypes.c_void_p), ("y", ctypes.c_void_p),
        ("x", ctypes.c_void_p), ("x_t", ctypes.c_void_p), ("bp", ctypes.c_void_p),
        ("bp_t", ctypes.c_void_p), ("emap", ctypes.c_void_p), ("grid", ctypes.c_int32 * 3),
        ("center", ctypes.c_float * 3), ("size", ctypes.c_float * 3),
    ]


class Study:
    """One study: LORs (N, 7) on the device, image geometry and an x-fastest sensitivity."""

    def __init__(self, lors: torch.Tensor, shape: Sequence[int], center: Sequence[float],
                 size: Sequence[float], emap_xfast: torch.Tensor, y: Optional[torch.Tensor] = None):
        kernels.check_lors(lors, True)
        self.lors, self.y = lors, y
        self.shape, self.center, self.size = list(shape), list(center), list(size)
        self.emap = emap_xfast
        dev = lors.device
        self.state = kernels.SubsetState(shape, center, size, dev)


def _to_device_bytes(obj, device) -> torch.Tensor:
    raw = bytes(obj)
    return torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(device)


class StudyBatch:
    def __init__(self, studies: List[Study], n_sub: int, tof: Tuple[float, float],
                 tof_nsigma: float = 3.0, seed: int = 0, rule: int = SRF_RATIO_DIV_NO_NAN,
                 eps: float = 1e-5):
        if not studies:
            raise ValueError("no studies")
        self.studies, self.n_sub = studies, n_sub
        self.tof, self.tof_nsigma, self.rule, self.eps = tof, tof_nsigma, rule, eps
        dev = studies[0].lors.device
        self.device = dev
        rng = np.random.default_rng(seed)
        for st in studies:
            perm = torch.as_tensor(rng.permutation(st.lors.shape[0]), device=dev)
            st.lors = st.lors.index_select(0, perm).contiguous()
            if st.y is not None:
                st.y = st.y.index_select(0, perm).contiguous()
        # per-subset descriptor arrays and batch offsets
        self.desc, self.boff, self.total = [], [], []
        for k in range(n_sub):
            arr = (SrfStudy * len(studies))()
            off = [0]
            for j, st in enumerate(studies):
                n = st.lors.shape[0]
                per = n // n_sub
                sl = st.lors[k * per:(k + 1) * per]
                d = arr[j]
                d.lors = sl.data_ptr() if per else st.lors.data_ptr()
                d.n = per
                d.lor_stride = st.lors.stride(0)
                d.tof_stride = st.lors.stride(0)
                d.tof = (sl.data_ptr() if per else st.lors.data_ptr()) + 24
                d.y = (st.y[k * per:(k + 1) * per].data_ptr() if (st.y is not None and per) else None)
                s = st.state
                d.x, d.x_t, d.bp, d.bp_t = (s.x.data_ptr(), s.x_t.data_ptr(), s.bp.data_ptr(),
                                            s.bp_t.data_ptr())
                d.emap = st.emap.data_ptr()
                d.grid[:] = st.shape
                d.center[:] = st.center
                d.size[:] = st.size
                off.append(off[-1] + (per + 31) // 32)
            self.desc.append(_to_device_bytes(arr, dev))
            # two zeroed work counters follow the offsets (the batch kernel's batch tickets)
            self.boff.append(torch.as_tensor(off + [0, 0], dtype=torch.int64, device=dev))
            self.total.append(off[-1])
        toff = [0]
        for st in studies:
            nx, ny, nz = st.shape
            toff.append(toff[-1] + ((nx + 31) // 32) * ((ny + 31) // 32) * nz)
        self.toff = torch.as_tensor(toff, dtype=torch.int64, device=dev)
        self.total_tiles = toff[-1]
        self.graph = None

    def subset(self, k: int) -> None:
        s = stream_ptr(self.device)
        call("srf_osem_subset_batch", ptr(self.desc[k]), i32(len(self.studies)), ptr(self.boff[k]),
             i64(self.total[k]), i32(1), f32(self.tof[0]), f32(self.tof[1]), f32(self.tof_nsigma),
             i32(self.rule), f32(self.eps), None, s)
        call("srf_osem_update_batch", ptr(self.desc[k]), i32(len(self.studies)), ptr(self.toff),
             i64(self.total_tiles), i32(1), s)

    def iteration(self) -> None:
        for k in range(self.n_sub):
            self.subset(k)

    def iteration_concurrent(self, n_streams: int = 8) -> None:
        """One iteration as independent per-study chains (each study's subset and update kernels
        in order) spread over ``n_streams`` streams forked from the current one and joined at the
        end (largest studies first, balanced by event count): the studies' kernels run side by
        side, each at the single-study kernel's efficiency, and small studies fill the GPU together
        instead of one at a time."""
        main = torch.cuda.current_stream(self.device)
        streams = self._streams(n_streams)
        for st_ in streams:
            st_.wait_stream(main)
        for j, st in self._assignment(len(streams)):
            with torch.cuda.stream(streams[j]):
                per = st.lors.shape[0] // self.n_sub
                for k in range(self.n_sub):
                    if per:
                        st.state.subset(st.lors[k * per:(k + 1) * per],
                                        None if st.y is None else st.y[k * per:(k + 1) * per],
                                        rule=self.rule, eps=self.eps, tof=self.tof, tof_nsigma=self.tof_nsigma)
                    st.state.update(st.emap, guard_zero=True)
        for st_ in streams:
            main.wait_stream(st_)

    def _assignment(self, n: int):
        """(stream, study) pairs: studies by event count, largest first, each onto the stream with
        the fewest events so far (longest-processing-time-first), so that the chains end together
        instead of one stream carrying several large studies."""
        load = [0] * n
        out = []
        for st in sorted(self.studies, key=lambda s_: -int(s_.lors.shape[0])):
            j = min(range(n), key=lambda i: load[i])
            load[j] += int(st.lors.shape[0])
            out.append((j, st))
        return out

    def _streams(self, n: int) -> List[torch.cuda.Stream]:
        have = getattr(self, "_pool", [])
        while len(have) < n:
            have.append(torch.cuda.Stream(self.device))
        self._pool = have
        return have[:n]

    def capture(self, concurrent: bool = False, n_streams: int = 8) -> None:
        """Record one iteration into a CUDA graph (after one eager warm-up iteration): the two
        batch kernels per subset, or with ``concurrent`` the per-study chains as parallel branches."""
        run = (lambda: self.iteration_concurrent(n_streams)) if concurrent else self.iteration
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            run()
        torch.cuda.current_stream(self.device).wait_stream(side)
        torch.cuda.synchronize(self.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            run()

    def replay(self) -> None:
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def images(self) -> List[torch.Tensor]:
        return [st.state.x.contiguous() for st in self.studies]

    def reset(self) -> None:
        for st in self.studies:
            st.state.x.fill_(1.0)
            st.state.x_t.fill_(1.0)
            st.state.bp.zero_()
            st.state.bp_t.zero_()
