"""ctypes binding of ``libsrf_gb300.so`` (the C ABI in include/srf_gb300.h).

The library is loaded from the package directory (built in-tree by ``srf_gb300.build``). There is
no fallback: if the library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import contextlib
import ctypes
import os
import threading
from typing import Optional, Sequence

import torch

from . import build as _build

_f32p = ctypes.c_void_p
_lock = threading.Lock()
_lib = None

SRF_RATIO_DIV_NO_NAN = 0
SRF_RATIO_PLAIN = 1

# every symbol include/srf_gb300.h declares
EXPORTS = (
    "srf_last_error", "srf_version", "srf_set_group_lanes", "srf_set_tuning", "srf_projection", "srf_backprojection",
    "srf_projection_tof", "srf_backprojection_tof", "srf_projection_adjoint", "srf_fold_views",
    "srf_copy_view", "srf_count_pairs", "srf_projection_batch", "srf_projection_adjoint_batch", "srf_osem_subset", "srf_osem_update", "srf_osem_subset_batch",
    "srf_osem_update_batch", "srf_emap_block_full", "srf_sss",
    "srf_backprojection_tof_noalloc", "srf_listmode_snap", "srf_lm2sino", "srf_attenuation",
    "srf_conv3d_fwd", "srf_conv3d_wgrad", "srf_conv3d_flip_weights", "srf_cnn_relu_bwd",
    "srf_set_conv_tc", "srf_conv_tc_status", "srf_conv_last_path",
    "srf_cnn_bias_grad", "srf_cnn_pool2", "srf_cnn_upsample2", "srf_cnn_add", "srf_cnn_head8", "srf_calib_l2", "srf_calib_sink_size",
    "srf_cnn_rel_mse", "srf_cnn_adam", "srf_spot_fit", "srf_scale_by_basis",
    "srf_deform", "srf_shift", "srf_shift_z", "srf_rotate", "srf_deform_invert",
)


class SrfError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the library once. Raises if it is missing (no CPU fallback exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(
                    f"{path} is missing: build it with `python -m srf_gb300.build` "
                    "(srf_gb300 has no CPU fallback)")
            _build.build()
        lib = ctypes.CDLL(path)
        lib.srf_last_error.restype = ctypes.c_char_p
        lib.srf_version.restype = ctypes.c_int
        for name in EXPORTS:
            getattr(lib, name)  # raises AttributeError if a symbol is missing
        _lib = lib
        return lib


def _check(fn: str, rc: int) -> None:
    if rc != 0:
        msg = _lib.srf_last_error().decode(errors="replace")
        raise SrfError(fn, rc, msg)


def call(fn: str, *args) -> None:
    lib = load()
    _check(fn, getattr(lib, fn)(*args))


# ------------------------------------------------------------------ argument helpers

def ptr(t: Optional[torch.Tensor]):
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def i64x3(v: Sequence[int]):
    return (ctypes.c_int64 * 3)(*[int(x) for x in v])


def i32x3(v: Sequence[int]):
    return (ctypes.c_int32 * 3)(*[int(x) for x in v])


def f32x3(v: Sequence[float]):
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def f32(v: float):
    return ctypes.c_float(float(v))


def f64(v: float):
    return ctypes.c_double(float(v))


def i32(v: int):
    return ctypes.c_int32(int(v))


def i64(v: int):
    return ctypes.c_int64(int(v))


def stream_ptr(device: torch.device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def xfast_strides(shape):
    nx, ny, nz = shape
    return (1, nx, nx * ny)


def yfast_strides(shape):
    nx, ny, nz = shape
    return (ny, 1, nx * ny)


_TUNING = {"lanes": 32, "slabs": 4}  # the library's defaults, mirrored by the setters below


def set_group_lanes(lanes: int) -> None:
    call("srf_set_group_lanes", ctypes.c_int(lanes))
    _TUNING["lanes"] = lanes


def set_tuning(lanes: int, slabs_per_lane: int) -> None:
    call("srf_set_tuning", ctypes.c_int(lanes), ctypes.c_int(slabs_per_lane))
    _TUNING.update(lanes=lanes, slabs=slabs_per_lane)


@contextlib.contextmanager
def tuning(lanes: int, slabs_per_lane: int):
    """Launch variant for the calls inside the block (lanes per LOR, slabs per lane), restored
    afterwards: e.g. 16 lanes for LORs that cross at most 64 slabs of a small grid."""
    prev = (_TUNING["lanes"], _TUNING["slabs"])
    set_tuning(lanes, slabs_per_lane)
    try:
        yield
    finally:
        set_tuning(*prev)
