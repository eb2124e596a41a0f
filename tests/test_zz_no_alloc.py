"""srf_backprojection_tof_noalloc: the TOF backprojection for callers that cannot allocate device
memory (a plugin inside a framework that owns the device memory, or an acquisition service with a
fixed device-memory reservation). It keeps its y-dominant accumulator in a static device array
instead of asking for one, so its output must equal srf_backprojection_tof's, call after call
(the array keeps the previous call's contents and must be cleared by every call).

The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _noalloc(lib, lors, vals, out, shape, center, size, tof, n=None):
    dev = lors.device
    n = lors.shape[0] if n is None else n
    grid = (ctypes.c_int32 * 3)(*shape)
    c = (ctypes.c_float * 3)(*center)
    s = (ctypes.c_float * 3)(*size)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rc = lib.srf_backprojection_tof_noalloc(
        ctypes.c_void_p(lors.data_ptr()), ctypes.c_int64(n), 7, ctypes.c_void_p(lors.data_ptr() + 24), 7,
        ctypes.c_float(tof[0]), ctypes.c_float(tof[1]), ctypes.c_float(0.0),
        ctypes.c_void_p(vals.data_ptr()), ctypes.c_void_p(out.data_ptr()), grid, c, s, stream)
    assert rc == 0, lib.srf_last_error()


def test_noalloc_matches_backprojection_tof_twice(cuda_lib, small_case):
    from srf_gb300 import _lib, kernels
    lib = _lib.load()
    ic, sc = small_case["ic"], small_case["scanner"]
    dev = torch.device("cuda", 0)
    lors = torch.as_tensor(small_case["lors"], device=dev).contiguous()
    n = lors.shape[0]
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    nx, ny, nz = ic.shape
    for call in range(2):
        vals = torch.as_tensor(np.random.default_rng(10 + call).random(n).astype(np.float32), device=dev)
        # the existing entry point, with the caller providing the second accumulator
        want = kernels.backproject(lors, vals, ic.shape, ic.center, ic.size, tof=tof)
        # the new one: output image only (x-fastest), zero-filled by the caller
        out = torch.zeros((nz, ny, nx), dtype=torch.float32, device=dev)
        _noalloc(lib, lors, vals, out, ic.shape, ic.center, ic.size, tof)
        got = out.permute(2, 1, 0).cpu().numpy()
        assert rel_l2(got, want.cpu().numpy()) <= TOL, f"call {call}"


def test_noalloc_accumulates_and_clears_per_grid(cuda_lib, small_case):
    """The output is accumulated into (like srf_backprojection_tof); a smaller grid after a larger
    one sees none of the larger call's scratch; n == 0 leaves the image unchanged."""
    from srf_gb300 import _lib, kernels
    lib = _lib.load()
    ic, sc = small_case["ic"], small_case["scanner"]
    dev = torch.device("cuda", 0)
    lors = torch.as_tensor(small_case["lors"], device=dev).contiguous()
    n = lors.shape[0]
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    vals = torch.as_tensor(np.random.default_rng(21).random(n).astype(np.float32), device=dev)
    # a larger grid first (same field of view, finer voxels), leaving its scratch behind
    big = [2 * ic.shape[0], 2 * ic.shape[1], ic.shape[2]]
    out_big = torch.zeros((big[2], big[1], big[0]), dtype=torch.float32, device=dev)
    _noalloc(lib, lors, vals, out_big, big, ic.center, ic.size, tof)
    want_big = kernels.backproject(lors, vals, big, ic.center, ic.size, tof=tof)
    assert rel_l2(out_big.permute(2, 1, 0).cpu().numpy(), want_big.cpu().numpy()) <= TOL
    # then the smaller grid, into a pre-filled image
    nx, ny, nz = ic.shape
    prefill = torch.as_tensor(np.random.default_rng(22).random((nz, ny, nx)).astype(np.float32), device=dev)
    out = prefill.clone()
    _noalloc(lib, lors, vals, out, ic.shape, ic.center, ic.size, tof)
    want = kernels.backproject(lors, vals, ic.shape, ic.center, ic.size, tof=tof)
    expect = prefill.permute(2, 1, 0).cpu().numpy() + want.cpu().numpy()
    assert rel_l2(out.permute(2, 1, 0).cpu().numpy(), expect) <= TOL
    # no events: the image stays as it was, bit for bit
    before = out.clone()
    _noalloc(lib, lors, vals, out, ic.shape, ic.center, ic.size, tof, n=0)
    torch.cuda.synchronize()
    assert torch.equal(out, before)


def test_noalloc_rejects_oversized_grid(cuda_lib):
    from srf_gb300 import _lib
    lib = _lib.load()
    big = (ctypes.c_int32 * 3)(256, 256, 80)  # 5.2e6 voxels > SRF_NOALLOC_MAX_VOXELS
    center = (ctypes.c_float * 3)(0, 0, 0)
    size = (ctypes.c_float * 3)(512, 512, 160)
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the size check fails first
    rc = lib.srf_backprojection_tof_noalloc(fake, ctypes.c_int64(10), 7, fake, 7,
                                            ctypes.c_float(3.66), ctypes.c_float(1000.0),
                                            ctypes.c_float(0.0), fake, fake, big, center, size, None)
    assert rc == 5
    assert b"at most" in lib.srf_last_error()
