"""The C-ABI library loads and exports every symbol include/srf_gb300.h declares, and its
argument checks return error codes before touching a device (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "srf_gb300.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(srf_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from srf_gb300 import _lib, build
    build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    from srf_gb300._lib import EXPORTS
    assert sorted(EXPORTS) == names


def test_version_and_lanes(lib):
    assert lib.srf_version() == 100
    assert lib.srf_set_group_lanes(12) == 1
    assert b"lanes" in lib.srf_last_error()
    assert lib.srf_set_group_lanes(32) == 0


def _geom():
    grid = (ctypes.c_int32 * 3)(8, 8, 4)
    center = (ctypes.c_float * 3)(0, 0, 0)
    size = (ctypes.c_float * 3)(16, 16, 8)
    st = (ctypes.c_int64 * 3)(1, 8, 64)
    return grid, center, size, st


def test_argument_checks(lib):
    grid, center, size, st = _geom()
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: every call below fails its checks
    p = lib.srf_projection
    # NULL lors with n > 0
    assert p(None, ctypes.c_int64(5), 6, fake, st, None, None, grid, center, size, fake, None) == 1
    # stride < 6
    assert p(fake, ctypes.c_int64(5), 5, fake, st, None, None, grid, center, size, fake, None) == 1
    # negative count
    assert p(fake, ctypes.c_int64(-1), 6, fake, st, None, None, grid, center, size, fake, None) == 1
    # bad grid
    bad = (ctypes.c_int32 * 3)(0, 8, 4)
    assert p(fake, ctypes.c_int64(5), 6, fake, st, None, None, bad, center, size, fake, None) == 2
    # non-finite center
    nanc = (ctypes.c_float * 3)(float("nan"), 0, 0)
    assert p(fake, ctypes.c_int64(5), 6, fake, st, None, None, grid, nanc, size, fake, None) == 3
    # negative stride of the image view
    nst = (ctypes.c_int64 * 3)(-1, 8, 64)
    assert p(fake, ctypes.c_int64(5), 6, fake, nst, None, None, grid, center, size, fake, None) == 2
    # TOF parameters
    pt = lib.srf_projection_tof
    assert pt(fake, ctypes.c_int64(5), 7, fake, 7, ctypes.c_float(3.66), ctypes.c_float(float("inf")),
              ctypes.c_float(0), fake, st, None, None, grid, center, size, fake, None) == 3
    assert pt(fake, ctypes.c_int64(5), 7, fake, 7, ctypes.c_float(3.66), ctypes.c_float(1000),
              ctypes.c_float(-1), fake, st, None, None, grid, center, size, fake, None) == 1
    # unknown ratio rule
    assert lib.srf_osem_subset(fake, ctypes.c_int64(5), 7, None, 7, ctypes.c_float(0), ctypes.c_float(0),
                               ctypes.c_float(0), None, None, 7, ctypes.c_float(0), fake, None, fake,
                               None, grid, center, size, None, None) == 1
    assert b"ratio" in lib.srf_last_error()
    # empty input succeeds without a launch
    assert p(None, ctypes.c_int64(0), 6, fake, st, None, None, grid, center, size, None, None) == 0
    # surrogate spot check: basis size, sample count, ridge, NULL pointers
    fit = lib.srf_spot_fit
    i64, i32, f64 = ctypes.c_int64, ctypes.c_int32, ctypes.c_double
    assert fit(fake, i64(100), fake, fake, i32(64), fake, i32(13), f64(1e-6), fake, None) == 1
    assert fit(fake, i64(100), fake, fake, i32(1), fake, i32(9), f64(1e-6), fake, None) == 1
    assert fit(fake, i64(100), fake, fake, i32(64), fake, i32(9), f64(-1.0), fake, None) == 1
    assert fit(fake, i64(100), None, fake, i32(64), fake, i32(9), f64(1e-6), fake, None) == 1
    sb = lib.srf_scale_by_basis
    assert sb(fake, i64(100), fake, i32(0), fake, None) == 1
    assert sb(fake, i64(100), None, i32(9), fake, None) == 1
    assert sb(fake, i64(0), fake, i32(9), fake, None) == 0
    # convolution: channel counts not multiples of 16, a slice past the channel stride, shapes that differ
    a6 = lambda *v: (ctypes.c_int32 * 6)(*v)
    conv = lib.srf_conv3d_fwd
    assert conv(fake, a6(1, 4, 4, 4, 16, 0), i32(12), fake, None, i32(16), i32(1), fake, a6(1, 4, 4, 4, 16, 0),
                None, None) == 1
    assert conv(fake, a6(1, 4, 4, 4, 16, 8), i32(16), fake, None, i32(16), i32(1), fake, a6(1, 4, 4, 4, 16, 0),
                None, None) == 2
    assert conv(fake, a6(1, 4, 4, 4, 16, 0), i32(16), fake, None, i32(16), i32(1), fake, a6(1, 4, 4, 5, 16, 0),
                None, None) == 2


def test_study_descriptor_layout_matches_header(tmp_path):
    """srf_gb300.studies.SrfStudy (ctypes) must lay out exactly like the C srf_study."""
    import shutil
    import subprocess
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    from srf_gb300.studies import SrfStudy
    src = tmp_path / "sz.cc"
    src.write_text('#include <cstdio>\n#include <cstddef>\n#include "srf_gb300.h"\n'
                   'int main(){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(srf_study),'
                   ' offsetof(srf_study, n), offsetof(srf_study, emap), offsetof(srf_study, grid),'
                   ' offsetof(srf_study, center), offsetof(srf_study, size));}\n')
    exe = tmp_path / "sz"
    subprocess.run([cxx, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    want = [ctypes.sizeof(SrfStudy), SrfStudy.n.offset, SrfStudy.emap.offset, SrfStudy.grid.offset,
            SrfStudy.center.offset, SrfStudy.size.offset]
    assert [int(v) for v in got] == want
