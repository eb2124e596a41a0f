"""CPU oracle for the list-mode reconstruction hot path. TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this module, and
only as the reference the GPU results are compared with. The product package srf_gb300 never
imports it.

* ``projection`` / ``backprojection`` / ``projection_adjoint`` -- ctypes bindings of the C
  restatement in siddon_oracle.c (built by ``make -C oracle`` into oracle/_build/liboracle.so);
* ``ref_*`` -- the reference's own device functions compiled on the host (oracle/_ref, built by
  ``make -C oracle ref`` where the reference sources exist); used to pin the restatement;
* ``mlem`` / ``osem`` -- numpy float32 restatements of the update loops
  (srfnef/functions/mlem.py:28-45, mlem_full.py:47-72, mlem_full_tof.py:43-69, osem_full.py:49-87);
* ``emap_block_full`` -- srfnef/functions/emap_generator.py:77-111 over the oracle backprojector;
* ``sss`` -- ctypes binding of sss_oracle.c.

Images passed in and returned here are (nx, ny, nz) numpy arrays, as srfnef's ``Image.data``;
the C code works on the x-fastest flat layout, i.e. the transpose that srfnef's TF wrappers pass.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libsrf_ref.so")

RULES_PROJ, RULES_BACK = 0, 1
GATHER, SCATTER = 0, 1

_lib = None
_ref = None

# Host threads of the oracle traversals when a call does not say (1: the serial code path, whose
# backprojection sums in the reference's LOR order). Large parity cases raise it.
THREADS = 1


def set_threads(n: int) -> int:
    """Set the default thread count of the oracle traversals; returns the previous one."""
    global THREADS
    prev, THREADS = THREADS, max(1, int(n))
    return prev

_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int)


def build(ref: bool = False) -> None:
    """Compile the oracle (and, with ref=True and the reference present, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.or_trace.restype = ctypes.c_int64
        _lib.or_trace.argtypes = [
            _f32p, ctypes.c_int64, ctypes.c_int, _f32p, ctypes.c_int, ctypes.c_float,
            ctypes.c_float, ctypes.c_float, _i32p, _f32p, _f32p, ctypes.c_int, ctypes.c_int,
            _f32p, _f32p, _f32p, _f32p]
        _lib.or_trace_mt.restype = ctypes.c_int64
        _lib.or_trace_mt.argtypes = _lib.or_trace.argtypes + [ctypes.c_int]
        _lib.or_sss.restype = None
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_LIB_PATH)
        _ref.ref_take_atomic_count.restype = ctypes.c_int64
    return _ref


def _p(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(_f32p)


def _geom(shape, center, size):
    grid = np.ascontiguousarray(np.asarray(shape, dtype=np.int32))
    c = np.ascontiguousarray(np.asarray(center, dtype=np.float32))
    s = np.ascontiguousarray(np.asarray(size, dtype=np.float32))
    return grid, c, s


def _xfast(img: np.ndarray) -> np.ndarray:
    """(nx, ny, nz) -> flat x-fastest float32 (the layout srfnef's TF ops receive)."""
    return np.ascontiguousarray(np.asarray(img, dtype=np.float32).transpose(2, 1, 0))


def _from_xfast(flat: np.ndarray, shape) -> np.ndarray:
    nx, ny, nz = shape
    return np.ascontiguousarray(flat.reshape(nz, ny, nx).transpose(2, 1, 0))


def _lor_args(lors: np.ndarray, tof: bool):
    lors = np.ascontiguousarray(lors, dtype=np.float32)
    stride = lors.shape[1]
    tof_ptr = None
    if tof:
        assert stride >= 7, "TOF needs a 7th column"
        tof_ptr = ctypes.cast(lors.ctypes.data + 6 * 4, _f32p)
    return lors, stride, tof_ptr


def trace(lors, shape, center, size, rules, action, *, tof=False, tof_bin=0.0, tof_sigma2=0.0,
          tof_nsigma=0.0, image=None, values=None, threads=None):
    """Generic traversal; returns (result, pairs). result is (N,) for GATHER, (nx,ny,nz) for SCATTER.
    threads > 1 uses the OpenMP variant (backprojection summed in a different order); None takes
    the module default THREADS."""
    L = lib()
    threads = THREADS if threads is None else threads
    fn = L.or_trace if threads <= 1 else (lambda *a: L.or_trace_mt(*a, threads))
    lors, stride, tof_ptr = _lor_args(lors, tof)
    n = lors.shape[0]
    grid, c, s = _geom(shape, center, size)
    if action == GATHER:
        img = _xfast(image)
        out = np.zeros(n, dtype=np.float32)
        pairs = fn(_p(lors), n, stride, tof_ptr, stride, tof_bin, tof_sigma2, tof_nsigma,
                   grid.ctypes.data_as(_i32p), _p(c), _p(s), rules, action, None, None,
                   _p(img), _p(out))
        return out, pairs
    vals = np.ascontiguousarray(values, dtype=np.float32)
    acc = np.zeros(int(np.prod(shape)), dtype=np.float32)
    pairs = fn(_p(lors), n, stride, tof_ptr, stride, tof_bin, tof_sigma2, tof_nsigma,
               grid.ctypes.data_as(_i32p), _p(c), _p(s), rules, action, _p(vals),
               _p(acc), None, None)
    return _from_xfast(acc, shape), pairs


def projection(image, lors, shape, center, size, *, tof=False, tof_bin=0.0, tof_sigma2=0.0,
               tof_nsigma=0.0):
    return trace(lors, shape, center, size, RULES_PROJ, GATHER, tof=tof, tof_bin=tof_bin,
                 tof_sigma2=tof_sigma2, tof_nsigma=tof_nsigma, image=image)[0]


def backprojection(values, lors, shape, center, size, *, tof=False, tof_bin=0.0, tof_sigma2=0.0,
                   tof_nsigma=0.0):
    return trace(lors, shape, center, size, RULES_BACK, SCATTER, tof=tof, tof_bin=tof_bin,
                 tof_sigma2=tof_sigma2, tof_nsigma=tof_nsigma, values=values)[0]


def projection_adjoint(values, lors, shape, center, size, *, tof=False, tof_bin=0.0,
                       tof_sigma2=0.0, tof_nsigma=0.0):
    return trace(lors, shape, center, size, RULES_PROJ, SCATTER, tof=tof, tof_bin=tof_bin,
                 tof_sigma2=tof_sigma2, tof_nsigma=tof_nsigma, values=values)[0]


# ---------------------------------------------------------------- reference (oracle/_ref)

def ref_projection(image, lors, shape, center, size, *, tof=False, tof_bin=0.0, tof_sigma2=0.0):
    R = ref_lib()
    lors, stride, tof_ptr = _lor_args(lors, tof)
    n = lors.shape[0]
    grid, c, s = _geom(shape, center, size)
    img = _xfast(image)
    out = np.zeros(n, dtype=np.float32)
    if tof:
        R.ref_projection_tof(_p(lors), ctypes.c_int64(n), stride, tof_ptr, stride,
                             ctypes.c_float(tof_bin), ctypes.c_float(tof_sigma2),
                             grid.ctypes.data_as(_i32p), _p(c), _p(s), _p(img), _p(out))
    else:
        R.ref_projection(_p(lors), ctypes.c_int64(n), stride, grid.ctypes.data_as(_i32p), _p(c),
                         _p(s), _p(img), _p(out))
    return out


def ref_backprojection(values, lors, shape, center, size, *, tof=False, tof_bin=0.0,
                       tof_sigma2=0.0):
    R = ref_lib()
    lors, stride, tof_ptr = _lor_args(lors, tof)
    n = lors.shape[0]
    grid, c, s = _geom(shape, center, size)
    vals = np.ascontiguousarray(values, dtype=np.float32)
    acc = np.zeros(int(np.prod(shape)), dtype=np.float32)
    R.ref_take_atomic_count()
    if tof:
        R.ref_backprojection_tof(_p(lors), ctypes.c_int64(n), stride, tof_ptr, stride,
                                 ctypes.c_float(tof_bin), ctypes.c_float(tof_sigma2), _p(vals),
                                 grid.ctypes.data_as(_i32p), _p(c), _p(s), _p(acc))
    else:
        R.ref_backprojection(_p(lors), ctypes.c_int64(n), stride, _p(vals),
                             grid.ctypes.data_as(_i32p), _p(c), _p(s), _p(acc))
    pairs = R.ref_take_atomic_count()
    return _from_xfast(acc, shape), pairs


# ---------------------------------------------------------------- update loops (numpy float32)

def div_no_nan(num, den):
    """tf.div_no_nan: 0 where the denominator is 0."""
    num = np.asarray(num, dtype=np.float32)
    den = np.asarray(den, dtype=np.float32)
    out = np.zeros(np.broadcast(num, den).shape, dtype=np.float32)
    nz = den != 0
    out[nz] = (num[nz] / den[nz]).astype(np.float32)
    return out


def guard_emap(emap):
    """zeros -> 1e8 (mlem_full_tof.py:56-58, mlem_full.py:60-61, mlem.py:33-34)."""
    e = np.array(emap, dtype=np.float32, copy=True)
    e[e == 0.0] = np.float32(1e8)
    return e


def mlem(lors, values, emap, shape, center, size, n_iter, *, rule="full_tof", tof=False,
         tof_bin=0.0, tof_sigma2=0.0, tof_nsigma=0.0, x0=None):
    """MLEM with the reference's update rule:
    rule 'mlem'     : p + mean(y)*1e-8, plain divide             (mlem.py:40-43)
    rule 'full'     : div_no_nan(y, p)                           (mlem_full.py:66-70)
    rule 'full_tof' : div_no_nan(y, p + 1e-5)                    (mlem_full_tof.py:62-67)
    x <- x * bp / emap with the zero-guarded emap, float32 throughout."""
    y = np.asarray(values, dtype=np.float32)
    em = guard_emap(emap)
    x = np.ones(shape, dtype=np.float32) if x0 is None else np.array(x0, dtype=np.float32)
    kw = dict(tof=tof, tof_bin=tof_bin, tof_sigma2=tof_sigma2, tof_nsigma=tof_nsigma)
    for _ in range(n_iter):
        p = projection(x, lors, shape, center, size, **kw)
        r = ratio(y, p, rule)
        bp = backprojection(r, lors, shape, center, size, **kw)
        x = (x * bp / em).astype(np.float32)
    return x


def ratio(y, p, rule):
    y = np.asarray(y, dtype=np.float32)
    p = np.asarray(p, dtype=np.float32)
    if rule == "mlem":
        return (y / (p + np.float32(np.mean(y) * 1e-8))).astype(np.float32)
    if rule == "full":
        return div_no_nan(y, p)
    if rule == "full_tof":
        return div_no_nan(y, p + np.float32(1e-5))
    if rule == "osem":
        return (y / (p + np.float32(1e-8))).astype(np.float32)
    raise ValueError(rule)


def osem_subsets(n, n_sub, perm):
    """Contiguous subsets of a permutation, n // n_sub events each (osem_full.py:63-69)."""
    n_per = n // n_sub
    return [perm[i * n_per:(i + 1) * n_per] for i in range(n_sub)]


def osem(lors, values, emap, shape, center, size, n_iter, n_sub, perm, *, rule="full_tof",
         emap_scale=1.0, guard=True, subset_index="mod", tof=False, tof_bin=0.0, tof_sigma2=0.0,
         tof_nsigma=0.0, x0=None, add=None):
    """OSEM: per step i the subset is i // n_sub ('reference' literal, osem_full.py:68) or
    i % n_sub ('mod'); n_iter counts subset steps as in the reference loop. The emap is the full
    sensitivity times emap_scale, zero-guarded when guard=True."""
    y = np.asarray(values, dtype=np.float32)
    em = np.asarray(emap, dtype=np.float32) * np.float32(emap_scale)
    if guard:
        em = guard_emap(em)
    x = np.ones(shape, dtype=np.float32) if x0 is None else np.array(x0, dtype=np.float32)
    subs = osem_subsets(len(y), n_sub, perm)
    kw = dict(tof=tof, tof_bin=tof_bin, tof_sigma2=tof_sigma2, tof_nsigma=tof_nsigma)
    for i in range(n_iter):
        k = (i // n_sub) if subset_index == "reference" else (i % n_sub)
        idx = subs[k]
        sl = np.ascontiguousarray(lors[idx])
        p = projection(x, sl, shape, center, size, **kw)
        if add is not None:
            p = (p + np.asarray(add, np.float32)[idx]).astype(np.float32)
        r = ratio(y[idx], p, rule)
        bp = backprojection(r, sl, shape, center, size, **kw)
        x = (x * bp / em).astype(np.float32)
    return x


def emap_block_full(crystal_table, n_blocks, shape, center, size):
    """Sensitivity image over all ordered crystal pairs, block column by block column
    (emap_generator.py:77-111); crystal_table from srf_gb300.geometry.block_full_crystal_table."""
    m = crystal_table.shape[0] // n_blocks
    acc = np.zeros(shape, dtype=np.float32)
    ones = np.ones(m * m, dtype=np.float32)
    for i in range(n_blocks):
        p1 = np.repeat(crystal_table[i * m:(i + 1) * m], m, axis=0)
        for j in range(n_blocks):
            p2 = np.tile(crystal_table[j * m:(j + 1) * m], (m, 1))
            lors = np.hstack((p1, p2)).astype(np.float32)
            acc = acc + backprojection(ones, lors, shape, center, size)
    return acc.astype(np.float32)


def sss(pairs, crystal_pos, scatter_pos, sumup_emission, atten, umap, umap_size,
        nb_crystals_per_ring, nb_blocks_per_ring, grid_block, low_energy, high_energy,
        resolution):
    """Raw SSS sums and scales for crystal pairs (scatter_fraction.py:40-136); float64 outputs."""
    L = lib()
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    cp = np.ascontiguousarray(crystal_pos, dtype=np.float32)
    sp = np.ascontiguousarray(scatter_pos, dtype=np.float32)
    em = np.ascontiguousarray(sumup_emission, dtype=np.float32)
    at = np.ascontiguousarray(atten, dtype=np.float32)
    um = np.ascontiguousarray(umap, dtype=np.float32)
    ushape = np.ascontiguousarray(np.asarray(um.shape, dtype=np.int32))
    usize = np.ascontiguousarray(np.asarray(umap_size, dtype=np.float32))
    gb = np.ascontiguousarray(np.asarray(grid_block, dtype=np.int32))
    n = pairs.shape[0]
    sc = np.zeros(n, dtype=np.float64)
    sl = np.zeros(n, dtype=np.float64)
    d = ctypes.POINTER(ctypes.c_double)
    L.or_sss(pairs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.c_int64(n), _p(cp),
             ctypes.c_int(cp.shape[0]), _p(sp), ctypes.c_int(sp.shape[0]), _p(em), _p(at), _p(um),
             ushape.ctypes.data_as(_i32p), _p(usize), ctypes.c_int(nb_crystals_per_ring),
             ctypes.c_int(nb_blocks_per_ring), gb.ctypes.data_as(_i32p), ctypes.c_int(low_energy),
             ctypes.c_int(high_energy), ctypes.c_double(np.sqrt(511.0) * resolution),
             sc.ctypes.data_as(d), sl.ctypes.data_as(d))
    return sc, sl


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


# ---------------------------------------------------------------- scatter correction pipeline

def umap_project(umap, lors):
    """UmapProject (attenuation_correct.py:31-40) over the oracle projector."""
    lors = np.ascontiguousarray(lors, dtype=np.float32)
    p = projection(umap.data, np.ascontiguousarray(lors[:, :6]), umap.shape, umap.center, umap.size)
    L = np.sqrt((lors[:, 0] - lors[:, 3]) ** 2 + (lors[:, 1] - lors[:, 4]) ** 2 + (lors[:, 2] - lors[:, 5]) ** 2)
    return np.exp(-(p * L * L / umap.unit_size[0]))


def scatter_preprocess(scanner, listmode, emission, umap):
    """scatter.py:57-73 / preprocess.py:6-75 with every projection done by the oracle. The numpy
    helpers for sinogram bins and scatter points come from srf_gb300.scatter (checked against the
    reference's own host code by tests/test_host_logic.py)."""
    from srf_gb300 import scatter as S
    lors = S.get_all_lors_id(scanner.nb_crystals)
    sinogram = S.lm2sino(listmode, scanner)
    index = np.where(sinogram > 0)[0].astype(np.int32)
    scat = S.pre_all_scatter_position(emission)
    cryst = S.get_all_crystal_position(scanner)
    L = S.get_lors(cryst, scat).data
    em = projection(emission.data, np.ascontiguousarray(L[:, :6]), emission.shape, emission.center,
                    emission.size)
    len2 = (L[:, 3] - L[:, 0]) ** 2 + (L[:, 4] - L[:, 1]) ** 2 + (L[:, 5] - L[:, 2]) ** 2
    atten = umap_project(umap, L)
    p1, p2 = cryst[lors[index, 0]], cryst[lors[index, 1]]
    lors7 = np.hstack((p1, p2, np.ones((p1.shape[0], 1), np.float32))).astype(np.float32)
    atten_lors = umap_project(umap * 1.3, lors7).reshape(-1, 1)
    return dict(lors=lors, sinogram=sinogram, index=index, scatter_position=scat,
                crystal_position=cryst, sumup_emission=em * len2, atten=atten,
                atten_lors=atten_lors)


def scatter_correct(corr, emission, umap, scanner, pre):
    """ScatterCorrect.__call__ (scatter.py:25-55) with the oracle's SSS sums."""
    import sys as _sys
    from srf_gb300 import scatter as S
    from srf_gb300.data import Listmode, Lors
    index = pre["index"]
    ns = pre["scatter_position"].shape[0]
    nc = pre["crystal_position"].shape[0]
    grid_block = np.array(scanner.blocks.shape, dtype=np.int32)
    size_block = np.array(scanner.blocks.size, dtype=np.float32)
    raw, scale = sss(pre["lors"][index, :2], pre["crystal_position"], pre["scatter_position"],
                     pre["sumup_emission"].reshape(nc, ns), pre["atten"].reshape(nc, ns),
                     umap.data, umap.size, scanner.nb_blocks_per_ring * scanner.blocks.shape[1],
                     scanner.nb_blocks_per_ring, grid_block, int(corr.low_energy),
                     int(corr.high_energy), float(corr.resolution))
    frac, scl = S.scatter_scaling(raw.reshape(-1, 1), scale.reshape(-1, 1), int(corr.low_energy),
                                  int(corr.high_energy), float(corr.resolution), grid_block,
                                  size_block)
    sino = pre["sinogram"]
    out = np.zeros_like(sino)
    out[index] = (sino[index] - frac / np.sum(frac) * np.sum(sino[index]) * corr.scatter_fraction) \
        * scl / (pre["atten_lors"] + _sys.float_info.min)
    data = S.sino2lm(scanner, out, pre["lors"])
    return Listmode(data[:, 6].astype(np.float32), Lors(data.astype(np.float32)))
