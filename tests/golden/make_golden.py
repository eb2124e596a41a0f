"""Generate the golden fixtures under tests/golden/ from the reference's own code.

Run in a checkout that has the reference sources (``--reference``, default: the environment
variable SRF_REFERENCE, else /root/reference):

* siddon.npz -- the reference's Siddon device functions (srfnef/cc/siddon/siddon.cu.cc:12-656,
  srfnef/cc/siddon_tof/siddon_tof.cu.cc:14-707), compiled on the host by ``make -C oracle ref``
  into oracle/_ref/libsrf_ref.so, run over seeded LORs (events of the 640-crystal scanner plus
  hand-made edge cases) on a 32 x 32 x 8 image and a non-square 40 x 32 x 12 image;
* sss.npz -- the reference's single-scatter functions ``loop_all_s`` / ``get_scale``
  (srfnef/corrections/scattering/scatter_fraction/scatter_fraction.py:64-91, kn_formula.py:6-46)
  executed as plain Python with stub ``numba`` and ``tensorflow`` modules (the decorators become
  identities), on a few crystal pairs and scatter points;
* host.npz -- the reference's host-side SSS helpers (listmode2sinogram.py:17-35 get_all_lors_id,
  change_id, cal_sinogram; preprocess.py:6-18 pre_all_scatter_position) run the same way.

The fixtures are what the tests read; this script is only needed to regenerate them.
"""
from __future__ import annotations

import argparse
import importlib
import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def edge_lors(rng, n_rand=300):
    rows = [
        [-100, 0, 0, 100, 0, 0], [-100, -100, -10, 100, 100, 10], [-3, 0, 0, 4, 1, 0],
        [-50, 0, -200, 50, 0, 200], [-120, 30, 5, 10, -5, 2], [15, 5, -3, 130, -60, 8],
        [-100, 36, 0, 100, 36, 0], [0, -120, 3, 0, 120, -3], [60, 60, 0, -60, -59, 0],
    ]
    rand = rng.uniform(-150, 150, size=(n_rand, 6))
    lors = np.vstack([np.asarray(rows, np.float64), rand]).astype(np.float32)
    tof = rng.normal(0, 40, size=(len(lors), 1)).astype(np.float32)
    return np.hstack([lors, tof]).astype(np.float32)


def make_siddon(out_path):
    import oracle as O
    from srf_gb300 import synth
    O.build(ref=True)
    rng = np.random.default_rng(1234)
    sc = synth.scanner_small()
    ic = synth.image_small()
    act = synth.phantom_cylinder(ic)
    ev = synth.sample_events(sc, ic, act, 1500, seed=9, tof_fwhm_ps=530.0).numpy()
    cases = {
        "a": dict(lors=ev, shape=[32, 32, 8], center=[0.0, 0.0, 0.0], size=[128.0, 128.0, 32.0]),
        "b": dict(lors=edge_lors(rng), shape=[40, 32, 12], center=[1.5, -2.0, 0.5], size=[80.0, 72.0, 30.0]),
    }
    arrays = {"tof_bin": np.float32(3.66), "tof_sigma2": np.float32(sc.tof.tof_sigma2)}
    for name, c in cases.items():
        lors, sh, ce, si = c["lors"], c["shape"], c["center"], c["size"]
        img = rng.random(sh).astype(np.float32)
        vals = rng.random(len(lors)).astype(np.float32)
        kw = dict(tof_bin=float(arrays["tof_bin"]), tof_sigma2=float(arrays["tof_sigma2"]))
        arrays[f"{name}_lors"] = lors
        arrays[f"{name}_shape"] = np.asarray(sh, np.int32)
        arrays[f"{name}_center"] = np.asarray(ce, np.float32)
        arrays[f"{name}_size"] = np.asarray(si, np.float32)
        arrays[f"{name}_image"] = img
        arrays[f"{name}_values"] = vals
        arrays[f"{name}_proj"] = O.ref_projection(img, lors[:, :6], sh, ce, si)
        arrays[f"{name}_proj_tof"] = O.ref_projection(img, lors, sh, ce, si, tof=True, **kw)
        arrays[f"{name}_bp"], arrays[f"{name}_bp_pairs"] = O.ref_backprojection(vals, lors[:, :6], sh, ce, si)
        arrays[f"{name}_bp_tof"], arrays[f"{name}_bp_tof_pairs"] = O.ref_backprojection(vals, lors, sh, ce, si, tof=True, **kw)
    np.savez_compressed(out_path, **arrays)


def _stub_modules():
    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba = types.ModuleType("numba")
    numba.jit = jit
    cuda = types.ModuleType("numba.cuda")
    cuda.jit = jit
    numba.cuda = cuda
    tf = types.ModuleType("tensorflow")
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = cuda
    sys.modules["tensorflow"] = tf


def load_reference_sss(reference):
    _stub_modules()
    d = os.path.join(reference, "srfnef", "corrections", "scattering", "scatter_fraction")
    pkg = types.ModuleType("srfnef_sss")
    pkg.__path__ = [d]
    sys.modules["srfnef_sss"] = pkg
    return importlib.import_module("srfnef_sss.scatter_fraction")


def make_sss(out_path, reference):
    from srf_gb300 import synth
    from srf_gb300.geometry import EcatIndexToCrystalPos
    ref = load_reference_sss(reference)
    rng = np.random.default_rng(77)
    sc = synth.scanner_small()
    crystal = EcatIndexToCrystalPos(sc)(np.arange(sc.nb_crystals)).astype(np.float32)
    n_s = 12
    scatter = rng.uniform([-40, -40, -10], [40, 40, 10], size=(n_s, 3)).astype(np.float32)
    sumup = rng.uniform(0.5, 2.0, size=(sc.nb_crystals, n_s)).astype(np.float32)
    atten = rng.uniform(0.3, 1.0, size=(sc.nb_crystals, n_s)).astype(np.float32)
    umap = rng.uniform(0.0, 0.02, size=(16, 16, 8)).astype(np.float32)
    usize = np.asarray([128.0, 128.0, 32.0], np.float32)
    ushape = np.asarray(umap.shape, np.int32)
    pairs = rng.integers(0, sc.nb_crystals, size=(40, 2)).astype(np.int32)
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    ncpr = sc.nb_blocks_per_ring * sc.blocks.shape[1]
    nbpr = sc.nb_blocks_per_ring
    grid_block = np.asarray(sc.blocks.shape, np.int32)
    low, high, res = 350, 650, 0.15
    out_s, out_c = [], []
    for a, b in pairs:
        s = ref.loop_all_s(scatter, crystal[a], crystal[b], low, high, math.sqrt(511) * res,
                           sumup[a], sumup[b], atten[a], atten[b], ncpr, nbpr, grid_block, umap,
                           usize, ushape)
        c = ref.get_scale(crystal[a], crystal[b], ncpr, nbpr, grid_block)
        out_s.append(float(s))
        out_c.append(float(c))
    eff0 = ref.eff_without_scatter(low, high, math.sqrt(511) * res)
    np.savez_compressed(out_path, pairs=pairs, crystal=crystal, scatter=scatter, sumup=sumup,
                        atten=atten, umap=umap, usize=usize, ncpr=np.int32(ncpr),
                        nbpr=np.int32(nbpr), grid_block=grid_block, low=np.int32(low),
                        high=np.int32(high), res=np.float64(res), sss=np.asarray(out_s),
                        scale=np.asarray(out_c), eff_without_scatter=np.float64(eff0))


def load_reference_host(reference):
    """listmode2sinogram.py and preprocess.py with stub numba/tensorflow/srfnef modules."""
    _stub_modules()
    srfnef = types.ModuleType("srfnef")
    srfnef.__path__ = []
    sys.modules.setdefault("srfnef", srfnef)
    d = os.path.join(reference, "srfnef", "corrections", "scattering")
    pkg = types.ModuleType("srfnef_scat")
    pkg.__path__ = [d]
    sys.modules["srfnef_scat"] = pkg
    l2s = importlib.import_module("srfnef_scat.listmode2sinogram")
    pre = importlib.import_module("srfnef_scat.preprocess")
    return l2s, pre


def make_host(out_path, reference):
    """Golden vectors of the reference's host-side SSS helpers."""
    l2s, pre = load_reference_host(reference)
    rng = np.random.default_rng(5)
    n = 37
    all_ids = l2s.get_all_lors_id(n)
    id1 = rng.integers(0, n, 500)
    id2 = rng.integers(0, n, 500)
    keep = id1 != id2
    id1, id2 = id1[keep], id2[keep]
    w = rng.random(id1.size).astype(np.float32)
    a, b = l2s.change_id(id1.copy(), id2.copy())
    sino = l2s.cal_sinogram(np.hstack((np.hstack((a, b)), w.reshape(-1, 1))), n)

    class Img:
        def __init__(self, shape, size):
            self.shape, self.size = list(shape), list(size)
            self.unit_size = [s / n for s, n in zip(size, shape)]
    img = Img([64, 64, 32], [256.0, 256.0, 128.0])
    scat = pre.pre_all_scatter_position(img)
    P1 = rng.uniform(-100, 100, (5, 3)).astype(np.float32)
    P2 = rng.uniform(-50, 50, (4, 3)).astype(np.float32)
    np.savez_compressed(out_path, n=np.int32(n), all_ids=all_ids, id1=id1, id2=id2, w=w,
                        sino=sino, img_shape=np.asarray(img.shape), img_size=np.asarray(img.size),
                        scatter_position=scat, P1=P1, P2=P2)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("SRF_REFERENCE", "/root/reference"))
    a = ap.parse_args()
    make_siddon(os.path.join(HERE, "siddon.npz"))
    make_sss(os.path.join(HERE, "sss.npz"), a.reference)
    make_host(os.path.join(HERE, "host.npz"), a.reference)
    for f in ("siddon.npz", "sss.npz", "host.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
