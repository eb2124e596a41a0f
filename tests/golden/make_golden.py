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


# ---------------------------------------------------------------- reference framework under stubs

class _Tensor(np.ndarray):
    """Eager TF tensor stand-in: a numpy array with .numpy(); Python and NumPy scalars take the
    array's dtype, as TF converts them (float32 stays float32)."""

    def numpy(self):
        return np.asarray(self)

    def _bin(self, other, op):
        if np.isscalar(other):
            other = np.asarray(other, dtype=self.dtype)
        return op(np.asarray(self), np.asarray(other)).view(_Tensor)

    __add__ = lambda s, o: s._bin(o, np.add)
    __radd__ = lambda s, o: s._bin(o, lambda a, b: np.add(b, a))
    __sub__ = lambda s, o: s._bin(o, np.subtract)
    __mul__ = lambda s, o: s._bin(o, np.multiply)
    __rmul__ = lambda s, o: s._bin(o, lambda a, b: np.multiply(b, a))
    __truediv__ = lambda s, o: s._bin(o, np.divide)


def _t(a):
    return np.asarray(a).view(_Tensor)


def _tf_stub(oracle):
    """tensorflow with the reference's op libraries bound to the reference's own Siddon device
    functions compiled for the host (oracle/_ref). The ops take what the srfnef wrappers pass:
    transposed LORs (6 or 7 x N) and images (nz, ny, nx), grid/center/size as lists."""
    tf = types.ModuleType("tensorflow")
    tf.Variable = lambda x: _t(np.array(x))
    tf.constant = lambda x: _t(np.array(x))
    tf.transpose = lambda x: _t(np.ascontiguousarray(np.asarray(x).T))

    def div_no_nan(a, b):
        a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
        out = np.zeros(np.broadcast(a, b).shape, np.float32)
        nz = b != 0
        out[nz] = a[nz] / b[nz]
        return _t(out)

    tf.div_no_nan = div_no_nan

    def geo(grid, center, size):
        return [int(v) for v in grid], [float(v) for v in center], [float(v) for v in size]

    class Ops:
        def projection(self, lors, image, grid, center, size):
            g, c, s = geo(grid, center, size)
            return _t(oracle.ref_projection(np.asarray(image).T, np.asarray(lors).T, g, c, s))

        def backprojection(self, image, lors, lors_value, grid, center, size):
            g, c, s = geo(grid, center, size)
            bp, _ = oracle.ref_backprojection(np.asarray(lors_value), np.asarray(lors).T, g, c, s)
            return _t(np.ascontiguousarray(bp.T))

        def projection_tof(self, lors, image, grid, center, size, tof_values, tof_bin, tof_sigma2):
            g, c, s = geo(grid, center, size)
            return _t(oracle.ref_projection(np.asarray(image).T, np.asarray(lors).T, g, c, s, tof=True,
                                            tof_bin=float(tof_bin), tof_sigma2=float(tof_sigma2)))

        def backprojection_tof(self, image, lors, lors_value, grid, center, size, tof_values, tof_bin,
                               tof_sigma2):
            g, c, s = geo(grid, center, size)
            bp, _ = oracle.ref_backprojection(np.asarray(lors_value), np.asarray(lors).T, g, c, s, tof=True,
                                              tof_bin=float(tof_bin), tof_sigma2=float(tof_sigma2))
            return _t(np.ascontiguousarray(bp.T))

    tf.load_op_library = lambda path: Ops()
    return tf


def load_reference_framework(reference):
    """The reference's own containers (nef_class, Image/Listmode/Lors/Emap, Block, PetEcatScanner
    properties), geometry functions, projector wrappers and MLEM/OSEM loops, imported from the
    reference tree under stub modules for what this container lacks (TensorFlow and its op
    libraries, tqdm, IO and plotting mixins, corrections). Returns the srfnef namespace."""
    import oracle
    oracle.build(ref=True)
    for name in [m for m in sys.modules if m == "srfnef" or m.startswith("srfnef.")]:
        del sys.modules[name]
    sys.modules["tensorflow"] = _tf_stub(oracle)
    root = os.path.join(reference, "srfnef")

    def pkg(name, path=None):
        m = types.ModuleType(name)
        m.__path__ = [path] if path else []
        sys.modules[name] = m
        return m

    def stub(name, **attrs):
        m = types.ModuleType(name)
        m.__dict__.update(attrs)
        sys.modules[name] = m
        return m

    top = pkg("srfnef", root)
    top.__version__ = "reference"
    pkg("srfnef.base", os.path.join(root, "base"))
    bt = importlib.import_module("srfnef.base.basic_types")
    bb = importlib.import_module("srfnef.base.base")
    for k in ("Optional", "List", "Any", "Tuple", "isinstance_", "NoneType", "eq_"):
        setattr(top, k, getattr(bt, k))
    top.nef_class, top.NefBaseClass = bb.nef_class, bb.NefBaseClass
    pkg("srfnef.ops", os.path.join(root, "ops"))
    pkg("srfnef.ops.common", os.path.join(root, "ops", "common"))
    pkg("srfnef.ops.geometry", os.path.join(root, "ops", "geometry"))
    for m in ("property_mixins", "arithmetic_mixins", "magic_method_mixins"):
        importlib.import_module("srfnef.ops.common." + m)
    stub("srfnef.ops.common.imshow_mixin", ImshowMixin=type("ImshowMixin", (), {}))
    stub("srfnef.io", LoadMixin=type("LoadMixin", (), {}), SaveMixin=type("SaveMixin", (), {}))
    stub("srfnef.utils", tqdm=lambda it, *a, **k: it, declare_eager_execution=lambda: None)
    stub("srfnef.config", TF_USER_OP_PATH="")
    geo = pkg("srfnef.geometry", os.path.join(root, "geometry"))
    for m, names in (("pet_scanner", ["PetScanner"]), ("block", ["Block"]), ("tof_config", ["TofConfig"]),
                     ("image_config", ["ImageConfig"]), ("pet_ecat_scanner", ["PetEcatScanner"])):
        mod = importlib.import_module("srfnef.geometry." + m)
        for nm in names:
            setattr(geo, nm, getattr(mod, nm))
            setattr(top, nm, getattr(mod, nm))
    geo.PetCylindricalScanner = type("PetCylindricalScanner", (), {})
    data = pkg("srfnef.data", os.path.join(root, "data"))
    for m, nm in (("lors", "Lors"), ("listmode", "Listmode"), ("image", "Image"), ("emap", "Emap")):
        cls = getattr(importlib.import_module("srfnef.data." + m), nm)
        setattr(data, nm, cls)
        setattr(top, nm, cls)
    top.Sinogram = type("Sinogram", (), {})
    fn = pkg("srfnef.functions", os.path.join(root, "functions"))
    pkg("srfnef.functions.geometry", os.path.join(root, "functions", "geometry"))
    g = importlib.import_module("srfnef.functions.geometry.pet_ecat_scanner")
    dtp = pkg("srfnef.functions.data_transform", os.path.join(root, "functions", "data_transform"))
    pe = importlib.import_module("srfnef.functions.data_transform.pet_ecat")

    class PetListmodeTrans:  # functions/data_transform/__init__.py:41-48, ECAT branch only
        def __init__(self, scanner):
            self.scanner = scanner

        def __call__(self, listmode):
            return pe.PetEcatListmodeTrans(self.scanner)(listmode)

    dtp.PetListmodeTrans = PetListmodeTrans
    for m, nm in (("project", "Project"), ("back_project", "BackProject"), ("project_tof", "ProjectTof"),
                  ("back_project_tof", "BackProjectTof")):
        setattr(fn, nm, getattr(importlib.import_module("srfnef.functions." + m), nm))
    fn.EmapGenerator = None
    corr = stub("srfnef.corrections", AttenuationCorrect=type("AttenuationCorrect", (), {}))
    corr.__path__ = []
    stub("srfnef.corrections.scattering", ScatterCorrect=type("ScatterCorrect", (), {}))
    stub("srfnef.corrections.psf", PsfCorrect=type("PsfCorrect", (), {}))
    for m, nm in (("mlem", "Mlem"), ("mlem_full", "MlemFull"), ("mlem_full_tof", "MlemFullTof"),
                  ("osem_full", "OsemFull")):
        setattr(fn, nm, getattr(importlib.import_module("srfnef.functions." + m), nm))
    top.EcatCrystalPosToIndex = g.EcatCrystalPosToIndex
    top.EcatIndexToCrystalPos = g.EcatIndexToCrystalPos
    top.PetEcatListmodeTrans = pe.PetEcatListmodeTrans
    top.functions = fn
    return top


def _ref_scanner(R, sc):
    """The reference's PetEcatScanner with the fields of an srf_gb300 scanner."""
    b = sc.blocks
    return R.PetEcatScanner(sc.inner_radius, sc.outer_radius, sc.nb_rings, sc.nb_blocks_per_ring, sc.gap,
                            R.Block(list(b.size), list(b.shape)),
                            R.TofConfig(sc.tof.tof_bin, sc.tof.tof_sigma2))


def make_geometry(out_path, R):
    """Crystal index <-> position and list-mode snapping from the reference's own functions
    (functions/geometry/pet_ecat_scanner.py:15-89, functions/data_transform/pet_ecat.py:43-60),
    on the small and the clinical scanner, at crystal centres and at jittered positions."""
    from srf_gb300 import synth
    rng = np.random.default_rng(2024)
    arrays = {}
    for name, sc in (("small", synth.scanner_small()), ("clinical", synth.scanner_clinical())):
        rs = _ref_scanner(R, sc)
        n = sc.nb_crystals
        ind = np.arange(n) if n <= 4096 else np.sort(rng.choice(n, 4096, replace=False))
        pos = R.EcatIndexToCrystalPos(rs)(ind)
        # jittered hits: within +-0.45 crystal of a centre transaxially and axially, and up to
        # half the crystal depth radially
        k = len(ind)
        u = np.stack([rng.uniform(-0.5, 0.5, k) * (rs.outer_radius - rs.inner_radius),
                      rng.uniform(-0.45, 0.45, k) * rs.blocks.unit_size[1],
                      rng.uniform(-0.45, 0.45, k) * rs.blocks.unit_size[2]], 1)
        iblock = (ind // rs.blocks.shape[1] // rs.blocks.shape[2]) % rs.nb_blocks_per_ring
        th = iblock * rs.angle_per_block
        jit = pos.astype(np.float64).copy()
        jit[:, 0] += u[:, 0] * np.cos(th) - u[:, 1] * np.sin(th)
        jit[:, 1] += u[:, 0] * np.sin(th) + u[:, 1] * np.cos(th)
        jit[:, 2] += u[:, 2]
        jit = jit.astype(np.float32)
        ids = R.EcatCrystalPosToIndex(rs)(jit)
        ids_c = R.EcatCrystalPosToIndex(rs)(pos)
        m = k // 2
        tof = rng.normal(0, 60, (m, 1)).astype(np.float32)
        lors7 = np.hstack([jit[:m], jit[m:2 * m], tof]).astype(np.float32)
        lm = R.Listmode(np.ones(m, np.float32), R.Lors(lors7))
        snapped7 = R.PetEcatListmodeTrans(rs)(lm).lors.data
        lm6 = R.Listmode(np.ones(m, np.float32), R.Lors(np.ascontiguousarray(lors7[:, :6])))
        snapped6 = R.PetEcatListmodeTrans(rs)(lm6).lors.data
        arrays.update({f"{name}_ind": ind, f"{name}_pos": pos, f"{name}_jit": jit, f"{name}_ids": ids,
                       f"{name}_ids_centres": ids_c, f"{name}_lors7": lors7, f"{name}_snapped7": snapped7,
                       f"{name}_snapped6": snapped6,
                       f"{name}_props": np.array([rs.average_radius, rs.axial_length, rs.angle_per_block,
                                                  rs.nb_crystals_per_block, rs.nb_crystals_per_ring,
                                                  rs.nb_crystals], np.float64)})
    np.savez_compressed(out_path, **arrays)


def make_loops(out_path, R):
    """Images of the reference's own update loops (functions/mlem.py:28-45, mlem_full.py:47-72,
    mlem_full_tof.py:43-69, osem_full.py:49-87) with its projector wrappers, the TF op calls
    served by the reference's compiled device functions, on a small seeded case."""
    import oracle
    from srf_gb300 import synth
    from srf_gb300.geometry import ImageConfig
    sc = synth.scanner_small()
    rs = _ref_scanner(R, sc)
    shape, center, size = [32, 32, 8], [0.0, 0.0, 0.0], [128.0, 128.0, 32.0]
    ic = ImageConfig(shape, center, size)
    lors = synth.sample_events(sc, ic, synth.phantom_cylinder(ic), 2000, seed=606, tof_fwhm_ps=530.0).numpy()
    lors6 = np.ascontiguousarray(lors[:, :6])
    rng = np.random.default_rng(607)
    emap = (0.5 + rng.random(shape)).astype(np.float32)
    emap[0, :, :] = 0.0  # exercises the zero guard
    counts = rng.integers(1, 4, len(lors)).astype(np.float32)
    ric = R.ImageConfig(shape, center, size)
    em = R.Emap(emap, center, size)
    F = R.functions
    ones = np.ones(len(lors), np.float32)
    out = {"lors": lors, "emap": emap, "counts": counts, "shape": np.asarray(shape, np.int32),
           "center": np.asarray(center, np.float32), "size": np.asarray(size, np.float32)}
    out["mlem_full_tof"] = F.MlemFullTof(3, ric, rs, R.Listmode(ones, R.Lors(lors)), None, None, None, em)().data
    out["mlem_full"] = F.MlemFull(3, ric, rs, R.Listmode(ones, R.Lors(lors6)), None, None, None, em)().data
    out["mlem"] = F.Mlem(3, em)(R.Listmode(counts, R.Lors(lors6))).data
    # OsemFull shuffles with numpy's global generator: seed it, and record the permutation drawn
    np.random.seed(608)
    perm = np.arange(len(lors))
    np.random.shuffle(perm)
    np.random.seed(608)
    em_pos = R.Emap((emap + np.float32(0.25)).astype(np.float32), center, size)  # no zero guard in OsemFull
    out["osem_full"] = F.OsemFull(4, 2, ric, rs, R.Listmode(ones, R.Lors(lors6)), None, None, None, None,
                                  em_pos, None)().data
    out["osem_perm"] = perm
    out["osem_emap"] = em_pos.data
    # the projector wrappers themselves (transposes and all), on the first events
    img = rng.random(shape).astype(np.float32)
    out["wrap_image"] = img
    out["wrap_proj"] = F.Project("tf-eager")(R.Image(img, center, size), R.Lors(lors6[:300])).data
    out["wrap_proj_tof"] = F.ProjectTof("tf-eager", rs.tof)(R.Image(img, center, size), R.Lors(lors[:300])).data
    vals = rng.random(300).astype(np.float32)
    out["wrap_values"] = vals
    out["wrap_bp"] = F.BackProject("tf-eager")(R.Listmode(vals, R.Lors(lors6[:300])),
                                             R.Image(img, center, size)).data
    out["wrap_bp_tof"] = F.BackProjectTof("tf-eager", rs.tof)(R.Listmode(vals, R.Lors(lors[:300])),
                                                           R.Image(img, center, size)).data
    np.savez_compressed(out_path, **{k: np.asarray(v) for k, v in out.items()})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("SRF_REFERENCE", "/root/reference"))
    a = ap.parse_args()
    make_siddon(os.path.join(HERE, "siddon.npz"))
    make_sss(os.path.join(HERE, "sss.npz"), a.reference)
    make_host(os.path.join(HERE, "host.npz"), a.reference)
    R = load_reference_framework(a.reference)
    make_geometry(os.path.join(HERE, "geometry.npz"), R)
    make_loops(os.path.join(HERE, "loops.npz"), R)
    for f in ("siddon.npz", "sss.npz", "host.npz", "geometry.npz", "loops.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
