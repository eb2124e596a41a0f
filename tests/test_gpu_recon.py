"""GPU parity of the MLEM/OSEM loops and the sensitivity image against the CPU oracle.

Tolerance: 1e-5 relative L2 on the final images (FP32; multiplicative iterations of the fused
GPU subset step against the oracle's separate projection/ratio/backprojection passes).
"""
import numpy as np
import pytest

from conftest import rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def emap_small(oracle, small_case):
    from srf_gb300.geometry import block_full_crystal_table
    sc, ic = small_case["scanner"], small_case["ic"]
    table = block_full_crystal_table(sc)
    return oracle.emap_block_full(table, sc.nb_blocks_per_ring, ic.shape, ic.center, ic.size)


def test_emap_block_full_matches_oracle(cuda_lib, emap_small, small_case):
    import srf_gb300 as nef
    sc, ic = small_case["scanner"], small_case["ic"]
    em = nef.EmapGenerator("block-full", sc)(ic)
    assert isinstance(em, nef.Emap) and em.data.shape == tuple(ic.shape)
    assert rel_l2(em.data, emap_small) <= TOL
    assert (em.data > 0).sum() == (emap_small > 0).sum()


@pytest.mark.parametrize("cls,rule,tof", [("MlemFull", "full", False), ("MlemFullTof", "full_tof", True)])
def test_mlem_full_matches_oracle(cuda_lib, oracle, small_case, emap_small, cls, rule, tof):
    import srf_gb300 as nef
    sc, ic, lors = small_case["scanner"], small_case["ic"], small_case["lors"]
    lors_in = lors if tof else np.ascontiguousarray(lors[:, :6])
    y = np.ones(len(lors), dtype=np.float32)
    lm = nef.Listmode(y, nef.Lors(lors_in))
    em = nef.Emap(emap_small, ic.center, ic.size)
    out = getattr(nef, cls)(10, ic, sc, lm, None, None, None, em)()
    kw = dict(tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2) if tof else {}
    ref = oracle.mlem(lors_in, y, emap_small, ic.shape, ic.center, ic.size, 10, rule=rule, **kw)
    assert out.data.shape == tuple(ic.shape)
    assert rel_l2(out.data, ref) <= TOL


def test_mlem_plain_matches_oracle(cuda_lib, oracle, small_case, emap_small):
    import srf_gb300 as nef
    ic, lors = small_case["ic"], small_case["lors"]
    lors6 = np.ascontiguousarray(lors[:, :6])
    y = np.random.default_rng(2).integers(1, 4, len(lors)).astype(np.float32)
    out = nef.Mlem(5, nef.Emap(emap_small, ic.center, ic.size))(nef.Listmode(y, nef.Lors(lors6)))
    ref = oracle.mlem(lors6, y, emap_small, ic.shape, ic.center, ic.size, 5, rule="mlem")
    assert rel_l2(out.data, ref) <= TOL


@pytest.mark.parametrize("subset_rule", ["reference", "cyclic"])
def test_osem_full_matches_oracle(cuda_lib, oracle, small_case, emap_small, subset_rule):
    import srf_gb300 as nef
    from srf_gb300.geometry import PetEcatListmodeTrans
    sc, ic, lors = small_case["scanner"], small_case["ic"], small_case["lors"]
    lors6 = np.ascontiguousarray(lors[:, :6])
    lm = nef.Listmode(np.ones(len(lors), np.float32), nef.Lors(lors6))
    em = nef.Emap(emap_small, ic.center, ic.size)
    out = nef.OsemFull(6, 4, ic, sc, lm, None, None, None, None, em, None,
                       subset_rule=subset_rule, seed=11)()
    perm = np.random.default_rng(11).permutation(len(lors))
    y = PetEcatListmodeTrans(sc)(lm).data
    ref = oracle.osem(lors6, y, emap_small, ic.shape, ic.center, ic.size, 6, 4, perm,
                      rule="osem", guard=False,
                      subset_index="reference" if subset_rule == "reference" else "mod")
    assert rel_l2(out.data, ref) <= TOL


@pytest.mark.parametrize("nsigma", [0.0, 3.0])
def test_osem_tof_matches_oracle(cuda_lib, oracle, small_case, emap_small, nsigma):
    import srf_gb300 as nef
    sc, ic, lors = small_case["scanner"], small_case["ic"], small_case["lors"]
    lm = nef.Listmode(np.ones(len(lors), np.float32), nef.Lors(lors))
    em = nef.Emap(emap_small, ic.center, ic.size)
    out = nef.OsemFullTof(2, 5, ic, sc, lm, em, tof_nsigma=nsigma, seed=3)()
    perm = np.random.default_rng(3).permutation(len(lors))
    ref = oracle.osem(lors, lm.data, emap_small, ic.shape, ic.center, ic.size, 10, 5, perm,
                      rule="full_tof", emap_scale=1.0 / 5, guard=True, subset_index="mod",
                      tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2,
                      tof_nsigma=nsigma)
    assert rel_l2(out.data, ref) <= TOL


@pytest.mark.parametrize("lanes,spl", [(32, 2), (16, 4), (16, 2), (8, 4), (8, 2)])
def test_osem_tuning_variants_match_oracle(cuda_lib, oracle, small_case, emap_small, lanes, spl):
    import srf_gb300 as nef
    from srf_gb300 import _lib
    sc, ic, lors = small_case["scanner"], small_case["ic"], small_case["lors"]
    lm = nef.Listmode(np.ones(len(lors), np.float32), nef.Lors(lors))
    em = nef.Emap(emap_small, ic.center, ic.size)
    _lib.set_tuning(lanes, spl)
    try:
        out = nef.OsemFullTof(1, 4, ic, sc, lm, em, tof_nsigma=3.0, seed=5)()
    finally:
        _lib.set_tuning(32, 4)
    perm = np.random.default_rng(5).permutation(len(lors))
    ref = oracle.osem(lors, lm.data, emap_small, ic.shape, ic.center, ic.size, 4, 4, perm,
                      rule="full_tof", emap_scale=1.0 / 4, guard=True, subset_index="mod",
                      tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2,
                      tof_nsigma=3.0)
    assert rel_l2(out.data, ref) <= TOL


def test_osem_tof_additive_term_matches_oracle(cuda_lib, oracle, small_case, emap_small):
    """Per-event additive expected counts (a scatter estimate) enter the ratio as y / (p + s)."""
    import srf_gb300 as nef
    sc, ic, lors = small_case["scanner"], small_case["ic"], small_case["lors"]
    lm = nef.Listmode(np.ones(len(lors), np.float32), nef.Lors(lors))
    em = nef.Emap(emap_small, ic.center, ic.size)
    add = (np.random.default_rng(8).random(len(lors)) * 1e-3).astype(np.float32)
    out = nef.OsemFullTof(1, 4, ic, sc, lm, em, tof_nsigma=3.0, seed=2, add=add)()
    zero = nef.OsemFullTof(1, 4, ic, sc, lm, em, tof_nsigma=3.0, seed=2, add=np.zeros_like(add))()
    none = nef.OsemFullTof(1, 4, ic, sc, lm, em, tof_nsigma=3.0, seed=2)()
    assert np.array_equal(zero.data, none.data) or rel_l2(zero.data, none.data) <= 1e-6
    perm = np.random.default_rng(2).permutation(len(lors))
    ref = oracle.osem(lors, lm.data, emap_small, ic.shape, ic.center, ic.size, 4, 4, perm,
                      rule="full_tof", emap_scale=1.0 / 4, guard=True, subset_index="mod",
                      tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2,
                      tof_nsigma=3.0, add=add)
    assert rel_l2(out.data, ref) <= TOL
    assert rel_l2(out.data, none.data) > 1e-4  # the term matters


@pytest.mark.parametrize("shape,offset", [((36, 20, 3), 0), ((36, 20, 3), 1), ((37, 21, 2), 0), ((200, 200, 2), 0)])
def test_osem_update_paths_bit_exact(cuda_lib, shape, offset):
    """srf_osem_update on both of its kernels: 16-byte accesses (nx, ny multiples of 4, aligned
    arrays) and the scalar tile kernel (odd sizes, or arrays one float off alignment). Both are
    x * (bp + bp_t) / emap in FP32 with emap zeros -> 1e8, x_t the transposed copy, both
    accumulators zeroed; compared bit for bit with numpy's FP32 arithmetic."""
    import torch
    from srf_gb300._lib import call, i32, i32x3, ptr, stream_ptr
    nx, ny, nz = shape
    v = nx * ny * nz
    rng = np.random.default_rng(nx * 131 + offset)
    x = rng.uniform(0.5, 2.0, (nz, ny, nx)).astype(np.float32)
    bp = rng.uniform(0.0, 3.0, (nz, ny, nx)).astype(np.float32)
    bpt = rng.uniform(0.0, 3.0, (nz, nx, ny)).astype(np.float32)
    em = rng.uniform(0.5, 1.5, (nz, ny, nx)).astype(np.float32)
    em[rng.random(em.shape) < 0.1] = 0.0
    dev = torch.device("cuda", 0)

    def put(a):
        buf = torch.zeros(v + offset, dtype=torch.float32, device=dev)
        buf[offset:] = torch.as_tensor(a.reshape(-1), device=dev)
        return buf[offset:]

    dx, dxt, dbp, dbpt, dem = put(x), put(np.ascontiguousarray(x.transpose(0, 2, 1))), put(bp), put(bpt), put(em)
    call("srf_osem_update", ptr(dx), ptr(dxt), ptr(dbp), ptr(dbpt), ptr(dem), i32(1), i32x3(shape),
         stream_ptr(dev))
    b = bp + bpt.transpose(0, 2, 1)
    e = np.where(em == 0.0, np.float32(1e8), em)
    want = (x * b) / e
    got = dx.cpu().numpy().reshape(nz, ny, nx)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))
    got_t = dxt.cpu().numpy().reshape(nz, nx, ny)
    assert np.array_equal(got_t.view(np.int32), np.ascontiguousarray(want.transpose(0, 2, 1)).view(np.int32))
    assert not dbp.any().item() and not dbpt.any().item()


def test_osem_tof_interleaved_subsets_match_oracle(cuda_lib, oracle, small_case, emap_small):
    """subsets='interleaved': subset k holds events k, k + n_sub, ... (no reordering of the LORs;
    the values and the additive term are regrouped by subset); uneven n (the remainder is left
    out), per-event values and an additive term."""
    import srf_gb300 as nef
    sc, ic, lors = small_case["scanner"], small_case["ic"], small_case["lors"]
    n_sub = 4
    lors = np.ascontiguousarray(lors[: (len(lors) // n_sub) * n_sub - 3])  # 3 events past the last full row
    rng = np.random.default_rng(12)
    y = (0.5 + rng.random(len(lors))).astype(np.float32)
    add = (rng.random(len(lors)) * 1e-3).astype(np.float32)
    lm = nef.Listmode(y, nef.Lors(lors))
    em = nef.Emap(emap_small, ic.center, ic.size)
    out = nef.OsemFullTof(2, n_sub, ic, sc, lm, em, tof_nsigma=3.0, add=add, subsets="interleaved")()
    n_used = (len(lors) // n_sub) * n_sub
    order = np.concatenate([np.arange(k, n_used, n_sub) for k in range(n_sub)] +
                           [np.arange(n_used, len(lors))])
    ref = oracle.osem(lors, y, emap_small, ic.shape, ic.center, ic.size, 2 * n_sub, n_sub, order,
                      rule="full_tof", emap_scale=1.0 / n_sub, guard=True, subset_index="mod",
                      tof=True, tof_bin=sc.tof.tof_bin, tof_sigma2=sc.tof.tof_sigma2,
                      tof_nsigma=3.0, add=add)
    assert rel_l2(out.data, ref) <= TOL
    with pytest.raises(ValueError):
        nef.OsemFullTof(1, n_sub, ic, sc, lm, em, subsets="blocks")()


@pytest.mark.parametrize("tof, nsigma, n_ev", [(False, 0.0, 20000), (True, 0.0, 20000), (True, 3.0, 20000),
                                                (True, 3.0, 33), (False, 0.0, 33)])
def test_osem_subset_step_nonsquare_voxels(cuda_lib, oracle, small_case, tof, nsigma, n_ev):
    """One fused subset step and the update on a grid with dy != dx (2.0 x 1.8 mm, off-centre): the
    subset kernel's variant with the reference's in-plane division by dy for x-dominant LORs
    (siddon.cu.cc:59-73), against the oracle's projection, MlemFullTof ratio and backprojection;
    also with 33 events (a second warp batch holding one LOR). The bound is an image-level one: the
    axial crossing fractions carry a few ulp of the linear z form, which a single LOR's image does
    not average (one non-TOF LOR measured 1.4e-5)."""
    import torch
    from srf_gb300 import kernels
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    sc, lors = small_case["scanner"], np.ascontiguousarray(small_case["lors"][:n_ev])
    sh, c, s = [48, 40, 12], [1.5, -2.0, 0.5], [96.0, 72.0, 30.0]
    rng = np.random.default_rng(31)
    img = (0.2 + rng.random(sh)).astype(np.float32)
    emap = (0.5 + rng.random(sh)).astype(np.float32)
    emap[0, 0, :] = 0.0  # guarded voxels
    t = (sc.tof.tof_bin, sc.tof.tof_sigma2) if tof else None
    dev = torch.device("cuda", 0)
    st = kernels.SubsetState(sh, c, s, dev, x0=torch.as_tensor(img, device=dev))
    st.subset(torch.as_tensor(lors, device=dev), None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=t,
              tof_nsigma=nsigma)
    st.update(kernels.xfast(torch.as_tensor(emap, device=dev)), guard_zero=True)
    got = st.x.contiguous().cpu().numpy()
    kw = dict(tof=True, tof_bin=t[0], tof_sigma2=t[1], tof_nsigma=nsigma) if tof else {}
    p = oracle.projection(img, lors, sh, c, s, **kw)
    r = oracle.ratio(np.ones(len(lors), np.float32), p, "full_tof")
    bp = oracle.backprojection(r, lors, sh, c, s, **kw)
    want = (img * bp / oracle.guard_emap(emap)).astype(np.float32)
    assert rel_l2(got, want) <= TOL
