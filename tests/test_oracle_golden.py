"""The CPU oracle reproduces the golden vectors made from the reference's own code.

siddon.npz comes from the reference's Siddon device functions compiled on the host; the oracle
must match it bit for bit (same operand order, no FMA contraction, sequential accumulation).
sss.npz comes from the reference's Python SSS functions; the oracle evaluates in double, the
reference partly in float32 scalars, so it is checked to 1e-5 relative.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def siddon():
    return dict(np.load(os.path.join(GOLD, "siddon.npz")))


def _case(g, name):
    return (g[f"{name}_lors"], list(g[f"{name}_shape"]), list(g[f"{name}_center"]),
            list(g[f"{name}_size"]), g[f"{name}_image"], g[f"{name}_values"])


@pytest.mark.parametrize("name", ["a", "b"])
def test_projection_bitexact(oracle, siddon, name):
    lors, sh, c, s, img, _ = _case(siddon, name)
    got = oracle.projection(img, np.ascontiguousarray(lors[:, :6]), sh, c, s)
    assert np.array_equal(got.view(np.int32), siddon[f"{name}_proj"].view(np.int32))
    kw = dict(tof=True, tof_bin=float(siddon["tof_bin"]), tof_sigma2=float(siddon["tof_sigma2"]))
    got_t = oracle.projection(img, lors, sh, c, s, **kw)
    assert np.array_equal(got_t.view(np.int32), siddon[f"{name}_proj_tof"].view(np.int32))


@pytest.mark.parametrize("name", ["a", "b"])
def test_backprojection_bitexact_and_pairs(oracle, siddon, name):
    lors, sh, c, s, _, vals = _case(siddon, name)
    got, pairs = oracle.trace(np.ascontiguousarray(lors[:, :6]), sh, c, s, oracle.RULES_BACK,
                              oracle.SCATTER, values=vals)
    assert np.array_equal(got.view(np.int32), siddon[f"{name}_bp"].view(np.int32))
    assert pairs == int(siddon[f"{name}_bp_pairs"])
    kw = dict(tof=True, tof_bin=float(siddon["tof_bin"]), tof_sigma2=float(siddon["tof_sigma2"]))
    got_t, pairs_t = oracle.trace(lors, sh, c, s, oracle.RULES_BACK, oracle.SCATTER, values=vals, **kw)
    assert np.array_equal(got_t.view(np.int32), siddon[f"{name}_bp_tof"].view(np.int32))
    assert pairs_t == int(siddon[f"{name}_bp_tof_pairs"])


def test_multithreaded_oracle_agrees(oracle, siddon):
    lors, sh, c, s, img, vals = _case(siddon, "a")
    p1, n1 = oracle.trace(lors, sh, c, s, 0, 0, image=img, tof=True, tof_bin=3.66, tof_sigma2=1138.0)
    p4, n4 = oracle.trace(lors, sh, c, s, 0, 0, image=img, tof=True, tof_bin=3.66, tof_sigma2=1138.0, threads=4)
    assert np.array_equal(p1, p4) and n1 == n4
    b1, _ = oracle.trace(lors, sh, c, s, 1, 1, values=vals)
    b4, _ = oracle.trace(lors, sh, c, s, 1, 1, values=vals, threads=4)
    assert oracle.rel_l2(b4, b1) < 1e-6


def test_truncation_only_removes_slabs(oracle, siddon):
    lors, sh, c, s, img, _ = _case(siddon, "a")
    kw = dict(tof=True, tof_bin=3.66, tof_sigma2=1138.0)
    full, nf = oracle.trace(lors, sh, c, s, 0, 0, image=img, **kw)
    cut, nc = oracle.trace(lors, sh, c, s, 0, 0, image=img, tof_nsigma=3.0, **kw)
    assert nc < nf and np.all(cut <= full + 1e-6)
    assert oracle.rel_l2(cut, full) < 0.02


def test_sss_matches_reference_python(oracle):
    g = dict(np.load(os.path.join(GOLD, "sss.npz")))
    sc, sl = oracle.sss(g["pairs"], g["crystal"], g["scatter"], g["sumup"], g["atten"], g["umap"],
                        g["usize"], int(g["ncpr"]), int(g["nbpr"]), g["grid_block"], int(g["low"]),
                        int(g["high"]), float(g["res"]))
    ref = g["sss"]
    assert np.all(np.isfinite(ref))
    np.testing.assert_allclose(sc, ref, rtol=1e-5, atol=1e-12 * np.abs(ref).max())
    # get_scale = (|AB| / area)^2: for two crystals of one block the area is a cancellation
    # residue (~1e-8 |AB|), so only well-conditioned pairs are compared to 1e-5; the degenerate
    # ones must be huge (or infinite) in both.
    ok = np.isfinite(g["scale"]) & (g["scale"] < 1e6)
    assert ok.sum() >= len(ok) // 2
    np.testing.assert_allclose(sl[ok], g["scale"][ok], rtol=1e-5)
    assert np.all(~np.isfinite(sl[~ok]) | (sl[~ok] > 1e6))
