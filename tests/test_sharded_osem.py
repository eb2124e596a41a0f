"""Event-sharded OSEM (srf_gb300.distributed) on CPU ranks.

Two `gloo` processes each run their shard of every subset and sum their backprojections with one
all-reduce per subset; the image must equal the single-process OSEM's. The subset step of each
rank is computed by a CPU stand-in engine over the oracle (test infrastructure: the product
engine is the GPU kernel, which these ranks do not have). Shards are uneven (1001 events per
subset over 2 ranks).
"""
import os
import socket
import sys
import tempfile

import numpy as np
import pytest
import torch

from conftest import ROOT, rel_l2

N_EVENTS, N_SUB, N_ITER = 3003, 3, 2
TOL = 1e-5


class OracleEngine:
    """The subset-step engine interface of srf_gb300.distributed, computed by the oracle:
    MlemFullTof's ratio div_no_nan(y, p + 1e-5), backprojection into a flat accumulator, update
    x * bp / emap with the zero guard."""

    def __init__(self, ic, tof):
        import oracle as O
        self.O = O
        self.ic, self.tof = ic, tof
        self.x = np.ones(ic.shape, np.float32)
        self.acc = torch.zeros(int(np.prod(ic.shape)), dtype=torch.float32)

    def subset(self, lors, y, **kw):
        O, ic = self.O, self.ic
        t = dict(tof=True, tof_bin=self.tof[0], tof_sigma2=self.tof[1], tof_nsigma=kw.get("tof_nsigma", 0.0))
        lors = np.ascontiguousarray(lors.numpy())
        p = O.projection(self.x, lors, ic.shape, ic.center, ic.size, **t)
        yv = np.ones(len(lors), np.float32) if y is None else y.numpy()
        r = O.ratio(yv, p, "full_tof")
        bp = O.backprojection(r, lors, ic.shape, ic.center, ic.size, **t)
        self.acc += torch.from_numpy(np.ascontiguousarray(bp).reshape(-1))

    def accumulators(self):
        return self.acc

    def update(self, emap, guard_zero=True):
        bp = self.acc.numpy().reshape(self.ic.shape)
        em = self.O.guard_emap(emap) if guard_zero else emap
        self.x = (self.x * bp / em).astype(np.float32)
        self.acc.zero_()


def _case():
    from srf_gb300 import synth
    sc, ic = synth.scanner_small(), synth.image_small()
    lors = synth.sample_events(sc, ic, synth.phantom_cylinder(ic), N_EVENTS, seed=77,
                               tof_fwhm_ps=530.0).numpy()
    emap = (0.5 + np.random.default_rng(78).random(ic.shape)).astype(np.float32)
    return sc, ic, lors, emap


def _run(rank, world):
    """Sharded OSEM on this rank; returns the final image."""
    from srf_gb300.distributed import ShardedOsem, subset_shards
    sc, ic, lors, emap = _case()
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    eng = OracleEngine(ic, tof)
    drv = ShardedOsem(eng)
    assert (drv.rank, drv.world) == (rank, world)
    t = torch.from_numpy(lors)
    shards = [t[lo:hi] for lo, hi in subset_shards(len(lors), N_SUB, rank, world)]
    for _ in range(N_ITER):
        drv.iteration(shards, None, emap * np.float32(1.0 / N_SUB), tof_nsigma=3.0)
    return eng.x


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        x = _run(rank, world)
        np.save(os.path.join(out_dir, f"x{rank}.npy"), x)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_ranges_cover_each_subset():
    from srf_gb300.distributed import shard_range, subset_shards
    for n in (0, 1, 7, 1001, 4096):
        for world in (1, 2, 3, 8):
            parts = [shard_range(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    got = [subset_shards(3003, 3, r, 2) for r in range(2)]
    assert got[0] == [(0, 501), (1001, 1502), (2002, 2503)]
    assert got[1] == [(501, 1001), (1502, 2002), (2503, 3003)]
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_sharded_osem_two_gloo_ranks_match_one_process(oracle):
    import torch.multiprocessing as mp
    single = _run(0, 1)
    sc, ic, lors, emap = _case()
    perm = np.arange(len(lors))
    ref = oracle.osem(lors, np.ones(len(lors), np.float32), emap, ic.shape, ic.center, ic.size,
                      N_ITER * N_SUB, N_SUB, perm, rule="full_tof", emap_scale=1.0 / N_SUB,
                      guard=True, subset_index="mod", tof=True, tof_bin=sc.tof.tof_bin,
                      tof_sigma2=sc.tof.tof_sigma2, tof_nsigma=3.0)
    assert rel_l2(single, ref) <= TOL
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_worker, args=(2, _free_port(), d), nprocs=2, join=True, start_method="spawn")
        x0, x1 = np.load(os.path.join(d, "x0.npy")), np.load(os.path.join(d, "x1.npy"))
    assert np.array_equal(x0, x1)  # every rank applies the identical update
    assert rel_l2(x0, single) <= TOL
