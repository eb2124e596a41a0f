"""GATE list-mode ingestion (srf_gb300.adapters; srfnef/adapters/listmode_from_gate_out.py).

CPU: the host part (sub-run file names, reading, bed split). GPU: the snapped LORs equal the
host restatement PetEcatListmodeTrans, which is pinned bit for bit to the reference's own
snapping (tests/golden/geometry.npz), for plain, TOF and multi-bed files.
"""
import os

import numpy as np
import pytest


def _write_runs(tmp, scanner, counts, seed, beds=None):
    """GATE-like sub-runs: jittered hits on crystals, a TOF column and optionally a bed id."""
    from srf_gb300.geometry import EcatIndexToCrystalPos
    rng = np.random.default_rng(seed)
    paths = []
    for i, m in enumerate(counts):
        ids = rng.integers(0, scanner.nb_crystals, (m, 2))
        p1 = EcatIndexToCrystalPos(scanner)(ids[:, 0]).astype(np.float64)
        p2 = EcatIndexToCrystalPos(scanner)(ids[:, 1]).astype(np.float64)
        p1 += rng.uniform(-0.4, 0.4, p1.shape) * scanner.blocks.unit_size[1]
        p2 += rng.uniform(-0.4, 0.4, p2.shape) * scanner.blocks.unit_size[1]
        cols = [p1, p2, rng.normal(0, 50, (m, 1))]
        if beds is not None:
            cols.append(rng.choice(beds, (m, 1)).astype(np.float64))
        a = np.hstack(cols).astype(np.float32)
        path = os.path.join(tmp, f"sub.{i}", "result.npy")
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.save(path, a)
        paths.append(a)
    return os.path.join(tmp, "sub.?", "result.npy"), paths


def test_gate_host_reading_and_bed_split(tmp_path):
    from srf_gb300 import adapters, synth
    sc = synth.scanner_small()
    path, arrays = _write_runs(str(tmp_path), sc, [5, 0, 7], 3, beds=[0.0, 1.0, 2.0])
    assert adapters.gate_paths(path, 3)[1].endswith(os.path.join("sub.1", "result.npy"))
    parts = adapters.read_gate_rows(path, 3)
    assert [p.shape[0] for p in parts] == [5, 0, 7]
    beds = adapters.split_by_bed(parts)
    assert sum(sum(len(x) for x in v) for v in beds.values()) == 12
    for b, rows in beds.items():
        assert all(np.all(r[:, -1] == b) for r in rows)
    with pytest.raises(ValueError):
        adapters.gate_paths(path, 0)
    np.save(os.path.join(str(tmp_path), "bad.npy"), np.zeros((3, 5), np.float32))
    with pytest.raises(ValueError):
        adapters.read_gate_rows(os.path.join(str(tmp_path), "bad.npy"), 1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["small", "clinical"])
def test_gate_ingestion_matches_host_snapping(cuda_lib, tmp_path, name):
    from srf_gb300 import adapters, synth
    from srf_gb300.data import Listmode, Lors
    from srf_gb300.geometry import PetEcatListmodeTrans
    sc = synth.scanner_small() if name == "small" else synth.scanner_clinical()
    path, arrays = _write_runs(str(tmp_path), sc, [3000, 1, 0, 2500], 11, beds=[0.0, 1.0])
    full = np.vstack(arrays)
    want7 = PetEcatListmodeTrans(sc)(Listmode(np.ones(len(full), np.float32), Lors(full[:, :7]))).lors.data
    lm = adapters.listmode_from_gate_out(path, sc, 4)
    assert np.array_equal(lm.lors.data.cpu().numpy().view(np.int32), want7[:, :6].view(np.int32))
    assert float(lm.data.sum()) == len(full)
    lmt = adapters.listmode_tof_from_gate_out(path, sc, 4, tof_scale=0.5)
    got = lmt.lors.data.cpu().numpy()
    assert np.array_equal(got[:, :6].view(np.int32), want7[:, :6].view(np.int32))
    assert np.array_equal(got[:, 6], (full[:, 6] * np.float32(0.5)).astype(np.float32))
    beds = adapters.listmode_from_gate_out_multi_bed(path, sc, 4)
    assert sorted(beds) == [0.0, 1.0]
    for b, lmb in beds.items():
        rows = full[full[:, -1] == b]
        w = PetEcatListmodeTrans(sc)(Listmode(np.ones(len(rows), np.float32), Lors(rows[:, :6]))).lors.data
        assert np.array_equal(lmb.lors.data.cpu().numpy().view(np.int32), w.view(np.int32))
