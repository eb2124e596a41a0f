import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O  # the CPU oracle (oracle/oracle.py)
    O.build()
    return O


@pytest.fixture(scope="session")
def small_case():
    """Small scanner (640 crystals), 64x64x16 image, seeded TOF events and a random image."""
    import torch
    from srf_gb300 import synth
    sc = synth.scanner_small()
    ic = synth.image_small()
    act = synth.phantom_cylinder(ic)
    lors = synth.sample_events(sc, ic, act, 20000, seed=1, tof_fwhm_ps=530.0).numpy()
    img = np.random.default_rng(0).random(ic.shape).astype(np.float32)
    return dict(scanner=sc, ic=ic, act=act.numpy(), lors=lors, img=img)


@pytest.fixture(scope="session")
def cuda_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from srf_gb300 import _lib
    _lib.load()
    return _lib


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))
