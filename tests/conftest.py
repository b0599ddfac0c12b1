import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU case")


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files}


GOLDEN_CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def uniform_case(n, L, nrhs, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, L, size=(n, 3))
    f = rng.standard_normal((nrhs, 3 * n)).astype(dtype)
    return pos, f


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; on a GPU machine it must load (no fallback)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import spme_gb300
    return spme_gb300.load()
