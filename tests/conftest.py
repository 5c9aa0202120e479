import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load_golden(name):
    """Return (Batch, npz dict) for a golden fixture."""
    from kronmult_gb300.workloads import Batch

    z = dict(np.load(os.path.join(GOLDEN_DIR, f"{name}.npz")))
    b = Batch(name, int(z["d"]), int(z["n"]), int(z["stride"]), int(z["block"]), z["factors"], z["inputs"],
              z["out_init"], z["fac_index"], z["out_index"])
    return b, z


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import kronmult_gb300

    kronmult_gb300.lib()
    return torch.device("cuda:0")
