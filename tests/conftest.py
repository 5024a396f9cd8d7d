import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def native_built():
    """Build (or reuse) the in-tree native libraries."""
    from cunfft_adjoint_gb300 import build
    build.build()
    return build.LIB


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def golden_cases(kind=None):
    import numpy as np
    out = []
    for f in sorted(os.listdir(GOLDEN_DIR)):
        if not f.endswith(".npz"):
            continue
        d = dict(np.load(os.path.join(GOLDEN_DIR, f)))
        is_boot = "nbs" in d
        if kind == "plain" and is_boot:
            continue
        if kind == "boot" and not is_boot:
            continue
        d["name"] = f[:-4]
        out.append(d)
    return out


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
