import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU visible")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(GOLDEN / name)

    return load


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle

    return Oracle("strict")


@pytest.fixture(scope="session")
def gala_ref():
    """gala's own compiled code, where its sources were available to build it."""
    from oracle import Oracle, ref_available

    if not ref_available():
        pytest.skip("gala's own objects are not built here (no gala sources)")
    return Oracle("ref")


@pytest.fixture(scope="session")
def gala_ref_strict():
    from oracle import Oracle, ref_available

    if not ref_available():
        pytest.skip("gala's own objects are not built here (no gala sources)")
    return Oracle("ref_strict")


def rel_err(a, b, axis=0):
    """Per-point relative error |a - b| / |b| of vectors stacked along `axis`."""
    num = np.linalg.norm(np.asarray(a) - np.asarray(b), axis=axis)
    den = np.linalg.norm(np.asarray(b), axis=axis)
    return num / np.where(den == 0, 1.0, den)
