"""Shared test set-up: import paths, the `gpu` marker, the in-tree build."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "nematic-worms_gb300"))
sys.path.insert(0, str(REPO / "oracle"))
sys.path.insert(0, str(REPO))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs through libnwgb.so")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libnwgb.so, the oracle and (where the reference tree exists) the
    reference-kernel emulation once per session; no-op when up to date."""
    from nwgb import build

    build.build_all()
    yield


@pytest.fixture(scope="session")
def lib(_built):
    import nwgb

    return nwgb.load_library()


@pytest.fixture(scope="session")
def orc(_built):
    import oracle

    return oracle


def have_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def rel_err(a, b) -> float:
    """max |a - b| / max |b| over the xyz components (the force tolerance metric)."""
    a = np.asarray(a, dtype=np.float64)[..., :3]
    b = np.asarray(b, dtype=np.float64)[..., :3]
    return float(np.abs(a - b).max() / (np.abs(b).max() + 1e-300))


def rel_err_rows(a, b, floor_frac: float = 1e-3) -> float:
    """max over beads of |a_i - b_i| / (|b_i| + floor), floor = floor_frac * rms|b|."""
    a = np.asarray(a, dtype=np.float64)[..., :3]
    b = np.asarray(b, dtype=np.float64)[..., :3]
    nb = np.linalg.norm(b, axis=-1)
    floor = floor_frac * (np.sqrt((nb ** 2).mean()) + 1e-300)
    return float((np.linalg.norm(a - b, axis=-1) / (nb + floor)).max())
