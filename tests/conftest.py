import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the product library and the oracle once per session."""
    from ascent_gb300 import build as B
    from oracle import oracle as O
    B.build()
    O.build()


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def image_error(a: np.ndarray, b: np.ndarray) -> dict:
    """Per-channel error statistics of two RGBA float images."""
    d = np.abs(a.astype(np.float64) - b.astype(np.float64))
    within = (d <= 2.0 / 255.0 + 1e-7).all(axis=-1)
    return {"max": float(d.max()) if d.size else 0.0, "mae": float(d.mean()) if d.size else 0.0,
            "frac_within_2": float(within.mean()) if within.size else 1.0,
            "frac_gt_4_255": float((d > 4.0 / 255.0).any(axis=-1).mean()) if d.size else 0.0}


def assert_parity(a, b, frac=0.999, mae=1e-3):
    e = image_error(a, b)
    assert e["frac_within_2"] >= frac and e["mae"] <= mae, e
    return e
