"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU.

The native library and the oracle are built (incrementally) once per session,
so a fresh checkout can run ``pytest`` directly.
"""

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


_built = {}


def _ensure_built():
    if _built:
        return
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    from mallard_gb300 import build as B
    B.build()
    _built["ok"] = True


@pytest.fixture(scope="session", autouse=True)
def built():
    _ensure_built()
    yield


@pytest.fixture(scope="session")
def golden():
    import json
    return json.loads((ROOT / "tests" / "golden" / "reference_unit_vectors.json").read_text())


@pytest.fixture(scope="session")
def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(autouse=True)
def _skip_gpu_without_device(request):
    if request.node.get_closest_marker("gpu") is not None:
        if os.environ.get("MALLARD_FORCE_GPU_TESTS") == "1":
            return
        try:
            import torch
            ok = torch.cuda.is_available()
        except Exception:
            ok = False
        if not ok:
            pytest.skip("no CUDA device")


def rel_err(a, b, floor_frac=1e-3):
    """Per-entry |a-b| / max(|b|, floor_frac * max|b| of that variable).

    The per-variable floor keeps near-zero residuals (cancelling fluxes) from
    dividing by round-off."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    b2 = b.reshape(len(b), -1) if b.ndim > 1 else b.reshape(-1, 1)
    a2 = a.reshape(b2.shape)
    scale = np.maximum(np.abs(b2), floor_frac * np.nanmax(np.abs(b2), axis=0, keepdims=True))
    scale = np.where(scale > 0, scale, 1.0)
    return np.abs(a2 - b2) / scale
