import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def max_abs(a, b) -> float:
    return float(np.max(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))))


def load_golden(name):
    path = GOLDEN / f"{name}.npz"
    if not path.exists():
        pytest.skip(f"golden vectors {path.name} not generated")
    z = np.load(path)
    g = {k[2:]: z[k] for k in z.files if k.startswith("g_")}
    for k in ("det_shape", "det_spacing", "det_offset", "DSO", "DSD", "COR"):
        if k in g and g[k].ndim == 0:
            g[k] = g[k].item()
    return z, g


@pytest.fixture(scope="session")
def cuda_device():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from curadon_gb300 import _build

    _build.build()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def ref_ops(cuda_device):
    import oracle
    from oracle import build_ref

    try:
        build_ref.build()
    except Exception as e:  # pragma: no cover - reported as a skip
        pytest.skip(f"reference shim did not build: {e}")
    if not oracle.ref_available():
        pytest.skip("reference headers not available; reference comparison skipped")
    return oracle.RefOps()


def gpu_threads():
    return max(1, os.cpu_count() or 1)


@pytest.fixture(autouse=True)
def _no_wait_timeouts(request):
    """After every GPU test: no bounded wait in this library's kernels gave up
    (a give-up leaves that launch's results untrustworthy)."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    import torch

    if not torch.cuda.is_available():
        return
    from curadon_gb300.backend import wait_timeouts

    assert wait_timeouts() == 0, "a kernel's bounded wait for its bulk copies gave up"
