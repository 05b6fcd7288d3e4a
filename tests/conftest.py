import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103); runs the CUDA decode path")


@pytest.fixture(scope="session")
def golden():
    return json.loads((GOLDEN / "golden.json").read_text())


@pytest.fixture(scope="session")
def rans_blob():
    return (GOLDEN / "rans_vectors.bin").read_bytes()


def golden_stream(name: str) -> bytes:
    return (GOLDEN / name).read_bytes()


@pytest.fixture(scope="session")
def gpu_ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gst_gb300 import decoder
    ctx = decoder.GPUContext(0)
    yield ctx
    ctx.close()


def as_blocks(dxt: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(dxt, dtype=np.uint8).view(np.uint64)
