"""pytest configuration: the `gpu` marker and shared fixtures.

Tests marked `gpu` need a CUDA device (sm_100 family) and the built
liboctgb.so; everything else runs on the CPU.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built liboctgb.so")


@pytest.fixture(scope="session")
def telesto():
    return dict(np.load(GOLDEN / "telesto_case.npz"))


@pytest.fixture(scope="session")
def spectral_case():
    return dict(np.load(GOLDEN / "spectral_case.npz"))


@pytest.fixture(scope="session")
def gpu_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oct_recon_af_v1_gb300 as pkg
    pkg.build()
    from oct_recon_af_v1_gb300._lib import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
