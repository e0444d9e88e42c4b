"""The C ABI: the shared library builds, loads, and exports every function
include/octgb.h declares (symbol lookup only; no compute call without a GPU)."""
from __future__ import annotations

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    txt = (ROOT / "include" / "octgb.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(octgb_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    import oct_recon_af_v1_gb300 as pkg
    from oct_recon_af_v1_gb300 import _lib
    pkg.build()
    declared = _declared()
    assert len(declared) >= 18
    assert sorted(_lib.SIGNATURES) == declared, "ctypes signatures and header disagree"
    import ctypes
    lib = ctypes.CDLL(str(pkg.LIB))
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing


def test_library_loads_without_gpu_and_create_fails_cleanly():
    """Without a usable GPU octgb_create must return an error code, not crash."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from oct_recon_af_v1_gb300 import _lib
    with pytest.raises(_lib.OctgbError) as e:
        _lib.Context(0)
    assert e.value.code in (_lib.ERR_CUDA, _lib.ERR_STATE)
