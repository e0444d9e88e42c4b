"""Import helper for tests that drive the reference octrecon package itself.

octrecon is taken from baseline/_ref (an offline `pip install --no-deps` of
the reference; absent -> the calling test skips).  Its TIFF writer imports
tifffile at module level; when tifffile is missing an empty stand-in module is
registered (only the TIFF writer would use it and these tests never write
TIFFs).
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF = ROOT / "baseline" / "_ref"


def import_octrecon():
    if not (REF / "octrecon" / "pipeline.py").exists():
        pytest.skip("octrecon is not installed in baseline/_ref")
    if str(REF) not in sys.path:
        sys.path.insert(0, str(REF))
    try:
        import tifffile  # noqa: F401
    except ImportError:
        sys.modules.setdefault("tifffile", types.ModuleType("tifffile"))
    import octrecon.pipeline  # noqa: F401
    return sys.modules["octrecon"]
