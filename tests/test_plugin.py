"""Registration of device "gb300" in the reference's octrecon (CPU only:
mechanics of the drop-in boundary, no device work)."""
from __future__ import annotations

import pytest

from octrecon_ref import import_octrecon


def test_register_adds_device_without_breaking_others():
    import_octrecon()
    import octrecon.backend as backend
    import octrecon.estimation._common as common
    import octrecon.pipeline as pipeline

    from oct_recon_af_v1_gb300 import plugin
    plugin.register()
    plugin.register()                           # idempotent
    xp, name = backend.get_xp("gb300")
    assert name == "gb300" and backend.is_torch(xp)
    assert str(xp.device).startswith("cuda")
    assert pipeline.get_xp is backend.get_xp and common.get_xp is backend.get_xp
    import numpy as np
    assert backend.get_xp("cpu") == (np, "cpu")
    with pytest.raises(ValueError):
        backend.get_xp("no-such-device")
    assert pipeline.Reconstructor.__init__.__name__ == "init"


def test_cli_entry_point_imports():
    import_octrecon()
    from oct_recon_af_v1_gb300 import octrecon_cli
    assert callable(octrecon_cli.main)
