"""The reference's own Reconstructor driving device "gb300" end to end on the
`telesto` format-test volume (the on-disk scan the reference's generator
writes): reads, geometry, parameter resolution and the public
process_planes/process_row API are octrecon's; the hot path is liboctgb.
Criteria as in the reference's tests (tests/test_formats.py:171-180,
tests/test_torch_backend.py:63-71)."""
from __future__ import annotations

import tarfile
import threading

import numpy as np
import pytest

from octrecon_ref import import_octrecon

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def volume(tmp_path_factory):
    d = tmp_path_factory.mktemp("vol")
    with tarfile.open(__import__("conftest").GOLDEN / "telesto_volume.tar.gz") as tf:
        tf.extractall(d, filter="data")
    return d / "telesto"


def _cfg(ReconConfig, vol, **kw):
    import json
    info = json.loads((vol / "synthetic_info.json").read_text())
    return ReconConfig(volume_folder=str(vol), device="gb300", precision="float32", dispersion_quadratic_term=8.949e7,
                       focus_positions=float(info["focus_pix"]), focus_sigma=10, crop_z_range_mm="none",
                       output_pixel_size_um=info.get("pixel_um", 2), interp_method="sinc5", batch_frames=4,
                       io_threads=2, write_tiff=False, **kw)


def test_reconstructor_on_gb300_matches_golden(volume, telesto):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import_octrecon()
    from octrecon.pipeline import ReconConfig, Reconstructor

    from oct_recon_af_v1_gb300 import plugin
    plugin.register()
    calls = []
    R = Reconstructor(_cfg(ReconConfig, volume), log=lambda *a: None)
    assert R.device == "gb300" and hasattr(R, "_gb300")
    n0 = R._gb300.ctx.launches
    p = R.process_row(0, frames=[1], on_batch=lambda i, n: calls.append((i, n)))[0].astype(float)
    assert R._gb300.ctx.launches > n0
    assert calls and calls[-1][0] == calls[-1][1]
    ref32 = telesto["plane_fp32"].astype(float)
    m = telesto["matlab_plane"].astype(float)
    assert np.array_equal(np.isfinite(p), np.isfinite(ref32))
    assert not np.any((np.isfinite(p) != np.isfinite(m)) & ~telesto["matlab_tie"])
    fin = np.isfinite(p) & np.isfinite(m)
    err, err_ref = np.abs(p - m)[fin].max(), np.abs(ref32 - m)[fin].max()
    assert err <= 1.5 * err_ref + 1e-4, (err, err_ref)
    # the public API around process_row is the reference's
    both = R.process_planes([0, 1])
    np.testing.assert_array_equal(both[1], R.process_row(0, frames=[1])[0])
    assert set(R.timers) >= {"io_wait", "spectral", "finalise"}


def test_cancel_stops_the_row(volume):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import_octrecon()
    from octrecon.pipeline import Cancelled, ReconConfig, Reconstructor

    from oct_recon_af_v1_gb300 import plugin
    plugin.register()
    ev = threading.Event()
    R = Reconstructor(_cfg(ReconConfig, volume), log=lambda *a: None, cancel=ev)
    ev.set()
    with pytest.raises(Cancelled):
        R.process_row(0)
