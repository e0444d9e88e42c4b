"""Device "gb300" for the reference's octrecon package.

`register()` adds the device to an imported octrecon without editing its
files, so `Reconstructor`, the CLI (`--set device=gb300`) and the web app
(config `device`) drive the GB300 kernels unchanged:

* octrecon/backend.py:61-83 `get_xp` accepts "gb300" and returns a TorchXP-
  like namespace on the CUDA device (`is_torch` true, :86), so the pipeline
  builds its host-side operators exactly as for its torch backend
  (octrecon/pipeline.py:172-189) and never imports CuPy.  The name is bound by
  value in pipeline.py:33 and estimation/_common.py:14, so those module
  globals are patched too.
* `Reconstructor.__init__` (pipeline.py:96-192) is wrapped: when the device is
  "gb300" it uploads the geometry the reference built (self.sg: sinc band and
  window, geometry.py:84-128; self.stitchers: TileStitcher operators,
  stitching.py:84-120; self.oc: optical-path correction, :54-78) into an
  octgb context and binds `process_row` to the GB300 row engine below.
* The bound `process_row` keeps the reference's contract (pipeline.py:223-302):
  same arguments, threaded read-ahead of raw batches through the reference's
  own readers, cancellation checked per batch (raises octrecon's Cancelled),
  `on_batch(done, total)` callbacks, the `timers` keys, and returns float32 dB
  (nFrames, nOutZ, nOutX) on the host.  Tiles are processed x-major/z-minor
  and every batch is added in that order, as in the reference.
* Estimators asked for device gb300 (estimate_dispersion, detect_focus,
  octrecon/estimation) keep their host logic; their spectral processors and
  the DispersionScorer run on the GB300 kernels (`_register_estimators`).
* Thorlabs SRR scans (io/srr.py): the read-ahead threads read each file's
  words as stored and the 12-bit decode plus the apodisation / scan line
  gather run on the device (`_srr_words`, octgb_srr_decode); only the used
  lines cross the link.
* The legacy TIFF writer (io/tiff_writer.py:53-71, called by
  Reconstructor.run) is replaced by `tiff.write_legacy_tiff`: same file
  layout, codes and PackBits packets computed on the GPU.
* The web app's GPU card only lights up when CuPy imports
  (webapp/server.py:74-85); `register()` patches its `system_info` to report
  the gb300 device.

There is no CPU fallback: if the CUDA library or device is unusable the
Reconstructor construction fails with the library's error.
"""
from __future__ import annotations

import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor

import numpy as np

DEVICE = "gb300"
_registered = False


def _torch_xp_class():
    from octrecon.core.torch_backend import TorchXP

    class GB300XP(TorchXP):
        """TorchXP on CUDA: satisfies the pipeline's array duck-type for the
        host-side operator construction; the hot path runs in liboctgb."""

        def __init__(self, device_index: int = 0):
            super().__init__(f"cuda:{device_index}")
            self.name = DEVICE

    return GB300XP


def register(device_index: int = 0) -> None:
    """Register device "gb300" with the imported octrecon (idempotent)."""
    global _registered
    if _registered:
        return
    import octrecon.backend as backend
    import octrecon.pipeline as pipeline

    GB300XP = _torch_xp_class()
    orig_get_xp = backend.get_xp

    def get_xp(device: str = "auto"):
        if device == DEVICE:
            return GB300XP(device_index), DEVICE
        return orig_get_xp(device)

    get_xp.__doc__ = orig_get_xp.__doc__
    backend.get_xp = get_xp
    pipeline.get_xp = get_xp
    try:
        _register_estimators(get_xp, device_index)
    except ImportError:
        pass

    orig_init = pipeline.Reconstructor.__init__

    def init(self, cfg, *a, **kw):
        orig_init(self, cfg, *a, **kw)
        if self.device == DEVICE:
            _attach(self, device_index)

    pipeline.Reconstructor.__init__ = init

    try:
        # the legacy TIFF (tiff_writer.py:53-71) written from the GPU codes and
        # PackBits packets; needs neither tifffile nor imagecodecs
        import octrecon.io.tiff_writer as tiff_writer

        from .tiff import write_legacy_tiff as gb300_write

        def write_legacy_tiff(path, db_volume, clim, metadata, legacy_double_quantization=False, plane_clims=None,
                              progress=None):
            return gb300_write(path, db_volume, clim, metadata, legacy_double_quantization, plane_clims, progress,
                               device=device_index)

        write_legacy_tiff.__doc__ = tiff_writer.write_legacy_tiff.__doc__
        tiff_writer.write_legacy_tiff = write_legacy_tiff
    except ImportError:
        pass

    try:
        import octrecon.webapp.server as server
        orig_info = server.system_info

        def system_info():
            info = dict(orig_info())
            try:
                import torch
                if torch.cuda.is_available():
                    info.update(gpu_available=True, gpu_kind=DEVICE, gpu_name=torch.cuda.get_device_name(device_index))
            except Exception:
                pass
            return info

        server.system_info = system_info
    except Exception:
        pass
    _registered = True


class _GB300Processor:
    """SpectralProcessor.magnitude (octrecon/core/spectral.py:136-153) of one
    geometry on the GB300 kernels; host arrays in and out, as the estimators'
    CPU path."""

    def __init__(self, sg, apod_size: int, device_index: int, binning: int = 1, apod_mode: int = 0,
                 apod_group: int = 1):
        from ._lib import Context
        self.ctx = Context(device_index)
        self.ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
        self.apod_size = int(apod_size)
        self.binning, self.apod_mode, self.apod_group = int(binning), int(apod_mode), int(apod_group)
        self.n = len(sg.lambda_nm)
        self.nz = self.n // 2

    def prepare(self, raw):
        """prepare_raw (core/spectral.py:48-68) on the device; raw itself when nothing applies."""
        if self.binning == 1 and self.apod_mode == 0:
            return np.asarray(raw)
        return self.ctx.prepare_raw(np.asarray(raw), self.apod_size, self.binning, self.apod_mode, self.apod_group)

    def magnitude(self, raw):
        x = self.prepare(raw)
        a = 1 if self.apod_mode == 1 else self.apod_size
        return self.ctx.magnitude(x, a)


def _register_estimators(get_xp, device_index: int) -> None:
    """Estimators on device gb300 (octrecon/estimation): VolumeContext
    (_common.py:38-118) keeps its host readers and NumPy namespace, its
    processors run the GB300 magnitude kernel, and DispersionScorer
    (dispersion.py:66-107) becomes the GB300 scorer; estimate_dispersion and
    detect_focus themselves run unchanged."""
    import octrecon.estimation._common as common
    import octrecon.estimation.dispersion as disp

    from .estimation import DispersionScorer as GB300Scorer
    common.get_xp = get_xp
    VC = common.VolumeContext
    orig_ctx_init, orig_processor = VC.__init__, VC.processor

    def ctx_init(self, volume_folder, device="cpu", dtype=np.float32):
        gb = device == DEVICE
        orig_ctx_init(self, volume_folder, "cpu" if gb else device, dtype)
        self._gb300 = {} if gb else None
        if gb:
            self.device = DEVICE

    def processor(self, dispersion, n_medium=None):
        cache = getattr(self, "_gb300", None)
        if cache is None:
            return orig_processor(self, dispersion, n_medium)
        key = (float(dispersion), self.si.tissue_ri if n_medium is None else float(n_medium))
        sp = cache.get(key)
        if sp is None:
            h = self.hdr
            sp = cache[key] = _GB300Processor(self.geometry(dispersion, n_medium), h.apod_size, device_index,
                                              max(1, h.spectra_avg), 1 if h.apod_mode == "frame_mean" else 0,
                                              max(1, h.bscan_avg))
        return sp

    VC.__init__ = ctx_init
    VC.processor = processor
    orig_scorer = disp.DispersionScorer

    def scorer(ctx, raw_list, metric):
        if getattr(ctx, "_gb300", None) is not None:
            return GB300Scorer.from_context(ctx, raw_list, metric, device_index)
        return orig_scorer(ctx, raw_list, metric)

    disp.DispersionScorer = scorer


class _RowEngine:
    """The octgb context of one Reconstructor: geometry, stitch plans."""

    def __init__(self, R, device_index: int):
        from ._lib import Context
        hdr = R.hdr
        self.ctx = Context(device_index)
        self.ctx.set_geometry(R.sg.sinc_idx, R.sg.sinc_w, R.sg.window)
        # rare formats (core/spectral.py:20-82,168-177): prepared and averaged on the device
        self.binning = max(1, int(hdr.spectra_avg))
        self.apod_mode = 1 if hdr.apod_mode == "frame_mean" else 0
        self.bscan_avg = max(1, int(hdr.bscan_avg))
        self.ascan_avg = max(1, int(hdr.ascan_avg))
        self.rare = self.binning > 1 or self.apod_mode == 1 or self.bscan_avg > 1 or self.ascan_avg > 1
        self.plans = {}
        for key, st in R.stitchers.items():
            if st.empty:
                continue
            Wz = st.WzT.detach().cpu().numpy().T if hasattr(st, "WzT") else np.asarray(st.Wz)
            WxT = st.WxT.detach().cpu().numpy() if hasattr(st.WxT, "detach") else np.asarray(st.WxT)
            fz = st.fz.detach().cpu().numpy() if hasattr(st.fz, "detach") else np.asarray(st.fz)
            oc = R.oc
            self.plans[key] = self.ctx.stitch_plan(
                len(R.sg.z_um), st.r0, st.r1, st.c0, st.c1, Wz, WxT, fz,
                None if oc is None else oc.shift, None if oc is None else oc.pdz)
        from .stitching import min_weight_threshold
        self.threshold = min_weight_threshold(np.float32)
        self._srr_buf = None

    def srr_raw(self, sw: _SrrWords):
        """Device int16 (files, interf, n) of one batch of SRR words, in a
        buffer reused batch after batch (every use is on the context's stream)."""
        import torch
        a0, a1 = sw.apod_range
        s0, s1 = sw.scan_range
        shape = (sw.words.shape[0], (a1 - a0) + (s1 - s0), sw.words.shape[2])
        if self._srr_buf is None or tuple(self._srr_buf.shape) != shape:
            self._srr_buf = torch.empty(shape, dtype=torch.int16, device=f"cuda:{self.ctx.device}")
        return self.ctx.srr_decode(sw.words, sw.apod_range, sw.scan_range, out=self._srr_buf)


class _SrrWords:
    """The files of one batch as stored, (files, file_lines, n) uint16, and
    the header's line ranges."""

    def __init__(self, words, apod_range, scan_range):
        self.words, self.apod_range, self.scan_range = words, apod_range, scan_range


def _srr_words(reader, file_indices, n_lambda: int) -> _SrrWords:
    """SRRTileReader.read_file without the decode (io/srr.py:108-118): each
    file's words after its header, the same size check; the decode and the
    line gather of read_bscans (:120-125) run on the device."""
    from pathlib import Path
    h = reader.srr
    file_lines = int(reader.file_lines)
    words = np.empty((len(file_indices), file_lines, n_lambda), np.uint16)
    for k, fi in enumerate(file_indices):
        p = Path(reader.dir) / reader.file_name(fi)
        b = p.read_bytes()
        data = np.frombuffer(b, dtype="<u2", offset=h["headerTotalBytes"], count=(len(b) - h["headerTotalBytes"]) // 2)
        if data.size != n_lambda * file_lines:
            raise IOError(f"{p}: expected {n_lambda * file_lines} samples, got {data.size}")
        words[k] = data.reshape(file_lines, n_lambda)
    return _SrrWords(words, (h["apodstart"], h["apodend"]), (h["scanstart"], h["scanend"]))


def _is_srr(reader) -> bool:
    return getattr(reader, "layout", None) == "srr" and hasattr(reader, "srr") and hasattr(reader, "file_lines")


def _attach(R, device_index: int) -> None:
    R._gb300 = _RowEngine(R, device_index)
    R.process_row = _process_row.__get__(R, type(R))


def _process_row(self, yi: int, frames=None, pool=None, on_batch=None):
    """GB300 body of Reconstructor.process_row (octrecon/pipeline.py:223-302)."""
    from octrecon.pipeline import Cancelled
    eng = self._gb300
    cfg, hdr = self.cfg, self.hdr
    frames = np.arange(self.si.n_y_px) if frames is None else np.asarray(frames)
    nF = len(frames)
    _, nz_out, nx_out = self.n_out
    B = cfg.batch_frames
    jobs = []
    for t in self.si.tiles_in_row(yi):
        if self.stitchers[(t.xi, t.zi)].empty:
            continue
        for s in range(0, nF, B):
            jobs.append((t, s, frames[s:s + B]))

    def read_job(job):
        t, s, fr = job
        files = [f for fr_ in fr for f in self.frame_files(int(fr_))]
        rd = self.reader(t.folder)
        if _is_srr(rd):
            return _srr_words(rd, files, hdr.n_lambda)
        buf = np.empty((len(files), hdr.interf_size, hdr.n_lambda), np.dtype(hdr.raw_dtype))
        rd.read_bscans(files, buf)
        return buf

    ctx = eng.ctx
    ctx.row_begin(nF, nz_out, nx_out)
    own_pool = pool is None
    pool = pool or ThreadPoolExecutor(cfg.io_threads)
    pending = deque()
    it = iter(jobs)
    for _ in range(self.prefetch):
        j = next(it, None)
        if j is None:
            break
        pending.append((j, pool.submit(read_job, j)))
    n_done = 0
    try:
        while pending:
            if self.cancel.is_set():
                raise Cancelled()
            job, fut = pending.popleft()
            t0 = time.perf_counter()
            raw = fut.result()
            t1 = time.perf_counter()
            self.timers["io_wait"] += t1 - t0
            nxt = next(it, None)
            if nxt is not None:
                pending.append((nxt, pool.submit(read_job, nxt)))
            t, s, fr = job
            if isinstance(raw, _SrrWords):
                raw = eng.srr_raw(raw)
            # spectral stage + stitching + accumulation of this batch on the device
            if eng.rare:
                ctx.row_add_batch_ex(eng.plans[(t.xi, t.zi)], raw, hdr.apod_size, fr, s, eng.binning, eng.apod_mode,
                                     eng.bscan_avg, eng.ascan_avg)
            else:
                ctx.row_add_batch(eng.plans[(t.xi, t.zi)], raw, hdr.apod_size, fr, s)
            t2 = time.perf_counter()
            self.timers["spectral"] += t2 - t1
            n_done += 1
            if on_batch:
                on_batch(n_done, len(jobs))
    finally:
        if own_pool:
            pool.shutdown(wait=True, cancel_futures=True)
        else:
            for _, f in pending:
                f.cancel()
    t0 = time.perf_counter()
    out = ctx.row_finalise(eng.threshold, (nF, nz_out, nx_out))
    self.timers["finalise"] += time.perf_counter() - t0
    return out
