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
  same arguments, cancellation checked per batch (raises octrecon's
  Cancelled), `on_batch(done, total)` callbacks over the reference's (tile,
  frame batch) jobs, the `timers` keys, and float32 dB (nFrames, nOutZ,
  nOutX) on the host.  It runs on the frame API: the reference's readers
  fill pinned host slots for a chunk of frames of every tile of the row,
  copy streams carry them to the device and back, and one call per chunk
  reconstructs and stitches all tiles with num/den on chip (`_RowRun`).
  Each voxel sums its tiles x-major/z-minor, as the reference does.
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
        self.staging = None

    def ensure_staging(self, torch):
        if self.staging is None:
            self.staging = _Staging(torch, f"cuda:{self.ctx.device}")
        return self.staging

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
    """GB300 body of Reconstructor.process_row (octrecon/pipeline.py:223-302):
    same arguments, float32 dB (nFrames, nOutZ, nOutX) on the host, per-batch
    cancellation (octrecon's Cancelled), on_batch(done, total) over the
    reference's (tile, frame batch) jobs, and its timer keys."""
    return _RowRun(self, yi, frames, pool, on_batch).run()


def _frame_chunks(frames: np.ndarray, batch: int):
    """(output offset, frames) of consecutive-valued runs of at most `batch`
    frames (the frame API takes frames f0 .. f0 + B - 1 in one call)."""
    out, start = [], 0
    for i in range(1, len(frames) + 1):
        if i == len(frames) or frames[i] != frames[i - 1] + 1 or i - start == batch:
            out.append((start, frames[start:i]))
            start = i
    return out


class _Staging:
    """Rings of the row pipeline, kept by the engine across rows and grown on
    demand: pinned host slots the readers fill (one per chunk in flight) and
    the device slots they are copied to.  Events order every reuse."""

    def __init__(self, torch, device: str, depth: int = 3):
        self.torch, self.device, self.depth = torch, device, depth
        self.host = [None] * depth
        self.dev = [None] * depth
        self.copied = [torch.cuda.Event() for _ in range(depth)]     # host slot free again
        self.consumed = [torch.cuda.Event() for _ in range(depth)]   # device slot free again
        self.h2d = torch.cuda.Stream(device)
        self.d2h = torch.cuda.Stream(device)
        self.compute = torch.cuda.Stream(device)

    def _fit(self, bufs, k, numel, dtype, **kw):
        b = bufs[k]
        if b is None or b.numel() < numel or b.dtype != dtype:
            bufs[k] = b = self.torch.empty(numel, dtype=dtype, **kw)
        return b[:numel]

    def host_slot(self, k, numel, dtype):
        return self._fit(self.host, k, numel, dtype, pin_memory=True)

    def dev_slot(self, k, numel, dtype):
        return self._fit(self.dev, k, numel, dtype, device=self.device)


_TORCH_RAW = {"uint16": "int16", "int16": "int16", "float32": "float32"}


class _RowRun:
    """One process_row call.  The unit of work is a chunk of consecutive frames
    over every non-empty tile of the y-row (x-major, z-minor: the order the
    tiles are summed in, as in the reference).  The I/O pool reads a chunk's
    raw B-scans straight into a pinned host slot while earlier chunks are on
    the device; a copy stream moves the slot to a device slot; one
    octgb_frames_process call reconstructs the chunk (spectral stage, focus-
    weighted stitching and finalise with num/den on chip) into the device row;
    its planes return through a pinned output slot on a third stream.  Rare
    formats (binning, frame-mean background, repeats) add each tile of a
    chunk through the row API instead, and finalise once."""

    def __init__(self, R, yi, frames, pool, on_batch):
        import torch
        self.torch, self.R, self.eng = torch, R, R._gb300
        self.hdr, self.cfg = R.hdr, R.cfg
        self.frames = np.arange(R.si.n_y_px) if frames is None else np.asarray(frames)
        self.tiles = [t for t in R.si.tiles_in_row(yi) if not R.stitchers[(t.xi, t.zi)].empty]
        self.chunks = _frame_chunks(self.frames, max(1, int(self.cfg.batch_frames)))
        self.pool, self.on_batch = pool, on_batch
        self.n_jobs = len(self.tiles) * len(self.chunks)
        self.srr = bool(self.tiles) and _is_srr(R.reader(self.tiles[0].folder))
        self.files_per_frame = max(1, int(self.hdr.bscan_avg))
        self.raw_np = np.dtype(self.hdr.raw_dtype)

    # ---- reads (I/O threads) ---------------------------------------------
    def _files(self, fr):
        return [f for v in fr for f in self.R.frame_files(int(v))]

    def _slot_view(self, k, n_files):
        """Pinned host slot k as (tiles, files, interf, n) in the raw dtype, and
        the torch tensor behind it."""
        per_tile = n_files * self.hdr.interf_size * self.hdr.n_lambda
        slot = self.eng.staging.host_slot(k, per_tile * len(self.tiles),
                                          getattr(self.torch, _TORCH_RAW[self.raw_np.name]))
        view = slot.numpy().view(self.raw_np).reshape(len(self.tiles), n_files, self.hdr.interf_size,
                                                      self.hdr.n_lambda)
        return slot, view

    def _read_tile(self, k, chunk, j):
        """One tile's raw B-scans of a chunk: into pinned slot k (regular
        readers; the slot's previous chunk has left for the device first), or
        the SRR words as stored."""
        files = self._files(chunk[1])
        t = self.tiles[j]
        if self.srr:
            return _srr_words(self.R.reader(t.folder), files, self.hdr.n_lambda)
        self.eng.staging.copied[k].synchronize()
        _, view = self._slot_view(k, len(files))
        self.R.reader(t.folder).read_bscans(files, view[j])
        return None

    def _submit_reads(self, pool, k, chunk):
        if not self.srr:
            self._slot_view(k, len(self._files(chunk[1])))       # size the slot once, before the tile jobs
        return [pool.submit(self._read_tile, k, chunk, j) for j in range(len(self.tiles))]

    def _wait_reads(self, k, chunk, futures):
        got = [f.result() for f in futures]
        return got if self.srr else self._slot_view(k, len(self._files(chunk[1])))[0]

    # ---- device side (the calling thread) ----------------------------------
    def _device_raws(self, k, chunk, got):
        """The chunk's raws as device tensors (B files, interf, n), one per tile."""
        torch, st, eng = self.torch, self.eng.staging, self.eng
        n_files = len(chunk[1]) * self.files_per_frame
        shape = (n_files, self.hdr.interf_size, self.hdr.n_lambda)
        if self.srr:
            raws = []
            for j, words in enumerate(got):
                a0, a1 = words.apod_range
                s0, s1 = words.scan_range
                n_lines = (a1 - a0) + (s1 - s0)
                dev = st.dev_slot(k, len(got) * n_files * n_lines * self.hdr.n_lambda, torch.int16)
                one = dev.view(len(got), n_files, n_lines, self.hdr.n_lambda)[j]
                eng.ctx.srr_decode(words.words, words.apod_range, words.scan_range, out=one)
                raws.append(one)
            return raws
        dev = st.dev_slot(k, got.numel(), got.dtype)
        st.h2d.wait_event(st.consumed[k])
        with torch.cuda.stream(st.h2d):
            dev.copy_(got, non_blocking=True)
        st.copied[k].record(st.h2d)
        st.compute.wait_event(st.copied[k])
        return list(dev.view((len(self.tiles),) + shape))

    def run(self):
        from octrecon.pipeline import Cancelled
        torch, R, eng = self.torch, self.R, self.eng
        nF = len(self.frames)
        _, nz, nx = R.n_out
        if not self.tiles:
            return np.full((nF, nz, nx), np.nan, np.float32)
        eng.ensure_staging(torch)
        st = eng.staging
        ctx = eng.ctx
        # the result lives in pinned memory, so each chunk's planes go to the
        # host by DMA while later chunks reconstruct (torch's pinned-memory
        # cache recycles it once the caller drops the array)
        host_out = torch.empty((nF, nz, nx), dtype=torch.float32, pin_memory=True)
        out = host_out.numpy()
        dtype = 1 if self.srr else (0 if self.raw_np == np.uint16 else (1 if self.raw_np == np.int16 else 2))
        ids = [eng.plans[(t.xi, t.zi)] for t in self.tiles]
        apod = int(self.hdr.apod_size)
        own_pool = self.pool is None
        pool = self.pool or ThreadPoolExecutor(self.cfg.io_threads)
        depth = st.depth
        reads = {}
        with torch.cuda.device(st.device):
            prev_stream = torch.cuda.current_stream()
            torch.cuda.set_stream(st.compute)
            ctx.follow_torch_stream()
            try:
                if eng.rare:
                    ctx.row_begin(nF, nz, nx)
                else:
                    row = torch.empty((nF, nz, nx), dtype=torch.float32, device=st.device)
                for c in range(min(depth, len(self.chunks))):
                    reads[c] = self._submit_reads(pool, c % depth, self.chunks[c])
                done = 0
                for c, chunk in enumerate(self.chunks):
                    if R.cancel.is_set():
                        raise Cancelled()
                    k = c % depth
                    t0 = time.perf_counter()
                    got = self._wait_reads(k, chunk, reads.pop(c))
                    t1 = time.perf_counter()
                    R.timers["io_wait"] += t1 - t0
                    raws = self._device_raws(k, chunk, got)
                    t2 = time.perf_counter()
                    R.timers["h2d"] += t2 - t1
                    off, fr = chunk
                    if eng.rare:
                        for pid, raw in zip(ids, raws):
                            ctx.row_add_batch_ex(pid, raw, apod, fr, off, eng.binning, eng.apod_mode,
                                                 eng.bscan_avg, eng.ascan_avg, raw_dtype=dtype)
                    else:
                        planes = row[off:off + len(fr)]
                        ctx.frames_process(ids, raws, apod, int(fr[0]), nz, nx, eng.threshold, out=planes,
                                           raw_dtype=dtype)
                        st.d2h.wait_stream(st.compute)
                        with torch.cuda.stream(st.d2h):
                            host_out[off:off + len(fr)].copy_(planes, non_blocking=True)
                    st.consumed[k].record(st.compute)
                    R.timers["spectral"] += time.perf_counter() - t2
                    if c + depth < len(self.chunks):
                        reads[c + depth] = self._submit_reads(pool, k, self.chunks[c + depth])
                    done += len(self.tiles)
                    if self.on_batch:
                        self.on_batch(done, self.n_jobs)
                t0 = time.perf_counter()
                if eng.rare:
                    ctx.row_finalise(eng.threshold, (nF, nz, nx), out)
                st.d2h.synchronize()
                R.timers["finalise"] += time.perf_counter() - t0
            finally:
                left = [f for fs in reads.values() for f in fs]
                for f in left:
                    f.cancel()
                if own_pool:
                    pool.shutdown(wait=True, cancel_futures=True)
                # reads still running would write into the rings: let them end
                for f in left:
                    if not f.cancelled():
                        try:
                            f.result()
                        except Exception:
                            pass
                st.compute.synchronize()
                st.h2d.synchronize()
                st.d2h.synchronize()
                torch.cuda.set_stream(prev_stream)
                ctx.set_stream(None)
        return out
