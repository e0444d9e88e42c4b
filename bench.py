"""Throughput benchmark: A-scans/s of the GB300 reconstruction.

Workload (default, `--config 1`): synthetic tiled scan, 2 x 2 lateral tiles x
3 depth stacks, each tile 270 B-scans x (25 apodisation + 1000) A-scans x 2048
uint16 spectral samples (~1.1 GB, 13.3 GB in all, 3.24 M A-scans), generated
on the device with the package's seeded spectrum model.  Focus at z = 400 +
U[-30, 30] px per depth, focus_sigma 80 px, 10 % lateral overlap, refractive
index 1.33, output 1 um pixels, no optical-path correction.  One step is the
whole volume: for each y-tile row, every tile's spectral stage, focus-weighted
stitching, row finalise (dB + per-plane clim); then the global clim and the
legacy uint16 quantisation of the volume.

`--config 0`: one tile, 50 B-scans x (25 + 500) A-scans, z-crop 1000 px:
spectral stage to dB, global clim, quantisation.
`--config 2`: the config-1 tiles through the precision form of the spectral
stage (exact background, tcgen05 split-FP16 sinc), beside the float32 form.
`--config 3`: 64 tiles of uneven size in one persistent launch (device work
queue, CUDA graph, autotuned grab / order), beside per-tile launches.
`--config 4`: the learned beta/focus estimator trained on the device (20 k
probe images), timed on 500 held-out B-scans against the GPU plain search.

`value` is measured with inputs resident in HBM (inputs are larger than L2, so
no flush is needed); `e2e` repeats the step through the same API with the raw
spectra in pinned host memory (H2D inside the timed region) and reads the
uint16 volume back (D2H).  Volumes are processed back to back: a volume's
codes need its global clim, so their read-back overlaps the next volume's
upload and reconstruction (second stream, double-buffered codes); the timed
region holds max(8, K) volumes and ends after the last read-back; `e2e_link`
gives this box's pinned host<->device copy bandwidth measured just before.
`roofline` is the spectral stage's against HBM; its `fp32_ceiling` is the same
launch against the CUDA cores' nominal FP32 rate.  `--impl reference` times the reference
algorithm's CPU restatement (the oracle: Numba kernel restated in C/OpenMP +
pocketfft + NumPy stitching) on the host cores over bounded samples.

Run:  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "A-scans/s on 1 GB300 (fused vs plain FP32; learned vs search β) at ≤1 LSB"
APOD = 25
# DRAM bytes per A-scan of the spectral kernel from one ncu capture
# (profiles/k_spectral_config1_small.md: (49.43 + 7.16) MB over 12 000 A-scans;
# caches flushed before the kernel, magnitudes partly still in L2 at its end)
SPECTRAL_DRAM_BYTES_PER_ASCAN = (49.433856e6 + 7.155456e6) / 12000


# ------------------------------------------------------------------------ workload description
def config1_layout(seed=1, bscans=270):
    """Config-1 scan layout; `bscans` < 270 gives a small case of the same
    geometry (used for profiling captures)."""
    from oct_recon_af_v1_gb300 import synthetic
    return synthetic.config1_layout(seed, bscans)


def config1_desc(bscans=270):
    """The workload alone (the same dict in both arms); how an arm runs it
    (parallelism, batch, the A-scans one timed step covers) is its `execution`."""
    return {"workload": f"config1: 2x2 tiles x 3 depths, tile {bscans} B-scans x 1000 A-scans x 2048 uint16, "
                        "focus 400+-30 px sigma 80, 10% overlap, n 1.33, 1 um output, uint16 legacy codes",
            "a_scans_per_volume": 12 * bscans * 1000, "tiles": 12, "bscans_per_tile": bscans,
            "ascans_per_bscan": 1000,
            "apod_lines": APOD, "spectral_samples": 2048, "l2_flush": "inputs (13.3 GB) larger than L2"}


def config0_desc():
    return {"workload": "config0: 1 tile, 50 B-scans x 500 A-scans x 2048 uint16, z-crop 1000, uint16 codes",
            "a_scans_per_step": 50 * 500, "l2_flush": "spectral inputs 107 MB + outputs 100 MB cycled over "
            "8 resident copies (856 MB) so each step reads inputs not left in L2"}


# ------------------------------------------------------------------------ clocks sampler
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons, pw = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                pw.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": float(max(pw)) if pw else None}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------------ GPU arm
class Volume:
    """Config-1 scan: geometry, stitch plans and the raw tiles (device and/or pinned host)."""

    def __init__(self, ctx, torch, dev, host_copy: bool, seed: int = 1, bscans: int = 270):
        from oct_recon_af_v1_gb300 import geometry as G
        from oct_recon_af_v1_gb300 import stitching as S
        from oct_recon_af_v1_gb300 import synthetic
        self.lay, self.focus = config1_layout(seed, bscans)
        lam = synthetic.lambda_nm()
        self.sg = G.build_spectral_geometry(lam, synthetic.beta_ref_from_px(1e-5), 1.33)
        ctx.set_geometry(self.sg.sinc_idx, self.sg.sinc_w, self.sg.window)
        self.tg = S.tiled_geometry(self.lay, self.sg.z_um, self.focus, 1.0)
        self.nz, self.nx = len(self.tg.out_z_mm), len(self.tg.out_x_mm)
        self.ny = self.lay.n_y_px
        self.order = [(xi, zi) for xi in range(2) for zi in range(3)]   # x-major, z-minor
        self.st = {}
        for xi, zi in self.order:
            st = S.TileStitcher.build(self.tg, self.lay.x_centers_mm[xi], self.lay.z_depths_mm[zi],
                                      self.focus[zi], 80.0)
            st.upload(ctx)
            self.st[(xi, zi)] = st
        self.raw = {}
        self.host = {}
        k = 0
        for yi in range(2):
            for xi, zi in self.order:
                t = synthetic.u16_bits(synthetic.generate(self.ny, self.lay.n_x_px, APOD, seed=seed * 1000 + k,
                                                          device=dev, chunk=30))
                if host_copy:
                    h = torch.empty(t.shape, dtype=torch.int16, pin_memory=True)
                    h.copy_(t)
                    self.host[(yi, xi, zi)] = h
                self.raw[(yi, xi, zi)] = t
                k += 1
        torch.cuda.synchronize()
        self.thr = S.min_weight_threshold(np.float32)
        self.frames = np.arange(self.ny)

    def raw_bytes(self):
        return sum(int(t.numel()) * 2 for t in self.raw.values())


def run_step(ctx, vol, src, db_vol, bits, batch=54):
    """One whole-volume reconstruction through the frame-batch API: for each
    y-row and each batch of `batch` frames, every tile's spectral stage and
    the stitched, finalised planes (num/den never leave the chip; the
    magnitudes of a batch are read back right after they are written, largely
    from L2); then the legacy quantisation with the
    running (global) clim read on the device.  src maps tile keys to device or
    pinned-host int16 tensors holding uint16 spectra."""
    ids = [vol.st[k].plan for k in vol.order]
    ctx.clim_reset()
    for yi in range(2):
        for s in range(0, vol.ny, batch):
            raws = [src[(yi, xi, zi)][s:s + batch] for xi, zi in vol.order]
            o = yi * vol.ny + s
            ctx.frames_process(ids, raws, APOD, s, vol.nz, vol.nx, vol.thr, out=db_vol[o:o + len(raws[0])],
                               raw_dtype=0)
    ctx.quantise_running(db_vol, bits)


FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12     # SMs x FP32 lanes x FMA x max SM clock


def fp32_ceiling(ascans_per_s, sg):
    """Nominal FLOP of one A-scan's spectral stage (background 2N, banded sinc
    2 T N with T the geometry's taps, complex window 2N, 2048-point FFT
    5 N log2 N, |.| 3 N/2) at the measured rate, against the CUDA cores'
    nominal FP32 peak."""
    n = 2048
    taps = int(np.asarray(sg.sinc_idx).shape[1])
    flops = 2 * n + 2 * taps * n + 2 * n + 5 * n * 11 + 3 * n // 2
    achieved = ascans_per_s * flops / 1e12
    return {"flops_per_ascan": flops, "achieved_tflops": achieved, "peak_tflops": FP32_NOMINAL_TFLOPS,
            "frac": achieved / FP32_NOMINAL_TFLOPS,
            "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 x 2.07 GHz (no measured FP32 peak on this pool)"}


def link_bandwidth(torch, stream, dev, nbytes=1 << 30):
    """Host<->device copy bandwidth (GB/s) of this box between pinned host
    memory and the device, CUDA events around 3 copies each way."""
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    out = {}
    for name, (dst, src) in (("h2d_gbs", (d, h)), ("d2h_gbs", (h, d))):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = 3 * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9
    del h, d
    return out


def time_spectral_kernel(ctx, torch, raw_tile, stream, reps=10):
    """CUDA-event time of the spectral stage (apod mean + fused kernel) on a slab of one tile."""
    B = raw_tile.shape[0]
    nxa = raw_tile.shape[1] - APOD
    out = torch.empty((B, nxa, 1024), dtype=torch.float32, device="cuda")
    for _ in range(2):
        ctx.magnitude(raw_tile, APOD, out, raw_dtype=0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        ctx.magnitude(raw_tile, APOD, out, raw_dtype=0)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    bytes_per_launch = B * raw_tile.shape[1] * 2048 * 2 + B * nxa * 1024 * 4
    return ms, bytes_per_launch, B * nxa


def gpu_arm(args, rank, world):
    import torch
    from oct_recon_af_v1_gb300 import build
    from oct_recon_af_v1_gb300._lib import Context
    build()
    dev = f"cuda:{int(os.environ.get('LOCAL_RANK', 0))}"
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()            # a real stream handle: the library launches on it
    torch.cuda.set_stream(stream)
    ctx = Context(torch.cuda.current_device())
    ctx.set_stream(stream.cuda_stream)
    if args.config == 0:
        return gpu_arm_config0(args, rank, world, torch, ctx)
    if args.config == 2:
        return gpu_arm_config2(args, rank, world, torch, ctx, stream, dev)
    if args.config == 3:
        return gpu_arm_config3(args, rank, world, torch, ctx, stream, dev)
    if args.config == 4:
        return gpu_arm_config4(args, rank, world, torch, ctx, stream, dev)
    vol = Volume(ctx, torch, dev, host_copy=not args.no_e2e, bscans=args.bscans)
    n_out = (2 * vol.ny, vol.nz, vol.nx)
    db_vol = torch.empty(n_out, dtype=torch.float32, device=dev)
    bits = torch.empty(n_out, dtype=torch.int16, device=dev)
    ascans = 12 * vol.ny * vol.lay.n_x_px

    # the stitch kernel's tile shape (output rows per block), autotuned on this volume
    from oct_recon_af_v1_gb300 import autotune
    if args.stitch_rows:
        stitch_rows, stitch_ms = args.stitch_rows, None
        ctx.set_stitch_rows(stitch_rows)
    else:
        stitch_rows, stitch_ms = autotune.tune_stitch_rows(
            ctx, lambda: run_step(ctx, vol, vol.raw, db_vol, bits, args.batch), stream,
            key=("config1", vol.ny, vol.nz, vol.nx, args.batch))
    graph = None
    if not args.no_graph:
        run_step(ctx, vol, vol.raw, db_vol, bits, args.batch)      # sizes every buffer
        ctx.synchronize()
        ctx.graph_begin()
        run_step(ctx, vol, vol.raw, db_vol, bits, args.batch)
        graph = ctx.graph_end()

    # end to end, volumes back to back: the codes of a volume need its global
    # clim, so their read-back cannot overlap the volume's own reconstruction;
    # it runs on a second stream (the other link direction) while the next
    # volume's raws stream in and reconstruct, from a double-buffered code volume
    e2e_bits = [bits, torch.empty_like(bits)] if not args.no_e2e else [bits]
    d2h = torch.cuda.Stream()
    d2h_done = [torch.cuda.Event(), torch.cuda.Event()]
    for ev in d2h_done:
        ev.record(d2h)

    def step(src, e2e=False, host_bits=None, k=0):
        if graph is not None and not e2e:
            ctx.graph_launch(graph)
            return
        if not e2e:
            run_step(ctx, vol, src, db_vol, bits, args.batch)
            return
        b = k % 2
        stream.wait_event(d2h_done[b])                  # the copy of two volumes ago has left this buffer
        run_step(ctx, vol, src, db_vol, e2e_bits[b], args.batch)
        end = torch.cuda.Event()
        end.record(stream)
        d2h.wait_event(end)
        with torch.cuda.stream(d2h):
            host_bits[b].copy_(e2e_bits[b], non_blocking=True)
        d2h_done[b].record(d2h)

    def timed(src, steps, warm, e2e=False):
        host_bits = [torch.empty(n_out, dtype=torch.int16, pin_memory=True) for _ in range(2)] if e2e else None
        for k in range(warm):
            step(src, e2e, host_bits, k)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        n0 = ctx.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(steps):
            step(src, e2e, host_bits, k)
        if e2e:                                          # every read-back is inside the timed region
            stream.wait_event(d2h_done[0])
            stream.wait_event(d2h_done[1])
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return e0.elapsed_time(e1) / steps, ctx.launches - n0

    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms, launches = timed(vol.raw, args.steps, args.warmup)
    clk = clocks.stop()
    e2e_ms = None
    link = None
    if not args.no_e2e:
        link = link_bandwidth(torch, stream, dev)
        # at least 8 volumes back to back: the last volume's code read-back (no
        # next volume to overlap with) is inside the timed region
        e2e_ms, _ = timed(vol.host, max(8, args.steps), 1, e2e=True)
    # roofline of the dominant kernel, measured live on a 30-B-scan slab of one tile
    kms, kbytes, kascans = time_spectral_kernel(ctx, torch, vol.raw[(0, 0, 0)][:30], stream)
    ms_all = reduce_max(ms, world)
    hbm, src = peaks()
    achieved = kbytes / (kms * 1e-3) / 1e9
    value = ascans * world / (ms_all * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": "A-scans/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_all, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (uint16 in, uint16 out)", "data": "synthetic (seeded, generated on device)",
        "config": config1_desc(vol.ny),
        "execution": {"parallelism": f"replicas x{world} (independent volumes)", "frame_batch": args.batch,
                      "cuda_graph": graph is not None, "a_scans_per_step": ascans,
                      "stitch_rows": stitch_rows, "stitch_rows_ms": stitch_ms},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": SPECTRAL_DRAM_BYTES_PER_ASCAN * kascans,
                     "kernel": "spectral stage (apod mean + k_spectral, magnitude out)",
                     "bytes_per_launch": kbytes, "ms_per_launch": kms, "a_scans_per_launch": kascans,
                     "peak_source": src + " (burst copy)",
                     # the arithmetic intensity (~21 flop/B) is above the FP32 ridge: the same
                     # launch against the CUDA cores' nominal FP32 rate
                     "fp32_ceiling": fp32_ceiling(kascans / (kms * 1e-3), vol.sg)},
        "clocks": clk,
    }
    if e2e_ms is not None:
        h2d, d2h = vol.raw_bytes(), int(bits.numel()) * 2
        line["e2e_link"] = dict(link, h2d_floor_ms=h2d / (link["h2d_gbs"] * 1e6),
                                note="pinned-memory copy bandwidth measured on this box just before the e2e run; "
                                     "the volume's raw upload alone needs h2d_floor_ms")
    if e2e_ms is not None:
        line["e2e"] = {"value": ascans / (e2e_ms * 1e-3), "unit": "A-scans/s", "ms_per_step": e2e_ms,
                       "h2d_bytes_per_step": vol.raw_bytes(), "d2h_bytes_per_step": int(bits.numel()) * 2}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_config1(vol, torch, budget_s=args.cpu_budget)
        first = {k: vol.raw[(0,) + k][:1].cpu().numpy().view(np.uint16) for k in vol.order}
        line["cpu_numpy_path"] = numpy_path_baseline(vol, vol.tg, first, frames=1)
    if rank == 0 and not args.no_precision:
        torch.cuda.synchronize()
        line["precision_form"] = precision_leg(ctx, vol, torch, stream, args)
    if rank == 0 and not args.no_plugin:
        torch.cuda.synchronize()
        line["plugin_process_row"] = plugin_arm(vol, torch, dev)
    if rank == 0 and not args.no_plain:
        torch.cuda.synchronize()
        pf = plain_form_arm(vol, torch, dev)
        if "value" in pf:
            pf["speedup_of_value"] = value / world / pf["value"]
        line["plain_fp32_gpu_form"] = pf
    if rank == 0 and not args.no_learned:
        torch.cuda.synchronize()
        line["learned_vs_search"] = learned_leg(args, torch, stream, dev)
    return line


def precision_leg(ctx, vol, torch, stream, args, sample_bscans=2):
    """The precision form (exact integer background, tcgen05 split-FP16 sinc,
    FFT, |.|) over every tile of the resident volume, beside the float32 form
    (the same tiles through the fused kernel), and the legacy codes of both
    against the float64 oracle on a sample (B-scans 0..1 of one tile, one
    shared clim)."""
    from oracle import numerics as O
    from oct_recon_af_v1_gb300 import synthetic
    tiles = list(vol.raw.values())
    B, interf = tiles[0].shape[0], tiles[0].shape[1]
    nxa = interf - APOD
    mag = torch.empty((B, nxa, 1024), dtype=torch.float32, device="cuda")

    def run(fn):
        for t in tiles:
            fn(t, APOD, mag, raw_dtype=0)

    def timed(fn, steps=3, warm=1):
        for _ in range(warm):
            run(fn)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            run(fn)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_p = timed(ctx.magnitude_precision)
    ms_f = timed(ctx.magnitude)
    ms_x = timed(ctx.magnitude_exact, steps=1, warm=1)
    ascans = len(tiles) * B * nxa
    sample = tiles[0][:sample_bscans]
    raw = sample.cpu().numpy().view(np.uint16)
    og = O.spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    with np.errstate(divide="ignore"):
        d64 = 20 * np.log10(O.magnitude_numpy(raw, og, APOD, np.float64))
        dp = 20 * np.log10(np.asarray(ctx.magnitude_precision(sample, APOD, raw_dtype=0), np.float64))
        df = 20 * np.log10(np.asarray(ctx.magnitude(sample, APOD, raw_dtype=0), np.float64))
        dx = 20 * np.log10(np.asarray(ctx.magnitude_exact(sample, APOD, raw_dtype=0), np.float64))
    fin = np.isfinite(d64)
    clim = (float(d64[fin].min()), float(d64[fin].max()))
    rp, rf, rx = (O.lsb_levels(d, d64, clim)[-1] for d in (dp, df, dx))
    return {"value": ascans / (ms_p * 1e-3), "unit": "A-scans/s", "ms_per_volume": ms_p,
            "float32_form": {"value": ascans / (ms_f * 1e-3), "ms_per_volume": ms_f},
            "float64_form": {"value": ascans / (ms_x * 1e-3), "ms_per_volume": ms_x,
                             "note": "exact integer background, float64 sinc / window / FFT, |X| to float32"},
            "codes_vs_float64": {"precision_exact": rp["exact_frac"], "precision_max_lsb": rp["max_lsb"],
                                 "float32_exact": rf["exact_frac"], "float32_max_lsb": rf["max_lsb"],
                                 "float64_form_exact": rx["exact_frac"], "float64_form_max_lsb": rx["max_lsb"],
                                 "voxels": rp["n"], "sample": f"B-scans 0..{sample_bscans - 1} of one tile, "
                                 "all 1024 depth bins, one clim (the float64 oracle's)"},
            "work": "the volume's 12 tiles, spectral stage only (magnitudes out)"}


def learned_leg(args, torch, stream, dev):
    """The learned estimator against the plain search at a reduced, stated
    size (4 000 training images, 6 epochs, 200 held-out B-scans): both
    estimators' time per B-scan, the speed-up and the sharpness reached."""
    import copy
    from oct_recon_af_v1_gb300._lib import Context
    a = copy.copy(args)
    a.train4, a.epochs4, a.test4, a.steps, a.warmup = 4000, 6, 200, 3, 2
    ctx4 = Context(torch.cuda.current_device())
    ctx4.set_stream(stream.cuda_stream)
    try:
        r = gpu_arm_config4(a, 0, 1, torch, ctx4, stream, dev)
    finally:
        ctx4.close()
    n = r["config"]["held_out_bscans"]
    return {"learned_ms_per_bscan": r["ms_per_step"] / n, "search_ms_per_bscan": r["search"]["seconds"] * 1e3 / n,
            "speedup": r["search"]["learned_speedup"], "learned_a_scans_per_s": r["value"],
            "search_a_scans_per_s": r["search"]["value"], "accuracy": r["accuracy"],
            "training": {k: r["training"][k] for k in ("train_s", "epochs", "batch", "kernels", "loss_per_epoch")},
            "config": r["config"]["workload"]}


def config3_specs(seed=3, n_tiles=64):
    """64 tiles: A-scans U[300,1200], B-scans U[50,300], z-crop U[400,1500] px (1 um rows)."""
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(50, 301)), int(rng.integers(300, 1201)), int(rng.integers(400, 1501)))
            for _ in range(n_tiles)]


def config3_desc(specs):
    a = sum(b * nx for b, nx, _ in specs)
    return {"workload": f"config3: {len(specs)} tiles of uneven size (A-scans U[300,1200], B-scans U[50,300], "
                        "z-crop U[400,1500] px at 1 um), 2048 uint16 spectra, one persistent launch",
            "a_scans_per_step": a, "tiles": len(specs), "l2_flush": "inputs larger than L2"}


def gpu_arm_config3(args, rank, world, torch, ctx, stream, dev):
    from oct_recon_af_v1_gb300 import autotune
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    specs = config3_specs(n_tiles=args.tiles3)
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    rng = np.random.default_rng(33)
    plans, raws, nzs = [], [], []
    for k, (B, nx, crop) in enumerate(specs):
        lay = S.ScanLayout(np.array([0.0]), np.array([0.0]), np.array([0.0]), nx, B, nx * 1e-3, B * 1e-3)
        full = S.tiled_geometry(lay, sg.z_um, [np.nan], 1.0)
        n_av = len(full.out_z_mm)
        crop = min(crop, n_av)
        z0 = int(rng.integers(0, n_av - crop + 1))
        zlo, zhi = full.out_z_mm[z0], full.out_z_mm[z0 + crop - 1]
        tg = S.tiled_geometry(lay, sg.z_um, [np.nan], 1.0, (zlo - 1e-9, zhi + 1e-9))
        st = S.TileStitcher.build(tg, 0.0, 0.0, np.nan, 80.0)
        plans.append(st.upload(ctx))
        nzs.append(len(tg.out_z_mm))
        raws.append(synthetic.u16_bits(synthetic.generate(B, nx, APOD, seed=3000 + k, device=dev, chunk=30)))
    sizes = [b * nx * nz for (b, nx, _), nz in zip(specs, nzs)]
    db_all = torch.empty(sum(sizes), dtype=torch.float32, device=dev)
    bits = torch.empty(sum(sizes), dtype=torch.int16, device=dev)
    tiles, off = [], 0
    for (B, nx, _), nz, sz, raw, plan in zip(specs, nzs, sizes, raws, plans):
        tiles.append((raw, APOD, plan, db_all[off:off + sz].view(B, nx, nz)))
        off += sz
    torch.cuda.synchronize()
    thr = S.min_weight_threshold(np.float32)
    grab, order, tune_ms = autotune.tune_batch(ctx, tiles, thr, stream)
    work = autotune.ordered(tiles, order)
    ascans = sum(b * nx for b, nx, _ in specs)

    def step():
        ctx.clim_reset()
        ctx.batch_process(work, thr, grab=grab)
        ctx.quantise_running(db_all, bits)

    def per_tile_step():
        ctx.clim_reset()
        for t in tiles:
            ctx.batch_process([t], thr, grab=grab)
        ctx.quantise_running(db_all, bits)

    step()
    ctx.synchronize()
    ctx.graph_begin()
    step()
    gid_queue = ctx.graph_end()
    per_tile_step()
    ctx.synchronize()
    ctx.graph_begin()
    per_tile_step()
    gid_tiles = ctx.graph_end()

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        n0 = ctx.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, ctx.launches - n0

    # the last tuning choice: the persistent queue launch or one launch per
    # tile, both captured in a graph (the same kernels and results)
    # (five interleaved rounds of 3 steps each, medians, with the SM clock
    # sampled meanwhile: the two forms differ by a few per cent)
    q_ms, t_ms = [], []
    choice_clk = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    choice_clk.start()
    for _ in range(5):
        q_ms.append(timed(lambda: ctx.graph_launch(gid_queue), 3, 1)[0])
        t_ms.append(timed(lambda: ctx.graph_launch(gid_tiles), 3, 1)[0])
    choice_clock = choice_clk.stop()
    ms_queue, ms_tiles = float(np.median(q_ms)), float(np.median(t_ms))
    form = "queue" if ms_queue <= ms_tiles else "per-tile"
    gid = gid_queue if form == "queue" else gid_tiles
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms, launches = timed(lambda: ctx.graph_launch(gid), args.steps, args.warmup)
    clk = clocks.stop()
    # e2e: raw tiles from page-locked host memory each step, codes back.  The
    # tiles go up on a copy stream in processing order and each tile is
    # reconstructed as soon as it has arrived (per-tile launches); the next
    # step's upload of a tile waits until this step has read it.  The codes
    # (which need the volume's clim) come back on a third stream, overlapping
    # the next step's uploads; the last read-back is inside the timed region.
    host = [t[0].cpu().pin_memory() for t in tiles]
    host_bits = torch.empty(bits.shape, dtype=torch.int16, pin_memory=True)
    up, d2h = torch.cuda.Stream(), torch.cuda.Stream()
    arrived = [torch.cuda.Event() for _ in tiles]
    read = [torch.cuda.Event() for _ in tiles]
    bits_free, quantised = torch.cuda.Event(), torch.cuda.Event()
    for ev in read:
        ev.record(stream)
    bits_free.record(stream)

    def e2e_step():
        for i, (h, t) in enumerate(zip(host, tiles)):
            up.wait_event(read[i])
            with torch.cuda.stream(up):
                t[0].copy_(h, non_blocking=True)
            arrived[i].record(up)
        ctx.clim_reset()
        for i, t in enumerate(tiles):
            stream.wait_event(arrived[i])
            ctx.batch_process([t], thr, grab=grab)
            read[i].record(stream)
        stream.wait_event(bits_free)                    # the previous read-back has left the codes
        ctx.quantise_running(db_all, bits)
        quantised.record(stream)
        d2h.wait_event(quantised)
        with torch.cuda.stream(d2h):
            host_bits.copy_(bits, non_blocking=True)
        bits_free.record(d2h)

    def e2e_timed(steps):
        e2e_step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            e2e_step()
        stream.wait_event(bits_free)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_e2e = e2e_timed(max(2, args.steps // 2))
    hbm, src = peaks()
    raw_bytes = sum(int(t[0].numel()) * 2 for t in tiles)
    out_bytes = int(bits.numel()) * 2
    alg = raw_bytes + out_bytes
    line = {"metric": METRIC, "value": ascans / (ms * 1e-3), "unit": "A-scans/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (uint16 in, uint16 out)",
            "data": "synthetic (seeded, generated on device)",
            "config": dict(config3_desc(specs), cuda_graph=True, grab=grab, order=order, autotune_ms=tune_ms,
                           form=form),
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": alg / (ms * 1e-3) / 1e9 / hbm, "traffic": None,
                         "kernel": "whole step (apod + persistent spectral/resample + quantise)",
                         "bytes_per_launch": alg, "peak_source": src + " (burst copy)"},
            "clocks": clk,
            "forms": {"chosen": form, "queue_ms": ms_queue, "per_tile_ms": ms_tiles,
                      "queue_ms_rounds": q_ms, "per_tile_ms_rounds": t_ms, "clocks": choice_clock,
                      "note": "both CUDA graphs: the persistent queue launch over all tiles, or one apodisation "
                              "+ one spectral launch per tile; medians of 5 interleaved rounds, the faster one "
                              "is timed"},
            "e2e": {"value": ascans / (ms_e2e * 1e-3), "unit": "A-scans/s", "ms_per_step": ms_e2e,
                    "h2d_bytes_per_step": raw_bytes, "d2h_bytes_per_step": out_bytes}}
    return line


def gpu_arm_config2(args, rank, world, torch, ctx, stream, dev):
    """Config 2: the config-1 tiles through the precision form of the spectral
    stage (tensor-core sinc, float64 background), beside the float32 form."""
    vol = Volume(ctx, torch, dev, host_copy=False, bscans=args.bscans)
    tiles = list(vol.raw.values())
    B, interf = tiles[0].shape[0], tiles[0].shape[1]
    nxa = interf - APOD
    mag = torch.empty((B, nxa, 1024), dtype=torch.float32, device=dev)
    X = torch.empty((B, nxa, 2048), dtype=torch.float32, device=dev)
    ascans = len(tiles) * B * nxa

    def prec_step():
        for t in tiles:
            ctx.magnitude_precision(t, APOD, mag, raw_dtype=0)

    def sinc_step():
        for t in tiles:
            ctx.linearise_precision(t, APOD, X, raw_dtype=0)

    def f32_step():
        for t in tiles:
            ctx.magnitude(t, APOD, mag, raw_dtype=0)

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        n0 = ctx.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, ctx.launches - n0

    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms, launches = timed(prec_step, args.steps, args.warmup)
    clk = clocks.stop()
    ms_sinc, _ = timed(sinc_step, args.steps, 1)
    ms_f32, _ = timed(f32_step, args.steps, 1)
    hbm, src = peaks()
    flops_per_ascan = 32 * 3 * 2 * 64 * 96                     # dense MMA tiles executed per A-scan
    sinc_bytes = ascans * (interf / nxa * 2048 * 2 + 2048 * 4)   # raw in, X out
    try:
        tf_peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("bf16_tflops"))
    except Exception:
        tf_peak = 1900.0
    return {"metric": METRIC, "value": ascans / (ms * 1e-3), "unit": "A-scans/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (split-fp16 tensor-core sinc, uint16 in)",
            "data": "synthetic (seeded, generated on device)",
            "config": dict(config1_desc(args.bscans),
                           workload="config2: config-1 tiles (12 x 270 B-scans x 1000 A-scans x 2048 uint16) through "
                                    "the precision form of the spectral stage (float64 background, tcgen05 "
                                    "split-FP16 sinc, FFT, |.|), magnitudes out"),
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": sinc_bytes / (ms_sinc * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": sinc_bytes / (ms_sinc * 1e-3) / 1e9 / hbm, "traffic": None,
                         "kernel": "precision stage (c): float64 background + split + tcgen05 sinc, raw in / X out",
                         "ms_per_step": ms_sinc, "peak_source": src + " (burst copy)",
                         "tensor": {"achieved_tflops": ascans * flops_per_ascan / (ms_sinc * 1e-3) / 1e12,
                                    "peak_tflops": tf_peak, "flops_per_ascan": flops_per_ascan,
                                    "note": "dense 128x64x96 MMA tiles x 3 split products; time of the whole stage"}},
            "clocks": clk,
            "float32_form": {"value": ascans / (ms_f32 * 1e-3), "unit": "A-scans/s", "ms_per_step": ms_f32}}


def config4_desc(n_train, n_base, epochs, n_test=500):
    return {"workload": f"config4: learned beta/focus vs plain search; {n_train} training images from {n_base} "
                        f"dispersion-free B-scans x 10 synthetic dispersions (phase trick), {n_test} held-out B-scans "
                        "x 500 A-scans x 2048 uint16 with beta_px ~ U[-5e-5, 5e-5] in the spectra and a confocal "
                        "focus ~ U[100, 900] px (reflector amplitude x exp(-((d - f)/150)^2)); 3 probe "
                        "reconstructions -> 256x256 dB images -> CNN",
            "ascans_per_bscan": 500, "training_images": n_train, "epochs": epochs,
            "search": "per-B-scan: 41-point grid over +-1.2 x 7.5e7 nm^2/rad (one launch) + batched zoom "
                      "refinement (9 candidates per launch, to 2e-5 of the largest |bound|), top_percentile; "
                      "focus: x-mean profile rules",
            "l2_flush": "held-out raw (1.05 GB) and magnitudes larger than L2"}


def gpu_arm_config4(args, rank, world, torch, ctx, stream, dev):
    from oct_recon_af_v1_gb300 import estimation as E
    from oct_recon_af_v1_gb300 import learned as L
    from oct_recon_af_v1_gb300 import synthetic as S
    from oct_recon_af_v1_gb300._lib import U16
    lam = S.lambda_nm()
    NX, n_test, shifts = 500, int(getattr(args, "test4", 500)), 10
    n_base = max(1, args.train4 // shifts)
    n_train = n_base * shifts
    rng = np.random.default_rng(404)
    # ---- training images: dispersion-free B-scans rendered at 10 dispersions each
    t0 = time.perf_counter()
    mk = L.ImageMaker(lam, APOD)
    X = torch.empty((n_train, 3, L.IMG, L.IMG), dtype=torch.float32, device=dev)
    Y = np.empty((n_train, 2), np.float32)
    focus_base = rng.uniform(100, 900, n_base)
    k, chunk = 0, 50
    for c0 in range(0, n_base, chunk):
        nb = min(chunk, n_base - c0)
        raw = S.u16_bits(S.generate(nb, NX, APOD, seed=10_000 + c0, device=dev, beta_px=0.0,
                                    focus_px=focus_base[c0:c0 + nb], chunk=nb, precision="float32"))
        mk.load(raw, raw_dtype=U16)
        for _ in range(shifts):
            bc = -S.beta_ref_from_px(rng.uniform(-5e-5, 5e-5))
            mk.render(bc, out=X[k:k + nb])
            Y[k:k + nb] = L.targets(np.full(nb, bc), focus_base[c0:c0 + nb])
            k += nb
        del raw
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    # ---- training (hand-written kernels; torch only holds tensors and shuffles)
    from oct_recon_af_v1_gb300._lib import Context
    net_ctx = Context(torch.cuda.current_device())
    net_ctx.set_stream(stream.cuda_stream)
    train_tc = not getattr(args, "train_fp32", False)
    net = L.BetaFocusNet(net_ctx, seed=0, train_tensor_cores=train_tc)
    Yd = torch.tensor(Y, device=dev)
    bs, epochs = 128, args.epochs4
    steps_per_epoch = n_train // bs
    total = epochs * steps_per_epoch
    losses = []
    t0 = time.perf_counter()
    it = 0
    for ep in range(epochs):
        perm = torch.randperm(n_train, device=dev)
        for i in range(steps_per_epoch):
            idx = perm[i * bs:(i + 1) * bs]
            lr = 1e-5 + 0.5 * (2e-3 - 1e-5) * (1 + np.cos(np.pi * it / total))
            loss = net.train_step(X.index_select(0, idx), Yd.index_select(0, idx), float(lr))
            it += 1
        losses.append(float(loss.item()))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del X, Yd
    # ---- held-out B-scans with the dispersion in their spectra
    beta_px_t = rng.uniform(-5e-5, 5e-5, n_test)
    focus_t = rng.uniform(100, 900, n_test)
    truth_beta = -np.asarray(beta_px_t) / S.dk_per_px() ** 2
    raw_t = S.u16_bits(S.generate(n_test, NX, APOD, seed=777, device=dev, beta_px=beta_px_t, focus_px=focus_t,
                                  chunk=50, precision="float32"))
    img_buf = torch.empty((n_test, 3, L.IMG, L.IMG), dtype=torch.float32, device=dev)
    pred_host = torch.empty((n_test, 2), dtype=torch.float32, pin_memory=True)

    def learned_step(src):
        imgs = mk.images(src, out=img_buf, raw_dtype=U16)
        pred = net.predict(imgs)
        pred_host.copy_(pred, non_blocking=True)

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        n0 = mk.ctx.launches + net_ctx.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, mk.ctx.launches + net_ctx.launches - n0

    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ms_learned, launches = timed(lambda: learned_step(raw_t), args.steps, args.warmup)
    clk = clocks.stop()
    beta_l, focus_l = L.decode(pred_host.numpy())
    host_raw = raw_t.cpu().pin_memory()
    dev_raw = torch.empty_like(raw_t)
    # end to end: the step's raw B-scans go up in 5 chunks on a copy stream and
    # the probe images of a chunk are made as soon as it has arrived (uploads
    # overlap image making); the CNN then runs on all of them and the
    # predictions come back.  The next step's uploads wait until this step's
    # image making has finished reading the buffer.
    up = torch.cuda.Stream()
    n_chunks = 5
    bounds = [n_test * c // n_chunks for c in range(n_chunks + 1)]
    arrived = [torch.cuda.Event() for _ in range(n_chunks)]
    raw_free = torch.cuda.Event()
    raw_free.record(stream)

    def e2e_step():
        up.wait_event(raw_free)
        with torch.cuda.stream(up):
            for c in range(n_chunks):
                sl = slice(bounds[c], bounds[c + 1])
                dev_raw[sl].copy_(host_raw[sl], non_blocking=True)
                arrived[c].record(up)
        for c in range(n_chunks):
            sl = slice(bounds[c], bounds[c + 1])
            stream.wait_event(arrived[c])
            mk.images(dev_raw[sl], out=img_buf[sl], raw_dtype=U16)
        raw_free.record(stream)
        pred = net.predict(img_buf)
        pred_host.copy_(pred, non_blocking=True)

    ms_e2e, _ = timed(e2e_step, args.steps, 1)
    # ---- the plain search on the same B-scans (GPU scorer + host Brent + focus rules)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sc = E.DispersionScorer(lam, raw_t, "top_percentile", APOD, rep=1, raw_dtype=U16)
    lo, hi = -1.2 * L.beta_scale(), 1.2 * L.beta_scale()
    beta_s, grid, Sg = L.search_per_bscan(sc, lo, hi, 41)
    mag0 = torch.empty((1, n_test, NX, 1024), dtype=torch.float32, device=dev)
    sc.ctx.disp_eval([0.0], 0, n_test, 0, mag=mag0)
    focus_s = L.focus_plain(sc.ctx, mag0[0])
    torch.cuda.synchronize()
    t_search = time.perf_counter() - t0
    n_evals = sc.n_evals
    # ---- sharpness at the chosen betas (not timed)
    s_l = np.array([sc.scores(beta_l[j], j)[0] for j in range(n_test)])
    s_s = np.array([sc.scores(beta_s[j], j)[0] for j in range(n_test)])
    s_t = np.array([sc.scores(truth_beta[j], j)[0] for j in range(n_test)])
    rng_j = Sg.max(0) - Sg.min(0)
    gap = (s_s - s_l) / rng_j
    sc.close()
    ascans = n_test * NX
    v_l = ascans / (ms_learned * 1e-3)
    v_s = ascans / t_search
    hbm, src = peaks()
    raw_bytes = int(raw_t.numel()) * 2
    return {"metric": METRIC, "value": v_l, "unit": "A-scans/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_learned, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (uint16 in)", "data": "synthetic (seeded, generated on device)",
            "config": dict(config4_desc(n_train, n_base, epochs, n_test), held_out_bscans=n_test),
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": raw_bytes / (ms_learned * 1e-3) / 1e9, "peak": hbm,
                         "unit": "GB/s", "frac": raw_bytes / (ms_learned * 1e-3) / 1e9 / hbm, "traffic": None,
                         "kernel": "whole learned step (linearise, 3 probe FFT passes, pooling, CNN forward on the tensor cores)",
                         "bytes_per_launch": raw_bytes, "peak_source": src + " (burst copy)"},
            "clocks": clk,
            "search": {"value": v_s, "unit": "A-scans/s", "seconds": t_search, "evaluations": n_evals,
                       "learned_speedup": v_l / v_s},
            "accuracy": {"beta_rmse_learned": float(np.sqrt(np.mean((beta_l - truth_beta) ** 2))),
                         "beta_rmse_search": float(np.sqrt(np.mean((beta_s - truth_beta) ** 2))),
                         "beta_unit": "nm^2/rad (training range +-7.49e7)",
                         "sharpness_gap_mean": float(np.mean(gap)),
                         "sharpness_gap_p95": float(np.quantile(gap, 0.95)),
                         "sharpness_gap_unit": "(S(search) - S(learned)) / (max - min of the B-scan's grid curve)",
                         "sharpness_truth_minus_search_mean": float(np.mean((s_t - s_s) / rng_j)),
                         # the score is log(mean of the top 1 % of |A|^2): exp of the score difference is
                         # the ratio of the top-1 % mean intensities at the predicted and searched betas
                         "sharpness_gap_relative_mean": float(np.mean((s_s - s_l) / np.abs(s_s))),
                         "top1pct_intensity_ratio_mean": float(np.mean(np.exp(s_l - s_s))),
                         "top1pct_intensity_ratio_p05": float(np.quantile(np.exp(s_l - s_s), 0.05)),
                         "fraction_within_1pct_intensity": float(np.mean(np.exp(s_l - s_s) >= 0.99)),
                         "focus_mae_learned_px": float(np.mean(np.abs(focus_l - focus_t))),
                         "focus_mae_plain_px": float(np.mean(np.abs(focus_s - focus_t)))},
            "training": {"images_s": t_data, "train_s": t_train, "epochs": epochs, "batch": bs,
                         "loss_per_epoch": losses,
                         "kernels": "tensor cores (FP16 forward, BF16 weight and data gradients, float32 "
                                    "accumulation)" if train_tc else "float32 SIMT"},
            "e2e": {"value": ascans / (ms_e2e * 1e-3), "unit": "A-scans/s", "ms_per_step": ms_e2e,
                    "h2d_bytes_per_step": raw_bytes, "d2h_bytes_per_step": n_test * 2 * 4}}


def gpu_arm_config0(args, rank, world, torch, ctx):
    from oct_recon_af_v1_gb300 import geometry as G
    from oct_recon_af_v1_gb300 import synthetic
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    ctx.set_geometry(sg.sinc_idx, sg.sinc_w, sg.window)
    copies = [synthetic.u16_bits(synthetic.generate(50, 500, APOD, seed=k, device="cuda", chunk=50)) for k in range(8)]
    db = torch.empty((50, 500, 1000), dtype=torch.float32, device="cuda")
    bits = torch.empty((50, 500, 1000), dtype=torch.int16, device="cuda")

    def step(i):
        _, clim = ctx.db(copies[i % len(copies)], APOD, 0, 1000, db, raw_dtype=0)
        ctx.quantise(db, clim, bits)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    n0 = ctx.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks()
    clocks.start()
    e0.record()
    for i in range(args.steps):
        step(i)
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    hbm, src = peaks()
    per = 2048 * 2 * (525 / 500) + 1000 * 4 + 1000 * 4 + 1000 * 2
    return {"metric": METRIC, "value": 25000 / (ms * 1e-3), "unit": "A-scans/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (uint16 in, uint16 out)",
            "data": "synthetic (seeded)", "config": config0_desc(), "gpu_launches": ctx.launches - n0,
            "roofline": {"bound": "hbm", "achieved": 25000 * per / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": 25000 * per / (ms * 1e-3) / 1e9 / hbm, "traffic": None,
                         "peak_source": src}, "clocks": clk}


def _import_reference_octrecon():
    """The reference package from baseline/_ref (offline install), or None."""
    import types
    ref = ROOT / "baseline" / "_ref"
    if not (ref / "octrecon" / "core" / "torch_backend.py").exists():
        return None
    if str(ref) not in sys.path:
        sys.path.insert(0, str(ref))
    try:
        import tifffile  # noqa: F401
    except ImportError:
        sys.modules.setdefault("tifffile", types.ModuleType("tifffile"))
    import octrecon.core.torch_backend  # noqa: F401
    return sys.modules["octrecon"]


def write_scan_folder(root: Path, vol, beta_ref: float):
    """The tiled workload as an on-disk scan the reference's Reconstructor
    opens: ScanInfo.json and, per tile, Header.xml (Thorlabs OCITY: 25
    apodisation + 1000 scan lines of 2048 int16 samples, 270 B-scans) and
    data/Chirp.data (the spectrometer's chirp: with the gan632 wavelength
    range, chirp_j = q_j maps to the synthetic spectrometer's wavelengths).
    The spectra themselves are served from memory (`_MemTileReader`)."""
    from oct_recon_af_v1_gb300 import synthetic
    lay = vol.lay
    folders, gx, gy, gz = [], [], [], []
    for yi, yc in enumerate(lay.y_centers_mm):
        for xi, xc in enumerate(lay.x_centers_mm):
            for zi, zd in enumerate(lay.z_depths_mm):
                folders.append(f"Data{len(folders) + 1:02d}")
                gx.append(float(xc)), gy.append(float(yc)), gz.append(float(zd))
    info = {"octSystem": "gan632", "tissueRefractiveIndex": 1.33, "pixelSize_um": 1.0, "units": "mm",
            "zDepths": [float(z) for z in lay.z_depths_mm], "xCenters_mm": [float(x) for x in lay.x_centers_mm],
            "yCenters_mm": [float(y) for y in lay.y_centers_mm], "nXPixelsInEachTile": lay.n_x_px,
            "nYPixelsInEachTile": lay.n_y_px, "tileRangeX_mm": lay.tile_range_x_mm,
            "tileRangeY_mm": lay.tile_range_y_mm, "xOffset": 0, "yOffset": 0, "nBScanAvg": 1,
            "galvoPhaseDelayXOffsetCorrection_mm": 0.0, "gridXcc": gx, "gridYcc": gy, "gridZcc": gz,
            "scanOrder": list(range(1, len(folders) + 1)), "octFolders": folders,
            "octProbe": {"DefaultDispersionQuadraticTerm": beta_ref,
                         "OpticalPathCorrectionPolynomial": [0.0, 0.0, 0.0, 0.0, 0.0]}}
    root.mkdir(parents=True, exist_ok=True)
    (root / "ScanInfo.json").write_text(json.dumps(info, indent=1))
    n, interf = 2048, APOD + lay.n_x_px
    header = f"""<?xml version='1.0' encoding='utf-8'?>
<Ocity version="1.0"><DataFiles>
<DataFile Type="Raw" SizeZ="{n}" SizeX="{interf}" BytesPerPixel="2" ApoRegionStart0="0" ApoRegionEnd0="{APOD}" ScanRegionStart0="{APOD}" ScanRegionEnd0="{interf}" SizeY="{lay.n_y_px}">data\\Spectral0.data</DataFile>
<DataFile Type="Real" SizeZ="{n}" BytesPerPixel="4">data\\Chirp.data</DataFile></DataFiles>
<Image Type="RawSpectra"><SizePixel Unit="px"><SizeZ>{n // 2}</SizeZ><SizeX>{lay.n_x_px}</SizeX><SizeY>{lay.n_y_px}</SizeY></SizePixel>
<SizeReal Unit="mm"><SizeZ>1.0</SizeZ><SizeX>{lay.tile_range_x_mm}</SizeX><SizeY>{lay.tile_range_y_mm}</SizeY></SizeReal></Image>
<Acquisition><IntensityAveraging><Spectra>1</Spectra><AScans>1</AScans><BScans>1</BScans></IntensityAveraging>
<SpeckleAveraging><FastAxis>1</FastAxis><SlowAxis>1</SlowAxis></SpeckleAveraging></Acquisition>
<Instrument><Model>GAN632</Model><Series>Ganymede</Series><SpectrometerElements>{n}</SpectrometerElements></Instrument>
</Ocity>"""
    chirp = synthetic.raw_position(synthetic.SpectrumParams()).astype("<f4").tobytes()
    for f in folders:
        (root / f / "data").mkdir(parents=True, exist_ok=True)
        (root / f / "Header.xml").write_text(header)
        (root / f / "data" / "Chirp.data").write_bytes(chirp)
    return folders


def plugin_arm(vol, torch, dev, batch=30, io_threads=16):
    """The drop-in path: the reference's own Reconstructor on device "gb300"
    (octrecon/pipeline.py:95-302 with the plug-in registered), process_row of
    both y-rows of the tiled workload, float32 dB planes back on the host.
    The scan folder is written by `write_scan_folder`; its B-scans are served
    from host memory by a reader whose read_bscans copies them into the
    plug-in's pinned slots (as a read from the page cache would), so the
    timed region holds that copy, the H2D copies, the kernels and the D2H of
    the float32 planes (2 x 270 x nOutZ x nOutX)."""
    import tempfile
    if _import_reference_octrecon() is None:
        return {"unavailable": "octrecon not installed in baseline/_ref"}
    if not vol.host:
        return {"unavailable": "needs the pinned host copy of the volume (run without --no-e2e)"}
    from octrecon.io.volume import TileReader
    from octrecon.pipeline import ReconConfig, Reconstructor

    from oct_recon_af_v1_gb300 import plugin, synthetic
    plugin.register(torch.cuda.current_device())

    class _MemTileReader(TileReader):
        """TileReader whose raw B-scans live in host memory."""

        def __init__(self, tile_dir, data):
            super().__init__(tile_dir)
            self.data = data

        def read_bscans(self, file_indices, out):
            for k, fi in enumerate(file_indices):
                np.copyto(out[k], self.data[int(fi)])
            return out

    beta = synthetic.beta_ref_from_px(1e-5)
    root = Path(tempfile.mkdtemp(prefix="octgb_scan_"))
    folders = write_scan_folder(root, vol, beta)
    cfg = ReconConfig(volume_folder=str(root), device="gb300", precision="float32", dispersion_quadratic_term=beta,
                      focus_positions=[float(f) for f in vol.focus], focus_sigma=80, crop_z_range_mm="none",
                      output_pixel_size_um=1.0, n_medium=1.33, apply_path_length_correction=False,
                      batch_frames=batch, io_threads=io_threads, write_tiff=False)
    R = Reconstructor(cfg, log=lambda *a: None)
    keys = [(yi, xi, zi) for yi in range(2) for xi in range(2) for zi in range(3)]
    for f, k in zip(folders, keys):
        R._readers[f] = _MemTileReader(root / f, vol.host[k].numpy())
    for yi in range(2):                                         # warm-up: rings, plans, pinned results
        R.process_row(yi)
    torch.cuda.synchronize()
    for key in R.timers:
        R.timers[key] = 0.0
    t0 = time.perf_counter()
    rows = [R.process_row(yi) for yi in range(2)]
    dt = time.perf_counter() - t0
    n_out = sum(int(r.size) for r in rows)
    del rows
    ascans = 12 * vol.ny * vol.lay.n_x_px
    # host memory traffic of the drop-in path per volume: the reader's copy into
    # the pinned slots (read + write), the DMA reads of those slots and the DMA
    # writes of the float32 planes
    host_bytes = 3 * vol.raw_bytes() + 4 * n_out
    return {"value": ascans / dt, "unit": "A-scans/s", "ms_per_volume": dt * 1e3,
            "h2d_bytes_per_volume": vol.raw_bytes(), "d2h_bytes_per_volume": 4 * n_out,
            "host_memory_bytes_per_volume": host_bytes,
            "timers_ms": {k: round(v * 1e3, 2) for k, v in R.timers.items()},
            "batch_frames": batch, "io_threads": io_threads,
            "source": "octrecon Reconstructor.process_row on device gb300 (reference pipeline, plug-in "
                      "registered), both y-rows; reader serves the B-scans from host memory; float32 dB out"}


def plain_form_arm(vol, torch, dev, batch=50):
    """The reference's own float32 GPU path, unmodified: octrecon's torch backend
    (TorchSpectralProcessor: gathers + torch.fft, TorchTileStitcher: gather +
    matmuls, core/torch_backend.py:66-165) on this GPU, driven as
    Reconstructor.process_row does (pipeline.py:223-300) over y-row 0 of the same
    volume (6 tiles x 270 frames).  Reported as the plain-FP32 GPU form."""
    if _import_reference_octrecon() is None:
        return {"unavailable": "octrecon not installed in baseline/_ref"}
    from octrecon.core.geometry import build_spectral_geometry
    from octrecon.core.stitching import TileStitcher, min_weight_threshold
    from octrecon.core.torch_backend import TorchSpectralProcessor, TorchTileStitcher, TorchXP

    from oct_recon_af_v1_gb300 import synthetic
    xp = TorchXP(dev)
    sg = build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33, "sinc5")
    sp = TorchSpectralProcessor(sg, APOD, xp)
    sts = {(xi, zi): TorchTileStitcher(TileStitcher(vol.tg, None, vol.lay.x_centers_mm[xi], vol.lay.z_depths_mm[zi],
                                                    vol.focus[zi], 80.0, xp=np, dtype=np.float32), None, xp)
           for xi, zi in vol.order}
    thr = min_weight_threshold(np.float32)

    def row(frames_total):
        num = torch.zeros((frames_total, vol.nz, vol.nx), dtype=torch.float32, device=dev)
        den = torch.zeros_like(num)
        for xi, zi in vol.order:
            st = sts[(xi, zi)]
            for s0 in range(0, frames_total, batch):
                raw16 = vol.raw[(0, xi, zi)][s0:s0 + batch]
                raw = raw16.to(torch.int32) & 0xFFFF          # the uint16 counts
                fr = torch.arange(s0, s0 + raw.shape[0], device=dev)
                mag = sp.magnitude(raw)
                n_, d_ = st.contribute(mag, fr)
                num[s0:s0 + raw.shape[0], :, st.c0:st.c1] += n_
                den[s0:s0 + raw.shape[0], :, st.c0:st.c1] += d_
        den[den < thr] = float("nan")
        return 20 * torch.log10(num / den)

    row(batch)                                  # warm-up (cuFFT plans, allocator)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    db = row(vol.ny)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    del db
    ascans = 6 * vol.ny * vol.lay.n_x_px
    return {"value": ascans / (ms * 1e-3), "unit": "A-scans/s", "ms": ms, "a_scans": ascans,
            "source": "reference octrecon torch backend (unmodified) on this GPU, y-row 0 of the volume, "
                      f"batch_frames {batch}; process_row's work (no quantisation)"}


def reduce_max(x, world):
    if world <= 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------ CPU (oracle) arm
def _cpu_sample(raw_tiles, vol, frames, g, sts):
    """Oracle reconstruction of `frames` of one y-row: returns the number of A-scans done."""
    from oracle import numerics as O
    nF = len(frames)
    num = np.zeros((nF, vol.nz, vol.nx), np.float32)
    den = np.zeros((nF, vol.nz, vol.nx), np.float32)
    n = 0
    for key, raw in raw_tiles.items():
        s = sts[key]
        mag = O.magnitude_numba(raw, g, APOD)
        n_, d_ = s.contribute(mag)
        num[:, :, s.c0:s.c1] += n_
        den[:, :, s.c0:s.c1] += d_
        n += raw.shape[0] * (raw.shape[1] - APOD)
    db = O.finalise(num, den, np.float32)
    fin = db[np.isfinite(db)]
    O.db_to_bits(db, (float(fin.min()), float(fin.max())))
    return n


def _oracle_setup(vol):
    from oracle import numerics as O
    from oct_recon_af_v1_gb300 import synthetic
    g = O.spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    sd = O.ScanDesc(vol.lay.x_centers_mm, vol.lay.y_centers_mm, vol.lay.z_depths_mm, vol.lay.n_x_px,
                    vol.lay.n_y_px, vol.lay.tile_range_x_mm, vol.lay.tile_range_y_mm)
    tg = O.tiled_geometry(sd, g.z_um, vol.focus, 1.0)
    sts = {(xi, zi): O.Stitcher(tg, vol.lay.x_centers_mm[xi], vol.lay.z_depths_mm[zi], vol.focus[zi], 80.0)
           for xi, zi in vol.order}
    return g, sts


def cpu_baseline_config1(vol, torch, budget_s=15.0, frames_max=64):
    """Time the oracle (reference algorithm restated) on a bounded sample of the
    workload: the first F frames of all 6 tiles of y-row 0, F grown until the
    run takes ~budget_s."""
    from oracle import numerics as O
    O.build()
    g, sts = _oracle_setup(vol)
    F = 1
    while True:
        tiles = {(xi, zi): vol.raw[(0, xi, zi)][:F].cpu().numpy().view(np.uint16) for xi, zi in vol.order}
        t0 = time.perf_counter()
        n = _cpu_sample(tiles, vol, np.arange(F), g, {k: sts[k] for k in vol.order})
        dt = time.perf_counter() - t0
        if dt >= budget_s / 3 or F >= frames_max:
            break
        F = min(frames_max, max(F + 1, int(F * budget_s / 3 / max(dt, 1e-3))))
    return {"value": n / dt, "unit": "A-scans/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"y-row 0, frames 0..{F - 1} of all 6 tiles ({n} A-scans): oracle Numba-kernel "
                      f"restatement (C/OpenMP) + pocketfft + NumPy stitch/finalise/quantise, {dt:.1f} s"}


def reference_arm(args, rank, world):
    """The reference algorithm (CPU restatement) timed on the host cores."""
    if rank != 0:
        return None
    import torch
    from oracle import numerics as O
    from oct_recon_af_v1_gb300 import geometry as G  # noqa: F401
    from oct_recon_af_v1_gb300 import stitching as S
    from oct_recon_af_v1_gb300 import synthetic
    O.build()
    lay, focus = config1_layout()

    class V:  # host-only description of the config-1 volume
        pass
    vol = V()
    vol.lay, vol.focus = lay, focus
    vol.order = [(xi, zi) for xi in range(2) for zi in range(3)]
    sg = G.build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33)
    tg = S.tiled_geometry(lay, sg.z_um, focus, 1.0)
    vol.nz, vol.nx = len(tg.out_z_mm), len(tg.out_x_mm)
    g, sts = _oracle_setup(vol)
    F = max(1, int(args.ref_frames))
    tiles = {(xi, zi): synthetic.generate_numpy(F, lay.n_x_px, APOD, seed=1000 + 10 * xi + zi)
             for xi, zi in vol.order}
    for _ in range(args.warmup):
        _cpu_sample(tiles, vol, np.arange(F), g, sts)
    t0 = time.perf_counter()
    n = 0
    for _ in range(args.steps):
        n += _cpu_sample(tiles, vol, np.arange(F), g, sts)
    dt = time.perf_counter() - t0
    v = n / dt
    per_step = n // args.steps
    sample = f"each step: frames 0..{F - 1} of the 6 tiles of y-row 0 ({per_step} A-scans)"
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "A-scans/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (Numba types)",
            "data": "synthetic (seeded)", "config": config1_desc(),
            "execution": {"parallelism": f"host cores ({os.cpu_count()} threads)", "a_scans_per_step": per_step,
                          "sample": sample},
            "cpu_baseline": {"value": v, "unit": "A-scans/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": sample},
            "numpy_path": numpy_path_baseline(vol, tg, tiles, frames=1),
            "e2e": {"value": v, "unit": "A-scans/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def numpy_path_baseline(vol, tg, tiles, frames=1):
    """The reference's own NumPy path (SpectralProcessor with use_numba=False,
    float32; TileStitcher.contribute; the row finalise of pipeline.py:296-300),
    unmodified, on the first `frames` frames of the 6 tiles of y-row 0."""
    if _import_reference_octrecon() is None:
        return {"unavailable": "octrecon is not installed in baseline/_ref"}
    from octrecon.core.geometry import build_spectral_geometry
    from octrecon.core.spectral import SpectralProcessor
    from octrecon.core.stitching import TileStitcher, min_weight_threshold

    from oct_recon_af_v1_gb300 import synthetic
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    sg = build_spectral_geometry(synthetic.lambda_nm(), synthetic.beta_ref_from_px(1e-5), 1.33, "sinc5")
    sp = SpectralProcessor(sg, APOD, xp=np, dtype=np.float32, use_numba=False)
    sts = {k: TileStitcher(tg, None, vol.lay.x_centers_mm[k[0]], vol.lay.z_depths_mm[k[1]], vol.focus[k[1]], 80.0,
                           xp=np, dtype=np.float32) for k in vol.order}

    def row():
        num = np.zeros((frames, vol.nz, vol.nx), np.float32)
        den = np.zeros_like(num)
        fr = np.arange(frames)
        for k in vol.order:
            n_, d_ = sts[k].contribute(sp.magnitude(tiles[k][:frames]), fr)
            num[:, :, sts[k].c0:sts[k].c1] += n_
            den[:, :, sts[k].c0:sts[k].c1] += d_
        den[den < min_weight_threshold(np.float32)] = np.nan
        with np.errstate(divide="ignore", invalid="ignore"):
            return 20 * np.log10(num / den)

    row()
    t0 = time.perf_counter()
    row()
    dt = time.perf_counter() - t0
    n = 6 * frames * vol.lay.n_x_px
    return {"value": n / dt, "unit": "A-scans/s", "cores": os.cpu_count(), "kind": "reference",
            "sample": f"frames 0..{frames - 1} of the 6 tiles of y-row 0 ({n} A-scans): the reference's NumPy "
                      "path (use_numba=False, float32), its TileStitcher and row finalise"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=1, choices=[0, 1, 2, 3, 4])
    ap.add_argument("--train4", type=int, default=20000, help="training images of the learned estimator (config 4)")
    ap.add_argument("--epochs4", type=int, default=8, help="training epochs (config 4)")
    ap.add_argument("--stitch-rows", type=int, default=0, choices=[0, 32, 64, 128],
                    help="fix the stitch kernel's rows per block instead of autotuning them (config 1)")
    ap.add_argument("--train-fp32", action="store_true",
                    help="train the learned estimator with the float32 SIMT kernels instead of the tensor cores")
    ap.add_argument("--tiles3", type=int, default=64, help="tiles of the batched workload (config 3)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the reference's plain float32 GPU path")
    ap.add_argument("--no-plugin", action="store_true", help="skip timing the reference's process_row on gb300")
    ap.add_argument("--no-precision", action="store_true", help="skip the precision-form leg of the default line")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-search leg of the default line")
    ap.add_argument("--test4", type=int, default=500, help="held-out B-scans of the learned estimator (config 4)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--ref-frames", type=int, default=4)
    ap.add_argument("--batch", type=int, default=54,
                    help="frames per frame-API call (config 1: 54 of the 270 B-scans; 9, 27, 54, 90 measured)")
    ap.add_argument("--bscans", type=int, default=270, help="B-scans per tile (270 = the full workload)")
    ap.add_argument("--no-graph", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    if args.impl == "reference":
        line = reference_arm(args, rank, world)
    else:
        line = gpu_arm(args, rank, world)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
