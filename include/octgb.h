/*
 * octgb — GB300-native (sm_103a) per-plane OCT reconstruction, C ABI.
 *
 * Drop-in boundary for the reference octrecon (atesfet/oct_recon_AF_v1) hot
 * path.  Every entry point returns an int status (OCTGB_OK = 0); no exception
 * crosses the ABI and nothing calls exit().  On failure the context keeps a
 * message readable through octgb_last_error().  A context owns one CUDA stream
 * (or uses the caller's, octgb_set_stream) and its device buffers; callers own
 * every host buffer and every device buffer they pass in.  Pointer arguments
 * come with a location flag: OCTGB_HOST (pageable or pinned host memory; the
 * library copies through its own device buffers) or OCTGB_DEVICE (used in
 * place, e.g. a torch CUDA tensor's data pointer).
 *
 * Threading: one context is driven by one host thread at a time (the reference
 * drives its backend from the main thread or a web Job thread,
 * octrecon/webapp/server.py:190-191); contexts are independent.  Not
 * re-entrant on one context.
 */
#ifndef OCTGB_H
#define OCTGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define OCTGB_OK 0
#define OCTGB_ERR_ARG 1        /* invalid argument (shape, dtype, pointer, range) */
#define OCTGB_ERR_CUDA 2       /* a CUDA runtime call failed */
#define OCTGB_ERR_STATE 3      /* call out of order (e.g. no geometry set) */
#define OCTGB_ERR_CANCELLED 4  /* octgb_cancel() was called; work was skipped */
#define OCTGB_ERR_TIMEOUT 5    /* a bounded device-side wait expired */
#define OCTGB_ERR_NOMEM 6      /* device or host allocation failed */

/* raw spectrum element types (the reference's SUPPORTED_RAW_DTYPES,
 * octrecon/core/gpu_kernels.py:39-41) */
#define OCTGB_U16 0
#define OCTGB_I16 1
#define OCTGB_F32 2

/* pointer locations */
#define OCTGB_HOST 0
#define OCTGB_DEVICE 1

typedef struct octgb_ctx octgb_ctx;

/* ---------------------------------------------------------------- context */

/* Create a context on CUDA device `device` (replaces the device selection of
 * octrecon/backend.py:61-83 get_xp for the "gb300" device). */
int octgb_create(int device, octgb_ctx **out);
int octgb_destroy(octgb_ctx *ctx);
/* Last error message of this context ("" if none).  Valid until the next call
 * on the context.  Accepts NULL (returns the message of the last failed
 * octgb_create). */
const char *octgb_last_error(const octgb_ctx *ctx);
/* Launch on `cuda_stream` (a cudaStream_t) instead of the context's own stream;
 * NULL restores the context stream.  The context's own stream is a blocking
 * stream: its work is ordered with the legacy default stream (work a caller
 * queues there before a call is done before the call's kernels run, and vice
 * versa).  Capture graphs on a caller's non-default stream. */
int octgb_set_stream(octgb_ctx *ctx, void *cuda_stream);
int octgb_synchronize(octgb_ctx *ctx);
/* Cancellation (the reference's threading.Event, octrecon/pipeline.py:45-46,
 * 262-263): every later batch call returns OCTGB_ERR_CANCELLED without work
 * until octgb_reset_cancel().  Safe to call from another host thread. */
int octgb_cancel(octgb_ctx *ctx);
int octgb_reset_cancel(octgb_ctx *ctx);
/* Number of kernels this context has launched (instrumentation). */
int64_t octgb_launch_count(const octgb_ctx *ctx);

/* ---------------------------------------------------------------- spectral */

/* Upload the spectral geometry (SpectralProcessor.__init__,
 * octrecon/core/spectral.py:91-110; built by geometry.py:84-128).
 *   sinc_idx (n, taps) int64 row-major: source indices of output i, each row a
 *            contiguous increasing run padded with index 0 / weight 0;
 *   sinc_w   (n, taps) float64: weights (rounded to float32 on upload, as
 *            `sg.sinc_w.astype(float32)` does);
 *   window   (n, 2) float64 re/im: Hann/rms * exp(i*phase) (rounded to
 *            complex64).
 * n must be 2048 (the kernels' FFT length); taps <= 32.
 * Refused (OCTGB_ERR_STATE) while a graph is being captured or while the
 * context holds captured graphs: a graph replays the geometry buffers it was
 * captured with, and a new geometry may reallocate them.  Release the graphs
 * first (octgb_graphs_release). */
int octgb_set_geometry(octgb_ctx *ctx, int n, int taps, const int64_t *sinc_idx, const double *sinc_w,
                       const double *window);

/* Fused pre-FFT stage only: apodisation mean, line mean, sinc
 * k-linearisation, window — the operator of octrecon/core/gpu_kernels.py:54-68
 * and core/cpu_kernels.py:12-41.  raw (B, interf, n) -> spec (B, interf-apod,
 * n) complex64 as interleaved float pairs. */
int octgb_fused_pre_fft(octgb_ctx *ctx, const void *raw, int raw_dtype, int raw_loc, int B, int interf,
                        int apod_size, float *spec, int spec_loc);

/* SpectralProcessor.magnitude (octrecon/core/spectral.py:136-153): raw (B,
 * interf, n) -> |ifft(spec)|[..., :n/2] float32 (B, interf-apod, n/2). */
int octgb_magnitude(octgb_ctx *ctx, const void *raw, int raw_dtype, int raw_loc, int B, int interf,
                    int apod_size, float *mag, int mag_loc);

/* Spectral stage to log-magnitude with a depth crop: db[a, z] =
 * 20*log10(|X[z0 + z]|) for z < nz (float32, (B, interf-apod, nz)), the
 * per-voxel value the reference writes after magnitude + crop + log.  When
 * minmax is non-NULL it receives [min, max] of the finite values (host
 * doubles), the plane clim of octrecon/io/tiff_writer.py:48-50. */
int octgb_db(octgb_ctx *ctx, const void *raw, int raw_dtype, int raw_loc, int B, int interf, int apod_size,
             int z0, int nz, float *db, int db_loc, double *minmax);

/* Float64 form of SpectralProcessor.magnitude: the reference's NumPy path at
 * precision "float64" (octrecon/core/spectral.py:91-95,123-165).  The
 * background is exact (integer apodisation sums; the line mean from the integer
 * sum of the numerators), the sinc runs in float64 over the float64 band
 * weights given to octgb_set_geometry, then the float64 window and a float64
 * inverse FFT; |X| (n/2 bins) is rounded once to float32.  raw must be uint16
 * or int16.  Several times slower than octgb_magnitude (GB300's float64 rate is
 * a small fraction of its float32 rate); its codes match the reference's
 * float64 path to within 1 LSB. */
int octgb_magnitude_exact(octgb_ctx *ctx, const void *raw, int raw_dtype, int raw_loc, int B, int interf,
                          int apod_size, float *mag, int mag_loc);

/* Precision form of the spectral stage: the sinc k-linearisation as a banded
 * GEMM on the tensor cores (tcgen05.mma, split-FP16 with three products,
 * float32 accumulation in TMEM; 128 A-scans x 64 output samples x a
 * 96-sample source window per block).  The background (apodisation mean, line
 * mean) is exact (integer sums; float64 for float32 raws): this form is
 * closer to the float64 path than the reference's float32 path, which rounds
 * the apodisation mean to float32 (core/cpu_kernels.py:20-25).  Requires
 * every 64-output block's
 * sinc band to fit in 96 source samples (OCTGB_ERR_STATE otherwise) and
 * |raw - apod - mean| < 65504 (the fp16 range).
 * octgb_linearise_precision: stage (c) only, the linearised interferogram
 *   (B, interf-apod, n) float32 without the window (SpectralProcessor.linearise,
 *   core/spectral.py:118-134);
 * octgb_magnitude_precision: the magnitude of octgb_magnitude
 *   (core/spectral.py:136-153).
 * With device input and device output neither call synchronises. */
int octgb_linearise_precision(octgb_ctx *ctx, const void *raw, int raw_dtype, int raw_loc, int B, int interf,
                              int apod_size, float *x, int x_loc);
int octgb_magnitude_precision(octgb_ctx *ctx, const void *raw, int raw_dtype, int raw_loc, int B, int interf,
                              int apod_size, float *mag, int mag_loc);

/* ---------------------------------------------------------------- quantisation */

/* Legacy quantisation db_to_bits (octrecon/io/tiff_writer.py:26-38):
 * bits = min(round_half_away((db-c1)/(c2-c1)*65534) + 1, 65535) with the
 * value clipped to [0, 65535] first, NaN -> 0; c1 < c2 (sorted by the caller
 * or here).  Evaluated in float64 as write_legacy_tiff does (:62). */
int octgb_quantise(octgb_ctx *ctx, const float *db, int64_t n, int db_loc, double c1, double c2,
                   uint16_t *bits, int bits_loc);
/* Legacy double quantisation (write_legacy_tiff with
 * legacy_double_quantization, tiff_writer.py:62-64): bits =
 * db_to_bits(bits_to_db(db_to_bits(db, pc), pc), clim), pc = [p1, p2] the
 * plane's clim, clim = [c1, c2] the volume's; float64 like the reference
 * (the second pass is an exact 65 536-entry table of the first code).  A
 * plane whose clim is not finite takes the single quantisation. */
int octgb_quantise_double(octgb_ctx *ctx, const float *db, int64_t n, int db_loc, double p1, double p2, double c1,
                          double c2, uint16_t *bits, int bits_loc);
/* PackBits (TIFF compression 32773) of a (rows, cols) uint16 image, every row
 * packed on its own from its little-endian bytes: out (host, `capacity`
 * bytes) receives the rows' packets back to back, row_sizes (host, rows
 * ints) each row's byte count, *total their sum.  A row never exceeds
 * 2 cols + ceil(2 cols / 128) bytes.  Synchronises. */
int octgb_packbits(octgb_ctx *ctx, const uint16_t *img, int img_loc, int rows, int cols, uint8_t *out,
                   int64_t capacity, int *row_sizes, int64_t *total);
/* [min, max] of the finite values of db (plane_clim, tiff_writer.py:48-50);
 * NaN pair when none is finite. */
int octgb_minmax(octgb_ctx *ctx, const float *db, int64_t n, int db_loc, double *minmax);

/* ---------------------------------------------------------------- stitching */

/* One tile position (xi, zi) of the output grid: TileStitcher.__init__
 * (octrecon/core/stitching.py:84-120).  Wz (n_out_z, r1-r0) and WxT
 * (n_tile_x, c1-c0) are the reference's dense linear-interpolation operators
 * restricted to the rows/columns that receive data; each row of Wz and each
 * column of WxT has at most two adjacent non-zeros (MATLAB linear
 * interpolation), which the library verifies and stores in compact form.
 * fz (r1-r0): focus weight.  shift/pdz (n_y, n_tile_x): optical-path
 * correction (OpticalPathCorrection, stitching.py:54-78), or NULL/NULL when it
 * is off.  n_rows: depth samples per A-scan (n/2).  Returns a plan id. */
int octgb_stitch_plan(octgb_ctx *ctx, int n_rows, int r0, int r1, int c0, int c1, int n_out_z, int n_tile_x,
                      const double *Wz, const double *WxT, const double *fz, const int64_t *shift,
                      const double *pdz, int n_y, int *plan_id);

/* ---------------------------------------------------------------- rare raw formats */

/* prepare_raw (octrecon/core/spectral.py:48-68): raw (B, n_lines, n) ->
 * float32 (B, *out_lines, n): apod_mode 0 keeps the first apod_size lines as
 * the apodisation, apod_mode 1 (Wasatch, no apodisation lines) prepends the
 * frame mean (mean over a file's lines, then over the apod_group files of its
 * frame, :59-63); the scan lines are AScanBinning-averaged (filter2 'same',
 * zero padded, decimated from max(1, binning/2) - 1, :20-45) when binning > 1.
 * Same float32 operation order as the reference, so equal to its arrays. */
int octgb_prepare_raw(octgb_ctx *ctx, const void *raw, int raw_dtype, int raw_loc, int B, int n_lines,
                      int apod_size, int binning, int apod_mode, int apod_group, float *out, int out_loc,
                      int *out_lines);
/* Thorlabs SRR raw files on the device (octrecon/io/srr.py:108-125, the
 * reader's read_file + read_bscans): words (n_files, file_lines, n) uint16 as
 * stored after each file's header; only the low 12 bits are data (data %
 * 4096).  Writes out (n_files, (apod_end - apod_start) + (scan_end -
 * scan_start), n) int16: the apodisation lines [apod_start, apod_end) then the
 * scan lines [scan_start, scan_end) of each file, decoded — the (B, interf, n)
 * int16 layout every entry reads with raw_dtype OCTGB_I16.  From host words
 * only the used lines are copied. */
int octgb_srr_decode(octgb_ctx *ctx, const uint16_t *words, int words_loc, int n_files, int file_lines, int n,
                     int apod_start, int apod_end, int scan_start, int scan_end, int16_t *out, int out_loc);
/* average_repeats (core/spectral.py:168-177): mag (n_frames * bscan_avg,
 * size_x * ascan_avg, nz) -> (n_frames, size_x, nz), mean over B-scan repeats
 * then A-scan repeats, float32 as the reference. */
int octgb_average_repeats(octgb_ctx *ctx, const float *mag, int mag_loc, int n_frames, int bscan_avg, int size_x,
                          int ascan_avg, int nz, float *out, int out_loc);

/* Start a y-tile row (Reconstructor.process_row, octrecon/pipeline.py:230-232):
 * zero the device accumulators num/den of shape (n_frames, n_out_z, n_out_x). */
int octgb_row_begin(octgb_ctx *ctx, int n_frames, int n_out_z, int n_out_x);

/* One batch of one tile (pipeline.py:274-285): spectral stage of raw (B,
 * interf, n) then TileStitcher.contribute (stitching.py:122-139) and
 * num/den[frame_offset : frame_offset+B, :, c0:c1] += contribution.
 * frame_idx (B, host int64): tile-local y frame of each B-scan (selects the
 * optical-path shift row). */
int octgb_row_add_batch(octgb_ctx *ctx, int plan_id, const void *raw, int raw_dtype, int raw_loc, int B,
                        int interf, int apod_size, const int64_t *frame_idx, int frame_offset);

/* octgb_row_add_batch for the rare formats (pipeline.py:274-285 with
 * hdr.spectra_avg, apod_mode, bscan_avg, ascan_avg): n_files = n_frames x
 * bscan_avg raw files (B-scan repeats consecutive, Reconstructor.frame_files,
 * pipeline.py:217-220) are prepared (octgb_prepare_raw with apod_group =
 * bscan_avg), reconstructed, averaged over repeats (octgb_average_repeats) and
 * stitched for frames frame_idx[0 .. n_frames-1]. */
int octgb_row_add_batch_ex(octgb_ctx *ctx, int plan_id, const void *raw, int raw_dtype, int raw_loc, int n_files,
                           int n_lines, int apod_size, int binning, int apod_mode, int bscan_avg, int ascan_avg,
                           const int64_t *frame_idx, int n_frames, int frame_offset);

/* Finalise the row (pipeline.py:296-300): den < threshold -> NaN, db =
 * 20*log10(num/den) as float32 (n_frames, n_out_z, n_out_x) into db (host or
 * device).  plane_minmax (optional, host, n_frames*2 doubles) receives each
 * plane's clim (tiff_writer.py:48-50). */
int octgb_row_finalise(octgb_ctx *ctx, float threshold, float *db, int db_loc, double *plane_minmax);


/* ---------------------------------------------------------------- frame batches */

/* One batch of frames across all tiles of a y-tile row (the body of
 * Reconstructor.process_row, octrecon/pipeline.py:261-300, with the loop
 * order frames-outer / tiles-inner, which gives every voxel the same tile
 * summation order as the reference's tiles-outer loop):
 *   spectral stage of raws[t] (B, interf, n) for t < n_tiles (one launch);
 *   stitching of every tile in array order (plan_ids[t], TileStitcher.contribute,
 *   stitching.py:122-139), with num/den kept on chip;
 *   finalise (pipeline.py:296-300) into db (B, n_out_z, n_out_x) float32.
 * f0: tile-local y frame of the batch's first B-scan (frames are consecutive).
 * The finite [min, max] of db folds into the context's running clim (see
 * octgb_clim_reset); plane_minmax (optional, host, B*2 doubles) receives each
 * plane's clim and forces a host sync.  With device raws, device db and no
 * plane_minmax the call does not synchronise and can be graph-captured.
 * Host raws are copied on a separate stream through a ring of three device
 * slots, so a batch's copy overlaps the previous batch's kernels; with device
 * db and no plane_minmax the call returns without waiting, so page-locked host
 * raws must stay unchanged until octgb_synchronize returns (pageable ones are
 * staged before the call returns).  n_tiles <= 32. */
int octgb_frames_process(octgb_ctx *ctx, int n_tiles, const int *plan_ids, const void *const *raws, int raw_dtype,
                         int raw_loc, int B, int interf, int apod_size, int f0, int n_out_z, int n_out_x,
                         float threshold, float *db, int db_loc, double *plane_minmax);

/* Running clim over everything octgb_frames_process wrote since the last reset
 * (the global clim of octrecon/pipeline.py:388). */
int octgb_clim_reset(octgb_ctx *ctx);
int octgb_clim_get(octgb_ctx *ctx, double *clim);
/* db_to_bits with the running clim read on the device (no host round trip;
 * device arrays only). */
int octgb_quantise_running(octgb_ctx *ctx, const float *db, int64_t n, int db_loc, uint16_t *bits, int bits_loc);

/* ---------------------------------------------------------------- CUDA graphs */

/* Capture the calls made between begin and end on the context's stream into a
 * CUDA graph, replayed by octgb_graph_launch.  Calls that read results on the
 * host or take host buffers are refused while capturing; run the sequence once
 * before capturing so every device buffer already has its size. */
int octgb_graph_begin(octgb_ctx *ctx);
int octgb_graph_end(octgb_ctx *ctx, int *graph_id);
int octgb_graph_launch(octgb_ctx *ctx, int graph_id);
/* Self-test of the bounded device waits (no counterpart in the reference):
 * runs the spectral kernel (which = 0) or the precision form's tensor-core
 * sinc (which = 1, integer raws; needs a geometry with precision tiles) on a
 * small internal batch of zero raws, with the waits' limit cut to
 * wait_limit_us (100 .. 2 000 000) and each CTA's first row-copy barrier
 * expecting 16 bytes more than its copies deliver.  Every copy still lands;
 * only that barrier never completes, so the wait runs out, the kernel drains
 * what it issued (and frees its tensor memory) and reports through the status
 * word.  Returns OCTGB_ERR_TIMEOUT when that happened (the expected result),
 * OCTGB_ERR_STATE if the wait did not expire; the limit and switch are
 * restored either way and the context stays usable. */
int octgb_selftest_wait_expiry(octgb_ctx *ctx, int which, int wait_limit_us);

/* Destroy every graph captured on the context (after the work already
 * launched has completed); their ids become invalid and octgb_set_geometry is
 * accepted again.  No counterpart in the reference (its loop has no graphs). */
int octgb_graphs_release(octgb_ctx *ctx);
/* Tile shape of octgb_frames_process's stitch kernel: output rows per block
 * (32, 64 or 128; each block is 32 columns wide; default 64).  Results do not
 * depend on it (every voxel sums its tiles in the same order); the
 * autotuner picks the fastest for a workload.  Graphs already captured keep
 * the shape they were captured with.  Not during graph capture. */
int octgb_set_stitch_rows(octgb_ctx *ctx, int rows);

/* ---------------------------------------------------------------- batched form */

/* One tile of a batch: raw (B, interf, n) and db (B, interf - apod_size,
 * n_out_z) are device buffers; db is A-scan major (the depth profile of each
 * A-scan contiguous).  plan_id: octgb_stitch_plan of the tile alone (the
 * single-tile TileStitcher of octrecon/core/stitching.py:84-120: depth
 * operator, focus weight, identity lateral operator, no optical-path
 * correction); n_out_z is the plan's. */
typedef struct octgb_tile {
    const void *raw;
    int B, interf, apod_size;
    int plan_id;
    float *db;
} octgb_tile;

/* Reconstruct n_tiles (<= 256) independent tiles of uneven sizes in ONE
 * persistent launch: every CTA takes `grab` groups of 4 A-scans at a time
 * from a device work queue spanning all tiles, runs the spectral stage and
 * resamples each depth profile with its tile's plan, finalising to dB
 * (threshold -> NaN, 20*log10(num/den), pipeline.py:296-300).  The finite
 * [min, max] folds into the running clim.  One apodisation launch precedes
 * it.  No host sync; graph-capturable once the same tile table has been run. */
int octgb_batch_process(octgb_ctx *ctx, int n_tiles, const octgb_tile *tiles, int raw_dtype, float threshold,
                        int grab);

/* ---------------------------------------------------------------- estimation */

/* Dispersion scorer (DispersionScorer, octrecon/estimation/dispersion.py:66-107).
 * octgb_disp_load replaces the constructor's linearisation (:80-85): the
 * context's geometry must be the dispersion-free one with a window of ones
 * (octgb_set_geometry with window = 1 + 0i), so the spectral stage yields the
 * plain linearised interferogram (SpectralProcessor.linearise, core/spectral.py:
 * 118-134), which is multiplied by hann (n doubles, Hann/rms) in float64 and
 * rounded once to float32 (dispersion.py:84).  raw holds n_bscans x rep
 * B-scans, repeats of one B-scan consecutive.  The result stays on the device. */
int octgb_disp_load(octgb_ctx *ctx, const void *raw, int raw_dtype, int raw_loc, int n_bscans, int rep, int interf,
                    int apod_size, const double *hann);
/* dk2[j] = (k_eq[j] - mean(k_eq))^2, n doubles (dispersion.py:78-79). */
/* The lines octgb_disp_load prepared: (n_bscans * rep, nX, n) float32, each
 * float32(float64(linearised sample) * hann[j]). */
int octgb_disp_lines(octgb_ctx *ctx, float *out, int out_loc);
int octgb_disp_set_dk2(octgb_ctx *ctx, const double *dk2);
/* Score n_beta candidate betas on loaded B-scans b0 .. b0+nb-1 in one launch
 * (DispersionScorer.magnitude + _metric, dispersion.py:46-63,91-107): phase
 * exp(-i beta dk2) formed in float64 and rounded to complex64, inverse FFT,
 * |.| of the first n/2 bins, mean over repeats.  metric: 0 none, 1
 * top_percentile (log of the mean of the top_k largest I = A^2 over depths >=
 * z_min; the reference's top_k = max(1, int(nX (n/2 - z_min) * 0.01))), 2
 * kurtosis, 3 entropy, 4 legacy_peak.  scores: host (n_beta, nb) doubles, or
 * NULL with metric 0.  mag (optional): the magnitudes (n_beta, nb, nX, n/2)
 * float32 at mag_loc.  Synchronises. */
int octgb_disp_eval(octgb_ctx *ctx, int n_beta, const double *betas, int b0, int nb, int metric, int64_t top_k,
                    int z_min, double *scores, float *mag, int mag_loc);
/* Median over x of every depth column of (n_frames, nx, nz) float32
 * magnitudes, as float64 (numpy.median(..., axis=x) of focus.py:146,156;
 * ignore_nan = 1 gives numpy.nanmedian, focus.py:215,255): out is host
 * (n_frames, nz) doubles.  nx <= 4096.  Synchronises. */
int octgb_xmedian(octgb_ctx *ctx, const float *mag, int mag_loc, int n_frames, int nx, int nz, int ignore_nan,
                  double *out);

/* Mean over x of every depth column of (n_frames, nx, nz) float32
 * magnitudes, as float64 (NaN ignored): the depth profile of sparse
 * reflectors, whose x-median is the noise floor.  No counterpart in the
 * reference.  nx <= 4096.  Synchronises. */
int octgb_xmean(octgb_ctx *ctx, const float *mag, int mag_loc, int n_frames, int nx, int nz, double *out);

/* ---------------------------------------------------------------- learned estimator */

/* A small CNN that predicts the dispersion term and the focus of a B-scan
 * from three probe reconstructions (the reference has no learned estimator;
 * its searches, octrecon/estimation/dispersion.py and focus.py, judge it).
 * Every pointer is a device pointer; tensors are float32 NCHW; all calls are
 * asynchronous on the context's stream. */

/* Probe images: mag (n_probe, nb, nx, n/2) (octgb_disp_eval magnitudes) ->
 * img (nb, n_probe, 256, 256) = 20 log10 of the adaptive average pool of
 * depths < z_keep (rows) x A-scans (columns); normalise = 1 standardises each
 * image over all its probes and pixels. */
int octgb_cnn_images(octgb_ctx *ctx, const float *mag, int n_probe, int nb, int nx, int z_keep, float *img,
                     int normalise);
/* The probe images straight from the loaded B-scans (octgb_disp_load): for
 * each of the n_beta probe betas the dispersion kernel's |X| is pooled over
 * depth inside the kernel (the magnitudes never reach memory), then over the
 * A-scans, as octgb_cnn_images of octgb_disp_eval's magnitudes; img is a
 * device buffer (nb, n_beta, 256, 256).  Asynchronous. */
int octgb_disp_images(octgb_ctx *ctx, int n_beta, const double *betas, int b0, int nb, int z_keep, float *img,
                      int normalise);
/* y = conv3x3(x, w) + b, stride 1, zero padding 1: x (n, cin, h, w), w (cout, cin, 3, 3), b (cout) or NULL. */
int octgb_cnn_conv3x3(octgb_ctx *ctx, const float *x, const float *w, const float *b, float *y, int n, int cin,
                      int cout, int h, int wd);
/* octgb_cnn_conv3x3 on the tensor cores (tcgen05.mma, FP16 operands, float32
 * accumulation in TMEM): the inference form of the learned estimator's
 * convolutions.  Shapes: 1 <= cin <= 32, cout a multiple of 32 up to 128, wd
 * a multiple of 128, or a divisor of 128 with h a multiple of 128 / wd.
 * Asynchronous; a bounded device wait that expires is reported by the next
 * synchronising call (OCTGB_ERR_TIMEOUT). */
int octgb_cnn_conv3x3_tc(octgb_ctx *ctx, const float *x, const float *w, const float *b, float *y, int n, int cin,
                         int cout, int h, int wd);
/* octgb_cnn_conv3x3_tc followed by octgb_cnn_relu_pool in one kernel (the
 * pre-activations never reach memory): p (n, cout, h/2, wd/2) = 0.25 *
 * ((relu + relu) + (relu + relu)) of each 2x2 block.  wd a multiple of 128, h
 * even. */
int octgb_cnn_conv3x3_relu_pool_tc(octgb_ctx *ctx, const float *x, const float *w, const float *b, float *p, int n,
                                   int cin, int cout, int h, int wd);
/* Gradients of octgb_cnn_conv3x3: dw, db from dy and x; dx (optional) with
 * w_scratch (cout * cin * 9 floats) for the flipped kernel. */
int octgb_cnn_conv3x3_bwd(octgb_ctx *ctx, const float *x, const float *w, const float *dy, float *dx, float *dw,
                          float *db, float *w_scratch, int n, int cin, int cout, int h, int wd);
/* octgb_cnn_conv3x3_bwd on the tensor cores (tcgen05.mma, BF16 operands,
 * float32 accumulation): dw as nine pixel-contracting GEMMs whose per-CTA
 * partial sums are added in a fixed order; dx as octgb_cnn_conv3x3_tc of dy
 * with the flipped kernel (the float32 kernel where that shape is not
 * supported); db as octgb_cnn_conv3x3_bwd.  Shapes: 1 <= cin <= 48, 1 <= cout
 * <= 128, and a band of rows dividing h whose staged input fits in shared
 * memory (wd up to about 1000).  Asynchronous; a bounded device wait that
 * expires is reported by the next synchronising call (OCTGB_ERR_TIMEOUT). */
int octgb_cnn_conv3x3_bwd_tc(octgb_ctx *ctx, const float *x, const float *w, const float *dy, float *dx, float *dw,
                             float *db, float *w_scratch, int n, int cin, int cout, int h, int wd);
/* p = 2x2 mean of relu(y) over `planes` planes of h x w (even), and its gradient. */
int octgb_cnn_relu_pool(octgb_ctx *ctx, const float *y, float *p, int64_t planes, int h, int wd);
int octgb_cnn_relu_pool_bwd(octgb_ctx *ctx, const float *dp, const float *y, float *dy, int64_t planes, int h,
                            int wd);
/* Dense layer: pre = x w^T + b (x (m, in), w (out, in)); act = relu(pre) when not NULL. */
int octgb_cnn_dense(octgb_ctx *ctx, const float *x, const float *w, const float *b, float *pre, float *act, int m,
                    int in, int out);
/* Its gradients: dy (m, out) is first masked by pre > 0 when pre is given
 * (in place); dw, db; dx (optional). */
int octgb_cnn_dense_bwd(octgb_ctx *ctx, const float *x, const float *w, float *dy, const float *pre, float *dx,
                        float *dw, float *db, int m, int in, int out);
/* loss (one device double) = mean((pred - target)^2) over n values; grad = 2 (pred - target) / n. */
int octgb_cnn_mse(octgb_ctx *ctx, const float *pred, const float *target, int n, float *grad, double *loss);
/* One Adam step (bias-corrected, `step` counted from 1) on n parameters. */
int octgb_cnn_adam(octgb_ctx *ctx, float *p, const float *g, float *m, float *v, int64_t n, float lr, float beta1,
                   float beta2, float eps, int step);

/* ---------------------------------------------------------------- allocation-free */

/* The magnitude of octgb_magnitude for callers that cannot allocate GPU
 * memory while they run (e.g. a frame-grabber callback, where cudaMalloc may
 * synchronise the device and stall acquisition, or a process whose GPU
 * memory belongs to another framework's pool).  This entry point has no
 * counterpart in the reference.  raw (B, interf, n) and mag (B, interf-apod,
 * n/2) must be device pointers owned by the caller; the only scratch (the
 * apodisation mean) lives in a fixed array of 64 B-scans x n floats
 * (512 KiB) in the library image, held by every GPU that loads the library
 * until the process exits; B > 64 is rejected with OCTGB_ERR_ARG.  The call
 * makes no cudaMalloc/cudaFree.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before
 * any stream capture.  All calls on a device share the array, so calls that
 * overlap on the GPU (other streams or contexts) race; serialise them.  The
 * call is asynchronous: octgb_synchronize reports device-side errors. */
int octgb_magnitude_noalloc(octgb_ctx *ctx, const void *raw, int raw_dtype, int B, int interf, int apod_size,
                            float *mag);

#ifdef __cplusplus
}
#endif
#endif /* OCTGB_H */
