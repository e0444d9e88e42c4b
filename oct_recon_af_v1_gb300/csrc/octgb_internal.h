// Internal declarations shared by the octgb CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace octgb {

constexpr int kN = 2048;          // spectral samples per A-scan (FFT length)
constexpr int kHalf = kN / 2;     // depth bins kept (core/spectral.py:153, nz = N/2)
constexpr int kMaxTaps = 32;      // sinc taps supported
constexpr int kTail = 32;         // zero tail after each line so padded taps stay in bounds
constexpr int kGroup = 128;       // threads per A-scan in the FFT (16 points each)
constexpr int kPerCta = 4;        // A-scans per CTA iteration
constexpr int kThreads = kGroup * kPerCta;

// device-side status word values
constexpr int kStatusOk = 0;
constexpr int kStatusTimeout = 1;

// kModeLinHann: the real linearised line times a float64 window, rounded once
// to float32 (the scorer's input, (eq * hann).astype(complex64) with a window of ones)
enum OutMode : int { kModeSpec = 0, kModeMag = 1, kModeDb = 2, kModeResample = 3, kModeLinHann = 4 };

constexpr int kBlk = 32;          // output rows / columns per stitch block
constexpr int kMaxSeg = 32;       // tiles per multi-tile launch

struct DevGeometry {
    const float* w;       // [taps][kN] sinc weights, tap-major, float32
    const int* start;     // [kN] first source sample of each output sample
    int taps;
    const float* wsh;     // [kThreads][4][U] shifted weights of outputs 4t..4t+3
    const int* s0;        // [kThreads] source window base of thread t
    int U;                // window width (16, 20 or 24)
    const float2* win;    // [kN] complex64 window scaled by 1/kN (ifft normalisation)
    const float2* tw;     // [kN] exp(+2*pi*i*k/kN), rounded from float64
};

struct StitchDev;

// One tile of the batched form: its raw B-scans, its depth operator (a stitch
// plan with the identity lateral operator) and its dB output (A-scan major).
struct QueueTile {
    const void* raw;          // (B, interf, kN) device
    float* out;               // (B * nx, nz) float32 dB
    const StitchDev* plan;    // device pointer into the context's plan table
    int B, interf, apod, nx, nz;
    int apod_row0;            // first row of the tile in the apodisation-mean buffer
    unsigned int quad0;       // first global quad (4 A-scans) of the tile
    unsigned int nquads;      // B * qpb
    int qpb;                  // quads per B-scan (quads never span two B-scans)
    int pad_;
};
constexpr int kMaxQueueTiles = 256;

// float64 form of the spectral stage (exact.cu)
struct ExactArgs {
    const void* raw;          // (B, interf, kN) device, uint16 or int16
    int B, interf, apod, nx;
    int64_t n_ascans;         // B * nx
    const int* apod_sum;      // (B, kN) integer sums of the apodisation lines (filled by launch_exact)
    const int* start;         // [kN] first source sample of each output
    const double* w;          // [taps][kN] float64 band weights, tap-major (padding 0)
    int taps;
    const double2* win;       // [kN] window / kN, float64 complex
    const double2* tw;        // [kN] exp(+2 pi i k / kN), float64
    float* mag;               // (n_ascans, kHalf) |X| rounded to float32
};
cudaError_t launch_exact(const ExactArgs& a, int dtype, int* sums, int num_sms, cudaStream_t st);

struct SpectralArgs {
    const void* raw;          // (B, interf, kN), segment 0
    const void* seg[kMaxSeg]; // raw batches of n_seg tiles, each (B, interf, kN); seg[0] == raw
    int n_seg;
    int B, interf, apod, nx;  // nx = interf - apod
    int64_t n_ascans;         // n_seg * B * nx
    const float* apod_mean;   // (n_seg * B, kN) float32 apodisation mean
    DevGeometry g;
    float* out;               // spec (M, kN, 2) | mag (M, kHalf) | db (M, nz) | windowed line (M, kN)
    const double* hann;       // kModeLinHann: the float64 window (kN)
    const float2* hann2;      // kModeLinHann: the window split hi + lo in float32 (kN)
    int z0, nz;               // depth crop (db mode)
    unsigned int* minmax;     // [2] ordered-uint min / max (db / resample modes), may be null
    int* status;              // device status word
    // work-queue mode (resample): tiles of uneven size, quads taken from a counter
    const QueueTile* qt;
    int n_qt;
    unsigned int* counter;    // queue head in quads, zero before the launch
    unsigned int total_quads;
    int grab;                 // quads taken per atomic grab
    float thr;                // weight threshold (pipeline.py:296-297)
    // static mode, set by the launcher: a CTA's grid stride (gridDim.x quads)
    // as whole B-scans plus A-scans, step_x < nx
    unsigned int step_bt, step_x;
};

// spectral.cu
cudaError_t launch_apod_mean(const SpectralArgs& a, int dtype, cudaStream_t st);
// apodisation mean of every B-scan of the queue tiles (rows by tile.apod_row0)
cudaError_t launch_apod_mean_tiles(const QueueTile* tiles_dev, int n_tiles, int total_rows, int dtype,
                                   float* apod_mean, cudaStream_t st);
cudaError_t launch_spectral(const SpectralArgs& a, int dtype, int mode, int grid, cudaStream_t st);
int spectral_max_ctas_per_sm(int dtype, int mode);
size_t spectral_smem_bytes(int dtype);

// stitch.cu
struct StitchDev {
    // compact 2-tap depth operator: for output row zo, rows zr[zo] and zr[zo]+1 (relative to r0)
    const int* zr;            // [n_out_z], -1 = no contribution
    const float* wz0;         // [n_out_z]
    const float* wz1;         // [n_out_z]
    // compact 2-tap lateral operator: output column c0+cc takes A-scans xr[cc], xr[cc]+1
    const int* xr;            // [C], -1 = none
    const float* wx0;         // [C]
    const float* wx1;         // [C]
    const float* fz;          // [R] focus weight of rows r0..r1-1
    const int* shift;         // [n_y, n_tile_x] optical-path row shift, or null
    const int* lo;            // [n_y, n_tile_x] smallest valid r (incl.), or null
    const int* hi;            // [n_y, n_tile_x] largest valid r (incl.), or null
    // per 32-row output block zb: input rows [x, y] (relative to r0) it reads; x = -1: none
    const int2* zblk;
    // per absolute 32-column output block cblk_first + i: A-scans [x, y] it reads; x = -1: none
    const int2* cblk;
    // per output row: {zr (int bits), wz0, wz1, d = fma(F1, wz1, F0 wz0)} and
    // {F0 = fz[zr], F1 = fz[zr + 1] or 0 past the window} (batched form)
    const float4* zrow;
    const float2* zf;
    // per output column c0 + cc: {xr (int bits), wx0, wx1, 0} (frame-batch form)
    const float4* xcol;
    int cblk_first, n_cblk;
    int r0, R, c0, C, n_out_z, n_tile_x, n_rows;
};

struct TileList {
    int n;
    int id[kMaxSeg];
};

// row API: one tile, accumulate into num/den (n_frames, n_out_z, n_out_x)
cudaError_t launch_stitch(const StitchDev& p, const float* mag, const int* frame_y, int f0, int B, float* num,
                          float* den, int frame_offset, int n_out_x, int xs_max, int rs_max, cudaStream_t st);
// frames API: all tiles of a frame batch, num/den kept on chip, dB + clim written
constexpr int kStitchRows = 64;   // default output rows per frame-batch stitch block (x 32 columns; 32, 64 or 128)
struct StitchSlot {               // one tile touching one output block
    int t;                        // index into the TileList
    int x_lo, xs;                 // A-scans read
    int r_lo, rs;                 // rows (relative to r0) read
    int off;                      // float offset of the patch in shared memory
    int opc;                      // optical-path correction on (patch of F follows)
    int rst;                      // patch stride per A-scan: rs + a zero row, made odd (distinct banks)
};
cudaError_t launch_stitch_frames(const StitchDev* plans_dev, const TileList& tiles, const StitchSlot* slots,
                                 const int* slot_count, int ns_max, size_t patch_smem_bytes, const float* mag,
                                 int64_t mag_tile_stride, int B, int n_tile_x, int f0, int n_out_z, int n_out_x,
                                 float thr, float* db, unsigned int* plane_mm, unsigned int* run_mm, int rows,
                                 cudaStream_t st);
cudaError_t launch_finalise(const float* num, const float* den, int64_t n_per_plane, int n_planes, float thr,
                            float* db, unsigned int* plane_minmax, cudaStream_t st);
// quantisation: `table` is scratch of kQuantTable floats (the code thresholds of the clim)
constexpr int kQuantTable = 65537;
cudaError_t launch_quantise(const float* db, int64_t n, double c1, double c2, float* table, uint16_t* bits,
                            cudaStream_t st);
cudaError_t launch_quantise_dev(const float* db, int64_t n, const unsigned int* clim_mm, float* table,
                                uint16_t* bits, cudaStream_t st);
cudaError_t launch_minmax(const float* x, int64_t n, unsigned int* minmax, cudaStream_t st);
cudaError_t launch_minmax_init(unsigned int* minmax, int count, cudaStream_t st);

// dispersion scorer: A[(gi * nb + bi) * nx + x][k] = mean over repeats of
// |ifft(X line * phase[gi])|[k], k < N/2, for B-scans b0 .. b0 + nb - 1
struct DispArgs {
    const float* X;        // (B, rep, nx, kN) linearised, windowed, real
    const float2* phase;   // (n_beta, kN) exp(-i beta dk^2) / N
    const float2* tw;      // (kN) e^(2 pi i k / N)
    float* A;              // (n_beta, nb, nx, kHalf), or null with zcol
    float* zcol;           // (n_beta, nb, nx, 256) depth-pooled sums of |X| (probe images), or null
    int z_keep;            // depths pooled into the 256 image rows
    int n_beta, nb, b0, nx, rep;
};
cudaError_t launch_disp_mag(const DispArgs& a, int num_sms, cudaStream_t st);
// per segment (n_seg rows of nx x kHalf magnitudes): metric 1 top_percentile
// (top_k elements), 2 kurtosis, 3 entropy, 4 legacy_peak, depths >= z_min
cudaError_t launch_disp_metric(const float* A, int n_seg, int nx, int z_min, int metric, unsigned int top_k,
                               double* score, cudaStream_t st);
// median over x of every (frame, z) column of (n_frames, nx, nz) float32, as float64
cudaError_t launch_xmedian(const float* mag, int n_frames, int nx, int nz, int ignore_nan, int mean_mode,
                           double* out, cudaStream_t st);

// rare raw formats (prepare.cu): AScanBinning, frame-mean apodisation, repeats
struct PrepArgs {
    const void* raw;      // (B, n_lines, kN)
    int B, n_lines;
    int a_out;            // apodisation lines of the output (apod_size, or 1 for frame mean)
    int n_kept;           // scan lines of the output
    int n_scan, scan0;    // scan lines of a file and the first one
    int s0, left;         // AScanBinning: first kept column, window lines before the column
    int binning, mode, group;   // mode 0: apodisation lines, 1: frame mean over `group` files
};
cudaError_t launch_prepare(const PrepArgs& p, int dtype, float* frame_apod, float* out, cudaStream_t st);
cudaError_t launch_srr_decode(const uint16_t* src, int64_t src_file, int a0, int na, int s0, int lines_out, int n,
                              int n_files, int16_t* out, cudaStream_t st);
cudaError_t launch_avg_repeats(const float* mag, int n_frames, int nb, int size_x, int na, int nz, float* out,
                               cudaStream_t st);

// legacy TIFF encoding (encode.cu)
cudaError_t launch_requant(uint16_t* bits, int64_t n, double p1, double p2, double c1, double c2, uint16_t* lut,
                           cudaStream_t st);
int packbits_slot(int cols);
cudaError_t launch_packbits(const uint16_t* img, int rows, int cols, uint8_t* out, int* sizes, cudaStream_t st);

// precision form (precision.cu): tensor-core sinc
constexpr int kPM = 128;                 // A-scans per tile (MMA M)
constexpr int kPN = 64;                  // output samples per block (MMA N)
constexpr int kPKW = 96;                 // source window per block (6 K-steps of 16)
constexpr int kPChunks = kPKW / 8;       // 8-sample column chunks of a window
constexpr int kPBlocks = kN / kPN;       // output blocks per A-scan
}  // namespace octgb
#include <cuda.h>
#include <cuda_fp16.h>
#include <vector>
namespace octgb {
// apod_scratch: B x kN int32 (integer raws) or float64 (float32 raws)
cudaError_t launch_prec_split(const SpectralArgs& a, int dtype, void* apod_scratch, __half* hi, __half* lo,
                              float* mline, int num_sms, cudaStream_t st);
cudaError_t launch_prec_sinc(const CUtensorMap& tm_hi, const CUtensorMap& tm_lo, const uint8_t* wtiles,
                             const int* kb, const float* mline, float* X, int64_t n_ascans, int* status, int num_sms,
                             cudaStream_t st);
bool encode_prec_map(CUtensorMap* map, const void* base, int64_t n_ascans);
// integer raws, fused: apodisation sums, line sums, then the tensor-core sinc
// reading the raw window directly (apod_sum: B x kN ints; sum_n, mline: per A-scan)
cudaError_t launch_prec_sinc_raw(const SpectralArgs& a, int dtype, const CUtensorMap& tm_raw, const uint8_t* wtiles,
                                 const int* kb, int* apod_sum, long long* sum_n, float* mline, float* X, int* status,
                                 int num_sms, cudaStream_t st);
bool encode_raw_map(CUtensorMap* map, const void* raw, int B, int interf, int apod);
// W tiles (per output block: hi then lo, canonical K-major no-swizzle, W x 64)
// and window starts kb; false when a block's band exceeds the window
bool build_prec_tiles(const int* start, const int* len, const float* wt, std::vector<uint16_t>& tiles,
                      std::vector<int>& kb);
size_t prec_smem_bytes();

// learned beta/focus estimator (cnn.cu)
cudaError_t launch_image_pool(const float* A, int n_probe, int nb, int nx, int z_keep, float* img, cudaStream_t st);
// the same images from k_disp_mag's depth-pooled column sums (n_probe, nb, nx, 256)
cudaError_t launch_image_cols(const float* zcol, int n_probe, int nb, int nx, int z_keep, float* img,
                              cudaStream_t st);
cudaError_t launch_image_norm(float* img, int n_images, int64_t per_image, cudaStream_t st);
// tensor-core 3x3 convolution (cnn_tc.cu): same contract as launch_conv3x3 for
// the shapes conv3x3_tc_supported accepts; FP16 operands (BF16 with bf16: the
// data gradient, whose values span float32's exponent range), float32
// accumulation (pool: ReLU + 2x2 mean fused, y is then (n, cout, H/2, W/2))
bool conv3x3_tc_supported(int cin, int cout, int H, int W);
bool conv3x3_tc_pool_supported(int cin, int cout, int H, int W);
cudaError_t launch_conv3x3_tc(const float* x, const float* w, const float* b, float* y, int n, int cin, int cout,
                              int H, int W, int pool, int* status, cudaStream_t st, bool bf16 = false);
// weight gradient of the 3x3 convolution on the tensor cores (cnn_tc.cu; BF16
// operands, float32 accumulation): dw (cout, cin, 3, 3) from x (n, cin, H, W)
// and dy (n, cout, H, W).  conv3x3_wgrad_tc_partials: the float count of the
// per-CTA partial sums the launch needs (0: shape not supported).
size_t conv3x3_wgrad_tc_partials(int n, int cin, int cout, int H, int W, int num_sms);
cudaError_t launch_conv3x3_wgrad_tc(const float* x, const float* dy, float* dw, int n, int cin, int cout, int H,
                                    int W, float* partials, int num_sms, int* status, cudaStream_t st);
cudaError_t launch_conv3x3(const float* x, const float* w, const float* b, float* y, int Nn, int C, int K, int H,
                           int W, cudaStream_t st);
cudaError_t launch_flip_weights(const float* w, int K, int C, float* wf, cudaStream_t st);
cudaError_t launch_conv3x3_wgrad(const float* x, const float* dy, float* dw, int Nn, int C, int K, int H, int W,
                                 cudaStream_t st);
cudaError_t launch_relu_pool(const float* y, int64_t nk, int H, int W, float* p, cudaStream_t st);
cudaError_t launch_relu_pool_bwd(const float* dp, const float* y, int64_t nk, int H, int W, float* dy,
                                 cudaStream_t st);
cudaError_t launch_gemm(const float* A, int64_t sa0, int64_t sa1, const float* B, int64_t sb0, int64_t sb1, float* C,
                        int64_t ldc, int M, int N, int K, int accumulate, cudaStream_t st);
// split-K form (S slices of K, partial: S x M x N floats of scratch); gemm_splits picks S
int gemm_splits(int M, int N, int K, int num_sms);
cudaError_t launch_gemm_split(const float* A, int64_t sa0, int64_t sa1, const float* B, int64_t sb0, int64_t sb1,
                              float* C, int64_t ldc, int M, int N, int K, int accumulate, int S, float* partial,
                              cudaStream_t st);
cudaError_t launch_bias_relu(float* y, const float* b, int M, int N, float* out, cudaStream_t st);
// db[k] = sum over n and inner of g[n][k][inner]; part (Nn * K floats, optional)
// takes the plane sums of the two-pass form used when inner is a multiple of 4
cudaError_t launch_bias_grad(const float* g, int Nn, int K, int64_t inner, float* db, float* part, cudaStream_t st);
cudaError_t launch_relu_bwd(float* g, const float* pre, int64_t n, cudaStream_t st);
cudaError_t launch_mse(const float* pred, const float* t, int n, float* grad, double* loss, cudaStream_t st);
cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                        float eps, float c1, float c2, cudaStream_t st);

// ordered-uint encoding of float32 for atomic min/max
__host__ __device__ inline unsigned int f2ord(float f) {
#ifdef __CUDA_ARCH__
    unsigned int u = __float_as_uint(f);
#else
    unsigned int u;
    __builtin_memcpy(&u, &f, 4);
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float ord2f(unsigned int u) {
    unsigned int v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(v);
#else
    float f;
    __builtin_memcpy(&f, &v, 4);
    return f;
#endif
}

// the bounded waits' limit and self-test switch of each kernel file (see
// octgb_device.cuh); only octgb_selftest_wait_expiry calls these
cudaError_t set_wait_test_spectral(unsigned long long limit_ns, int starve, cudaStream_t st);
cudaError_t set_wait_test_precision(unsigned long long limit_ns, int starve, cudaStream_t st);
cudaError_t set_wait_test_cnn(unsigned long long limit_ns, int starve, cudaStream_t st);

}  // namespace octgb
