// Output encoding of the legacy TIFF (octrecon/io/tiff_writer.py:53-71) on the
// device.
//
//   k_requant_lut   legacy double quantisation (tiff_writer.py:62-64): the
//                   re-quantised code of a plane depends only on its first
//                   code b = db_to_bits(db, plane clim), so one 65 536-entry
//                   table per plane, built in float64 with the reference's
//                   operations (bits_to_db then db_to_bits, :33-45), replaces
//                   the per-voxel float64 work; k_apply_lut maps the codes.
//   k_packbits_rows PackBits (TIFF compression 32773) of every image row on
//                   its own (TIFF 6.0 packs rows separately), one thread per
//                   row, little-endian sample bytes: a run of >= 3 equal bytes
//                   (up to 128) becomes a repeat packet, everything else
//                   literal packets of up to 128 bytes.  Each row is written to
//                   its own worst-case slot; its byte count goes to sizes[].
#include <cuda_runtime.h>
#include <stdint.h>

#include "octgb_internal.h"

namespace octgb {
namespace {

__device__ __forceinline__ uint16_t quantise_f64(double x, double c1, double span) {
    if (isnan(x)) return 0;
    const double v = (x - c1) / span * 65534.0;
    double r = floor(fabs(v) + 0.5);
    if (v < 0) r = -r;
    if (!(r > 0.0)) r = 0.0;
    if (r > 65535.0) r = 65535.0;
    const unsigned int u = static_cast<unsigned int>(r) + 1u;
    return static_cast<uint16_t>(u > 65535u ? 65535u : u);
}

__global__ void k_requant_lut(double p1, double p2, double c1, double c2, uint16_t* __restrict__ lut) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= 65536) return;
    if (b == 0) {
        lut[0] = 0;                                       // bits_to_db(0) is NaN -> 0
        return;
    }
    const double db = static_cast<double>(b - 1) * (p2 - p1) / 65534.0 + p1;
    lut[b] = quantise_f64(db, c1, c2 - c1);
}

__global__ void k_apply_lut(uint16_t* __restrict__ bits, int64_t n, const uint16_t* __restrict__ lut) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        bits[i] = lut[bits[i]];
}

__device__ __forceinline__ uint8_t row_byte(const uint16_t* row, int k) {
    return static_cast<uint8_t>(row[k >> 1] >> ((k & 1) * 8));
}

__global__ void k_packbits_rows(const uint16_t* __restrict__ img, int rows, int cols, uint8_t* __restrict__ out,
                                int slot, int* __restrict__ sizes) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const uint16_t* row = img + static_cast<int64_t>(r) * cols;
    uint8_t* o = out + static_cast<int64_t>(r) * slot;
    const int n = 2 * cols;
    int i = 0, w = 0;
    while (i < n) {
        const uint8_t b = row_byte(row, i);
        int run = 1;
        while (i + run < n && run < 128 && row_byte(row, i + run) == b) ++run;
        if (run >= 3) {
            o[w++] = static_cast<uint8_t>(1 - run);       // -(run - 1)
            o[w++] = b;
            i += run;
            continue;
        }
        int j = i;
        while (j < n && j - i < 128) {
            if (j + 2 < n) {
                const uint8_t c = row_byte(row, j);
                if (row_byte(row, j + 1) == c && row_byte(row, j + 2) == c) break;
            }
            ++j;
        }
        o[w++] = static_cast<uint8_t>(j - i - 1);
        for (int k = i; k < j; ++k) o[w++] = row_byte(row, k);
        i = j;
    }
    sizes[r] = w;
}

int grid_n(int64_t n) {
    int64_t g = (n + 255) / 256;
    return static_cast<int>(g > 65536 ? 65536 : (g < 1 ? 1 : g));
}

}  // namespace

cudaError_t launch_requant(uint16_t* bits, int64_t n, double p1, double p2, double c1, double c2, uint16_t* lut,
                           cudaStream_t st) {
    k_requant_lut<<<65536 / 256, 256, 0, st>>>(p1, p2, c1, c2, lut);
    k_apply_lut<<<grid_n(n), 256, 0, st>>>(bits, n, lut);
    return cudaGetLastError();
}

int packbits_slot(int cols) { return 2 * cols + (2 * cols + 127) / 128 + 1; }

cudaError_t launch_packbits(const uint16_t* img, int rows, int cols, uint8_t* out, int* sizes, cudaStream_t st) {
    k_packbits_rows<<<(rows + 127) / 128, 128, 0, st>>>(img, rows, cols, out, packbits_slot(cols), sizes);
    return cudaGetLastError();
}

}  // namespace octgb
