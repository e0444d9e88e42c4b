// Rare raw formats on the device: AScanBinning, the Wasatch frame-mean
// apodisation line and B-/A-scan repeat averaging (octrecon/core/spectral.py:
// 20-82 and 168-177), each with the reference's float32 operation order so the
// prepared spectra and averaged magnitudes equal its float32 arrays.
//
//   k_frame_apod   frame-mean apodisation (spectral.py:61-63): per frame of G
//                  files and sample j, the mean over a file's lines (sequential
//                  float32 sum, then / lines), then the mean of the G file
//                  means (sequential sum, then / G)
//   k_prepare      the prepared batch (B, a + kept, N) float32: the first a
//                  lines are the apodisation lines (as float) or the frame-mean
//                  line; then the scan lines, binned when B > 1 (spectral.py:
//                  27-45: filter2 'same' with zero padding, window lines
//                  [c - ceil(B/2) + 1, c + floor(B/2)] of kept column c, summed
//                  as acc = x_0 * h, acc = acc + x_t * h with h = float32(1/B),
//                  products and sums rounded separately as numpy does)
//   k_avg_repeats  (n_frames * nb, size_x * na, nz) -> (n_frames, size_x, nz):
//                  mean over the nb B-scan repeats, then over the na A-scan
//                  repeats (sequential float32 sums, then the division)
//   k_srr_decode   Thorlabs SRR files (octrecon/io/srr.py:108-125): uint16
//                  words whose low 12 bits are the sample (data % 4096, kept
//                  as int16); each file's apodisation lines [a0, a0 + na) and
//                  scan lines [s0, ...) gathered into the (files, na + scan, n)
//                  int16 layout the spectral stage reads
#include <cuda_runtime.h>
#include <stdint.h>

#include "octgb_internal.h"

namespace octgb {
namespace {

template <typename RawT>
__device__ __forceinline__ float ld(const void* raw, int64_t i) {
    return static_cast<float>(static_cast<const RawT*>(raw)[i]);
}

template <typename RawT>
__global__ void k_frame_apod(const PrepArgs p, float* __restrict__ apod) {
    const int64_t total = static_cast<int64_t>(p.B / p.group) * kN;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int j = static_cast<int>(i % kN);
        const int64_t fg = i / kN;
        float acc = 0.f;
        for (int g = 0; g < p.group; ++g) {
            const int64_t base = (fg * p.group + g) * p.n_lines * kN + j;
            float s = ld<RawT>(p.raw, base);
            for (int l = 1; l < p.n_lines; ++l) s = __fadd_rn(s, ld<RawT>(p.raw, base + static_cast<int64_t>(l) * kN));
            const float m = __fdiv_rn(s, static_cast<float>(p.n_lines));
            acc = g == 0 ? m : __fadd_rn(acc, m);
        }
        apod[i] = p.group == 1 ? acc : __fdiv_rn(acc, static_cast<float>(p.group));
    }
}

template <typename RawT>
__global__ void k_prepare(const PrepArgs p, const float* __restrict__ frame_apod, float* __restrict__ out) {
    const int lines_out = p.a_out + p.n_kept;
    const int64_t total = static_cast<int64_t>(p.B) * lines_out * kN;
    const float h = 1.0f / static_cast<float>(p.binning);        // float32(1/B), correctly rounded
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int j = static_cast<int>(i % kN);
        const int l = static_cast<int>((i / kN) % lines_out);
        const int64_t b = i / (static_cast<int64_t>(kN) * lines_out);
        const int64_t file = b * p.n_lines * kN + j;
        float v;
        if (l < p.a_out) {
            v = p.mode == 0 ? ld<RawT>(p.raw, file + static_cast<int64_t>(l) * kN)
                            : frame_apod[(b / p.group) * kN + j];
        } else if (p.binning == 1) {
            v = ld<RawT>(p.raw, file + static_cast<int64_t>(p.scan0 + l - p.a_out) * kN);
        } else {
            const int col = p.s0 + (l - p.a_out) * p.binning;
            v = 0.f;
            for (int t = 0; t < p.binning; ++t) {
                const int line = col + t - p.left;
                const float x = (line >= 0 && line < p.n_scan)
                                    ? ld<RawT>(p.raw, file + static_cast<int64_t>(p.scan0 + line) * kN)
                                    : 0.f;
                const float prod = __fmul_rn(x, h);
                v = t == 0 ? prod : __fadd_rn(v, prod);
            }
        }
        out[i] = v;
    }
}

__global__ void k_avg_repeats(const float* __restrict__ mag, int n_frames, int nb, int size_x, int na, int nz,
                              float* __restrict__ out) {
    const int64_t total = static_cast<int64_t>(n_frames) * size_x * nz;
    const int64_t per_file = static_cast<int64_t>(size_x) * na * nz;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int z = static_cast<int>(i % nz);
        const int x = static_cast<int>((i / nz) % size_x);
        const int64_t f = i / (static_cast<int64_t>(nz) * size_x);
        float acc = 0.f;
        for (int a = 0; a < na; ++a) {
            const int64_t col = (static_cast<int64_t>(x) * na + a) * nz + z;
            float m = mag[(f * nb) * per_file + col];
            for (int r = 1; r < nb; ++r) m = __fadd_rn(m, mag[(f * nb + r) * per_file + col]);
            if (nb > 1) m = __fdiv_rn(m, static_cast<float>(nb));
            acc = a == 0 ? m : __fadd_rn(acc, m);
        }
        out[i] = na > 1 ? __fdiv_rn(acc, static_cast<float>(na)) : acc;
    }
}

// Vec: eight samples per thread with 16-byte accesses (n a multiple of 8,
// both buffers 16-byte aligned).  src may equal out with the identity line map
// (each thread reads its own words before writing them), so no __restrict__.
template <bool Vec>
__global__ void k_srr_decode(const uint16_t* src, int64_t src_file, int a0, int na, int s0, int lines_out, int n,
                             int64_t total, int16_t* out) {
    constexpr int kV = Vec ? 8 : 1;
    const int nv = n / kV;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int jv = static_cast<int>(i % nv);
        const int64_t fl = i / nv;                        // file * lines_out + line
        const int l = static_cast<int>(fl % lines_out);
        const int64_t f = fl / lines_out;
        const int line = l < na ? a0 + l : s0 + (l - na);
        const int64_t si = f * src_file + static_cast<int64_t>(line) * n + static_cast<int64_t>(jv) * kV;
        const int64_t di = fl * n + static_cast<int64_t>(jv) * kV;
        if (Vec) {
            uint4 u = *reinterpret_cast<const uint4*>(src + si);
            u.x &= 0x0fff0fffu;
            u.y &= 0x0fff0fffu;
            u.z &= 0x0fff0fffu;
            u.w &= 0x0fff0fffu;
            *reinterpret_cast<uint4*>(out + di) = u;
        } else {
            out[di] = static_cast<int16_t>(src[si] & 0x0fffu);
        }
    }
}

int grid_of(int64_t n) {
    int64_t g = (n + 255) / 256;
    return static_cast<int>(g > 65536 ? 65536 : (g < 1 ? 1 : g));
}

template <typename RawT>
cudaError_t prepare_t(const PrepArgs& p, float* frame_apod, float* out, cudaStream_t st) {
    if (p.mode == 1) {
        k_frame_apod<RawT><<<grid_of(static_cast<int64_t>(p.B / p.group) * kN), 256, 0, st>>>(p, frame_apod);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_prepare<RawT><<<grid_of(static_cast<int64_t>(p.B) * (p.a_out + p.n_kept) * kN), 256, 0, st>>>(p, frame_apod,
                                                                                                   out);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_srr_decode(const uint16_t* src, int64_t src_file, int a0, int na, int s0, int lines_out, int n,
                              int n_files, int16_t* out, cudaStream_t st) {
    const bool vec = n % 8 == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(out) & 15) == 0 && src_file % 8 == 0;
    const int64_t total = static_cast<int64_t>(n_files) * lines_out * (vec ? n / 8 : n);
    if (total == 0) return cudaSuccess;
    if (vec)
        k_srr_decode<true><<<grid_of(total), 256, 0, st>>>(src, src_file, a0, na, s0, lines_out, n, total, out);
    else
        k_srr_decode<false><<<grid_of(total), 256, 0, st>>>(src, src_file, a0, na, s0, lines_out, n, total, out);
    return cudaGetLastError();
}

cudaError_t launch_prepare(const PrepArgs& p, int dtype, float* frame_apod, float* out, cudaStream_t st) {
    if (dtype == 0) return prepare_t<uint16_t>(p, frame_apod, out, st);
    if (dtype == 1) return prepare_t<int16_t>(p, frame_apod, out, st);
    return prepare_t<float>(p, frame_apod, out, st);
}

cudaError_t launch_avg_repeats(const float* mag, int n_frames, int nb, int size_x, int na, int nz, float* out,
                               cudaStream_t st) {
    k_avg_repeats<<<grid_of(static_cast<int64_t>(n_frames) * size_x * nz), 256, 0, st>>>(mag, n_frames, nb, size_x,
                                                                                         na, nz, out);
    return cudaGetLastError();
}

}  // namespace octgb
