// Focus-weighted tile stitching, row finalisation and the legacy uint16
// quantisation.
//
// Stitching (octrecon/core/stitching.py:122-139, pipeline.py:283-284): for
// one tile and one batch of B-scans,
//   a[f,x,r]  = mag[f, x, clip(r0 + r + shift)]   (optical-path gather)
//   F[f,x,r]  = valid * fz[r]
//   num[f0+f, zo, c0+c] += sum_x WxT[x,c] sum_r Wz[zo,r] a F
//   den[f0+f, zo, c0+c] += sum_x WxT[x,c] sum_r Wz[zo,r] F
// Wz / WxT are linear-interpolation operators with at most two adjacent
// non-zeros per output row / column, stored compactly.  One thread per output
// voxel; tiles are added one launch after the other on one stream, so each
// voxel sums its tile contributions in the same order as the reference loop.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "octgb_internal.h"

namespace octgb {
namespace {

__device__ __forceinline__ float gather(const float* __restrict__ mag_ax, const StitchDev& p, int fy, int x, int r,
                                        float& F) {
    // r: row relative to r0
    int src = p.r0 + r;
    bool ok = true;
    if (p.shift != nullptr) {
        const int64_t o = static_cast<int64_t>(fy) * p.n_tile_x + x;
        const int rr = p.r0 + r;
        ok = rr >= p.lo[o] && rr <= p.hi[o];
        src = rr + p.shift[o];
        src = src < 0 ? 0 : (src > p.n_rows - 1 ? p.n_rows - 1 : src);
    }
    F = ok ? p.fz[r] : 0.f;
    return mag_ax[static_cast<int64_t>(x) * kHalf + src] * F;
}

__global__ void k_stitch(const StitchDev p, const float* __restrict__ mag, const int* __restrict__ frame_y, int B,
                         float* __restrict__ num, float* __restrict__ den, int frame_offset, int n_out_x) {
    const int64_t n = static_cast<int64_t>(B) * p.n_out_z * p.C;
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < n;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int c = static_cast<int>(t % p.C);
        const int64_t t2 = t / p.C;
        const int zo = static_cast<int>(t2 % p.n_out_z);
        const int f = static_cast<int>(t2 / p.n_out_z);
        const int zr = p.zr[zo];
        const int xr = p.xr[c];
        if (zr < 0 || xr < 0) continue;
        const float wz0 = p.wz0[zo], wz1 = p.wz1[zo];
        const float wx0 = p.wx0[c], wx1 = p.wx1[c];
        const float* mf = mag + static_cast<int64_t>(f) * p.n_tile_x * kHalf;
        const int fy = frame_y[f];
        // depth interpolation (Wz) per contributing A-scan, then lateral (WxT)
        float un[2], ud[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int x = xr + q;
            un[q] = 0.f;
            ud[q] = 0.f;
            if (x >= p.n_tile_x || (q == 1 && wx1 == 0.f)) continue;
            float F0, F1 = 0.f;
            const float a0 = gather(mf, p, fy, x, zr, F0);
            float a1 = 0.f;
            if (wz1 != 0.f) a1 = gather(mf, p, fy, x, zr + 1, F1);
            un[q] = fmaf(a1, wz1, a0 * wz0);
            ud[q] = fmaf(F1, wz1, F0 * wz0);
        }
        const float cn = fmaf(un[1], wx1, un[0] * wx0);
        const float cd = fmaf(ud[1], wx1, ud[0] * wx0);
        const int64_t o = (static_cast<int64_t>(frame_offset + f) * p.n_out_z + zo) * n_out_x + p.c0 + c;
        num[o] += cn;
        den[o] += cd;
    }
}

// pipeline.py:296-300 plus plane_clim (io/tiff_writer.py:48-50)
__global__ void k_finalise(const float* __restrict__ num, const float* __restrict__ den, int64_t n_per_plane,
                           float thr, float* __restrict__ db, unsigned int* __restrict__ plane_mm) {
    const int plane = blockIdx.y;
    float mn = __int_as_float(0x7f800000), mx = -__int_as_float(0x7f800000);
    const int64_t base = static_cast<int64_t>(plane) * n_per_plane;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_per_plane;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float d = den[base + i];
        float v;
        if (d < thr || isnan(d)) {
            v = __int_as_float(0x7fc00000);
        } else {
            v = 20.0f * log10f(__fdiv_rn(num[base + i], d));
        }
        db[base + i] = v;
        if (isfinite(v)) {
            mn = fminf(mn, v);
            mx = fmaxf(mx, v);
        }
    }
    if (plane_mm == nullptr) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0 && mn <= mx) {
        atomicMin(&plane_mm[2 * plane], f2ord(mn));
        atomicMax(&plane_mm[2 * plane + 1], f2ord(mx));
    }
}

// db_to_bits (io/tiff_writer.py:26-38) in float64
__global__ void k_quantise(const float* __restrict__ db, int64_t n, double c1, double c2,
                           uint16_t* __restrict__ bits) {
    const double span = c2 - c1;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float x = db[i];
        uint16_t b;
        if (isnan(x)) {
            b = 0;
        } else {
            const double v = (static_cast<double>(x) - c1) / span * 65534.0;
            // MATLAB uint16(): round half away from zero, saturate to [0, 65535]
            double r = floor(fabs(v) + 0.5);
            if (v < 0) r = -r;
            if (!(r > 0.0)) r = 0.0;
            if (r > 65535.0) r = 65535.0;
            unsigned int u = static_cast<unsigned int>(r) + 1u;
            b = static_cast<uint16_t>(u > 65535u ? 65535u : u);
        }
        bits[i] = b;
    }
}

__global__ void k_minmax(const float* __restrict__ x, int64_t n, unsigned int* __restrict__ mm) {
    float mn = __int_as_float(0x7f800000), mx = -__int_as_float(0x7f800000);
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float v = x[i];
        if (isfinite(v)) {
            mn = fminf(mn, v);
            mx = fmaxf(mx, v);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0 && mn <= mx) {
        atomicMin(&mm[0], f2ord(mn));
        atomicMax(&mm[1], f2ord(mx));
    }
}

__global__ void k_minmax_init(unsigned int* mm, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) mm[i] = (i & 1) ? 0u : 0xffffffffu;
}

int grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    if (b > 152 * 32) b = 152 * 32;
    return static_cast<int>(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t launch_stitch(const StitchDev& p, const float* mag, const int* frame_y, int B, float* num, float* den,
                          int frame_offset, int n_out_x, cudaStream_t st) {
    const int64_t n = static_cast<int64_t>(B) * p.n_out_z * p.C;
    if (n == 0) return cudaSuccess;
    k_stitch<<<grid_for(n, 256), 256, 0, st>>>(p, mag, frame_y, B, num, den, frame_offset, n_out_x);
    return cudaGetLastError();
}

cudaError_t launch_finalise(const float* num, const float* den, int64_t n_per_plane, int n_planes, float thr,
                            float* db, unsigned int* plane_minmax, cudaStream_t st) {
    if (n_planes == 0 || n_per_plane == 0) return cudaSuccess;
    int gx = grid_for(n_per_plane, 256);
    if (gx > 64) gx = 64;
    k_finalise<<<dim3(gx, n_planes), 256, 0, st>>>(num, den, n_per_plane, thr, db, plane_minmax);
    return cudaGetLastError();
}

cudaError_t launch_quantise(const float* db, int64_t n, double c1, double c2, uint16_t* bits, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_quantise<<<grid_for(n, 256), 256, 0, st>>>(db, n, c1, c2, bits);
    return cudaGetLastError();
}

cudaError_t launch_minmax(const float* x, int64_t n, unsigned int* mm, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_minmax<<<grid_for(n, 256), 256, 0, st>>>(x, n, mm);
    return cudaGetLastError();
}

cudaError_t launch_minmax_init(unsigned int* mm, int count, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    k_minmax_init<<<(count + 255) / 256, 256, 0, st>>>(mm, count);
    return cudaGetLastError();
}

}  // namespace octgb
