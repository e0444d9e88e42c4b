// Focus-weighted tile stitching, row finalisation and the legacy uint16
// quantisation.
//
// Stitching (octrecon/core/stitching.py:122-139, pipeline.py:283-284): for
// one tile and one batch of B-scans,
//   a[f,x,r]  = mag[f, x, clip(r0 + r + shift)]   (optical-path gather)
//   F[f,x,r]  = valid * fz[r]
//   num[f, zo, c0+c] += sum_x WxT[x,c] sum_r Wz[zo,r] a F
//   den[f, zo, c0+c] += sum_x WxT[x,c] sum_r Wz[zo,r] F
// Wz / WxT are linear-interpolation operators with at most two adjacent
// non-zeros per output row / column, stored compactly.
//
// The work unit is a 32 x 32 block of output voxels (rows zo, columns c) of
// one frame.  The block reads a small patch of the tile's magnitudes (the
// A-scans feeding its columns x the depth rows feeding its rows) into shared
// memory with reads along depth (the magnitude layout), applies the depth
// interpolation per A-scan, then the lateral interpolation, and writes along
// x (the output layout): a transpose through shared memory, so both global
// sides are coalesced.
//
// Two kernels use it:
//   k_stitch_tile    one tile, num/den += contribution (per-tile row API);
//   k_stitch_frames  every tile of a frame batch in tile order, num/den kept in
//                    registers, then finalise (threshold -> NaN, 20 log10) and
//                    the plane / running clim: num/den never reach memory.
// In both the per-voxel floating-point operations and their order are those of
// the reference loop (tile contributions added one after the other).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "octgb_internal.h"

namespace octgb {
namespace {

constexpr int kStThreads = 256;          // 32 columns x 8 row groups
constexpr int kRowsPerThread = kBlk / 8; // 4 output rows per thread

struct PatchSmem {
    float* pa;   // [xs_max][rs_max] a * F
    float* pf;   // [xs_max][rs_max] F
    float* un;   // [xs_max][kBlk]   depth-interpolated a F
    float* ud;   // [xs_max][kBlk]   depth-interpolated F
};

__device__ __forceinline__ PatchSmem carve(float* sm, int xs_max, int rs_max) {
    PatchSmem s;
    s.pa = sm;
    s.pf = s.pa + xs_max * rs_max;
    s.un = s.pf + xs_max * rs_max;
    s.ud = s.un + xs_max * kBlk;
    return s;
}

// Contribution of one tile to the block (zb, cb) of frame f; adds it to
// an/ad (4 voxels per thread: rows zb + ty + 8q, column cb + tx).  Uniform
// control flow across the CTA; returns false when the tile misses the block.
__device__ bool block_contrib(const StitchDev& p, const float* __restrict__ mag_f, int fy, int zb, int cb,
                              const PatchSmem& s, int rs_max, float (&an)[kRowsPerThread],
                              float (&ad)[kRowsPerThread]) {
    const int cbi = cb / kBlk - p.cblk_first;
    if (cbi < 0 || cbi >= p.n_cblk) return false;
    const int2 xb = p.cblk[cbi];
    const int2 zr_b = p.zblk[zb / kBlk];
    if (xb.x < 0 || zr_b.x < 0) return false;
    const int x_lo = xb.x, xs = xb.y - xb.x + 1;
    const int r_lo = zr_b.x, rs = zr_b.y - zr_b.x + 1;
    const int tid = threadIdx.x;

    // 1. gather the patch: rows fastest (contiguous in the magnitude layout);
    //    magnitudes by asynchronous 4-byte copies (all in flight at once), the
    //    focus weight F beside them (a = magnitude * F is formed on read)
    for (int i = tid; i < xs * rs; i += kStThreads) {
        const int xx = i / rs, rr = i - xx * rs;
        const int x = x_lo + xx;
        const int r = r_lo + rr;
        const int ra = p.r0 + r;
        int src = ra;
        float F = p.fz[r];
        if (p.shift != nullptr) {
            const int64_t o = static_cast<int64_t>(fy) * p.n_tile_x + x;
            if (ra < p.lo[o] || ra > p.hi[o]) F = 0.f;
            src = ra + p.shift[o];
            src = src < 0 ? 0 : (src > p.n_rows - 1 ? p.n_rows - 1 : src);
        }
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                         static_cast<uint32_t>(__cvta_generic_to_shared(s.pa + xx * rs_max + rr))),
                     "l"(mag_f + static_cast<int64_t>(x) * kHalf + src)
                     : "memory");
        s.pf[xx * rs_max + rr] = F;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();

    // 2. depth interpolation (Wz) for every A-scan of the patch and row of the block
    for (int i = tid; i < xs * kBlk; i += kStThreads) {
        const int xx = i / kBlk, z = i - xx * kBlk;
        const int zo = zb + z;
        float un = 0.f, ud = 0.f;
        if (zo < p.n_out_z) {
            const int zr = p.zr[zo];
            if (zr >= 0) {
                const int rr = zr - r_lo;
                const float w0 = p.wz0[zo], w1 = p.wz1[zo];
                const float f0 = s.pf[xx * rs_max + rr], a0 = s.pa[xx * rs_max + rr] * f0;
                float a1 = 0.f, f1 = 0.f;
                if (rr + 1 < rs) {
                    f1 = s.pf[xx * rs_max + rr + 1];
                    a1 = s.pa[xx * rs_max + rr + 1] * f1;
                }
                un = fmaf(a1, w1, a0 * w0);
                ud = fmaf(f1, w1, f0 * w0);
            }
        }
        s.un[xx * kBlk + z] = un;
        s.ud[xx * kBlk + z] = ud;
    }
    __syncthreads();

    // 3. lateral interpolation (WxT) and accumulation
    const int tx = tid & (kBlk - 1), ty = tid / kBlk;
    const int cc = cb + tx - p.c0;
    if (cc >= 0 && cc < p.C) {
        const int xr = p.xr[cc];
        if (xr >= 0) {
            const int xx = xr - x_lo;
            const float w0 = p.wx0[cc], w1 = p.wx1[cc];
#pragma unroll
            for (int q = 0; q < kRowsPerThread; ++q) {
                const int z = ty + 8 * q;
                const int zo = zb + z;
                if (zo < p.n_out_z && p.zr[zo] >= 0) {
                    const float u0 = s.un[xx * kBlk + z], d0 = s.ud[xx * kBlk + z];
                    const float u1 = xx + 1 < xs ? s.un[(xx + 1) * kBlk + z] : 0.f;
                    const float d1 = xx + 1 < xs ? s.ud[(xx + 1) * kBlk + z] : 0.f;
                    an[q] += fmaf(u1, w1, u0 * w0);
                    ad[q] += fmaf(d1, w1, d0 * w0);
                }
            }
        }
    }
    __syncthreads();
    return true;
}

__global__ void __launch_bounds__(kStThreads) k_stitch_tile(const StitchDev p, const float* __restrict__ mag,
                                                            const int* __restrict__ frame_y, int f0,
                                                            float* __restrict__ num, float* __restrict__ den,
                                                            int frame_offset, int n_out_x, int xs_max, int rs_max) {
    extern __shared__ __align__(16) float sm[];
    const PatchSmem s = carve(sm, xs_max, rs_max);
    const int f = blockIdx.z;
    const int zb = blockIdx.y * kBlk;
    const int cb = (p.cblk_first + blockIdx.x) * kBlk;
    const int fy = frame_y ? frame_y[f] : f0 + f;
    float an[kRowsPerThread] = {0.f, 0.f, 0.f, 0.f}, ad[kRowsPerThread] = {0.f, 0.f, 0.f, 0.f};
    const float* mag_f = mag + static_cast<int64_t>(f) * p.n_tile_x * kHalf;
    if (!block_contrib(p, mag_f, fy, zb, cb, s, rs_max, an, ad)) return;
    const int tx = threadIdx.x & (kBlk - 1), ty = threadIdx.x / kBlk;
    const int c = cb + tx;
    const int cc = c - p.c0;
    if (cc < 0 || cc >= p.C || p.xr[cc] < 0) return;
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
        const int zo = zb + ty + 8 * q;
        if (zo >= p.n_out_z || p.zr[zo] < 0) continue;
        const int64_t o = (static_cast<int64_t>(frame_offset + f) * p.n_out_z + zo) * n_out_x + c;
        num[o] += an[q];
        den[o] += ad[q];
    }
}

__device__ __forceinline__ void warp_minmax(float& mn, float& mx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
}

// The fields of a tile's stitch plan that the frame-batch kernel reads,
// copied to shared memory once per CTA (one load round for all slots).
struct SlotPlan {
    const float4* zrow;       // per output row {zr, wz0, wz1, d}
    const float2* zf;         // per output row {F[zr], F[zr + 1]}
    const float4* xcol;       // per output column {xr, wx0, wx1, 0}
    const float* fz;
    const int* shift;         // null without the optical-path correction
    const int* lo;
    const int* hi;
    int r0, c0, C, n_out_z, n_tile_x, n_rows;
};

static_assert(sizeof(SlotPlan) % 16 == 0, "the row parameters after the slot plans need 16-byte alignment");

// asynchronous global -> shared copy of one 8- or 16-byte element (both addresses aligned to its size)
template <int kBytes>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
    static_assert(kBytes == 8 || kBytes == 16, "cp.async element size");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
                 "l"(src), "n"(kBytes)
                 : "memory");
}

// Frame-batch kernel: one CTA = one frame x kFZ output rows x 32 output
// columns.  The tiles touching each block and their patch extents come from a
// table built once per tile list on the host (StitchSlot); the CTA reads the
// table and each tile's plan fields in one round of loads, then stages every
// contributing patch and the tiles' per-row / per-column interpolation
// parameters (precomputed per plan) in shared memory by asynchronous copies:
// no load waits on another before the one barrier.  Then every voxel sums
// the tiles in order.
// kFZ output rows per CTA (the tile shape the autotuner picks: 32, 64 or 128)
template <int kFZ>
__global__ void __launch_bounds__(kStThreads) k_stitch_frames(const StitchDev* __restrict__ plans, const TileList tl,
                                                              const StitchSlot* __restrict__ slots,
                                                              const int* __restrict__ slot_count,
                                                              const float* __restrict__ mag, int64_t mag_tile_stride,
                                                              int n_tile_x, int f0, int n_out_z, int n_out_x,
                                                              float thr, float* __restrict__ db,
                                                              unsigned int* __restrict__ plane_mm,
                                                              unsigned int* __restrict__ run_mm, int ns_max) {
    constexpr int kFRows = kFZ / 8;          // rows per thread
    // dynamic shared memory: per-slot plan fields, row / column parameters, then the patches
    extern __shared__ __align__(16) float smem_all[];
    __shared__ StitchSlot slot[kMaxSeg];
    SlotPlan* spl = reinterpret_cast<SlotPlan*>(smem_all);              // [ns_max]
    float4* rowp = reinterpret_cast<float4*>(spl + ns_max);             // [ns_max][kFZ] {zr, w0, w1, F interpolated}
    float2* rowf = reinterpret_cast<float2*>(rowp + ns_max * kFZ);      // [ns_max][kFZ] {F of the row's two taps}
    float4* colp = reinterpret_cast<float4*>(rowf + ns_max * kFZ);      // [ns_max][kBlk] {xr, wx0, wx1, 0}
    float* sm = reinterpret_cast<float*>(colp + ns_max * kBlk);
    const int f = blockIdx.z;
    const int zb = blockIdx.y * kFZ;
    const int cb = blockIdx.x * kBlk;
    const int tid = threadIdx.x;
    const int blk = blockIdx.y * gridDim.x + blockIdx.x;
    const int ns = slot_count[blk];
    if (tid < ns) {
        const StitchSlot s = slots[static_cast<int64_t>(blk) * tl.n + tid];
        const StitchDev& p = plans[tl.id[s.t]];
        SlotPlan q;
        q.zrow = p.zrow;
        q.zf = p.zf;
        q.xcol = p.xcol;
        q.fz = p.fz;
        q.shift = p.shift;
        q.lo = p.lo;
        q.hi = p.hi;
        q.r0 = p.r0;
        q.c0 = p.c0;
        q.C = p.C;
        q.n_out_z = p.n_out_z;
        q.n_tile_x = p.n_tile_x;
        q.n_rows = p.n_rows;
        slot[tid] = s;
        spl[tid] = q;
    }
    __syncthreads();

    // 1. stage each contributing tile's interpolation parameters and its
    //    magnitude patch (a * F, and F when the optical-path correction makes
    //    it depend on the A-scan); depth fastest in the patch, one zero row
    //    after each A-scan's rows and one zero A-scan after the last (stride
    //    s.rst), so every 2 x 2 read below is in the patch
    for (int k = 0; k < ns; ++k) {
        const StitchSlot s = slot[k];
        const SlotPlan& p = spl[k];
        if (tid < kFZ) {
            // without the optical-path correction F depends on the row only:
            // its two taps and the depth-interpolated F (the den term) per row.
            // The slot's rows reach zr + 1 of every row, so the per-plan F[zr + 1]
            // (0 past the window) is the one the patch holds.
            const int zo = zb + tid;
            if (zo < p.n_out_z) {
                cp_async<16>(rowp + k * kFZ + tid, p.zrow + zo);
                cp_async<8>(rowf + k * kFZ + tid, p.zf + zo);
            } else {
                rowp[k * kFZ + tid] = make_float4(__int_as_float(-1), 0.f, 0.f, 0.f);
                rowf[k * kFZ + tid] = make_float2(0.f, 0.f);
            }
        } else if (tid < kFZ + kBlk) {
            // the slot's A-scans reach xr + 1 of every column of the block
            const int cc = cb + tid - kFZ - p.c0;
            if (cc >= 0 && cc < p.C)
                cp_async<16>(colp + k * kBlk + tid - kFZ, p.xcol + cc);
            else
                colp[k * kBlk + tid - kFZ] = make_float4(__int_as_float(-1), 0.f, 0.f, 0.f);
        }
        const float* mag_f = mag + s.t * mag_tile_stride + static_cast<int64_t>(f) * n_tile_x * kHalf;
        float* pa = sm + s.off;
        float* pf = pa + (s.xs + 1) * s.rst;
        const int fy = f0 + f;
        // zero rows (rst - rs of them after each A-scan's rows) and the zero
        // A-scan after the last (plain stores, before the barrier)
        {
            const int zr = s.rst - s.rs;                     // 1 or 2
            const int nz = s.xs * zr;
            for (int i = tid; i < nz + s.rst; i += kStThreads) {
                int o;
                if (i < nz) {
                    const int xx = zr == 1 ? i : i >> 1;
                    o = xx * s.rst + s.rs + (i - xx * zr);
                } else {
                    o = s.xs * s.rst + (i - nz);
                }
                pa[o] = 0.f;
                if (s.opc) pf[o] = 0.f;
            }
        }
        // the patch is copied as is (asynchronous 4-byte copies, every slot's
        // in flight at once); the focus weight multiplies it when it is read,
        // the same single product a * F.  64 consecutive threads copy 64
        // consecutive rows of one A-scan, four A-scans per pass
        if (p.shift == nullptr) {
            // source and destination advance by four A-scans a pass
            for (int rr = tid & 63; rr < s.rs; rr += 64) {
                const int xx0 = tid >> 6;
                const float* src = mag_f + static_cast<int64_t>(s.x_lo + xx0) * kHalf + p.r0 + s.r_lo + rr;
                uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(pa + xx0 * s.rst + rr));
                const uint32_t dstep = static_cast<uint32_t>(kStThreads / 64 * s.rst) * 4u;
                for (int xx = xx0; xx < s.xs; xx += kStThreads / 64) {
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
                    src += kStThreads / 64 * kHalf;
                    dst += dstep;
                }
            }
        } else {
            for (int rr = tid & 63; rr < s.rs; rr += 64)
                for (int xx = tid >> 6; xx < s.xs; xx += kStThreads / 64) {
                    const int i = xx * s.rst + rr;
                    const int x = s.x_lo + xx;
                    const int ra = p.r0 + s.r_lo + rr;
                    const int64_t o = static_cast<int64_t>(fy) * p.n_tile_x + x;
                    pf[i] = (ra < p.lo[o] || ra > p.hi[o]) ? 0.f : p.fz[s.r_lo + rr];
                    int src = ra + p.shift[o];
                    src = src < 0 ? 0 : (src > p.n_rows - 1 ? p.n_rows - 1 : src);
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                                     static_cast<uint32_t>(__cvta_generic_to_shared(pa + i))),
                                 "l"(mag_f + static_cast<int64_t>(x) * kHalf + src)
                                 : "memory");
                }
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();

    // 2. per voxel: tiles in order, depth (Wz) then lateral (WxT) interpolation.
    //    A tap outside the patch reads a zero, so a * F and F of it are the
    //    zeros the reference's operators give there.
    const int tx = tid & (kBlk - 1), ty = tid / kBlk;
    const int c = cb + tx;
    float an[kFRows], ad[kFRows];
#pragma unroll
    for (int q = 0; q < kFRows; ++q) an[q] = ad[q] = 0.f;
    for (int k = 0; k < ns; ++k) {
        const float4 cp = colp[k * kBlk + tx];
        const int xr = __float_as_int(cp.x);
        if (xr < 0) continue;
        const int rst = slot[k].rst;
        // this thread's first A-scan of the patch, rows indexed by zr directly
        const float* pa = sm + slot[k].off + (xr - slot[k].x_lo) * rst - slot[k].r_lo;
        const float wx0 = cp.y, wx1 = cp.z;
        const float4* rpk = rowp + k * kFZ + ty;
        const float2* rfk = rowf + k * kFZ + ty;
        if (slot[k].opc == 0) {
            // F depends on the row only: its two taps and the den term per row
#pragma unroll
            for (int q = 0; q < kFRows; ++q) {
                const float4 rp = rpk[8 * q];
                const int zr = __float_as_int(rp.x);
                if (zr < 0) continue;
                const float* p0 = pa + zr;
                const float* p1 = p0 + rst;
                const float w0 = rp.y, w1 = rp.z, d = rp.w;
                const float2 ff = rfk[8 * q];
                // a = magnitude * F (TileStitcher.contribute, stitching.py:136)
                const float a00 = p0[0] * ff.x, a01 = p0[1] * ff.y;
                const float a10 = p1[0] * ff.x, a11 = p1[1] * ff.y;
                const float u0 = fmaf(a01, w1, a00 * w0), u1 = fmaf(a11, w1, a10 * w0);
                an[q] += fmaf(u1, wx1, u0 * wx0);
                ad[q] += fmaf(d, wx1, d * wx0);
            }
        } else {
            // optical-path correction: F per A-scan and row, its patch after the magnitudes
            const float* pf = pa + (slot[k].xs + 1) * rst;
#pragma unroll
            for (int q = 0; q < kFRows; ++q) {
                const float4 rp = rpk[8 * q];
                const int zr = __float_as_int(rp.x);
                if (zr < 0) continue;
                const float w0 = rp.y, w1 = rp.z;
                const float f00 = pf[zr], f01 = pf[zr + 1], f10 = pf[zr + rst], f11 = pf[zr + rst + 1];
                const float d0 = fmaf(f01, w1, f00 * w0), d1 = fmaf(f11, w1, f10 * w0);
                const float a00 = pa[zr] * f00, a01 = pa[zr + 1] * f01;
                const float a10 = pa[zr + rst] * f10, a11 = pa[zr + rst + 1] * f11;
                const float u0 = fmaf(a01, w1, a00 * w0), u1 = fmaf(a11, w1, a10 * w0);
                an[q] += fmaf(u1, wx1, u0 * wx0);
                ad[q] += fmaf(d1, wx1, d0 * wx0);
            }
        }
    }

    // 3. finalise (pipeline.py:296-300) and clim (io/tiff_writer.py:48-50)
    float mn = __int_as_float(0x7f800000), mx = -__int_as_float(0x7f800000);
#pragma unroll
    for (int q = 0; q < kFRows; ++q) {
        const int zo = zb + ty + 8 * q;
        if (zo >= n_out_z || c >= n_out_x) continue;
        float v;
        if (ad[q] < thr || isnan(ad[q])) {
            v = __int_as_float(0x7fc00000);
        } else {
            v = 20.0f * log10f(__fdiv_rn(an[q], ad[q]));
        }
        db[(static_cast<int64_t>(f) * n_out_z + zo) * n_out_x + c] = v;
        if (isfinite(v)) {
            mn = fminf(mn, v);
            mx = fmaxf(mx, v);
        }
    }
    warp_minmax(mn, mx);
    if ((tid & 31) == 0 && mn <= mx) {
        if (plane_mm) {
            atomicMin(&plane_mm[2 * f], f2ord(mn));
            atomicMax(&plane_mm[2 * f + 1], f2ord(mx));
        }
        if (run_mm) {
            atomicMin(&run_mm[0], f2ord(mn));
            atomicMax(&run_mm[1], f2ord(mx));
        }
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
    warp_minmax(mn, mx);
    if ((threadIdx.x & 31) == 0 && mn <= mx) {
        atomicMin(&plane_mm[2 * plane], f2ord(mn));
        atomicMax(&plane_mm[2 * plane + 1], f2ord(mx));
    }
}

// MATLAB uint16() of (db - c1)/(c2 - c1) * 65534, then + 1 saturating, NaN -> 0
__device__ __forceinline__ uint16_t quantise_exact(float x, double c1, double span) {
    if (isnan(x)) return 0;
    const double v = (static_cast<double>(x) - c1) / span * 65534.0;
    double r = floor(fabs(v) + 0.5);
    if (v < 0) r = -r;
    if (!(r > 0.0)) r = 0.0;
    if (r > 65535.0) r = 65535.0;
    const unsigned int u = static_cast<unsigned int>(r) + 1u;
    return static_cast<uint16_t>(u > 65535u ? 65535u : u);
}

// The legacy code is a non-decreasing function of the float32 dB value
// (every float64 step is monotonic), so it is fully described by 65534
// thresholds T[k] = the smallest float32 x with code(x) >= k (k = 2..65535;
// T[1] = -inf, T[65536] = +inf).  k_quant_table finds each T[k] in float64:
// a float32 guess next to c1 + (k - 1.5) * span / 65534, then moved ulp by ulp
// until code(T[k]) >= k > code(prev(T[k])).  Per voxel a float32 estimate
// v32 = (x - c1f) * sf (error < 0.02 code) gives the code directly when v32
// is more than kGuard from a rounding boundary; otherwise two table
// comparisons decide.  Bit-exact, and no float64 work per voxel.
constexpr float kGuard = 0.05f;
constexpr int kTable = 65537;

__global__ void k_quant_table(const unsigned int* __restrict__ clim_mm, double c1_in, double c2_in,
                              float* __restrict__ T) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kTable) return;
    double c1 = c1_in, c2 = c2_in;
    if (clim_mm != nullptr) {
        c1 = static_cast<double>(ord2f(clim_mm[0]));
        c2 = static_cast<double>(ord2f(clim_mm[1]));
    }
    const double span = c2 - c1;
    if (k <= 1) {
        T[k] = -__int_as_float(0x7f800000);
        return;
    }
    if (k == kTable - 1) {
        T[k] = __int_as_float(0x7f800000);
        return;
    }
    float y = static_cast<float>(c1 + (k - 1.5) * span / 65534.0);
    const float lo = -__int_as_float(0x7f800000), hi = __int_as_float(0x7f800000);
    for (int i = 0; i < 256 && quantise_exact(y, c1, span) >= k; ++i) y = nextafterf(y, lo);
    for (int i = 0; i < 256 && quantise_exact(y, c1, span) < k; ++i) y = nextafterf(y, hi);
    T[k] = y;
}

struct QuantParams {
    float c1f, sf;
    bool fast;
};

__host__ __device__ inline QuantParams quant_params(double c1, double c2) {
    QuantParams q;
    const double span = c2 - c1;
    q.c1f = static_cast<float>(c1);
    q.sf = static_cast<float>(65534.0 / span);
    // three float32 roundings of values <= ~65535 plus the offset error of c1f
    const double off = fabs(c1 - static_cast<double>(q.c1f)) * (65534.0 / span);
    q.fast = (4.0 * 65536.0 * 5.96e-8 + off) < 0.5 * kGuard && span > 0.0;
    return q;
}

__device__ __forceinline__ uint16_t quantise_one(float x, const QuantParams& q, const float* __restrict__ T) {
    if (isnan(x)) return 0;
    int n;       // estimated code
    if (q.fast) {
        const float v = (x - q.c1f) * q.sf;
        if (v < 0.5f - kGuard) return 1;              // rounds to <= 0: clipped to 0, + 1
        if (v > 65534.5f + kGuard) return 65535;      // rounds to >= 65535: + 1 saturates
        const float f = v + 0.5f;
        const float fl = floorf(f);
        const float fr = f - fl;
        n = static_cast<int>(fl) + 1;
        if (fr > kGuard && fr < 1.0f - kGuard) return static_cast<uint16_t>(n);
        n = n < 1 ? 1 : (n > 65535 ? 65535 : n);
        // within one code of the truth: settle with the thresholds
        if (n < 65535 && x >= T[n + 1]) return static_cast<uint16_t>(n + 1);
        if (x >= T[n]) return static_cast<uint16_t>(n);
        return static_cast<uint16_t>(n - 1);
    }
    // no usable estimate: binary search of the thresholds
    int a = 1, b = 65535;        // code in [a, b]
    while (a < b) {
        const int m = (a + b + 1) >> 1;
        if (x >= T[m]) a = m; else b = m - 1;
    }
    return static_cast<uint16_t>(a);
}

// Grid-stride quantisation of n voxels: 4 per thread and iteration (one
// 16-byte load, one 8-byte store) when db and bits are aligned for it, so the
// pass streams at HBM rate; scalar otherwise and for the tail.
__device__ __forceinline__ void quantise_span(const float* __restrict__ db, int64_t n, const QuantParams& q,
                                              const float* __restrict__ T, uint16_t* __restrict__ bits) {
    const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    int64_t done = 0;
    if ((reinterpret_cast<uintptr_t>(db) & 15u) == 0 && (reinterpret_cast<uintptr_t>(bits) & 7u) == 0) {
        const int64_t n4 = n >> 2;
        const float4* d4 = reinterpret_cast<const float4*>(db);
        uint2* b4 = reinterpret_cast<uint2*>(bits);
        // four independent 16-byte loads in flight per thread
        int64_t i = tid;
        for (; i + 3 * stride < n4; i += 4 * stride) {
            float4 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = d4[i + u * stride];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const unsigned int c0 = quantise_one(v[u].x, q, T), c1 = quantise_one(v[u].y, q, T);
                const unsigned int c2 = quantise_one(v[u].z, q, T), c3 = quantise_one(v[u].w, q, T);
                b4[i + u * stride] = make_uint2(c0 | (c1 << 16), c2 | (c3 << 16));
            }
        }
        for (; i < n4; i += stride) {
            const float4 v = d4[i];
            const unsigned int c0 = quantise_one(v.x, q, T), c1 = quantise_one(v.y, q, T);
            const unsigned int c2 = quantise_one(v.z, q, T), c3 = quantise_one(v.w, q, T);
            b4[i] = make_uint2(c0 | (c1 << 16), c2 | (c3 << 16));
        }
        done = n4 << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) bits[i] = quantise_one(db[i], q, T);
}

// db_to_bits (io/tiff_writer.py:26-38), float64 semantics
__global__ void k_quantise(const float* __restrict__ db, int64_t n, double c1, double c2,
                           const float* __restrict__ T, uint16_t* __restrict__ bits) {
    quantise_span(db, n, quant_params(c1, c2), T, bits);
}

// same with the clim read from device memory (ordered-uint [min, max] of float32 dB)
__global__ void k_quantise_dev(const float* __restrict__ db, int64_t n, const unsigned int* __restrict__ clim_mm,
                               const float* __restrict__ T, uint16_t* __restrict__ bits) {
    quantise_span(db, n, quant_params(static_cast<double>(ord2f(clim_mm[0])), static_cast<double>(ord2f(clim_mm[1]))),
                  T, bits);
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
    warp_minmax(mn, mx);
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

size_t patch_smem(int xs_max, int rs_max) {
    return sizeof(float) * (2 * static_cast<size_t>(xs_max) * rs_max + 2 * static_cast<size_t>(xs_max) * kBlk);
}

}  // namespace

cudaError_t launch_stitch(const StitchDev& p, const float* mag, const int* frame_y, int f0, int B, float* num,
                          float* den, int frame_offset, int n_out_x, int xs_max, int rs_max, cudaStream_t st) {
    if (B == 0 || p.n_cblk == 0) return cudaSuccess;
    const size_t smem = patch_smem(xs_max, rs_max);
    cudaError_t e = cudaFuncSetAttribute(k_stitch_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    const dim3 grid(p.n_cblk, (p.n_out_z + kBlk - 1) / kBlk, B);
    k_stitch_tile<<<grid, kStThreads, smem, st>>>(p, mag, frame_y, f0, num, den, frame_offset, n_out_x, xs_max,
                                                   rs_max);
    return cudaGetLastError();
}

cudaError_t launch_stitch_frames(const StitchDev* plans_dev, const TileList& tiles, const StitchSlot* slots,
                                 const int* slot_count, int ns_max, size_t patch_smem_bytes, const float* mag,
                                 int64_t mag_tile_stride, int B, int n_tile_x, int f0, int n_out_z, int n_out_x,
                                 float thr, float* db, unsigned int* plane_mm, unsigned int* run_mm, int rows,
                                 cudaStream_t st) {
    if (B == 0) return cudaSuccess;
    if (rows != 32 && rows != 64 && rows != 128) return cudaErrorInvalidValue;
    const size_t smem = patch_smem_bytes +
                        static_cast<size_t>(ns_max) * (sizeof(SlotPlan) + sizeof(float) * (6 * rows + 4 * kBlk)) + 16;
    if (smem > 160 * 1024) return cudaErrorInvalidValue;
    auto kern = rows == 32 ? k_stitch_frames<32> : (rows == 64 ? k_stitch_frames<64> : k_stitch_frames<128>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    const dim3 grid((n_out_x + kBlk - 1) / kBlk, (n_out_z + rows - 1) / rows, B);
    kern<<<grid, kStThreads, smem, st>>>(plans_dev, tiles, slots, slot_count, mag, mag_tile_stride, n_tile_x, f0,
                                         n_out_z, n_out_x, thr, db, plane_mm, run_mm, ns_max);
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

cudaError_t launch_quantise(const float* db, int64_t n, double c1, double c2, float* table, uint16_t* bits,
                            cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_quant_table<<<(kTable + 255) / 256, 256, 0, st>>>(nullptr, c1, c2, table);
    k_quantise<<<grid_for(n, 256), 256, 0, st>>>(db, n, c1, c2, table, bits);
    return cudaGetLastError();
}

cudaError_t launch_quantise_dev(const float* db, int64_t n, const unsigned int* clim_mm, float* table,
                                uint16_t* bits, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_quant_table<<<(kTable + 255) / 256, 256, 0, st>>>(clim_mm, 0.0, 0.0, table);
    k_quantise_dev<<<grid_for(n, 256), 256, 0, st>>>(db, n, clim_mm, table, bits);
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
