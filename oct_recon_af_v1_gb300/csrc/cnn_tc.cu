// Tensor-core kernels of the learned estimator.
//
// k_conv3x3_tc: the 3x3 convolution (cnn.cu's k_conv3x3 on the tensor cores):
// stride 1, zero padding 1, + bias, NCHW float32 in and out, FP16 operands
// (BF16 for the data gradient) and float32 accumulation on the 5th-generation
// tensor cores (tcgen05.mma kind::f16, accumulator in TMEM).  Forward pass of
// training and inference, and the data gradient (the convolution of dy with
// the flipped kernel).  k_conv3x3_wgrad_tc (further down): the weight
// gradient.
//
// Implicit GEMM without an im2col copy: M = 128 output pixels of one image (a
// row segment when the width W >= 128, else 128 / W whole rows), N = the
// output channels, K = 3 x 3 taps x the input channels (chunks of 8, an even
// number of chunks).  The tile's input rows are staged once in shared memory
// as fp16, eight channels per 16 bytes, pixel rows contiguous per chunk, so
// the A operand of tap (dy, dx) is the staged block itself seen through a
// shifted matrix descriptor (canonical no-swizzle K-major layout, rows 16
// bytes apart):
//   W >= 128  rows y0 - 1 .. y0 + 1 with a one-pixel halo (columns x0 - 1 ..
//             x0 + 128, zero outside the image); tap (dy, dx) starts at pixel
//             dy * 130 + dx;
//   W < 128   rows y0 - 1 .. y0 + R without halo, in three copies shifted by
//             dx - 1 columns with the wrapped column zeroed; tap (dy, dx)
//             starts at pixel dy * W of copy dx.
// Per tile one thread issues 9 taps x (chunks / 2) K16 MMAs; the staged block
// and the accumulator (2 x N TMEM columns) are double-buffered, so tile j's
// MMAs run while the CTA writes tile j - 1's pre-activations (every warp its
// 32 TMEM lanes = pixels, + bias, coalesced along x) and stages tile j + 1.
// With ReLU + 2x2 mean fused (W >= 128) a unit is a vertical pair of tiles;
// where the CTAs per SM allow, the pair's four input rows are staged as one
// block (its halo rows read once) and the second tile's MMAs read it one row
// down.  Persistent over units.  Every mbarrier wait is bounded; on expiry the CTA
// records the status, waits (bounded) for its MMAs, frees its TMEM and
// returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "octgb_device.cuh"
#include "octgb_internal.h"

namespace octgb {
namespace {

constexpr int kCM = 128;                    // output pixels per tile (MMA M)
constexpr int kCThreads = 128;              // four warps = the 128 TMEM lanes
constexpr int kCSlots = 5;                  // staged pixels per thread (a staged block holds <= 640)

struct ConvGeom {
    int n, cin, cout, H, W;
    int cin8;          // channel chunks of 8, even (chunks past cin8r are zero)
    int cin8r;         // chunks holding channels
    int wseg, rows;    // tile: rows x wseg pixels
    int halo;          // 1: one staged copy with halo columns (W >= 128); 0: three shifted copies
    int cols_s;        // staged pixels per row
    int pix_c;         // staged pixels per chunk (one copy)
    int nbuf;          // staged buffers (2: the next block stages while the MMAs read the other)
    int sh;            // tiles per staged block: 2 = a pooled pair's rows and halo read once, else 1
    int pool;          // 1: ReLU + 2x2 mean fused into the epilogue (units = vertical tile pairs)
    int tiles_img;     // tiles per image
    int64_t n_units;   // tiles, or tile pairs with pool
    uint32_t xbytes;   // one staged buffer
    uint32_t off_b, smem;
    int tmem_cols;
};

struct ConvBars {
    uint64_t x[2], d[2], drain;
    uint32_t tmem;
    int abort;
    float bias[128];
};

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// two operand values in the kernel's 16-bit type, the first in the low half
template <bool kBf16>
__device__ __forceinline__ uint32_t pack2(float a, float b) {
    return kBf16 ? pack_bf2(a, b) : pack_h2(a, b);
}

// kind::f16 A and B formats: 0 = FP16, 1 = BF16 (both operands the same type)
constexpr uint32_t kIdescBf16 = (1u << 7) | (1u << 10);

__device__ __forceinline__ bool conv_wait(uint64_t* bar, uint32_t parity, ConvBars& S, int* status) {
    bool ok = true;
    if (*reinterpret_cast<volatile int*>(&S.abort) == 0) {
        ok = mbar_wait_bounded(bar, parity, status);
        if (!ok) atomicExch(&S.abort, 1);
    } else {
        ok = false;
    }
    return __syncthreads_and(ok ? 1 : 0) != 0;
}

// image and origin of tile h (0, or 1 = the row below with pool) of unit u
__device__ __forceinline__ void unit_tile(const ConvGeom& g, int64_t u, int h, int& img, int& y0, int& x0) {
    if (g.pool) {                                 // W >= 128: pairs of row segments
        const int per_row = g.W / kCM;
        const int64_t pairs = static_cast<int64_t>(g.H / 2) * per_row;
        img = static_cast<int>(u / pairs);
        const int pi = static_cast<int>(u - static_cast<int64_t>(img) * pairs);
        y0 = 2 * (pi / per_row) + h;
        x0 = (pi % per_row) * kCM;
        return;
    }
    img = static_cast<int>(u / g.tiles_img);
    const int ti = static_cast<int>(u - static_cast<int64_t>(img) * g.tiles_img);
    if (g.W >= kCM) {
        const int per_row = g.W / kCM;
        y0 = ti / per_row;
        x0 = (ti - y0 * per_row) * kCM;
    } else {
        y0 = ti * g.rows;
        x0 = 0;
    }
}

template <bool kBf16>
__global__ void __launch_bounds__(kCThreads, 4)
    k_conv3x3_tc(const float* __restrict__ x, const float* __restrict__ w, const float* __restrict__ bias,
                 float* __restrict__ y, const ConvGeom g, int* status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ ConvBars S;
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* B = base + g.off_b;                         // [9 taps][cin8][cout][16 B]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t b_chunk = static_cast<uint32_t>(g.cout) * 16;
    const int64_t hw = static_cast<int64_t>(g.H) * g.W;
    const int copies = g.halo ? 1 : 3;
    const int U = g.pool ? 2 : 1;                        // tiles per unit

    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(&S.x[b], 1);
            mbar_init(&S.d[b], 1);
        }
        mbar_init(&S.drain, 1);
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                     "r"(g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int co = tid; co < g.cout; co += kCThreads) S.bias[co] = bias != nullptr ? bias[co] : 0.f;
    // weights: B[tap][c8][co] = 8 fp16 of channels 8 c8 .. 8 c8 + 7 (zero past cin)
    for (int i = tid; i < 9 * g.cin8 * g.cout; i += kCThreads) {
        const int kb = i / g.cout, co = i - kb * g.cout;
        const int tap = kb / g.cin8, c8 = kb - tap * g.cin8;
        const int dy = tap / 3, dx = tap - 3 * dy;
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int c = 8 * c8 + e;
            v[e] = c < g.cin ? w[((static_cast<int64_t>(co) * g.cin + c) * 3 + dy) * 3 + dx] : 0.f;
        }
        *reinterpret_cast<uint4*>(B + static_cast<uint32_t>(kb) * b_chunk + co * 16) =
            make_uint4(pack2<kBf16>(v[0], v[1]), pack2<kBf16>(v[2], v[3]), pack2<kBf16>(v[4], v[5]),
                       pack2<kBf16>(v[6], v[7]));
    }
    // the padding chunks of every staged buffer (never rewritten)
    {
        const int npad = (g.cin8 - g.cin8r) * g.pix_c;
        for (int i = tid; i < g.nbuf * copies * npad; i += kCThreads) {
            const int bc = i / npad, r = i - bc * npad;                 // bc = buffer * copies + copy
            uint4* X = reinterpret_cast<uint4*>(base + (bc / copies) * g.xbytes);
            X[((bc % copies) * g.cin8 + g.cin8r) * g.pix_c + r] = make_uint4(0, 0, 0, 0);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    const uint32_t idesc = mma_idesc_f16(kCM, g.cout) | (kBf16 ? kIdescBf16 : 0u);
    // the staged source pixels this thread loads: p = tid + 128 k (row, column), -1 past the block
    int prs[kCSlots], pcs[kCSlots];
#pragma unroll
    for (int k = 0; k < kCSlots; ++k) {
        const int p = tid + kCThreads * k;
        prs[k] = p < g.pix_c ? p / g.cols_s : -1;
        pcs[k] = p < g.pix_c ? p - prs[k] * g.cols_s : 0;
    }

    // the tile origin (img, y0, x0) of the unit (its first tile with pool)
    auto epilogue = [&](int ab, int img, int y0, int x0) {
        const int m = 32 * warp + lane;
        const uint32_t taddr = tmem + (static_cast<uint32_t>(32 * warp) << 16) + static_cast<uint32_t>(ab * U * g.cout);
        if (!g.pool) {
            const int oy = y0 + m / g.wseg, ox = x0 + m % g.wseg;
            float* yo = y + static_cast<int64_t>(img) * g.cout * hw + static_cast<int64_t>(oy) * g.W + ox;
            for (int c0 = 0; c0 < g.cout; c0 += 32) {
                float v[32];
                tmem_ld32(taddr + static_cast<uint32_t>(c0), v);
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    *yo = v[i] + S.bias[c0 + i];
                    yo += hw;
                }
            }
        } else {
            // rows y0 (accumulator 0) and y0 + 1 (accumulator 1); lanes m, m + 1
            // are the two columns.  Per pair of channels each lane sums its
            // column's two ReLUs for both, swaps one with its neighbour and
            // writes one: the even lane the first channel, the odd lane the
            // second (0.25 x the 2x2 sum; the summation order is not
            // k_relu_pool's, the operands being FP16-rounded already)
            const int Ho = g.H / 2, Wo = g.W / 2;
            const int64_t pw = static_cast<int64_t>(Ho) * Wo;
            const int odd = lane & 1;
            float* po = y + static_cast<int64_t>(img) * g.cout * pw + static_cast<int64_t>(y0 / 2) * Wo + (x0 + m) / 2 +
                        odd * pw;
            for (int c0 = 0; c0 < g.cout; c0 += 32) {
                float v0[32], v1[32];
                tmem_ld32(taddr + static_cast<uint32_t>(c0), v0);
                tmem_ld32(taddr + static_cast<uint32_t>(g.cout + c0), v1);
#pragma unroll
                for (int i = 0; i < 32; i += 2) {
                    const float b0 = S.bias[c0 + i], b1 = S.bias[c0 + i + 1];
                    const float t0 = fmaxf(v0[i] + b0, 0.f) + fmaxf(v1[i] + b0, 0.f);
                    const float t1 = fmaxf(v0[i + 1] + b1, 0.f) + fmaxf(v1[i + 1] + b1, 0.f);
                    const float other = __shfl_xor_sync(0xffffffffu, odd ? t0 : t1, 1);
                    *po = 0.25f * ((odd ? t1 : t0) + other);
                    po += 2 * pw;
                }
            }
        }
        tc_fence_before();
    };

    uint32_t j = 0;            // blocks staged by this CTA so far
    uint32_t ju = 0;           // units so far (accumulator set ju & 1)
    bool have_prev = false;
    int prev_img = 0, prev_y0 = 0, prev_x0 = 0;  // origin of the previous unit
    bool ok = true;
    for (int64_t u = blockIdx.x; u < g.n_units && ok; u += gridDim.x, ++ju) {
        const int ab = static_cast<int>(ju & 1);
        int img, y0u, x0;
        unit_tile(g, u, 0, img, y0u, x0);
        for (int h0 = 0; h0 < U && ok; h0 += g.sh, ++j) {
            // one staged block per sh tiles (sh = 2: a pooled pair's rows and
            // their halo read once); nbuf is 1 or 2: the buffer and the parity
            // of its previous use
            const int b = g.nbuf == 2 ? static_cast<int>(j & 1u) : 0;
            if (j >= static_cast<uint32_t>(g.nbuf)) {
                // the MMAs of the block staged nbuf blocks ago have read X[b]
                const uint32_t use = g.nbuf == 2 ? (j - 2) >> 1 : j - 1;
                ok = conv_wait(&S.x[b], use & 1u, S, status);
                if (!ok) break;
            }
            const int y0 = y0u + h0;
            uint4* X = reinterpret_cast<uint4*>(base + b * g.xbytes);
            const float* xi = x + static_cast<int64_t>(img) * g.cin * hw;
            int off[kCSlots];
#pragma unroll
            for (int k = 0; k < kCSlots; ++k) {
                const int iy = y0 - 1 + prs[k];
                const int ix = g.halo ? x0 - 1 + pcs[k] : pcs[k];
                off[k] = (prs[k] >= 0 && iy >= 0 && iy < g.H && ix >= 0 && ix < g.W) ? iy * g.W + ix : -1;
            }
            // each source pixel is loaded once (eight channels in flight) and
            // stored into every copy that holds it: the halo block, or the
            // three shifted copies (copy dx holds column c + dx - 1; the
            // wrapped column is zero)
            for (int c8 = 0; c8 < g.cin8r; ++c8) {
                const float* xc = xi + static_cast<int64_t>(8 * c8) * hw;
                const int ne = g.cin - 8 * c8;
#pragma unroll
                for (int k = 0; k < kCSlots; ++k) {
                    if (prs[k] < 0) continue;
                    float v[8];
                    const float* pe = xc + (off[k] >= 0 ? off[k] : 0);
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        v[e] = (off[k] >= 0 && e < ne) ? __ldg(pe) : 0.f;
                        pe += hw;
                    }
                    const uint4 q = make_uint4(pack2<kBf16>(v[0], v[1]), pack2<kBf16>(v[2], v[3]),
                                               pack2<kBf16>(v[4], v[5]), pack2<kBf16>(v[6], v[7]));
                    const int p = tid + kCThreads * k;
                    if (g.halo) {
                        X[c8 * g.pix_c + p] = q;
                    } else {
                        const uint4 z = make_uint4(0, 0, 0, 0);
                        X[(1 * g.cin8 + c8) * g.pix_c + p] = q;
                        uint4* X0 = X + c8 * g.pix_c;
                        uint4* X2 = X + (2 * g.cin8 + c8) * g.pix_c;
                        if (pcs[k] + 1 < g.W) X0[p + 1] = q;
                        if (pcs[k] == 0) X0[p] = z;
                        if (pcs[k] >= 1) X2[p - 1] = q;
                        if (pcs[k] == g.W - 1) X2[p] = z;
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc_fence_before();
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
                const uint8_t* Xb = base + b * g.xbytes;
                const uint32_t lbo = static_cast<uint32_t>(g.pix_c) * 16;
                for (int h = h0; h < h0 + g.sh; ++h) {
                    // tile h of the unit: its rows start (h - h0) tile heights down the staged block
                    const uint32_t d_tmem = tmem + static_cast<uint32_t>((ab * U + h) * g.cout);
                    const uint8_t* Xh = Xb + static_cast<uint32_t>((h - h0) * g.rows * g.cols_s) * 16u;
                    for (int tap = 0; tap < 9; ++tap) {
                        const int dy = tap / 3, dx = tap - 3 * dy;
                        const uint8_t* a0 = g.halo ? Xh + (dy * g.cols_s + dx) * 16
                                                   : Xh + static_cast<uint32_t>(dx * g.cin8) * lbo + dy * g.W * 16;
                        for (int ks = 0; ks < g.cin8 / 2; ++ks) {
                            const uint64_t da = smem_desc(a0 + 2 * ks * lbo, lbo, 128);
                            const uint64_t db = smem_desc(B + static_cast<uint32_t>(tap * g.cin8 + 2 * ks) * b_chunk,
                                                          b_chunk, 128);
                            mma_f16_id(d_tmem, da, db, idesc, (tap > 0 || ks > 0) ? 1u : 0u);
                        }
                    }
                }
                mma_commit(&S.x[b]);
                if (h0 + g.sh == U) mma_commit(&S.d[ab]);
            }
        }
        if (!ok) break;
        if (have_prev) {
            const int pab = static_cast<int>((ju - 1) & 1);
            ok = conv_wait(&S.d[pab], ((ju - 1) >> 1) & 1u, S, status);
            if (!ok) break;
            tc_fence_after();
            epilogue(pab, prev_img, prev_y0, prev_x0);
        }
        have_prev = true;
        prev_img = img;
        prev_y0 = y0u;
        prev_x0 = x0;
    }
    if (ok && have_prev) {
        const int pab = static_cast<int>((ju - 1) & 1);
        ok = conv_wait(&S.d[pab], ((ju - 1) >> 1) & 1u, S, status);
        if (ok) {
            tc_fence_after();
            epilogue(pab, prev_img, prev_y0, prev_x0);
        }
    }
    // every MMA this CTA issued has completed before its TMEM is released
    __syncthreads();
    if (tid == 0) {
        mma_commit(&S.drain);
        mbar_wait_bounded(&S.drain, 0, status);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(g.tmem_cols)
                     : "memory");
}


// ---------------------------------------------------------------- weight gradient
// dw[k][c][ty][tx] = sum over the images and output pixels (oy, ox) of
//   dy[k](oy, ox) * x[c](oy + ty - 1, ox + tx - 1)          (x zero outside the image)
// as nine GEMMs that contract over pixels: M = 128 rows = the output channels
// (rows past cout read in-bounds data of the following chunks into
// accumulator rows that are never read), N = the input channels rounded up to
// 16, K = 16 pixels per MMA; BF16 operands (gradients span float32's exponent
// range), float32 accumulation.  A tile is R image rows.  Its input rows
// y0 - 1 .. y0 + R are staged with a zero column before each row and zeros
// after it up to the row pitch Wp (W + 2 rounded up to 4), channel-contiguous
// ([channel group][pixel][8 channels x 2 B], the MN-major B operand), and dy
// on the same pitch pixel-contiguous ([8-pixel chunk][output channel][8 pixels
// x 2 B], the K-major A operand) with zeros past each row's W pixels: output
// pixel q = r * Wp + ox meets input pixel q + ty * Wp + tx, so tap (ty, tx) is
// the staged input block seen from that pixel on (a descriptor offset of 16
// bytes a pixel, no shifted copies).  The pitch being a multiple of 4, dy's
// rows arrive as 16-byte loads, four pixels per half chunk.  The nine
// accumulators (9 x N TMEM columns) stay in TMEM over all the CTA's tiles; the
// staged blocks are double-buffered.  Warp 0 only issues the MMAs (one
// thread), so tile j's MMAs are issued while warps 1.. stage tile j + 1.  Each
// CTA then writes its partial sums and k_sum_partials adds them in CTA order
// (the result does not depend on timing).
constexpr int kWThreads = 512;
constexpr int kWStage = kWThreads - 32;       // staging threads (warps 1..)

struct WgradGeom {
    int n, C, K, H, W;
    int R, Wp, Q;        // rows per tile, staged row pitch (W + 2 rounded up to 4), pixels per tile (R Wp rounded up to 32)
    int N;               // MMA N: C rounded up to 16
    int cg, kg;          // channel groups of 8 staged (x: N / 8; dy: ceil(K / 8))
    int xpix;            // staged input pixels per channel group (Q + 2 Wp + 2, rounded up to 8)
    int nbuf;            // staged blocks: 2 (tile j + 1 stages while tile j's MMAs run), or 1 for wide rows
    int vec4;            // dy rows load as float4 (W a multiple of 4)
    int fold;            // C <= 8: the three column taps are one MMA (N = 32: copies of the block shifted by
                         // tx = 0, 1, 2 pixels as channel groups 0-2, group 3 zero): 3 MMAs a K step, not 9
    int acc_cols;        // TMEM columns of the accumulators (9 N, or 3 x 32 folded)
    int tiles_img;
    int64_t n_units;
    uint32_t xbytes, stage, smem;
    int tmem_cols;
};

struct WgradBars {
    uint64_t x[2], drain;
    uint32_t tmem;
    int abort;
    int drained;
};

__device__ __forceinline__ bool wg_wait(uint64_t* bar, uint32_t parity, WgradBars& S, int* status) {
    bool ok = true;
    if (*reinterpret_cast<volatile int*>(&S.abort) == 0) {
        ok = mbar_wait_bounded(bar, parity, status);
        if (!ok) atomicExch(&S.abort, 1);
    } else {
        ok = false;
    }
    return __syncthreads_and(ok ? 1 : 0) != 0;
}

__global__ void __launch_bounds__(kWThreads, 1)
    k_conv3x3_wgrad_tc(const float* __restrict__ x, const float* __restrict__ dy, float* __restrict__ part,
                       const WgradGeom g, int* status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ WgradBars S;
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int st = tid - 32;                       // staging thread index (warps 1..)
    const int64_t hw = static_cast<int64_t>(g.H) * g.W;
    const int kp = 8 * g.kg;

    if (tid == 0) {
        mbar_init(&S.x[0], 1);
        mbar_init(&S.x[1], 1);
        mbar_init(&S.drain, 1);
        S.abort = 0;
        S.drained = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                     "r"(g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    // BF16 A (K-major) and B (MN-major: bit 16)
    const uint32_t idesc = mma_idesc_f16(128, g.fold ? 32 : g.N) | kIdescBf16 | (1u << 16);
    const uint32_t lbo_a = static_cast<uint32_t>(kp) * 16;      // next 8-pixel chunk of dy
    // B is MN-major without swizzle: there the descriptor's leading offset is
    // the step along K (the next 8 pixels, 128 bytes on) and the stride offset
    // the step along N (the next channel group)
    const uint32_t sbo_b = static_cast<uint32_t>(g.xpix) * 16;
    const int ksteps = g.Q / 16;
    const int qw = g.Wp / 4;                       // half chunks (4 pixels) a staged row
    if (g.fold && warp > 0)                        // channel group 3 of every stage stays zero
        for (int i = st; i < g.nbuf * g.xpix; i += kWStage) {
            const int bb = i / g.xpix, p = i - bb * g.xpix;
            *reinterpret_cast<uint4*>(base + bb * g.stage + (3u * g.xpix + p) * 16u) = make_uint4(0, 0, 0, 0);
        }
    const int dtasks = g.Q / 4 * kp;               // (output channel, half chunk) pairs

    uint32_t j = 0;
    bool ok = true;
    for (int64_t u = blockIdx.x; u < g.n_units; u += gridDim.x, ++j) {
        const int b = g.nbuf == 2 ? static_cast<int>(j & 1u) : 0;
        if (j >= static_cast<uint32_t>(g.nbuf)) {
            // the MMAs of the tile staged nbuf tiles ago have read buffer b
            const uint32_t use = g.nbuf == 2 ? (j - 2) >> 1 : j - 1;
            ok = wg_wait(&S.x[b], use & 1u, S, status);
            if (!ok) break;
        }
        const int img = static_cast<int>(u / g.tiles_img);
        const int y0 = static_cast<int>(u - static_cast<int64_t>(img) * g.tiles_img) * g.R;
        uint8_t* Xs = base + b * g.stage;
        uint8_t* Ds = Xs + g.xbytes;
        if (warp > 0) {
            // input block: pixel i = r * Wp + cc is x(y0 - 1 + r, cc - 1); zero
            // outside the image, past each row's W + 1 columns and past the R + 2
            // staged rows.  Two channel groups (16 loads) in flight per pass.
            const float* xi = x + static_cast<int64_t>(img) * g.C * hw;
            if (g.fold) {
                // C <= 8: pixel i of the block goes to copy tx at pixel i - tx
                for (int i0 = st; i0 < g.xpix; i0 += 2 * kWStage) {
                    float v[2][8];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int i = i0 + h * kWStage;
                        const int r = i / g.Wp, cc = i - r * g.Wp;
                        const int iy = y0 - 1 + r, ix = cc - 1;
                        const bool in = i < g.xpix && r < g.R + 2 && iy >= 0 && iy < g.H && ix >= 0 && ix < g.W;
                        const float* px = xi + (in ? static_cast<int64_t>(iy) * g.W + ix : 0);
#pragma unroll
                        for (int e = 0; e < 8; ++e) v[h][e] = (in && e < g.C) ? __ldg(px + static_cast<int64_t>(e) * hw) : 0.f;
                    }
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int i = i0 + h * kWStage;
                        if (i >= g.xpix) continue;
                        const uint4 q = make_uint4(pack_bf2(v[h][0], v[h][1]), pack_bf2(v[h][2], v[h][3]),
                                                   pack_bf2(v[h][4], v[h][5]), pack_bf2(v[h][6], v[h][7]));
#pragma unroll
                        for (int tx = 0; tx < 3; ++tx)
                            if (i - tx >= 0)
                                *reinterpret_cast<uint4*>(Xs + (static_cast<uint32_t>(tx) * g.xpix + i - tx) * 16u) = q;
                    }
                }
            } else
            for (int i0 = st; i0 < g.xpix; i0 += 2 * kWStage) {
                // two pixels a pass, each with two channel groups: 32 loads in flight
                const float* px[2];
                bool in[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int i = i0 + h * kWStage;
                    const int r = i / g.Wp, cc = i - r * g.Wp;
                    const int iy = y0 - 1 + r, ix = cc - 1;
                    in[h] = i < g.xpix && r < g.R + 2 && iy >= 0 && iy < g.H && ix >= 0 && ix < g.W;
                    px[h] = xi + (in[h] ? static_cast<int64_t>(iy) * g.W + ix : 0);
                }
                for (int c8 = 0; c8 < g.cg; c8 += 2) {
                    float v[2][16];
#pragma unroll
                    for (int h = 0; h < 2; ++h)
#pragma unroll
                        for (int e = 0; e < 16; ++e) {
                            const int c = 8 * c8 + e;
                            v[h][e] = (in[h] && c < g.C) ? __ldg(px[h] + static_cast<int64_t>(c) * hw) : 0.f;
                        }
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int i = i0 + h * kWStage;
                        if (i >= g.xpix) continue;
#pragma unroll
                        for (int q = 0; q < 2; ++q)
                            *reinterpret_cast<uint4*>(Xs + (static_cast<uint32_t>(c8 + q) * g.xpix + i) * 16u) =
                                make_uint4(pack_bf2(v[h][8 * q], v[h][8 * q + 1]), pack_bf2(v[h][8 * q + 2], v[h][8 * q + 3]),
                                           pack_bf2(v[h][8 * q + 4], v[h][8 * q + 5]),
                                           pack_bf2(v[h][8 * q + 6], v[h][8 * q + 7]));
                    }
                }
            }
            // dy block: half chunk h4 (q = 4 h4 .. 4 h4 + 3, one row: the pitch is a
            // multiple of 4) of channel k.  A warp takes 8 channels x 4 half
            // chunks: each channel's 16 pixels are one 64-byte read, and the
            // 8-byte stores of two chunks fill two 128-byte rows of banks.
            const float* di = dy + static_cast<int64_t>(img) * g.K * hw + static_cast<int64_t>(y0) * g.W;
            constexpr int kDU = 4;                 // tasks a pass: four 16-byte loads in flight
            for (int i0 = st; i0 < dtasks; i0 += kDU * kWStage) {
                float v[kDU][4];
                uint32_t so[kDU];
#pragma unroll
                for (int t = 0; t < kDU; ++t) {
                    const int i = i0 + t * kWStage;
                    const int l = i & 31, w = i >> 5;
                    const int hb = w / g.kg, kgi = w - hb * g.kg;
                    const int k = 8 * kgi + (l >> 2);
                    const int h4 = 4 * hb + (l & 3);
                    const int r = h4 / qw;
                    const int ox = 4 * (h4 - r * qw);
                    so[t] = i < dtasks ? (static_cast<uint32_t>(h4 >> 1) * kp + k) * 16u + (h4 & 1) * 8u : ~0u;
#pragma unroll
                    for (int e = 0; e < 4; ++e) v[t][e] = 0.f;
                    if (i < dtasks && k < g.K && r < g.R && ox < g.W) {
                        const float* pr = di + static_cast<int64_t>(k) * hw + r * g.W + ox;
                        if (g.vec4) {
                            const float4 f = __ldg(reinterpret_cast<const float4*>(pr));
                            v[t][0] = f.x;
                            v[t][1] = f.y;
                            v[t][2] = f.z;
                            v[t][3] = f.w;
                        } else {
#pragma unroll
                            for (int e = 0; e < 4; ++e) v[t][e] = ox + e < g.W ? __ldg(pr + e) : 0.f;
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < kDU; ++t)
                    if (so[t] != ~0u)
                        *reinterpret_cast<uint2*>(Ds + so[t]) =
                            make_uint2(pack_bf2(v[t][0], v[t][1]), pack_bf2(v[t][2], v[t][3]));
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint64_t da0 = smem_desc(Ds, lbo_a, 128);
            const uint64_t db0 = smem_desc(Xs, 128, sbo_b);
            // K steps outer, taps inner: consecutive MMAs go to different
            // accumulators, so no MMA waits for the previous one's sum
            for (int ks = 0; ks < ksteps; ++ks) {
                const uint64_t da = da0 + static_cast<uint64_t>(ks) * (2u * lbo_a >> 4);
                // descriptor addresses are in 16-byte units: one unit per staged pixel of x
                const uint64_t dbk = db0 + static_cast<uint64_t>(16 * ks);
                const uint32_t acc = (j > 0 || ks > 0) ? 1u : 0u;
                if (g.fold) {
                    // one MMA per row tap: N = the three column taps x 8 channels (+ the zero group)
#pragma unroll
                    for (int ty = 0; ty < 3; ++ty)
                        mma_f16_id(tmem + static_cast<uint32_t>(32 * ty), da, dbk + static_cast<uint64_t>(ty * g.Wp),
                                   idesc, acc);
                } else {
#pragma unroll
                    for (int tap = 0; tap < 9; ++tap) {
                        const int ty = tap / 3, tx = tap - 3 * ty;
                        mma_f16_id(tmem + static_cast<uint32_t>(tap * g.N), da,
                                   dbk + static_cast<uint64_t>(ty * g.Wp + tx), idesc, acc);
                    }
                }
            }
            mma_commit(&S.x[b]);
        }
    }
    // every MMA this CTA issued has completed before the accumulators are read
    __syncthreads();
    if (tid == 0) {
        mma_commit(&S.drain);
        S.drained = mbar_wait_bounded(&S.drain, 0, status) ? 1 : 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (ok && S.drained) {
        // warp w reads TMEM lanes 32 (w % 4) .. + 31 (output channels), 32-column
        // chunks w / 4, w / 4 + 4, ...; column t * N + c is tap t of channel c
        const int quarter = warp & 3;
        const int k = 32 * quarter + lane;
        const int cols = g.acc_cols;
        const int64_t kc9 = static_cast<int64_t>(g.K) * g.C * 9;
        if (32 * quarter < g.K) {
            for (int ch = warp >> 2; 32 * ch < cols; ch += kWThreads / 128) {
                float v[32];
                tmem_ld32(tmem + (static_cast<uint32_t>(32 * quarter) << 16) + static_cast<uint32_t>(32 * ch), v);
                if (k < g.K) {
                    float* pk = part + blockIdx.x * kc9 + static_cast<int64_t>(k) * g.C * 9;
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const int col = 32 * ch + i;
                        int t, c;
                        if (g.fold) {              // column 32 ty + 8 tx + c
                            const int tx = (col & 31) >> 3;
                            t = tx < 3 ? 3 * (col >> 5) + tx : -1;
                            c = col & 7;
                        } else {
                            t = col / g.N;
                            c = col - t * g.N;
                        }
                        if (col < cols && t >= 0 && c < g.C) pk[c * 9 + t] = v[i];
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(g.tmem_cols)
                     : "memory");
}

// out[i] = sum over b < nb (in order) of part[b * n + i]
__global__ void k_sum_partials(const float* __restrict__ part, int nb, int64_t n, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nb; ++b) s += part[b * n + i];
        out[i] = s;
    }
}

// tile geometry: the band of R rows (R dividing H) with at least 512 pixels,
// or the tallest whose staged blocks fit (two, else one for wide rows)
bool wgrad_geom(int n, int cin, int cout, int H, int W, WgradGeom& g) {
    if (n < 1 || cin < 1 || cin > 48 || cout < 1 || cout > 128 || H < 1 || W < 1) return false;
    g = WgradGeom{};
    g.n = n;
    g.C = cin;
    g.K = cout;
    g.H = H;
    g.W = W;
    g.N = (cin + 15) / 16 * 16;
    g.cg = g.N / 8;
    g.kg = (cout + 7) / 8;
    g.Wp = (W + 2 + 3) / 4 * 4;
    g.vec4 = W % 4 == 0 ? 1 : 0;
    g.fold = cin <= 8 ? 1 : 0;
    const int xgroups = g.fold ? 4 : g.cg;          // staged channel groups of x
    const uint32_t budget = 227u * 1024u;
    g.R = 0;
    for (int nbuf = 2; nbuf >= 1 && g.R == 0; --nbuf) {
        for (int R = 1; R <= H; ++R) {
            if (H % R != 0) continue;
            const int Q = (R * g.Wp + 31) / 32 * 32;
            const int xpix = (Q + 2 * g.Wp + 2 + 7) / 8 * 8;
            const uint32_t xbytes = static_cast<uint32_t>(xgroups) * xpix * 16u;
            const uint32_t dbytes = static_cast<uint32_t>(Q / 8) * 8u * g.kg * 16u;
            const uint32_t stage = (xbytes + dbytes + 127u) & ~127u;
            // the stages, 2 KB past the last one for the unused A rows, 1 KB alignment
            const uint32_t smem = static_cast<uint32_t>(nbuf) * stage + 2048u + 1024u;
            if (smem > budget) break;
            g.R = R;
            g.Q = Q;
            g.xpix = xpix;
            g.xbytes = xbytes;
            g.stage = stage;
            g.smem = smem;
            g.nbuf = nbuf;
            if (Q >= 512) break;         // 32+ K steps a tap: enough per tile
        }
    }
    if (g.R == 0) return false;
    g.tiles_img = H / g.R;
    g.n_units = static_cast<int64_t>(n) * g.tiles_img;
    g.acc_cols = g.fold ? 3 * 32 : 9 * g.N;
    g.tmem_cols = g.acc_cols <= 128 ? 128 : (g.acc_cols <= 256 ? 256 : 512);
    return g.acc_cols <= 512;
}

int wgrad_grid(const WgradGeom& g, int num_sms) {
    const int per_sm = g.tmem_cols == 512 || g.smem > 113u * 1024u ? 1 : 2;   // TMEM and shared memory allow
    const int64_t slots = static_cast<int64_t>(per_sm) * num_sms;
    return static_cast<int>(g.n_units < slots ? g.n_units : slots);
}
}  // namespace

bool conv3x3_tc_supported(int cin, int cout, int H, int W) {
    if (cin < 1 || cin > 32 || cout < 32 || cout > 128 || cout % 32 != 0) return false;
    if (W >= kCM) return W % kCM == 0;
    return W >= 1 && kCM % W == 0 && H % (kCM / W) == 0;
}

bool conv3x3_tc_pool_supported(int cin, int cout, int H, int W) {
    return conv3x3_tc_supported(cin, cout, H, W) && W >= kCM && H % 2 == 0;
}

cudaError_t launch_conv3x3_tc(const float* x, const float* w, const float* b, float* y, int n, int cin, int cout,
                              int H, int W, int pool, int* status, cudaStream_t st, bool bf16) {
    if (!conv3x3_tc_supported(cin, cout, H, W)) return cudaErrorInvalidValue;
    if (pool && !conv3x3_tc_pool_supported(cin, cout, H, W)) return cudaErrorInvalidValue;
    ConvGeom g{};
    g.n = n;
    g.cin = cin;
    g.cout = cout;
    g.H = H;
    g.W = W;
    g.cin8r = (cin + 7) / 8;
    g.cin8 = (g.cin8r + 1) / 2 * 2;
    g.halo = W >= kCM ? 1 : 0;
    g.wseg = W >= kCM ? kCM : W;
    g.rows = kCM / g.wseg;
    g.cols_s = g.halo ? g.wseg + 2 : g.wseg;
    g.nbuf = g.halo ? 2 : 1;
    g.pool = pool ? 1 : 0;
    g.tiles_img = static_cast<int>(static_cast<int64_t>(H) * W / kCM);
    g.n_units = static_cast<int64_t>(n) * g.tiles_img / (pool ? 2 : 1);
    const int cols = 2 * (pool ? 2 : 1) * cout;                   // two units of accumulators
    g.tmem_cols = cols <= 32 ? 32 : (cols <= 64 ? 64 : (cols <= 128 ? 128 : (cols <= 256 ? 256 : 512)));
    if (g.n_units == 0) return cudaSuccess;
    auto kern = bf16 ? k_conv3x3_tc<true> : k_conv3x3_tc<false>;
    int dev = 0, sms = 0, smem_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaFuncAttributes fa{};
    cudaError_t e = cudaFuncGetAttributes(&fa, kern);
    if (e != cudaSuccess) return e;
    // staged layout for sh tiles per block, and the CTAs per SM it allows
    // (shared memory, registers, TMEM columns)
    auto layout = [&](int sh) -> int {
        g.sh = sh;
        g.pix_c = (sh * g.rows + 2) * g.cols_s;
        g.xbytes = static_cast<uint32_t>((g.halo ? 1 : 3) * g.cin8 * g.pix_c) * 16u;
        g.xbytes = (g.xbytes + 127u) & ~127u;
        g.off_b = static_cast<uint32_t>(g.nbuf) * g.xbytes;
        g.smem = g.off_b + 9u * static_cast<uint32_t>(g.cin8) * static_cast<uint32_t>(cout) * 16u + 1024u;
        if (g.smem > 227u * 1024u || g.pix_c > kCSlots * kCThreads) return 0;
        const int by_smem = smem_sm / static_cast<int>(g.smem + fa.sharedSizeBytes + 1024);
        const int regs = (fa.numRegs + 7) / 8 * 8;
        const int by_regs = 65536 / (regs * kCThreads);
        const int by_tmem = 512 / g.tmem_cols;
        int ps = by_smem < by_regs ? by_smem : by_regs;
        ps = ps < by_tmem ? ps : by_tmem;
        return ps;
    };
    // a pooled pair staged once (its halo rows read once) unless that costs CTAs per SM
    int per_sm = layout(1);
    if (g.pool && g.halo) {
        const int ps2 = layout(2);
        if (ps2 < per_sm || ps2 == 0) per_sm = layout(1);
        else per_sm = ps2;
    }
    if (per_sm == 0) return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(g.smem));
    if (e != cudaSuccess) return e;
    const int64_t slots = static_cast<int64_t>(per_sm) * sms;
    const int64_t grid = g.n_units < slots ? g.n_units : slots;
    kern<<<static_cast<unsigned int>(grid), kCThreads, g.smem, st>>>(x, w, b, y, g, status);
    return cudaGetLastError();
}

size_t conv3x3_wgrad_tc_partials(int n, int cin, int cout, int H, int W, int num_sms) {
    WgradGeom g;
    if (!wgrad_geom(n, cin, cout, H, W, g)) return 0;
    return static_cast<size_t>(wgrad_grid(g, num_sms)) * cout * cin * 9;
}

cudaError_t launch_conv3x3_wgrad_tc(const float* x, const float* dy, float* dw, int n, int cin, int cout, int H,
                                    int W, float* partials, int num_sms, int* status, cudaStream_t st) {
    WgradGeom g;
    if (!wgrad_geom(n, cin, cout, H, W, g) || partials == nullptr) return cudaErrorInvalidValue;
    if (reinterpret_cast<uintptr_t>(dy) % 16 != 0) g.vec4 = 0;          // 16-byte loads need an aligned base
    const int grid = wgrad_grid(g, num_sms);
    cudaError_t e = cudaFuncSetAttribute(k_conv3x3_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(g.smem));
    if (e != cudaSuccess) return e;
    k_conv3x3_wgrad_tc<<<grid, kWThreads, g.smem, st>>>(x, dy, partials, g, status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int64_t total = static_cast<int64_t>(cout) * cin * 9;
    k_sum_partials<<<static_cast<unsigned int>((total + 255) / 256), 256, 0, st>>>(partials, grid, total, dw);
    return cudaGetLastError();
}

cudaError_t set_wait_test_cnn(unsigned long long limit_ns, int starve, cudaStream_t st) {
    return set_wait_test_here(limit_ns, starve, st);
}

}  // namespace octgb
