// Kernels of the learned beta/focus estimator (no counterpart in the
// reference, whose estimators are the searches of octrecon/estimation): input
// images from the dispersion scorer's magnitudes, and the forward, backward
// and Adam steps of a small CNN.  All tensors are float32, NCHW, on the device.
//
//   k_image_pool    magnitudes (probes, B, nX, N/2) -> (B, probes, 256, 256)
//                   20 log10 of the area mean over z < z_keep (adaptive
//                   average pooling, the block-average of estimation/
//                   preview.py:49-53 with fractional edges)
//   k_image_cols    the same images from the dispersion kernel's depth-pooled
//                   column sums (the magnitudes never reach memory)
//   k_image_norm    per image: (v - mean) / std over all its probes and pixels
//   k_conv3x3       3x3 convolution, stride 1, zero padding 1, + bias: a CTA
//                   computes a 16x16 pixel tile of 16 output channels, input
//                   channels staged 8 at a time in shared memory; also the
//                   data gradient (weights flipped and transposed by
//                   k_flip_weights)
//   k_conv3x3_wgrad weight gradient: a CTA sums dY x shifted X over one image
//                   for 16 output x 8 input channels x 9 taps, then adds its
//                   partial sums atomically
//   k_relu_pool / k_relu_pool_bwd   ReLU then 2x2 mean, and its gradient
//   k_gemm          C = A B (+ C) with arbitrary strides, 64x64 tiles
//   k_bias_relu, k_bias_grad, k_mse, k_adam
#include <cuda_runtime.h>
#include <stdint.h>

#include "octgb_internal.h"

namespace octgb {
namespace {

constexpr int kImg = 256;

__global__ void k_image_pool(const float* __restrict__ A, int n_probe, int nb, int nx, int z_keep,
                             float* __restrict__ img) {
    const int64_t total = static_cast<int64_t>(nb) * n_probe * kImg * kImg;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int zi = static_cast<int>(i % kImg);
        const int xi = static_cast<int>((i / kImg) % kImg);
        const int p = static_cast<int>((i / (kImg * kImg)) % n_probe);
        const int b = static_cast<int>(i / (static_cast<int64_t>(kImg) * kImg * n_probe));
        const int z0 = zi * z_keep / kImg, z1 = ((zi + 1) * z_keep + kImg - 1) / kImg;
        const int x0 = xi * nx / kImg, x1 = ((xi + 1) * nx + kImg - 1) / kImg;
        const float* a = A + (static_cast<int64_t>(p) * nb + b) * nx * kHalf;
        float s = 0.f;
        for (int x = x0; x < x1; ++x)
            for (int z = z0; z < z1; ++z) s += a[static_cast<int64_t>(x) * kHalf + z];
        const float m = s / static_cast<float>((x1 - x0) * (z1 - z0));
        // image rows = depth, columns = A-scans (the preview orientation)
        img[((static_cast<int64_t>(b) * n_probe + p) * kImg + zi) * kImg + xi] = 20.0f * log10f(fmaxf(m, 1e-30f));
    }
}

// k_image_pool from depth-pooled column sums zcol (probes, B, nx, 256): the
// sum over the row's A-scans, divided by the window's element count.  A CTA
// makes 32 image rows of one (B-scan, probe) image, 32 columns at a time: the
// column sums of the A-scans those columns cover are staged in shared memory
// (rows of 32 depths, read along depth), summed per pixel and written along
// the image row.
constexpr int kColTile = 32;
__global__ void __launch_bounds__(256) k_image_cols(const float* __restrict__ zcol, int n_probe, int nb, int nx,
                                                     int z_keep, float* __restrict__ img) {
    extern __shared__ float T[];                         // [A-scans of the chunk][kColTile + 1]
    const int zb = blockIdx.x * kColTile;
    const int p = blockIdx.y % n_probe, b = blockIdx.y / n_probe;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float* c = zcol + (static_cast<int64_t>(p) * nb + b) * nx * kImg + zb;
    float* out = img + ((static_cast<int64_t>(b) * n_probe + p) * kImg + zb) * kImg;
    for (int xc = 0; xc < kImg; xc += kColTile) {
        const int xa = xc * nx / kImg, xe = ((xc + kColTile) * nx + kImg - 1) / kImg;
        for (int x = xa + warp; x < xe; x += 8) T[(x - xa) * (kColTile + 1) + lane] = c[static_cast<int64_t>(x) * kImg + lane];
        __syncthreads();
        const int xi = xc + lane;
        const int x0 = xi * nx / kImg, x1 = ((xi + 1) * nx + kImg - 1) / kImg;
        for (int zl = warp; zl < kColTile; zl += 8) {
            const int zi = zb + zl;
            const int z0 = zi * z_keep / kImg, z1 = ((zi + 1) * z_keep + kImg - 1) / kImg;
            float sum = 0.f;
            for (int x = x0; x < x1; ++x) sum += T[(x - xa) * (kColTile + 1) + zl];
            const float m = sum / static_cast<float>((x1 - x0) * (z1 - z0));
            out[static_cast<int64_t>(zl) * kImg + xi] = 20.0f * log10f(fmaxf(m, 1e-30f));
        }
        __syncthreads();
    }
}

// Sums in float64 of float32 partial sums over 16 pixels (four float4 loads),
// so the FP64 pipe sees a quarter of an operation per pixel; per_image is a
// multiple of 4 (probes x 256 x 256).
__global__ void __launch_bounds__(1024) k_image_norm(float* __restrict__ img, int64_t per_image) {
    __shared__ double red[32];
    float* v = img + blockIdx.x * per_image;
    const float4* v4 = reinterpret_cast<const float4*>(v);
    const int64_t n4 = per_image / 4;
    double s = 0.0, s2 = 0.0;
    for (int64_t i0 = threadIdx.x; i0 < n4; i0 += 4 * static_cast<int64_t>(blockDim.x)) {
        float fs = 0.f, fs2 = 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * static_cast<int64_t>(blockDim.x);
            if (i < n4) {
                const float4 q = v4[i];
                fs += (q.x + q.y) + (q.z + q.w);
                fs2 += fmaf(q.x, q.x, q.y * q.y) + fmaf(q.z, q.z, q.w * q.w);
            }
        }
        s += static_cast<double>(fs);
        s2 += static_cast<double>(fs2);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    __shared__ double red2[32];
    if (lane == 0) {
        red[w] = s;
        red2[w] = s2;
    }
    __syncthreads();
    if (w == 0) {
        s = lane < (blockDim.x >> 5) ? red[lane] : 0.0;
        s2 = lane < (blockDim.x >> 5) ? red2[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        if (lane == 0) {
            red[0] = s;
            red2[0] = s2;
        }
    }
    __syncthreads();
    const double mean = red[0] / per_image;
    const double var = red2[0] / per_image - mean * mean;
    const float inv = static_cast<float>(1.0 / sqrt(var > 1e-12 ? var : 1e-12));
    const float mf = static_cast<float>(mean);
    float4* w4 = reinterpret_cast<float4*>(v);
    for (int64_t i = threadIdx.x; i < n4; i += blockDim.x) {
        const float4 q = w4[i];
        w4[i] = make_float4((q.x - mf) * inv, (q.y - mf) * inv, (q.z - mf) * inv, (q.w - mf) * inv);
    }
}

// ---------------------------------------------------------------- convolution
constexpr int kTH = 16, kTW = 16, kKT = 16, kCT = 8;

__global__ void __launch_bounds__(256) k_conv3x3(const float* __restrict__ x, const float* __restrict__ w,
                                                 const float* __restrict__ bias, float* __restrict__ y, int C,
                                                 int K, int H, int W, int tiles_x) {
    __shared__ float xs[kCT][kTH + 2][kTW + 2];
    __shared__ float4 ws[kCT * 9][kKT / 4];
    const int n = blockIdx.z;
    const int ty0 = (blockIdx.x / tiles_x) * kTH, tx0 = (blockIdx.x % tiles_x) * kTW;
    const int ty = threadIdx.x / kTW, tx = threadIdx.x % kTW;
    const int k0 = blockIdx.y * kKT;
    float acc[kKT];
#pragma unroll
    for (int k = 0; k < kKT; ++k) acc[k] = (bias != nullptr && k0 + k < K) ? bias[k0 + k] : 0.f;
    for (int c0 = 0; c0 < C; c0 += kCT) {
        const int cn = min(kCT, C - c0);
        for (int e = threadIdx.x; e < kCT * (kTH + 2) * (kTW + 2); e += 256) {
            const int c = e / ((kTH + 2) * (kTW + 2));
            const int r = (e / (kTW + 2)) % (kTH + 2), q = e % (kTW + 2);
            const int ih = ty0 + r - 1, iw = tx0 + q - 1;
            float v = 0.f;
            if (c < cn && ih >= 0 && ih < H && iw >= 0 && iw < W)
                v = x[((static_cast<int64_t>(n) * C + c0 + c) * H + ih) * W + iw];
            xs[c][r][q] = v;
        }
        float* wsf = reinterpret_cast<float*>(ws);
        for (int e = threadIdx.x; e < kCT * 9 * kKT; e += 256) {
            const int k = e % kKT, ct = e / kKT;
            const int c = ct / 9, t = ct % 9;
            wsf[e] = (c < cn && k0 + k < K) ? w[(static_cast<int64_t>(k0 + k) * C + c0 + c) * 9 + t] : 0.f;
        }
        __syncthreads();
        for (int c = 0; c < cn; ++c)
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                const float v = xs[c][ty + t / 3][tx + t % 3];
#pragma unroll
                for (int kq = 0; kq < kKT / 4; ++kq) {
                    const float4 wv = ws[c * 9 + t][kq];
                    acc[4 * kq] = fmaf(v, wv.x, acc[4 * kq]);
                    acc[4 * kq + 1] = fmaf(v, wv.y, acc[4 * kq + 1]);
                    acc[4 * kq + 2] = fmaf(v, wv.z, acc[4 * kq + 2]);
                    acc[4 * kq + 3] = fmaf(v, wv.w, acc[4 * kq + 3]);
                }
            }
        __syncthreads();
    }
    const int oh = ty0 + ty, ow = tx0 + tx;
    if (oh < H && ow < W)
#pragma unroll
        for (int k = 0; k < kKT; ++k)
            if (k0 + k < K) y[((static_cast<int64_t>(n) * K + k0 + k) * H + oh) * W + ow] = acc[k];
}

// wf[c][k][t] = w[k][c][8 - t]: the data gradient is the convolution of dY
// with the flipped, transposed kernel
__global__ void k_flip_weights(const float* __restrict__ w, int K, int C, float* __restrict__ wf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K * C * 9) return;
    const int t = i % 9, c = (i / 9) % C, k = i / (9 * C);
    wf[(static_cast<int64_t>(c) * K + k) * 9 + (8 - t)] = w[i];
}

constexpr int kWK = 16, kWC = 8;

__global__ void __launch_bounds__(256) k_conv3x3_wgrad(const float* __restrict__ x, const float* __restrict__ dy,
                                                       float* __restrict__ dw, int C, int K, int H, int W,
                                                       int c_tiles) {
    __shared__ float dys[kWK][kTH * kTW];
    __shared__ float xs[kWC][kTH + 2][kTW + 2];
    const int n = blockIdx.z;
    const int k0 = (blockIdx.x / c_tiles) * kWK, c0 = (blockIdx.x % c_tiles) * kWC;
    const int pair = threadIdx.x & 127, half = threadIdx.x >> 7;
    const int kk = pair / kWC, cc = pair % kWC;
    const int t0 = half ? 5 : 0, tn = half ? 4 : 5;
    float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    const int tiles_x = (W + kTW - 1) / kTW, tiles_y = (H + kTH - 1) / kTH;
    for (int tile = 0; tile < tiles_x * tiles_y; ++tile) {
        const int ty0 = (tile / tiles_x) * kTH, tx0 = (tile % tiles_x) * kTW;
        for (int e = threadIdx.x; e < kWK * kTH * kTW; e += 256) {
            const int k = e / (kTH * kTW), p = e % (kTH * kTW);
            const int oh = ty0 + p / kTW, ow = tx0 + p % kTW;
            dys[k][p] = (k0 + k < K && oh < H && ow < W)
                            ? dy[((static_cast<int64_t>(n) * K + k0 + k) * H + oh) * W + ow]
                            : 0.f;
        }
        for (int e = threadIdx.x; e < kWC * (kTH + 2) * (kTW + 2); e += 256) {
            const int c = e / ((kTH + 2) * (kTW + 2));
            const int r = (e / (kTW + 2)) % (kTH + 2), q = e % (kTW + 2);
            const int ih = ty0 + r - 1, iw = tx0 + q - 1;
            xs[c][r][q] = (c0 + c < C && ih >= 0 && ih < H && iw >= 0 && iw < W)
                              ? x[((static_cast<int64_t>(n) * C + c0 + c) * H + ih) * W + iw]
                              : 0.f;
        }
        __syncthreads();
        for (int p = 0; p < kTH * kTW; ++p) {
            const float d = dys[kk][p];
            const int py = p / kTW, px = p % kTW;
#pragma unroll
            for (int j = 0; j < 5; ++j)
                if (j < tn) {
                    const int t = t0 + j;
                    acc[j] = fmaf(d, xs[cc][py + t / 3][px + t % 3], acc[j]);
                }
        }
        __syncthreads();
    }
    if (k0 + kk < K && c0 + cc < C)
        for (int j = 0; j < tn; ++j) atomicAdd(&dw[(static_cast<int64_t>(k0 + kk) * C + c0 + cc) * 9 + t0 + j], acc[j]);
}

__global__ void k_relu_pool(const float* __restrict__ y, int64_t nk, int H, int W, float* __restrict__ p) {
    const int Ho = H / 2, Wo = W / 2;
    const int64_t total = nk * Ho * Wo;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int ow = static_cast<int>(i % Wo), oh = static_cast<int>((i / Wo) % Ho);
        const int64_t plane = i / (static_cast<int64_t>(Ho) * Wo);
        const float* s = y + (plane * H + 2 * oh) * W + 2 * ow;
        p[i] = 0.25f * ((fmaxf(s[0], 0.f) + fmaxf(s[1], 0.f)) + (fmaxf(s[W], 0.f) + fmaxf(s[W + 1], 0.f)));
    }
}

__global__ void k_relu_pool_bwd(const float* __restrict__ dp, const float* __restrict__ y, int64_t nk, int H, int W,
                                float* __restrict__ dy) {
    const int64_t total = nk * H * W;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int w = static_cast<int>(i % W), h = static_cast<int>((i / W) % H);
        const int64_t plane = i / (static_cast<int64_t>(H) * W);
        const float g = dp[(plane * (H / 2) + h / 2) * (W / 2) + w / 2];
        dy[i] = y[i] > 0.f ? 0.25f * g : 0.f;
    }
}

// the same two kernels four pixels a thread (16-byte loads and stores) for
// widths that are a multiple of 4 on aligned buffers, rows = planes x H < 2^31 / (W / 4)
__global__ void k_relu_pool4(const float* __restrict__ y, int rows_out, int H, int W, float* __restrict__ p) {
    const int w4 = W / 4, Wo = W / 2, Ho = H / 2;
    const int total = rows_out * w4;                     // two outputs (four inputs of two rows) a thread
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int ro = i / w4, c = 4 * (i - ro * w4);
        const int plane = ro / Ho, oh = ro - plane * Ho;
        const float* s = y + (static_cast<int64_t>(plane) * H + 2 * oh) * W + c;
        const float4 a = *reinterpret_cast<const float4*>(s);
        const float4 b = *reinterpret_cast<const float4*>(s + W);
        const float p0 = 0.25f * ((fmaxf(a.x, 0.f) + fmaxf(a.y, 0.f)) + (fmaxf(b.x, 0.f) + fmaxf(b.y, 0.f)));
        const float p1 = 0.25f * ((fmaxf(a.z, 0.f) + fmaxf(a.w, 0.f)) + (fmaxf(b.z, 0.f) + fmaxf(b.w, 0.f)));
        *reinterpret_cast<float2*>(p + static_cast<int64_t>(ro) * Wo + c / 2) = make_float2(p0, p1);
    }
}

__global__ void k_relu_pool_bwd4(const float* __restrict__ dp, const float* __restrict__ y, int rows, int H, int W,
                                 float* __restrict__ dy) {
    const int w4 = W / 4, Wo = W / 2;
    const int total = rows * w4;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int row = i / w4, c = 4 * (i - row * w4);
        const int plane = row / H, h = row - plane * H;
        const float2 g = *reinterpret_cast<const float2*>(dp + (static_cast<int64_t>(plane) * (H / 2) + h / 2) * Wo +
                                                          c / 2);
        const int64_t o = static_cast<int64_t>(row) * W + c;
        const float4 v = *reinterpret_cast<const float4*>(y + o);
        const float g0 = 0.25f * g.x, g1 = 0.25f * g.y;
        *reinterpret_cast<float4*>(dy + o) =
            make_float4(v.x > 0.f ? g0 : 0.f, v.y > 0.f ? g0 : 0.f, v.z > 0.f ? g1 : 0.f, v.w > 0.f ? g1 : 0.f);
    }
}

// ---------------------------------------------------------------- dense layers
constexpr int kGT = 64, kGK = 16;

// C[i][j] (+)= sum_k A(i,k) B(k,j), A(i,k) = A[i*sa0 + k*sa1], B(k,j) = B[k*sb0 + j*sb1].
// Split K: blockIdx.z takes k in [z k_chunk, (z + 1) k_chunk) and writes its
// partial product to the slice Cm + z M ldc (k_sum_splits adds the slices in
// order).  Tiles are loaded along whichever index is contiguous in memory.
__global__ void __launch_bounds__(256) k_gemm(const float* __restrict__ A, int64_t sa0, int64_t sa1,
                                              const float* __restrict__ B, int64_t sb0, int64_t sb1,
                                              float* __restrict__ Cm, int64_t ldc, int M, int N, int Kd,
                                              int accumulate, int k_chunk) {
    __shared__ float as[kGK][kGT + 4];
    __shared__ float bs[kGK][kGT + 4];
    const int i0 = blockIdx.y * kGT, j0 = blockIdx.x * kGT;
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
    const int kb = blockIdx.z * k_chunk, ke = min(Kd, kb + k_chunk);
    Cm += static_cast<int64_t>(blockIdx.z) * M * ldc;
    const bool a_kfast = sa1 == 1, b_kfast = sb0 == 1;
    float acc[4][4] = {};
    for (int k0 = kb; k0 < ke; k0 += kGK) {
        for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
            const int kk = a_kfast ? e % kGK : e / kGT, r = a_kfast ? e / kGK : e % kGT;
            as[kk][r] = (i0 + r < M && k0 + kk < ke) ? A[(i0 + r) * sa0 + (k0 + kk) * sa1] : 0.f;
            const int kk2 = b_kfast ? e % kGK : e / kGT, r2 = b_kfast ? e / kGK : e % kGT;
            bs[kk2][r2] = (j0 + r2 < N && k0 + kk2 < ke) ? B[(k0 + kk2) * sb0 + (j0 + r2) * sb1] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kGK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = as[kk][ti + 16 * u];
                b[u] = bs[kk][tj + 16 * u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + ti + 16 * u, j = j0 + tj + 16 * v;
            if (i < M && j < N) {
                float* c = Cm + i * ldc + j;
                *c = accumulate ? *c + acc[u][v] : acc[u][v];
            }
        }
}

// C[i][j] (+)= sum over s in order of P[s][i][j] (the split-K slices)
__global__ void k_sum_splits(const float* __restrict__ P, int S, int M, int N, float* __restrict__ Cm, int64_t ldc,
                             int accumulate) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(M) * N) return;
    float v = P[i];
    for (int s = 1; s < S; ++s) v += P[static_cast<int64_t>(s) * M * N + i];
    float* c = Cm + (i / N) * ldc + i % N;
    *c = accumulate ? *c + v : v;
}

// y[i][j] += b[j]; out = relu(y) (out may be NULL)
__global__ void k_bias_relu(float* __restrict__ y, const float* __restrict__ b, int M, int N,
                            float* __restrict__ out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(M) * N) return;
    const float v = y[i] + b[i % N];
    y[i] = v;
    if (out != nullptr) out[i] = fmaxf(v, 0.f);
}

// db[k] = sum over n and inner of g[n][k][inner] (inner = 1 for dense layers)
__global__ void __launch_bounds__(256) k_bias_grad(const float* __restrict__ g, int Nn, int K, int64_t inner,
                                                   float* __restrict__ db) {
    __shared__ float red[8];
    const int k = blockIdx.x;
    float s = 0.f;
    for (int64_t e = threadIdx.x; e < static_cast<int64_t>(Nn) * inner; e += 256) {
        const int64_t n = e / inner, r = e % inner;
        s += g[(n * K + k) * inner + r];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < 8; ++w) t += red[w];
        db[k] = t;
    }
}

// part[n * K + k] = sum of the plane g[n][k][0 .. inner) (inner a multiple of
// 4): one block per plane, 16-byte loads, a fixed reduction order
__global__ void __launch_bounds__(256) k_plane_sums(const float* __restrict__ g, int K, int64_t inner,
                                                    float* __restrict__ part) {
    __shared__ float red[8];
    const int64_t plane = static_cast<int64_t>(blockIdx.y) * K + blockIdx.x;
    const float4* p = reinterpret_cast<const float4*>(g + plane * inner);
    float s = 0.f;
    for (int64_t e = threadIdx.x; e < inner / 4; e += 256) {
        const float4 v = p[e];
        s += (v.x + v.y) + (v.z + v.w);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < 8; ++w) t += red[w];
        part[plane] = t;
    }
}

// dense gradient through ReLU: g[i] = pre[i] > 0 ? g[i] : 0
__global__ void k_relu_bwd(float* __restrict__ g, const float* __restrict__ pre, int64_t n) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n && !(pre[i] > 0.f)) g[i] = 0.f;
}

// loss = mean((pred - t)^2) over n values; grad = 2 (pred - t) / n
__global__ void __launch_bounds__(256) k_mse(const float* __restrict__ pred, const float* __restrict__ t, int n,
                                             float* __restrict__ grad, double* __restrict__ loss) {
    __shared__ double red[8];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) {
        const float d = pred[i] - t[i];
        grad[i] = 2.0f * d / static_cast<float>(n);
        s += static_cast<double>(d) * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < 8; ++w) v += red[w];
        *loss = v / n;
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

int grid_for(int64_t n, int threads, int cap = 1 << 20) {
    int64_t g = (n + threads - 1) / threads;
    if (g > cap) g = cap;
    return static_cast<int>(g < 1 ? 1 : g);
}

}  // namespace

cudaError_t launch_image_pool(const float* A, int n_probe, int nb, int nx, int z_keep, float* img, cudaStream_t st) {
    k_image_pool<<<grid_for(static_cast<int64_t>(nb) * n_probe * kImg * kImg, 256, 65536), 256, 0, st>>>(
        A, n_probe, nb, nx, z_keep, img);
    return cudaGetLastError();
}

cudaError_t launch_image_cols(const float* zcol, int n_probe, int nb, int nx, int z_keep, float* img,
                              cudaStream_t st) {
    // A-scans of a 32-column chunk: at most 32 nx / 256 + 2
    const size_t smem = static_cast<size_t>(kColTile * nx / kImg + 2) * (kColTile + 1) * sizeof(float);
    if (smem > 48 * 1024 || static_cast<int64_t>(nb) * n_probe > 65535) return cudaErrorInvalidValue;
    k_image_cols<<<dim3(kImg / kColTile, nb * n_probe), 256, smem, st>>>(zcol, n_probe, nb, nx, z_keep, img);
    return cudaGetLastError();
}

cudaError_t launch_image_norm(float* img, int n_images, int64_t per_image, cudaStream_t st) {
    k_image_norm<<<n_images, 1024, 0, st>>>(img, per_image);
    return cudaGetLastError();
}

cudaError_t launch_conv3x3(const float* x, const float* w, const float* b, float* y, int Nn, int C, int K, int H,
                           int W, cudaStream_t st) {
    const int tx = (W + kTW - 1) / kTW, ty = (H + kTH - 1) / kTH;
    dim3 grid(tx * ty, (K + kKT - 1) / kKT, Nn);
    k_conv3x3<<<grid, 256, 0, st>>>(x, w, b, y, C, K, H, W, tx);
    return cudaGetLastError();
}

cudaError_t launch_flip_weights(const float* w, int K, int C, float* wf, cudaStream_t st) {
    k_flip_weights<<<grid_for(static_cast<int64_t>(K) * C * 9, 256), 256, 0, st>>>(w, K, C, wf);
    return cudaGetLastError();
}

cudaError_t launch_conv3x3_wgrad(const float* x, const float* dy, float* dw, int Nn, int C, int K, int H, int W,
                                 cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(dw, 0, static_cast<size_t>(K) * C * 9 * sizeof(float), st);
    if (e != cudaSuccess) return e;
    const int ct = (C + kWC - 1) / kWC;
    dim3 grid(((K + kWK - 1) / kWK) * ct, 1, Nn);
    k_conv3x3_wgrad<<<grid, 256, 0, st>>>(x, dy, dw, C, K, H, W, ct);
    return cudaGetLastError();
}

static bool aligned16(const void* p) { return reinterpret_cast<uintptr_t>(p) % 16 == 0; }

cudaError_t launch_relu_pool(const float* y, int64_t nk, int H, int W, float* p, cudaStream_t st) {
    const int64_t threads4 = nk * (H / 2) * (W / 4);
    if (W % 4 == 0 && threads4 < (int64_t(1) << 31) && aligned16(y) && reinterpret_cast<uintptr_t>(p) % 8 == 0) {
        k_relu_pool4<<<grid_for(threads4, 256, 65536), 256, 0, st>>>(y, static_cast<int>(nk * (H / 2)), H, W, p);
        return cudaGetLastError();
    }
    k_relu_pool<<<grid_for(nk * (H / 2) * (W / 2), 256, 65536), 256, 0, st>>>(y, nk, H, W, p);
    return cudaGetLastError();
}

cudaError_t launch_relu_pool_bwd(const float* dp, const float* y, int64_t nk, int H, int W, float* dy,
                                 cudaStream_t st) {
    const int64_t threads4 = nk * H * (W / 4);
    if (W % 4 == 0 && threads4 < (int64_t(1) << 31) && aligned16(y) && aligned16(dy) &&
        reinterpret_cast<uintptr_t>(dp) % 8 == 0) {
        k_relu_pool_bwd4<<<grid_for(threads4, 256, 65536), 256, 0, st>>>(dp, y, static_cast<int>(nk * H), H, W, dy);
        return cudaGetLastError();
    }
    k_relu_pool_bwd<<<grid_for(nk * H * W, 256, 65536), 256, 0, st>>>(dp, y, nk, H, W, dy);
    return cudaGetLastError();
}

cudaError_t launch_gemm(const float* A, int64_t sa0, int64_t sa1, const float* B, int64_t sb0, int64_t sb1, float* C,
                        int64_t ldc, int M, int N, int K, int accumulate, cudaStream_t st) {
    dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT);
    k_gemm<<<grid, 256, 0, st>>>(A, sa0, sa1, B, sb0, sb1, C, ldc, M, N, K, accumulate, K);
    return cudaGetLastError();
}

int gemm_splits(int M, int N, int K, int num_sms) {
    const int tiles = ((N + kGT - 1) / kGT) * ((M + kGT - 1) / kGT);
    int S = (2 * num_sms + tiles - 1) / tiles;
    const int max_s = K / 256;                       // at least 256 of K per slice
    S = S < max_s ? S : max_s;
    return S < 1 ? 1 : S;
}

cudaError_t launch_gemm_split(const float* A, int64_t sa0, int64_t sa1, const float* B, int64_t sb0, int64_t sb1,
                              float* C, int64_t ldc, int M, int N, int K, int accumulate, int S, float* partial,
                              cudaStream_t st) {
    if (S <= 1) return launch_gemm(A, sa0, sa1, B, sb0, sb1, C, ldc, M, N, K, accumulate, st);
    const int chunk = ((K + S - 1) / S + kGK - 1) / kGK * kGK;
    S = (K + chunk - 1) / chunk;
    dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT, S);
    k_gemm<<<grid, 256, 0, st>>>(A, sa0, sa1, B, sb0, sb1, partial, N, M, N, K, 0, chunk);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_sum_splits<<<grid_for(static_cast<int64_t>(M) * N, 256), 256, 0, st>>>(partial, S, M, N, C, ldc, accumulate);
    return cudaGetLastError();
}

cudaError_t launch_bias_relu(float* y, const float* b, int M, int N, float* out, cudaStream_t st) {
    k_bias_relu<<<grid_for(static_cast<int64_t>(M) * N, 256), 256, 0, st>>>(y, b, M, N, out);
    return cudaGetLastError();
}

cudaError_t launch_bias_grad(const float* g, int Nn, int K, int64_t inner, float* db, float* part, cudaStream_t st) {
    if (inner >= 4 && inner % 4 == 0 && part != nullptr) {
        // planes of a convolution gradient: one block per (image, channel),
        // then the Nn plane sums of each channel in order
        k_plane_sums<<<dim3(K, Nn), 256, 0, st>>>(g, K, inner, part);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        k_bias_grad<<<K, 256, 0, st>>>(part, Nn, K, 1, db);
        return cudaGetLastError();
    }
    k_bias_grad<<<K, 256, 0, st>>>(g, Nn, K, inner, db);
    return cudaGetLastError();
}

cudaError_t launch_relu_bwd(float* g, const float* pre, int64_t n, cudaStream_t st) {
    k_relu_bwd<<<grid_for(n, 256), 256, 0, st>>>(g, pre, n);
    return cudaGetLastError();
}

cudaError_t launch_mse(const float* pred, const float* t, int n, float* grad, double* loss, cudaStream_t st) {
    k_mse<<<1, 256, 0, st>>>(pred, t, n, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                        float eps, float c1, float c2, cudaStream_t st) {
    k_adam<<<grid_for(n, 256), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

}  // namespace octgb
