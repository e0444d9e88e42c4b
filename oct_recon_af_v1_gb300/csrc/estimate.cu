// Estimation kernels for sm_103a: the dispersion scorer and the depth
// profiles of the focus search.
//
// Dispersion (octrecon/estimation/dispersion.py:66-107): the B-scans are
// k-linearised and Hann/rms-windowed once (X, real); every candidate beta
// then costs one phase multiply, one inverse FFT and |.| per A-scan
// (dispersion.py:88-102), and a sharpness metric per B-scan over the depth
// pixels z >= 20 (dispersion.py:46-63).
//   k_disp_mag    one launch for a whole list of betas: 128 threads per
//                 A-scan load X and the beta's phase row straight into the
//                 registers of the first FFT stage, then the shared-memory
//                 Stockham FFT of the reconstruction kernel; |X| is averaged
//                 over the B-scan repeats (dispersion.py:101).
//   k_top_sum     top_percentile: one CTA per (beta, B-scan) finds the exact
//                 k-th largest magnitude by a three-digit radix select on the
//                 float bits (12 + 11 + 8 bits, histograms in shared memory),
//                 then sums I = float32(A^2) in float64 over the top k
//                 (elements above the threshold plus the ties needed), and
//                 returns log(sum / k).
//   k_moments     kurtosis, entropy, legacy_peak, one CTA per (beta, B-scan).
// Focus (octrecon/estimation/focus.py:146,156,255): k_xmedian takes the
// median over x of every depth column of (frames, nX, nZ) magnitudes, as
// float64, optionally ignoring NaN (nanmedian), by a bitonic sort per column
// in shared memory (one warp per column); or, in mean mode, the float64 mean
// of the column's non-NaN values.
#include <cuda_runtime.h>
#include <stdint.h>

#include "octgb_device.cuh"
#include "octgb_internal.h"

namespace octgb {
namespace {

struct DispSmem {
    alignas(16) float2 spec[kPerCta][kSpecStride];  // FFT work line per group
    alignas(16) float2 tw2[16][16];
    alignas(16) float2 tw3[8][256];
};

__global__ void __launch_bounds__(kThreads, 2) k_disp_mag(const DispArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    DispSmem& S = *reinterpret_cast<DispSmem*>(smem_raw);
    const int tid = threadIdx.x;
    const int g = tid / kGroup, lt = tid % kGroup;
    for (int k = tid; k < 16 * 16; k += kThreads) {
        const int r = k / 16, j = k % 16;
        S.tw2[r][j] = __ldg(a.tw + (r * j * (kN / 256)) % kN);
    }
    for (int k = tid; k < 8 * 256; k += kThreads) {
        const int r = k / 256, j = k % 256;
        S.tw3[r][j] = __ldg(a.tw + (r * j) % kN);
    }
    __syncthreads();
    // items < 2^32 - 2 kPerCta gridDim (the launcher checks): 32-bit item arithmetic
    const unsigned int nbx = static_cast<unsigned int>(a.nb) * static_cast<unsigned int>(a.nx);
    const unsigned int n_items = static_cast<unsigned int>(a.n_beta) * nbx;
    for (unsigned int item = blockIdx.x * kPerCta + g; item < n_items; item += gridDim.x * kPerCta) {
        const unsigned int gu = item / nbx, bx = item - gu * nbx;
        const unsigned int bu = bx / static_cast<unsigned int>(a.nx);
        const unsigned int x = bx - bu * static_cast<unsigned int>(a.nx);
        const float2* ph = a.phase + static_cast<int64_t>(gu) * kN;
        // repeat rp of A-scan x of B-scan b0 + bu: line0 + rp * nx * kN
        const float* line0 =
            a.X + ((static_cast<int64_t>(a.b0 + static_cast<int>(bu)) * a.rep) * a.nx + x) * kN;
        float acc[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[h][r] = 0.f;
        for (int rp = 0; rp < a.rep; ++rp) {
            const float* line = line0 + static_cast<int64_t>(rp) * a.nx * kN;
            float2 v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int j = lt + 128 * r;
                const float xv = __ldg(line + j);
                const float2 p = __ldg(ph + j);
                // complex64 (xv + 0i) * p, as numpy multiplies (dispersion.py:94)
                v[r] = make_float2(xv * p.x, xv * p.y);
            }
            float mag[2][4];
            ifft2048_low_mag_regs(v, S.spec[g], S.tw2, S.tw3, g, lt, mag);
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int r = 0; r < 4; ++r) acc[h][r] += mag[h][r];
        }
        if (a.zcol != nullptr) {
            // probe images: |X| into the group's (now free) line, then per image
            // row zi the sum over depths [zi z_keep / 256, ceil((zi + 1) z_keep / 256))
            float* M = reinterpret_cast<float*>(S.spec[g]);
            group_sync(g);                              // every thread has read the line's last stage
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    M[lt + 128 * h + 256 * r] = a.rep == 1 ? acc[h][r] : __fdiv_rn(acc[h][r], static_cast<float>(a.rep));
            group_sync(g);
            for (int zi = lt; zi < 256; zi += kGroup) {
                const int z0 = zi * a.z_keep / 256, z1 = ((zi + 1) * a.z_keep + 255) / 256;
                float sum = 0.f;
                for (int z = z0; z < z1; ++z) sum += M[z];
                a.zcol[static_cast<int64_t>(item) * 256 + zi] = sum;
            }
            continue;                                   // the next transform writes the line after a group barrier
        }
        float* out = a.A + static_cast<int64_t>(item) * kHalf;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int k = lt + 128 * h + 256 * r;
                // numpy's float32 mean over the repeats: sum, then divide
                out[k] = a.rep == 1 ? acc[h][r] : __fdiv_rn(acc[h][r], static_cast<float>(a.rep));
            }
    }
}

// ---------------------------------------------------------------- block helpers (1024 threads)
constexpr int kSelThreads = 1024;

// Inclusive prefix sum of one value per thread over the block.
__device__ __forceinline__ unsigned int block_inclusive_scan(unsigned int v, unsigned int* warp_tot) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
        unsigned int t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned int u = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += u;
        }
        warp_tot[lane] = t;                     // inclusive over warps
    }
    __syncthreads();
    const unsigned int off = w > 0 ? warp_tot[w - 1] : 0u;
    __syncthreads();
    return v + off;
}

// The bin (counted from the top) holding the need-th largest element, and the
// number of elements in the bins above it.  hist has nbins entries.
__device__ __forceinline__ void find_from_top(const unsigned int* hist, int nbins, unsigned int need,
                                              unsigned int* warp_tot, int* bin_out, unsigned int* above_out) {
    const int chunk = (nbins + kSelThreads - 1) / kSelThreads;
    const int lo = threadIdx.x * chunk, hi = min(lo + chunk, nbins);
    unsigned int c = 0;
    for (int b = lo; b < hi; ++b) c += hist[b];
    const unsigned int incl = block_inclusive_scan(c, warp_tot);
    __shared__ unsigned int total_s;
    if (threadIdx.x == kSelThreads - 1) total_s = incl;
    __syncthreads();
    const unsigned int above = total_s - incl;     // elements in bins >= hi
    if (c > 0 && above < need && above + c >= need) {
        unsigned int ab = above;
        for (int b = hi - 1; b >= lo; --b) {
            if (ab + hist[b] >= need) {
                *bin_out = b;
                *above_out = ab;
                break;
            }
            ab += hist[b];
        }
    }
    __syncthreads();
}

__device__ __forceinline__ double block_sum_f64(double v, double* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = red[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[0] = t;
    }
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

__device__ __forceinline__ double block_max_f64(double v, double* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = -__longlong_as_double(0x7ff0000000000000ll);
    if (w == 0) {
        t = red[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (lane == 0) red[0] = t;
    }
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

// One CTA per segment (beta, B-scan) of A (nx rows of kHalf magnitudes);
// thread t reads depth z_min + t of every row (z_min + 1024 >= kHalf).
__global__ void __launch_bounds__(kSelThreads, 1) k_top_sum(const float* __restrict__ A, int nx, int z_min,
                                                            unsigned int k, double* __restrict__ score) {
    __shared__ unsigned int hist[4096];
    __shared__ unsigned int warp_tot[32];
    __shared__ double red[32];
    __shared__ int bin_s;
    __shared__ unsigned int above_s;
    const float* seg = A + static_cast<int64_t>(blockIdx.x) * nx * kHalf;
    const int z = z_min + threadIdx.x;
    const bool act = z < kHalf;
    // pass 1: bits 31..19
    for (int b = threadIdx.x; b < 4096; b += kSelThreads) hist[b] = 0u;
    __syncthreads();
    if (act)
        for (int x = 0; x < nx; ++x) atomicAdd(&hist[__float_as_uint(seg[static_cast<int64_t>(x) * kHalf + z]) >> 19], 1u);
    __syncthreads();
    find_from_top(hist, 4096, k, warp_tot, &bin_s, &above_s);
    const unsigned int p1 = static_cast<unsigned int>(bin_s);
    unsigned int gt = above_s;
    __syncthreads();
    // pass 2: bits 18..8 among prefix p1
    for (int b = threadIdx.x; b < 2048; b += kSelThreads) hist[b] = 0u;
    __syncthreads();
    if (act)
        for (int x = 0; x < nx; ++x) {
            const unsigned int key = __float_as_uint(seg[static_cast<int64_t>(x) * kHalf + z]);
            if ((key >> 19) == p1) atomicAdd(&hist[(key >> 8) & 0x7ffu], 1u);
        }
    __syncthreads();
    find_from_top(hist, 2048, k - gt, warp_tot, &bin_s, &above_s);
    const unsigned int p2 = (p1 << 11) | static_cast<unsigned int>(bin_s);
    gt += above_s;
    __syncthreads();
    // pass 3: bits 7..0 among prefix p2
    for (int b = threadIdx.x; b < 256; b += kSelThreads) hist[b] = 0u;
    __syncthreads();
    if (act)
        for (int x = 0; x < nx; ++x) {
            const unsigned int key = __float_as_uint(seg[static_cast<int64_t>(x) * kHalf + z]);
            if ((key >> 8) == p2) atomicAdd(&hist[key & 0xffu], 1u);
        }
    __syncthreads();
    find_from_top(hist, 256, k - gt, warp_tot, &bin_s, &above_s);
    const unsigned int thr = (p2 << 8) | static_cast<unsigned int>(bin_s);
    gt += above_s;
    // pass 4: float64 sum of I = float32(A^2) above the threshold, in row order
    double s = 0.0;
    if (act)
        for (int x = 0; x < nx; ++x) {
            const float v = seg[static_cast<int64_t>(x) * kHalf + z];
            if (__float_as_uint(v) > thr) s += static_cast<double>(__fmul_rn(v, v));
        }
    s = block_sum_f64(s, red);
    if (threadIdx.x == 0) {
        const float tv = __uint_as_float(thr);
        const double top = s + static_cast<double>(k - gt) * static_cast<double>(__fmul_rn(tv, tv));
        score[blockIdx.x] = log(top / static_cast<double>(k));
    }
}

// metric 2 kurtosis: sum(I^2) / sum(I)^2; 3 entropy: sum(p log(p + 1e-30)),
// p = I / sum(I); 4 legacy_peak: max_z mean_x log(A + 1e-12) (float32 as the
// reference's arrays).  I = float64(float32(A^2)).
__global__ void __launch_bounds__(kSelThreads, 1) k_moments(const float* __restrict__ A, int nx, int z_min,
                                                            int metric, double* __restrict__ score) {
    __shared__ double red[32];
    const float* seg = A + static_cast<int64_t>(blockIdx.x) * nx * kHalf;
    const int z = z_min + threadIdx.x;
    const bool act = z < kHalf;
    if (metric == 4) {
        float L = 0.f;
        if (act)
            for (int x = 0; x < nx; ++x) L += logf(seg[static_cast<int64_t>(x) * kHalf + z] + 1e-12f);
        const double mean = act ? static_cast<double>(__fdiv_rn(L, static_cast<float>(nx)))
                                : -__longlong_as_double(0x7ff0000000000000ll);
        const double m = block_max_f64(mean, red);
        if (threadIdx.x == 0) score[blockIdx.x] = m;
        return;
    }
    double s1 = 0.0, s2 = 0.0;
    if (act)
        for (int x = 0; x < nx; ++x) {
            const float v = seg[static_cast<int64_t>(x) * kHalf + z];
            const double I = static_cast<double>(__fmul_rn(v, v));
            s1 += I;
            s2 += I * I;
        }
    s1 = block_sum_f64(s1, red);
    if (metric == 2) {
        s2 = block_sum_f64(s2, red);
        if (threadIdx.x == 0) score[blockIdx.x] = s2 / (s1 * s1);
        return;
    }
    double e = 0.0;
    if (act)
        for (int x = 0; x < nx; ++x) {
            const float v = seg[static_cast<int64_t>(x) * kHalf + z];
            const double p = static_cast<double>(__fmul_rn(v, v)) / s1;
            e += p * log(p + 1e-30);
        }
    e = block_sum_f64(e, red);
    if (threadIdx.x == 0) score[blockIdx.x] = e;
}

// ---------------------------------------------------------------- x-median
constexpr int kMedCols = 8;                       // depth columns per CTA (one warp each)
constexpr int kMedMaxX = 4096;

// mean_mode: the float64 mean of the non-NaN values instead of the median
__global__ void __launch_bounds__(kMedCols * 32) k_xmedian(const float* __restrict__ mag, int n_frames, int nx,
                                                          int nz, int p2, int ignore_nan, int mean_mode,
                                                          double* __restrict__ out) {
    extern __shared__ __align__(16) float col[];  // [kMedCols][p2]
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int f = blockIdx.y;
    const int z0 = blockIdx.x * kMedCols;
    // coalesced load of rows x, columns z0..z0+7; NaN and padding sort last
    __shared__ int n_nan[kMedCols];
    if (threadIdx.x < kMedCols) n_nan[threadIdx.x] = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < p2 * kMedCols; e += kMedCols * 32) {
        const int x = e / kMedCols, c = e % kMedCols;
        float v = __int_as_float(0x7f800000);
        if (x < nx && z0 + c < nz) {
            v = mag[(static_cast<int64_t>(f) * nx + x) * nz + z0 + c];
            if (isnan(v)) {
                atomicAdd(&n_nan[c], 1);
                v = __int_as_float(0x7f800000);
            }
        }
        col[c * p2 + x] = v;
    }
    __syncthreads();
    float* s = col + w * p2;
    if (mean_mode) {
        const int z = z0 + w;
        double acc = 0.0;
        for (int i = lane; i < nx; i += 32)
            if (!isinf(s[i])) acc += static_cast<double>(s[i]);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0 && z < nz) {
            const int n = nx - n_nan[w];
            out[static_cast<int64_t>(f) * nz + z] = n > 0 ? acc / n : __longlong_as_double(0x7ff8000000000000ll);
        }
        return;
    }
    for (int k = 2; k <= p2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < p2; i += 32) {
                const int l = i ^ j;
                if (l > i) {
                    const float a = s[i], b = s[l];
                    const bool up = (i & k) == 0;
                    if (up ? a > b : a < b) {
                        s[i] = b;
                        s[l] = a;
                    }
                }
            }
            __syncwarp();
        }
    const int z = z0 + w;
    if (lane == 0 && z < nz) {
        const int nn = n_nan[w];
        double m;
        if (nn > 0 && !ignore_nan) {
            m = __longlong_as_double(0x7ff8000000000000ll);
        } else {
            const int n = nx - nn;
            if (n == 0)
                m = __longlong_as_double(0x7ff8000000000000ll);
            else if (n & 1)
                m = static_cast<double>(s[n / 2]);
            else
                m = (static_cast<double>(s[n / 2 - 1]) + static_cast<double>(s[n / 2])) / 2.0;
        }
        out[static_cast<int64_t>(f) * nz + z] = m;
    }
}

}  // namespace

cudaError_t launch_disp_mag(const DispArgs& a, int num_sms, cudaStream_t st) {
    const size_t smem = sizeof(DispSmem);
    cudaError_t e = cudaFuncSetAttribute(k_disp_mag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    const int64_t items = static_cast<int64_t>(a.n_beta) * a.nb * a.nx;
    if (items >= (int64_t(1) << 32) - 2 * kPerCta * num_sms) return cudaErrorInvalidValue;   // 32-bit item index
    int64_t grid = (items + kPerCta - 1) / kPerCta;
    if (grid > 2 * num_sms) grid = 2 * num_sms;
    k_disp_mag<<<static_cast<int>(grid), kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_disp_metric(const float* A, int n_seg, int nx, int z_min, int metric, unsigned int top_k,
                               double* score, cudaStream_t st) {
    if (metric == 1)
        k_top_sum<<<n_seg, kSelThreads, 0, st>>>(A, nx, z_min, top_k, score);
    else
        k_moments<<<n_seg, kSelThreads, 0, st>>>(A, nx, z_min, metric, score);
    return cudaGetLastError();
}

cudaError_t launch_xmedian(const float* mag, int n_frames, int nx, int nz, int ignore_nan, int mean_mode,
                           double* out, cudaStream_t st) {
    int p2 = 32;
    while (p2 < nx) p2 <<= 1;
    if (p2 > kMedMaxX) return cudaErrorInvalidValue;
    const size_t smem = static_cast<size_t>(kMedCols) * p2 * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(k_xmedian, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    dim3 grid((nz + kMedCols - 1) / kMedCols, n_frames);
    k_xmedian<<<grid, kMedCols * 32, smem, st>>>(mag, n_frames, nx, nz, p2, ignore_nan, mean_mode, out);
    return cudaGetLastError();
}

}  // namespace octgb
