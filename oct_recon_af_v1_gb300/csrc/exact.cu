// Float64 form of the spectral stage for sm_103a: the reference's
// SpectralProcessor at precision "float64" (octrecon/core/spectral.py:123-165,
// NumPy path), raw integer counts -> |ifft| rounded once to float32.
//
// Per A-scan (group of 128 threads, two A-scans per CTA):
//   background, exactly: with S_j the integer sum of the apodisation lines and
//     A their count, interf_j = raw_j - S_j / A = n_j / A for the integer
//     n_j = A raw_j - S_j; the line mean is sum(n) / (2048 A) and the
//     background-free sample d_j = N_j / (2048 A) with the integer
//     N_j = 2048 n_j - sum(n) (|N_j| < 2^53: exact in float64);
//   sinc: lin_i = (sum_t w[t,i] N[start_i + t] + sum(n)) / (2048 A), float64
//     fused multiply-adds over the float64 band weights in the reference's
//     tap order (core/spectral.py:128-134);
//   window (Hann/rms x dispersion phase, 1/N folded in), float64 complex;
//   inverse FFT, Stockham radix 16, 16, 8 in float64 (last stage pruned to
//     k < N/2), |X| in float64 rounded to float32.
// Thread lt computes the sinc outputs its first FFT stage takes (samples
// lt + 128 r), so the line goes from the sinc to the FFT in registers; the
// band weights (tap-major, coalesced) are read through L1 for every A-scan.
// GB300 executes float64 at a small fraction of its float32 rate: this form is
// the accurate one, not the fast one.
#include <cuda_runtime.h>
#include <stdint.h>

#include "octgb_internal.h"

namespace octgb {
namespace {

constexpr int kXGroup = 128;                    // threads per A-scan
constexpr int kXPerCta = 2;                     // A-scans per CTA
constexpr int kXThreads = kXGroup * kXPerCta;
constexpr int kXStride = kN + (kN >> 4);        // padded complex line (one slot per 16)
constexpr int kXTail = 32;                      // zero tail of the integer line (padded taps)

__device__ __forceinline__ int xpad(int e) { return e + (e >> 4); }

__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 dsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 dmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 dmuli(double2 a) { return make_double2(-a.y, a.x); }

__device__ __forceinline__ void ddft4(double2& x0, double2& x1, double2& x2, double2& x3) {
    const double2 a = dadd(x0, x2), b = dsub(x0, x2), c = dadd(x1, x3), d = dmuli(dsub(x1, x3));
    x0 = dadd(a, c);
    x2 = dsub(a, c);
    x1 = dadd(b, d);
    x3 = dsub(b, d);
}

constexpr double kDC1 = 0.92387953251128675613;   // cos(pi/8)
constexpr double kDS1 = 0.38268343236508977173;   // sin(pi/8)
constexpr double kDC2 = 0.70710678118654752440;   // cos(pi/4)

// inverse DFT-16 as 4 x 4 (the float32 kernel's decomposition, in float64)
__device__ __forceinline__ void ddft16(double2 (&v)[16]) {
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) ddft4(v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]);
    v[1 + 4] = dmul(v[1 + 4], make_double2(kDC1, kDS1));
    v[1 + 8] = dmul(v[1 + 8], make_double2(kDC2, kDC2));
    v[1 + 12] = dmul(v[1 + 12], make_double2(kDS1, kDC1));
    v[2 + 4] = dmul(v[2 + 4], make_double2(kDC2, kDC2));
    v[2 + 8] = dmuli(v[2 + 8]);
    v[2 + 12] = dmul(v[2 + 12], make_double2(-kDC2, kDC2));
    v[3 + 4] = dmul(v[3 + 4], make_double2(kDS1, kDC1));
    v[3 + 8] = dmul(v[3 + 8], make_double2(-kDC2, kDC2));
    v[3 + 12] = dmul(v[3 + 12], make_double2(-kDC1, -kDS1));
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) ddft4(v[4 * k2], v[4 * k2 + 1], v[4 * k2 + 2], v[4 * k2 + 3]);
    double2 t;
    t = v[1]; v[1] = v[4]; v[4] = t;
    t = v[2]; v[2] = v[8]; v[8] = t;
    t = v[3]; v[3] = v[12]; v[12] = t;
    t = v[6]; v[6] = v[9]; v[9] = t;
    t = v[7]; v[7] = v[13]; v[13] = t;
    t = v[11]; v[11] = v[14]; v[14] = t;
}

__device__ __forceinline__ void ddft8_low(double2 (&v)[8], double2 (&X)[4]) {
    ddft4(v[0], v[2], v[4], v[6]);
    ddft4(v[1], v[3], v[5], v[7]);
    const double2 y1 = dmul(v[3], make_double2(kDC2, kDC2));
    const double2 y2 = dmuli(v[5]);
    const double2 y3 = dmul(v[7], make_double2(-kDC2, kDC2));
    X[0] = dadd(v[0], v[1]);
    X[1] = dadd(v[2], y1);
    X[2] = dadd(v[4], y2);
    X[3] = dadd(v[6], y3);
}

__device__ __forceinline__ void xgroup_sync(int g) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kXGroup) : "memory");
}

template <typename RawT>
__device__ __forceinline__ int raw_int(const RawT* p, int j) {
    return static_cast<int>(p[j]);
}

// integer sums of the apodisation lines, (B, N)
template <typename RawT>
__global__ void k_exact_apod_sum(const RawT* __restrict__ raw, int interf, int apod, int* __restrict__ sums) {
    const int b = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= kN) return;
    const RawT* p = raw + static_cast<int64_t>(b) * interf * kN + j;
    int s = 0;
    for (int k = 0; k < apod; ++k) s += static_cast<int>(p[static_cast<int64_t>(k) * kN]);
    sums[static_cast<int64_t>(b) * kN + j] = s;
}

template <typename RawT>
__global__ void __launch_bounds__(kXThreads, 1) k_exact(const ExactArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* dl = reinterpret_cast<double*>(smem_raw);                       // [kXPerCta][kN + kXTail]
    double2* L0 = reinterpret_cast<double2*>(dl + kXPerCta * (kN + kXTail));  // [kXPerCta][kXStride]
    double2* L1 = L0 + kXPerCta * kXStride;
    double2* tw2 = L1 + kXPerCta * kXStride;                                  // [16][16]
    double2* tw3 = tw2 + 16 * 16;                                             // [8][256]
    __shared__ long long red[kXPerCta][4];

    const int tid = threadIdx.x, g = tid / kXGroup, lt = tid % kXGroup;
    const int warp = tid >> 5, lane = tid & 31;
    for (int k = tid; k < 16 * 16; k += kXThreads) {
        const int r = k / 16, j = k % 16;
        tw2[k] = a.tw[(r * j * (kN / 256)) % kN];
    }
    for (int k = tid; k < 8 * 256; k += kXThreads) {
        const int r = k / 256, j = k % 256;
        tw3[k] = a.tw[(r * j) % kN];
    }
    for (int k = tid; k < kXPerCta * kXTail; k += kXThreads) dl[(k / kXTail) * (kN + kXTail) + kN + k % kXTail] = 0.0;
    __syncthreads();

    double* D = dl + g * (kN + kXTail);
    double2* X0 = L0 + g * kXStride;
    double2* X1 = L1 + g * kXStride;
    const double inv = 1.0 / (2048.0 * a.apod);            // one rounding, as the mean's division
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * kXPerCta; base < a.n_ascans;
         base += static_cast<int64_t>(gridDim.x) * kXPerCta) {
        const int64_t as = base + g;
        const bool valid = as < a.n_ascans;
        const int64_t asc = valid ? as : 0;
        const int64_t b = asc / a.nx, x = asc - b * a.nx;
        const RawT* row = static_cast<const RawT*>(a.raw) + ((b * a.interf + a.apod + x) * kN);
        const int* S = a.apod_sum + b * kN;
        // ---- background: integer n_j and their sum
        long long nj[16];
        long long sum = 0;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const int j = lt + 128 * r;
            nj[r] = static_cast<long long>(a.apod) * raw_int(row, j) - __ldg(S + j);
            sum += nj[r];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) red[g][warp & 3] = sum;
        xgroup_sync(g);
        const long long sn = (red[g][0] + red[g][1]) + (red[g][2] + red[g][3]);
#pragma unroll
        for (int r = 0; r < 16; ++r) D[lt + 128 * r] = static_cast<double>(2048LL * nj[r] - sn);
        xgroup_sync(g);
        // ---- sinc + window: the outputs lt + 128 r (this thread's first FFT stage)
        double2 v[16];
        const double dsn = static_cast<double>(sn);
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const int i = lt + 128 * r;
            const int s = __ldg(a.start + i);
            double acc = 0.0;
            for (int t = 0; t < a.taps; ++t) acc = fma(__ldg(a.w + static_cast<int64_t>(t) * kN + i), D[s + t], acc);
            const double lin = (acc + dsn) * inv;
            const double2 wv = __ldg(a.win + i);
            v[r] = make_double2(lin * wv.x, lin * wv.y);
        }
        // ---- inverse FFT: stage 1 from registers into X0, stage 2 into X1, stage 3
        ddft16(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) X0[xpad(16 * lt + r)] = v[r];
        xgroup_sync(g);
        {
            const int jm = lt & 15;
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = X0[xpad(lt + 128 * r)];
#pragma unroll
            for (int r = 1; r < 16; ++r) v[r] = dmul(v[r], tw2[r * 16 + jm]);
            ddft16(v);
            const int idxD = (lt >> 4) * 256 + jm;
#pragma unroll
            for (int r = 0; r < 16; ++r) X1[xpad(idxD + 16 * r)] = v[r];
        }
        xgroup_sync(g);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = lt + 128 * h;
            double2 w8[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) w8[r] = X1[xpad(j + 256 * r)];
#pragma unroll
            for (int r = 1; r < 8; ++r) w8[r] = dmul(w8[r], tw3[r * 256 + j]);
            double2 Xk[4];
            ddft8_low(w8, Xk);
            if (valid) {
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    a.mag[as * kHalf + j + 256 * r] =
                        static_cast<float>(sqrt(fma(Xk[r].x, Xk[r].x, Xk[r].y * Xk[r].y)));
            }
        }
        // the next A-scan writes D and X0 only after this group's barriers above,
        // and X1 after its own first barrier: every read of this one is done
    }
}

template <typename RawT>
cudaError_t launch_exact_t(const ExactArgs& a, int* sums, int num_sms, cudaStream_t st) {
    const dim3 sgrid(kN / 256, a.B);
    k_exact_apod_sum<RawT><<<sgrid, 256, 0, st>>>(static_cast<const RawT*>(a.raw), a.interf, a.apod, sums);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t smem = static_cast<size_t>(kXPerCta) * (kN + kXTail) * sizeof(double) +
                        static_cast<size_t>(2 * kXPerCta * kXStride + 16 * 16 + 8 * 256) * sizeof(double2);
    e = cudaFuncSetAttribute(k_exact<RawT>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    const int64_t pairs = (a.n_ascans + kXPerCta - 1) / kXPerCta;
    const int grid = static_cast<int>(pairs < num_sms ? pairs : num_sms);
    ExactArgs b = a;
    b.apod_sum = sums;
    k_exact<RawT><<<grid, kXThreads, smem, st>>>(b);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_exact(const ExactArgs& a, int dtype, int* sums, int num_sms, cudaStream_t st) {
    if (dtype == 0) return launch_exact_t<uint16_t>(a, sums, num_sms, st);
    if (dtype == 1) return launch_exact_t<int16_t>(a, sums, num_sms, st);
    return cudaErrorInvalidValue;
}

}  // namespace octgb
