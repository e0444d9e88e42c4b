// Precision form of the spectral stage: the banded sinc k-linearisation on
// the 5th-generation tensor cores (tcgen05), split-FP16 with three products.
//
//   k_apod_sum + k_prec_split_int  the background exactly (the float32 form
//                 keeps the reference's float32 apodisation store, whose
//                 rounding dominates its error against float64): for integer
//                 raws d' = raw - apod - m (core/cpu_kernels.py:20-36) is an
//                 exact int64 ratio rounded twice in float32 (float64 for
//                 float32 raws, k_apod_mean64 + k_prec_split_f32), then split
//                 into fp16 hi = rn(d') and lo = rn(d' - hi) (22 significant
//                 bits together).
//   k_prec_sinc   X[a][i] = sum_j W[i][j] d'[a][j] + m[a] (cpu_kernels.py:
//                 37-41 without the window): a GEMM with M = 128 A-scans, N =
//                 64 output samples, K = the 96-sample source window of the
//                 output block (the band follows the chirp; the window start
//                 kb is per block).  D = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T
//                 accumulates in TMEM (float32).  W is pre-scaled by 64 (exact;
//                 keeps the fp16 lo parts of small weights normal) and split on
//                 the host into hi/lo tiles already in the canonical no-swizzle
//                 K-major layout (core matrices of 8 rows x 16 bytes).
//                 Warp roles, one CTA per SM, persistent over 128-A-scan tiles:
//                   warp 4 lane 0  producer: per block, 12 + 12 two-dimensional
//                                  TMA loads (cp.async.bulk.tensor, 8 samples x
//                                  128 A-scans each) of d' hi/lo and two bulk
//                                  copies of the W tiles, into one of 2 stages;
//                   warp 5 lane 0  MMA issuer: 6 K-steps x 3 products of
//                                  tcgen05.mma (M128 N64 K16), commit to the
//                                  stage's empty barrier and the accumulator's
//                                  full barrier; 2 accumulators of 64 TMEM
//                                  columns alternate;
//                   warps 0-3      epilogue: tcgen05.ld of their 32 TMEM lanes
//                                  (A-scans) x 64 columns, X = D / 64 + m.
//                 Every mbarrier wait is bounded (2 s); on expiry the CTA
//                 records the status, drains its copies and MMAs, frees TMEM
//                 and returns.
// The FFT and |.| of the precision form are k_disp_mag's (estimate.cu) with
// the geometry's window as the phase row.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <vector>

#include "octgb_device.cuh"
#include "octgb_internal.h"

namespace octgb {
namespace {

constexpr uint32_t kAChunkBytes = kPM * 16;                  // 8 samples of 128 A-scans
constexpr uint32_t kATileBytes = kPChunks * kAChunkBytes;    // 24576
constexpr uint32_t kBChunkBytes = kPN * 16;                  // 8 samples of 64 outputs
constexpr uint32_t kBTileBytes = kPChunks * kBChunkBytes;    // 12288
constexpr uint32_t kStageBytes = 2 * kATileBytes + 2 * kBTileBytes;
constexpr int kPStages = 2;
constexpr int kPThreads = 192;

struct PrecSmem {
    alignas(1024) uint8_t stage[kPStages][kStageBytes];      // A_hi | A_lo | B_hi | B_lo
    // every byte a descriptor of either operand layout could address stays
    // inside the allocation
    uint8_t slack[16384];
    uint64_t full[kPStages], empty[kPStages], tfull[2], tempty[2], drain;
    uint32_t tmem_base;
    int abort;
};

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// kind::f16 instruction descriptor: f16 x f16 -> f32, K-major A and B, M = 128, N = 64
constexpr uint32_t kIdesc = mma_idesc_f16(kPM, kPN);

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    mma_f16_id(d_tmem, a, b, kIdesc, accumulate);
}

__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, PrecSmem& S, int* status) {
    if (*reinterpret_cast<volatile int*>(&S.abort)) return false;
    if (mbar_wait_bounded(bar, parity, status)) return true;
    atomicExch(&S.abort, 1);
    return false;
}

__global__ void __launch_bounds__(kPThreads, 1)
    k_prec_sinc(const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo,
                const uint8_t* __restrict__ wtiles, const int* __restrict__ kb, const float* __restrict__ mline,
                float* __restrict__ X, int64_t n_ascans, int* status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // tensor-copy destinations want 128-byte alignment: align the window by hand
    PrecSmem& S = *reinterpret_cast<PrecSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t n_tiles = (n_ascans + kPM - 1) / kPM;
    const int64_t my_tiles = blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t n_q = my_tiles * kPBlocks;                   // (tile, block) steps of this CTA

    if (tid == 0) {
        for (int s = 0; s < kPStages; ++s) {
            mbar_init(&S.full[s], 1);
            mbar_init(&S.empty[s], 1);
        }
        for (int d = 0; d < 2; ++d) {
            mbar_init(&S.tfull[d], 1);
            mbar_init(&S.tempty[d], 4);
        }
        mbar_init(&S.drain, 1);
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&S.tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;

    if (warp == 4 && lane == 0) {
        // ---------------- producer
        int64_t q = 0;
        for (; q < n_q; ++q) {
            const int s = static_cast<int>(q % kPStages);
            const uint32_t ph = static_cast<uint32_t>(q / kPStages) & 1u;
            if (!wait_or_abort(&S.empty[s], ph ^ 1u, S, status)) break;
            const int64_t tile = blockIdx.x + (q / kPBlocks) * gridDim.x;
            const int b = static_cast<int>(q % kPBlocks);
            uint8_t* st = S.stage[s];
            mbar_expect_tx(&S.full[s], kStageBytes + starved_bytes(q == 0));
            const int x0 = kb[b], y0 = static_cast<int>(tile * kPM);
            for (int c = 0; c < kPChunks; ++c) {
                tma_load_2d(st + c * kAChunkBytes, &tm_hi, x0 + 8 * c, y0, &S.full[s]);
                tma_load_2d(st + kATileBytes + c * kAChunkBytes, &tm_lo, x0 + 8 * c, y0, &S.full[s]);
            }
            const uint8_t* wsrc = wtiles + static_cast<size_t>(b) * 2 * kBTileBytes;
            tma_bulk_g2s(st + 2 * kATileBytes, wsrc, kBTileBytes, &S.full[s]);
            tma_bulk_g2s(st + 2 * kATileBytes + kBTileBytes, wsrc + kBTileBytes, kBTileBytes, &S.full[s]);
        }
        // drain: copies still in flight land before the CTA's memory is released
        for (int64_t r = q - kPStages; r < q; ++r) {
            if (r < 0) continue;
            mbar_wait_bounded(&S.full[r % kPStages], static_cast<uint32_t>(r / kPStages) & 1u, status);
        }
    } else if (warp == 5 && lane == 0) {
        // ---------------- MMA issuer
        for (int64_t q = 0; q < n_q; ++q) {
            const int s = static_cast<int>(q % kPStages);
            const uint32_t ph = static_cast<uint32_t>(q / kPStages) & 1u;
            const int d = static_cast<int>(q & 1);
            const uint32_t dph = static_cast<uint32_t>(q >> 1) & 1u;
            if (!wait_or_abort(&S.full[s], ph, S, status)) break;
            if (!wait_or_abort(&S.tempty[d], dph ^ 1u, S, status)) break;
            tc_fence_after();
            const uint32_t dt = tmem + static_cast<uint32_t>(d * kPN);
            const uint8_t* st = S.stage[s];
#pragma unroll
            for (int k = 0; k < kPKW / 16; ++k) {
                const uint64_t ah = smem_desc(st + k * 2 * kAChunkBytes, kAChunkBytes, 128);
                const uint64_t al = smem_desc(st + kATileBytes + k * 2 * kAChunkBytes, kAChunkBytes, 128);
                const uint64_t bh = smem_desc(st + 2 * kATileBytes + k * 2 * kBChunkBytes, kBChunkBytes, 128);
                const uint64_t bl = smem_desc(st + 2 * kATileBytes + kBTileBytes + k * 2 * kBChunkBytes, kBChunkBytes,
                                              128);
                mma_f16(dt, ah, bh, k > 0 ? 1u : 0u);
                mma_f16(dt, ah, bl, 1u);
                mma_f16(dt, al, bh, 1u);
            }
            mma_commit(&S.empty[s]);
            mma_commit(&S.tfull[d]);
        }
        // drain: every MMA issued has completed
        mma_commit(&S.drain);
        mbar_wait_bounded(&S.drain, 0, status);
    } else if (warp < 4) {
        // ---------------- epilogue
        const uint32_t lane_base = static_cast<uint32_t>(32 * warp) << 16;
        for (int64_t q = 0; q < n_q; ++q) {
            const int d = static_cast<int>(q & 1);
            const uint32_t dph = static_cast<uint32_t>(q >> 1) & 1u;
            bool ok = true;
            if (lane == 0) ok = wait_or_abort(&S.tfull[d], dph, S, status);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            tc_fence_after();
            float v[2][32];
            tmem_ld32(tmem + lane_base + static_cast<uint32_t>(d * kPN), v[0]);
            tmem_ld32(tmem + lane_base + static_cast<uint32_t>(d * kPN + 32), v[1]);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.tempty[d]);
            const int64_t tile = blockIdx.x + (q / kPBlocks) * gridDim.x;
            const int b = static_cast<int>(q % kPBlocks);
            const int64_t a = tile * kPM + 32 * warp + lane;
            if (a < n_ascans) {
                const float m = mline[a];
                float4* out = reinterpret_cast<float4*>(X + a * kN + b * kPN);
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                        out[h * 8 + c] = make_float4(fmaf(v[h][4 * c], 1.0f / 64, m), fmaf(v[h][4 * c + 1], 1.0f / 64, m),
                                                     fmaf(v[h][4 * c + 2], 1.0f / 64, m),
                                                     fmaf(v[h][4 * c + 3], 1.0f / 64, m));
            }
        }
    }
    __syncwarp();                                       // role lanes rejoin their warps
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
}

// ---------------------------------------------------------------------------
// Fused variant for integer raws (k_prec_sinc_raw): the raw uint16/int16
// window of each block arrives by three-dimensional tensor copies (samples x
// A-scans x B-scans, tiles of 128 A-scans inside one B-scan, rows past the
// B-scan zero-filled) and twelve converter warps form d' in shared memory
// from it: n = apod * raw - S is an exact integer below 2^24, so
// d' = fma(n, 1/apod, -m) takes one float32 rounding relative to
// max(|d|, |m|) (m from k_prec_rowsum); they write the fp16 hi/lo operand
// tiles in the canonical layout, so d' never reaches global memory.  Roles:
// warps 0-3 epilogue, 4-15 converters, warp 16 lane 0 copies, warp 17 lane 0
// MMAs.
constexpr int kRConvWarps = 12;
constexpr int kRThreads = (4 + kRConvWarps + 2) * 32;
constexpr uint32_t kRawTileBytes = kPChunks * kAChunkBytes;            // 12 chunks of 8 samples x 128 rows, 2 B
constexpr uint32_t kRStageBytes = kRawTileBytes + 2 * kATileBytes + 2 * kBTileBytes;
constexpr uint32_t kRLoadBytes = kRawTileBytes + 2 * kBTileBytes + kPKW * 4;   // bytes the copies deliver per block


struct RawSmem {
    alignas(1024) uint8_t stage[kPStages][kRStageBytes];   // raw | A_hi | A_lo | B_hi | B_lo
    alignas(16) int sw[kPStages][kPKW];                     // S[b][kb .. kb + 96) of the block
    uint64_t full[kPStages], conv[kPStages], empty[kPStages], tfull[2], tempty[2], drain;
    uint32_t tmem_base;
    int abort;
};

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool wait_or_abort_r(uint64_t* bar, uint32_t parity, RawSmem& S, int* status) {
    if (*reinterpret_cast<volatile int*>(&S.abort)) return false;
    if (mbar_wait_bounded(bar, parity, status)) return true;
    atomicExch(&S.abort, 1);
    return false;
}

template <typename RawT>
__global__ void __launch_bounds__(kRThreads, 1)
    k_prec_sinc_raw(const __grid_constant__ CUtensorMap tm_raw, const uint8_t* __restrict__ wtiles,
                    const int* __restrict__ kb, const int* __restrict__ apod_sum,
                    const long long* __restrict__ sum_n, const float* __restrict__ mline, float* __restrict__ X,
                    int B, int nx, int apod, int* status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    RawSmem& S = *reinterpret_cast<RawSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int xtiles = (nx + kPM - 1) / kPM;
    const int64_t n_tiles = static_cast<int64_t>(B) * xtiles;
    const int64_t my_tiles = blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t n_q = my_tiles * kPBlocks;
    const float inv_apod = 1.0f / static_cast<float>(apod);

    if (tid == 0) {
        for (int s = 0; s < kPStages; ++s) {
            mbar_init(&S.full[s], 1);
            mbar_init(&S.conv[s], kRConvWarps);
            mbar_init(&S.empty[s], 1);
        }
        for (int d = 0; d < 2; ++d) {
            mbar_init(&S.tfull[d], 1);
            mbar_init(&S.tempty[d], 4);
        }
        mbar_init(&S.drain, 1);
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&S.tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;

    if (warp == 4 + kRConvWarps && lane == 0) {
        // ---------------- copies
        int64_t q = 0;
        for (; q < n_q; ++q) {
            const int s = static_cast<int>(q % kPStages);
            const uint32_t ph = static_cast<uint32_t>(q / kPStages) & 1u;
            if (!wait_or_abort_r(&S.empty[s], ph ^ 1u, S, status)) break;
            const int64_t tile = blockIdx.x + (q / kPBlocks) * gridDim.x;
            const int b = static_cast<int>(q % kPBlocks);
            const int bs = static_cast<int>(tile / xtiles), xt = static_cast<int>(tile % xtiles);
            uint8_t* st = S.stage[s];
            mbar_expect_tx(&S.full[s], kRLoadBytes + starved_bytes(q == 0));
            for (int c = 0; c < kPChunks; ++c)
                tma_load_3d(st + c * kAChunkBytes, &tm_raw, kb[b] + 8 * c, xt * kPM, bs, &S.full[s]);
            const uint8_t* wsrc = wtiles + static_cast<size_t>(b) * 2 * kBTileBytes;
            uint8_t* bdst = st + kRawTileBytes + 2 * kATileBytes;
            tma_bulk_g2s(bdst, wsrc, kBTileBytes, &S.full[s]);
            tma_bulk_g2s(bdst + kBTileBytes, wsrc + kBTileBytes, kBTileBytes, &S.full[s]);
            // the window's apodisation sums (the buffer is padded past the last B-scan)
            tma_bulk_g2s(S.sw[s], apod_sum + static_cast<int64_t>(bs) * kN + kb[b], kPKW * 4, &S.full[s]);
        }
        for (int64_t r = q - kPStages; r < q; ++r) {
            if (r < 0) continue;
            mbar_wait_bounded(&S.full[r % kPStages], static_cast<uint32_t>(r / kPStages) & 1u, status);
        }
    } else if (warp >= 4 && warp < 4 + kRConvWarps) {
        // ---------------- converters: raw window -> d' hi/lo operand tiles
        const int ct = tid - 128;
        for (int64_t q = 0; q < n_q; ++q) {
            const int s = static_cast<int>(q % kPStages);
            const uint32_t ph = static_cast<uint32_t>(q / kPStages) & 1u;
            bool ok = true;
            if (lane == 0) ok = wait_or_abort_r(&S.full[s], ph, S, status);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            const int64_t tile = blockIdx.x + (q / kPBlocks) * gridDim.x;
            const int b = static_cast<int>(q % kPBlocks);
            const int bs = static_cast<int>(tile / xtiles), xt = static_cast<int>(tile % xtiles);
            const int j0 = kb[b];
            uint8_t* st = S.stage[s];
            const int* sw = S.sw[s];
            // a thread's items all lie in one row (the stride is a multiple of 128)
            const int row = ct % kPM;
            const int x = xt * kPM + row;
            const float m = x < nx ? mline[static_cast<int64_t>(bs) * nx + x] : 0.f;
            for (int i = ct; i < kPChunks * kPM; i += kRConvWarps * 32) {
                const int c = i / kPM;
                const uint4 rv = *reinterpret_cast<const uint4*>(st + c * kAChunkBytes + row * 16);
                const int4 sa = *reinterpret_cast<const int4*>(sw + 8 * c);
                const int4 sb = *reinterpret_cast<const int4*>(sw + 8 * c + 4);
                const int sv[8] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y, sb.z, sb.w};
                const uint32_t words[4] = {rv.x, rv.y, rv.z, rv.w};
                const bool in_row = j0 + 8 * c + 8 <= kN;         // samples past N are never used
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int e2 = 0; e2 < 4; ++e2) {
                    float v[2];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const uint32_t u = (words[e2] >> (16 * h)) & 0xffffu;
                        const int rawv = static_cast<RawT>(-1) < 0 ? static_cast<int>(static_cast<int16_t>(u))
                                                                   : static_cast<int>(u);
                        // n = apod (raw - apod mean), an exact integer below 2^24: exact in
                        // float32, so d' = n / apod - m takes one rounding (fma)
                        const int n = in_row ? apod * rawv - sv[2 * e2 + h] : 0;
                        v[h] = fmaf(static_cast<float>(n), inv_apod, -m);
                    }
                    const __half2 hv = __floats2half2_rn(v[0], v[1]);
                    const float2 hf = __half22float2(hv);
                    const __half2 lv = __floats2half2_rn(v[0] - hf.x, v[1] - hf.y);
                    hw[e2] = *reinterpret_cast<const uint32_t*>(&hv);
                    lw[e2] = *reinterpret_cast<const uint32_t*>(&lv);
                }
                *reinterpret_cast<uint4*>(st + kRawTileBytes + c * kAChunkBytes + row * 16) =
                    make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4*>(st + kRawTileBytes + kATileBytes + c * kAChunkBytes + row * 16) =
                    make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            // generic-proxy writes become visible to the tensor cores' (async) reads
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.conv[s]);
        }
    } else if (warp == 5 + kRConvWarps && lane == 0) {
        // ---------------- MMA issuer
        for (int64_t q = 0; q < n_q; ++q) {
            const int s = static_cast<int>(q % kPStages);
            const uint32_t ph = static_cast<uint32_t>(q / kPStages) & 1u;
            const int d = static_cast<int>(q & 1);
            const uint32_t dph = static_cast<uint32_t>(q >> 1) & 1u;
            if (!wait_or_abort_r(&S.conv[s], ph, S, status)) break;
            if (!wait_or_abort_r(&S.tempty[d], dph ^ 1u, S, status)) break;
            tc_fence_after();
            const uint32_t dt = tmem + static_cast<uint32_t>(d * kPN);
            const uint8_t* A = S.stage[s] + kRawTileBytes;
            const uint8_t* Bw = A + 2 * kATileBytes;
#pragma unroll
            for (int k = 0; k < kPKW / 16; ++k) {
                const uint64_t ah = smem_desc(A + k * 2 * kAChunkBytes, kAChunkBytes, 128);
                const uint64_t al = smem_desc(A + kATileBytes + k * 2 * kAChunkBytes, kAChunkBytes, 128);
                const uint64_t bh = smem_desc(Bw + k * 2 * kBChunkBytes, kBChunkBytes, 128);
                const uint64_t bl = smem_desc(Bw + kBTileBytes + k * 2 * kBChunkBytes, kBChunkBytes, 128);
                mma_f16(dt, ah, bh, k > 0 ? 1u : 0u);
                mma_f16(dt, ah, bl, 1u);
                mma_f16(dt, al, bh, 1u);
            }
            mma_commit(&S.empty[s]);
            mma_commit(&S.tfull[d]);
        }
        mma_commit(&S.drain);
        mbar_wait_bounded(&S.drain, 0, status);
    } else if (warp < 4) {
        // ---------------- epilogue
        const uint32_t lane_base = static_cast<uint32_t>(32 * warp) << 16;
        for (int64_t q = 0; q < n_q; ++q) {
            const int d = static_cast<int>(q & 1);
            const uint32_t dph = static_cast<uint32_t>(q >> 1) & 1u;
            bool ok = true;
            if (lane == 0) ok = wait_or_abort_r(&S.tfull[d], dph, S, status);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            tc_fence_after();
            float v[2][32];
            tmem_ld32(tmem + lane_base + static_cast<uint32_t>(d * kPN), v[0]);
            tmem_ld32(tmem + lane_base + static_cast<uint32_t>(d * kPN + 32), v[1]);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.tempty[d]);
            const int64_t tile = blockIdx.x + (q / kPBlocks) * gridDim.x;
            const int b = static_cast<int>(q % kPBlocks);
            const int bs = static_cast<int>(tile / xtiles), xt = static_cast<int>(tile % xtiles);
            const int x = xt * kPM + 32 * warp + lane;
            if (x < nx) {
                const int64_t a = static_cast<int64_t>(bs) * nx + x;
                const float m = mline[a];
                float4* out = reinterpret_cast<float4*>(X + a * kN + b * kPN);
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                        out[h * 8 + c] = make_float4(fmaf(v[h][4 * c], 1.0f / 64, m), fmaf(v[h][4 * c + 1], 1.0f / 64, m),
                                                     fmaf(v[h][4 * c + 2], 1.0f / 64, m),
                                                     fmaf(v[h][4 * c + 3], 1.0f / 64, m));
            }
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
}

// Line sums of the integer numerators: sum_n[a] = sum_j (apod raw_j - S_j),
// mline[a] = sum_n / (2048 apod) (the line mean of d).  One warp per A-scan.
template <typename RawT>
__global__ void __launch_bounds__(256) k_prec_rowsum(const SpectralArgs a, const int* __restrict__ apod_sum,
                                                     long long* __restrict__ sum_n, float* __restrict__ mline) {
    const int lane = threadIdx.x & 31;
    const float den = static_cast<float>(kN) * static_cast<float>(a.apod);
    for (int64_t as = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5; as < a.n_ascans;
         as += (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5) {
        const int64_t b = as / a.nx, x = as - b * a.nx;
        const RawT* row = static_cast<const RawT*>(a.raw) + (b * a.interf + a.apod + x) * kN;
        const int* Sb = apod_sum + b * kN;
        // eight samples a 16-byte load when the row is aligned (kN * 2 bytes a
        // row: rows are aligned when the buffer is); with apod < 256 a lane's
        // 64 terms, |apod raw - S| < 2^24 each, sum exactly in 32 bits
        long long s = 0;
        if ((reinterpret_cast<uintptr_t>(row) & 15u) == 0 && a.apod < 256) {
            int sl = 0;
            const uint4* r4 = reinterpret_cast<const uint4*>(row);
            const int4* s4 = reinterpret_cast<const int4*>(Sb);
            for (int c = lane; c < kN / 8; c += 32) {
                const uint4 rv = __ldg(r4 + c);
                const int4 sa = __ldg(s4 + 2 * c), sb = __ldg(s4 + 2 * c + 1);
                const uint32_t w[4] = {rv.x, rv.y, rv.z, rv.w};
                const int sv[8] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y, sb.z, sb.w};
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const uint32_t u = (w[e >> 1] >> (16 * (e & 1))) & 0xffffu;
                    const int rawv = static_cast<RawT>(-1) < 0 ? static_cast<int>(static_cast<int16_t>(u))
                                                               : static_cast<int>(u);
                    sl += a.apod * rawv - sv[e];
                }
            }
            s = sl;
        } else {
            for (int j = lane; j < kN; j += 32) s += a.apod * static_cast<int>(row[j]) - Sb[j];
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            sum_n[as] = s;
            mline[as] = static_cast<float>(s) / den;
        }
    }
}

// Integer raws: exact apodisation sums S[b][j] (int32).
template <typename RawT>
__global__ void k_apod_sum(const SpectralArgs a, int* __restrict__ out) {
    const int b = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= kN) return;
    const RawT* p = static_cast<const RawT*>(a.raw) + static_cast<int64_t>(b) * a.interf * kN + j;
    int s = 0;
    for (int k = 0; k < a.apod; ++k) s += static_cast<int>(p[static_cast<int64_t>(k) * kN]);
    out[static_cast<int64_t>(b) * kN + j] = s;
}

__device__ __forceinline__ void store_split(float v, __half* hi, __half* lo) {
    const __half h = __float2half_rn(v);
    *hi = h;
    *lo = __float2half_rn(v - __half2float(h));            // exact difference in float32
}

// Integer raws, 256 threads, persistent over A-scans.  With N_j = apod*raw_j
// - S_j (exact) the background-free line is d'_j = (2048 N_j - sum N) /
// (2048 apod): an exact int64 numerator and two float32 roundings, each
// relative to d'_j itself (the float32 form's apodisation store instead
// errs by ~1e-7 of the ~2e4-count background).  m = sum N / (2048 apod).
template <typename RawT>
__global__ void __launch_bounds__(256) k_prec_split_int(const SpectralArgs a, const int* __restrict__ apod_sum,
                                                        __half* __restrict__ hi, __half* __restrict__ lo,
                                                        float* __restrict__ mline) {
    __shared__ long long red[8];
    const float den = static_cast<float>(kN) * static_cast<float>(a.apod);   // exact
    for (int64_t as = blockIdx.x; as < a.n_ascans; as += gridDim.x) {
        const int64_t b = as / a.nx, x = as - b * a.nx;
        const RawT* row = static_cast<const RawT*>(a.raw) + (b * a.interf + a.apod + x) * kN;
        const int* S = apod_sum + b * kN;
        int n[8];
        long long s = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = threadIdx.x + 256 * k;
            n[k] = a.apod * static_cast<int>(row[j]) - S[j];
            s += n[k];
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        long long t = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) t += red[w];
        __syncthreads();
        if (threadIdx.x == 0) mline[as] = static_cast<float>(t) / den;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = threadIdx.x + 256 * k;
            const long long q = static_cast<long long>(kN) * n[k] - t;
            store_split(static_cast<float>(q) / den, hi + as * kN + j, lo + as * kN + j);
        }
    }
}

// float32 raws: the background in float64 (apodisation mean, line mean).
__global__ void k_apod_mean64(const SpectralArgs a, double* __restrict__ out) {
    const int b = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= kN) return;
    const float* p = static_cast<const float*>(a.raw) + static_cast<int64_t>(b) * a.interf * kN + j;
    double s = 0.0;
    for (int k = 0; k < a.apod; ++k) s += static_cast<double>(p[static_cast<int64_t>(k) * kN]);
    out[static_cast<int64_t>(b) * kN + j] = s / a.apod;
}

__global__ void __launch_bounds__(256) k_prec_split_f32(const SpectralArgs a, const double* __restrict__ apod64,
                                                        __half* __restrict__ hi, __half* __restrict__ lo,
                                                        float* __restrict__ mline) {
    __shared__ double red[8];
    for (int64_t as = blockIdx.x; as < a.n_ascans; as += gridDim.x) {
        const int64_t b = as / a.nx, x = as - b * a.nx;
        const float* row = static_cast<const float*>(a.raw) + (b * a.interf + a.apod + x) * kN;
        const double* ap = apod64 + b * kN;
        double d[8];
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = threadIdx.x + 256 * k;
            d[k] = static_cast<double>(row[j]) - ap[j];
            s += d[k];
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) t += red[w];
        __syncthreads();
        const double m = t / kN;
        if (threadIdx.x == 0) mline[as] = static_cast<float>(m);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = threadIdx.x + 256 * k;
            store_split(static_cast<float>(d[k] - m), hi + as * kN + j, lo + as * kN + j);
        }
    }
}

}  // namespace

cudaError_t launch_prec_split(const SpectralArgs& a, int dtype, void* apod_scratch, __half* hi, __half* lo,
                              float* mline, int num_sms, cudaStream_t st) {
    const int64_t n = a.n_ascans;
    if (n == 0) return cudaSuccess;
    const dim3 ga(kN / 256, a.B);
    const int64_t g64 = n < static_cast<int64_t>(num_sms) * 8 ? n : static_cast<int64_t>(num_sms) * 8;
    const unsigned int g = static_cast<unsigned int>(g64);
    int* isum = static_cast<int*>(apod_scratch);
    if (dtype == 0) {
        k_apod_sum<uint16_t><<<ga, 256, 0, st>>>(a, isum);
        k_prec_split_int<uint16_t><<<g, 256, 0, st>>>(a, isum, hi, lo, mline);
    } else if (dtype == 1) {
        k_apod_sum<int16_t><<<ga, 256, 0, st>>>(a, isum);
        k_prec_split_int<int16_t><<<g, 256, 0, st>>>(a, isum, hi, lo, mline);
    } else {
        double* a64 = static_cast<double*>(apod_scratch);
        k_apod_mean64<<<ga, 256, 0, st>>>(a, a64);
        k_prec_split_f32<<<g, 256, 0, st>>>(a, a64, hi, lo, mline);
    }
    return cudaGetLastError();
}

cudaError_t launch_prec_sinc(const CUtensorMap& tm_hi, const CUtensorMap& tm_lo, const uint8_t* wtiles,
                             const int* kb, const float* mline, float* X, int64_t n_ascans, int* status, int num_sms,
                             cudaStream_t st) {
    const size_t smem = sizeof(PrecSmem) + 1024;                  // + alignment of the dynamic window
    cudaError_t e = cudaFuncSetAttribute(k_prec_sinc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    const int64_t tiles = (n_ascans + kPM - 1) / kPM;
    const int grid = static_cast<int>(tiles < num_sms ? tiles : num_sms);
    if (grid < 1) return cudaSuccess;
    k_prec_sinc<<<grid, kPThreads, smem, st>>>(tm_hi, tm_lo, wtiles, kb, mline, X, n_ascans, status);
    return cudaGetLastError();
}

size_t prec_smem_bytes() { return sizeof(PrecSmem) + 1024; }

cudaError_t launch_prec_sinc_raw(const SpectralArgs& a, int dtype, const CUtensorMap& tm_raw, const uint8_t* wtiles,
                                 const int* kb, int* apod_sum, long long* sum_n, float* mline, float* X, int* status,
                                 int num_sms, cudaStream_t st) {
    if (a.n_ascans == 0) return cudaSuccess;
    const dim3 ga(kN / 256, a.B);
    const int64_t warps = a.n_ascans;
    int64_t g = (warps * 32 + 255) / 256;
    if (g > static_cast<int64_t>(num_sms) * 16) g = static_cast<int64_t>(num_sms) * 16;
    const size_t smem = sizeof(RawSmem) + 1024;
    const int xtiles = (a.nx + kPM - 1) / kPM;
    const int64_t tiles = static_cast<int64_t>(a.B) * xtiles;
    const int grid = static_cast<int>(tiles < num_sms ? tiles : num_sms);
    cudaError_t e;
    if (dtype == 0) {
        k_apod_sum<uint16_t><<<ga, 256, 0, st>>>(a, apod_sum);
        k_prec_rowsum<uint16_t><<<static_cast<unsigned int>(g), 256, 0, st>>>(a, apod_sum, sum_n, mline);
        e = cudaFuncSetAttribute(k_prec_sinc_raw<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        k_prec_sinc_raw<uint16_t><<<grid, kRThreads, smem, st>>>(tm_raw, wtiles, kb, apod_sum, sum_n, mline, X,
                                                                 a.B, a.nx, a.apod, status);
    } else {
        k_apod_sum<int16_t><<<ga, 256, 0, st>>>(a, apod_sum);
        k_prec_rowsum<int16_t><<<static_cast<unsigned int>(g), 256, 0, st>>>(a, apod_sum, sum_n, mline);
        e = cudaFuncSetAttribute(k_prec_sinc_raw<int16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        k_prec_sinc_raw<int16_t><<<grid, kRThreads, smem, st>>>(tm_raw, wtiles, kb, apod_sum, sum_n, mline, X,
                                                                a.B, a.nx, a.apod, status);
    }
    return cudaGetLastError();
}

// 3-D map of the scan lines of a raw batch: samples x A-scans x B-scans
// (uint16/int16 elements, rows of one B-scan consecutive, B-scans `interf`
// rows apart), boxes of 8 samples x 128 A-scans x 1 B-scan
bool encode_raw_map(CUtensorMap* map, const void* raw, int B, int interf, int apod) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (encode == nullptr) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || fn == nullptr)
            return false;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const void* base = static_cast<const uint16_t*>(raw) + static_cast<size_t>(apod) * kN;
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(kN), static_cast<cuuint64_t>(interf - apod),
                                static_cast<cuuint64_t>(B)};
    const cuuint64_t strides[2] = {static_cast<cuuint64_t>(kN) * 2, static_cast<cuuint64_t>(interf) * kN * 2};
    const cuuint32_t box[3] = {8, static_cast<cuuint32_t>(kPM), 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_prec_map(CUtensorMap* map, const void* base, int64_t n_ascans) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (encode == nullptr) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || fn == nullptr)
            return false;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(kN), static_cast<cuuint64_t>(n_ascans)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(kN) * sizeof(__half)};
    const cuuint32_t box[2] = {8, static_cast<cuuint32_t>(kPM)};
    const cuuint32_t estr[2] = {1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool build_prec_tiles(const int* start, const int* len, const float* wt, std::vector<uint16_t>& tiles,
                      std::vector<int>& kb) {
    tiles.assign(static_cast<size_t>(kPBlocks) * 2 * kBTileBytes / 2, 0);
    kb.assign(kPBlocks, 0);
    for (int b = 0; b < kPBlocks; ++b) {
        int lo = kN, hi = 0;
        for (int r = 0; r < kPN; ++r) {
            const int i = b * kPN + r;
            lo = lo < start[i] ? lo : start[i];
            hi = hi > start[i] + len[i] ? hi : start[i] + len[i];
        }
        const int k0 = lo & ~7;
        if (hi - k0 > kPKW) return false;
        kb[b] = k0;
        uint16_t* th = tiles.data() + static_cast<size_t>(b) * kBTileBytes;         // 2-byte units: hi then lo
        uint16_t* tl = th + kBTileBytes / 2;
        for (int r = 0; r < kPN; ++r) {
            const int i = b * kPN + r;
            for (int t = 0; t < len[i]; ++t) {
                const int col = start[i] + t - k0;                                    // 0 .. kPKW-1
                const float w = wt[static_cast<size_t>(t) * kN + i] * 64.0f;          // exact scaling
                const __half h = __float2half_rn(w);
                const __half l = __float2half_rn(w - __half2float(h));
                const size_t off = static_cast<size_t>(col >> 3) * (kBChunkBytes / 2) + static_cast<size_t>(r) * 8 +
                                   (col & 7);
                th[off] = __half_as_ushort(h);
                tl[off] = __half_as_ushort(l);
            }
        }
    }
    return true;
}

cudaError_t set_wait_test_precision(unsigned long long limit_ns, int starve, cudaStream_t st) {
    return set_wait_test_here(limit_ns, starve, st);
}

}  // namespace octgb
