// Fused spectral stage for sm_103a: raw camera counts -> |ifft| / dB.
//
// One CTA of 512 threads processes four A-scans per iteration of a persistent
// loop, one A-scan per group of 128 threads in the per-A-scan stages.
// Per A-scan (2048 samples):
//   (a) the raw row (4 KiB of uint16) and the B-scan's apodisation-mean row
//       reach shared memory by asynchronous 16-byte copies (through L2 only)
//       that the A-scan's 128 threads issue one quad ahead; one arrival per
//       thread on the group's mbarrier marks them landed (the bounded wait of
//       the next iteration); the raw copies start once the background has
//       read the current row, the apodisation copies once the sinc has read
//       the current lines, so both hide behind the sinc and the transform;
//   (b) d[j] = float(raw[j]) - apod[j] (float32 apodisation mean of the
//       B-scan, rounded from an exact sum as core/cpu_kernels.py:20-25 does),
//       line mean m removed before d reaches shared memory (cpu_kernels.py:
//       26-36);
//   (c) banded sinc k-linearisation, sum_t w[t,i] * d[start_i + t]
//       (cpu_kernels.py:37-40), float32 accumulation;
//   (d) (acc + m) * window[i] (Hann/rms * dispersion phase, scaled by 1/N for
//       the ifft normalisation, cpu_kernels.py:41, spectral.py:160-165);
//   (e) inverse FFT of length 2048 in shared memory: Stockham radix 16,16,8,
//       each radix butterfly in registers (128 threads, 16 points each);
//   (f) |X[k]| for k < N/2 (spectral.py:153), optionally 20*log10 with a
//       depth crop and a running min/max for the global clim; with 16-bit
//       raws each A-scan's row (magnitudes, or a dB crop of a multiple of 4
//       rows) leaves by one bulk copy from shared memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include "octgb_device.cuh"
#include "octgb_internal.h"

namespace octgb {
namespace {

template <typename RawT>
struct RawLoad;
template <>
struct RawLoad<uint16_t> {
    static __device__ __forceinline__ void load4(const uint16_t* p, float (&f)[4]) {
        const uint2 u = *reinterpret_cast<const uint2*>(p);
        f[0] = static_cast<float>(u.x & 0xffffu);
        f[1] = static_cast<float>(u.x >> 16);
        f[2] = static_cast<float>(u.y & 0xffffu);
        f[3] = static_cast<float>(u.y >> 16);
    }
};
template <>
struct RawLoad<int16_t> {
    static __device__ __forceinline__ void load4(const int16_t* p, float (&f)[4]) {
        const uint2 u = *reinterpret_cast<const uint2*>(p);
        f[0] = static_cast<float>(static_cast<int16_t>(u.x & 0xffffu));
        f[1] = static_cast<float>(static_cast<int16_t>(u.x >> 16));
        f[2] = static_cast<float>(static_cast<int16_t>(u.y & 0xffffu));
        f[3] = static_cast<float>(static_cast<int16_t>(u.y >> 16));
    }
};
template <>
struct RawLoad<float> {
    static __device__ __forceinline__ void load4(const float* p, float (&f)[4]) {
        const float4 u = *reinterpret_cast<const float4*>(p);
        f[0] = u.x;
        f[1] = u.y;
        f[2] = u.z;
        f[3] = u.w;
    }
};

constexpr int kDLine = kN + kTail;                        // d line incl. zero tail (16-byte rows)

// float32(float64(x) * h) for a float64 h given as float32 hi + lo (h2.x +
// h2.y, the rest below 2^-48 |h|) without the FP64 pipe: p + e1 = x * hi
// exactly (fma), q = x lo + e1 (one rounding), o = p + q rounded once.  The
// exact product differs from p + q by < 2^-46 |o|; when p + q lies more than
// 2^-40 |o| from a float32 rounding boundary (r = (p + q) - o exactly, by
// Fast2Sum), both the product and its float64 rounding round to o.  Otherwise
// (about one sample in 65 000), and for powers of two (asymmetric boundaries)
// and tiny values, the float64 product is formed as the reference does.  A
// window value of exactly zero (the Hann window's end points) gives the exact
// product x * 0 (signed zero, or NaN) in both forms and needs no float64 step:
// without this case the two warps holding the end points took the float64 path
// for every A-scan.
// The caller forms the float64 product for the lanes whose `safe` is false,
// behind a warp vote, so the FP64 pipe only runs in the rare warps that need it.
__device__ __forceinline__ float mul_window(float x, float2 h2, bool& safe) {
    const float p = x * h2.x;
    const float e1 = fmaf(x, h2.x, -p);
    const float q = fmaf(x, h2.y, e1);
    const float o = p + q;
    const float r = q - (o - p);
    const float ao = fabsf(o);
    const int bits = __float_as_int(ao);
    const float half_ulp = __int_as_float((bits & 0x7f800000) - (24 << 23));
    const bool zero_h = h2.x == 0.f && h2.y == 0.f;
    safe = zero_h || (ao > 1e-30f && (bits & 0x007fffff) != 0 && fabsf(fabsf(r) - half_ulp) > ao * 9.094947e-13f);
    // x * 0 keeps x's sign, as the float64 product does (p + q would give +0)
    return zero_h ? p : o;
}

// Where slot s of quad q reads its raw row and apodisation row and writes
// its result.  Static mode: quads of one batch (n_seg segments of B x nx
// A-scans).  Queue mode: quads of the tile table (quad0 prefix in shared
// memory, binary search).
struct SlotRef {
    const void* row;     // raw row (kN samples)
    unsigned int apod_row;   // row of the apodisation-mean buffer
    unsigned int as;     // static: global A-scan index; queue: A-scan index within the tile
    int tile;            // queue: tile index
    bool valid;
};

template <typename RawT>
struct Smem {
    uint64_t bar[kPerCta];                          // slot k: its group's copies of the rows have landed
    SlotRef slot[kPerCta];                          // queue mode: the next quad's slots (warp 0 fills them)
    float red[kPerCta][4];
    float mval[kPerCta];
    unsigned int mm[2];
    alignas(16) RawT stage[kPerCta][kN];            // raw rows (each thread copies the samples it reads)
    alignas(16) float d[kPerCta][kDLine];           // apodisation-mean row, then the background-free line
    alignas(16) float2 spec[kPerCta][kSpecStride];  // windowed spectrum / FFT work line
    // second FFT line of each A-scan (16-bit raws; float32 raws need the
    // shared memory for their larger staging rows and transform in place)
    alignas(16) float2 fft_y[sizeof(RawT) == 2 ? kPerCta : 1][kSpecStride];
    alignas(16) float2 tw2[16][16];                 // stage-2 twiddles [r][j mod 16]
    alignas(16) float2 tw3[8][256];                 // stage-3 twiddles [r][j]
    alignas(16) float4 win[2][kThreads];            // window of outputs 4t, 4t+1 ([0][t]) and 4t+2, 4t+3 ([1][t])
};

// dynamic + static shared memory of the kernel within the 227 KB a CTA may use
static_assert(sizeof(Smem<uint16_t>) + sizeof(int64_t) + kMaxQueueTiles * sizeof(unsigned) <= 232448,
              "spectral kernel shared memory (16-bit raws) exceeds 227 KB");
static_assert(sizeof(Smem<float>) + sizeof(int64_t) + kMaxQueueTiles * sizeof(unsigned) <= 232448,
              "spectral kernel shared memory (float32 raws) exceeds 227 KB");

// A launch holds fewer than 2^31 A-scans (the host checks), so the index
// arithmetic is 32-bit.  Queue mode: a CTA takes its quads in increasing
// order, so the tile holding quad q is found by stepping forward from the
// previous one (`hint`); a binary search is the fallback.
template <typename RawT, bool Queue>
__device__ __forceinline__ SlotRef slot_ref(const SpectralArgs& a, const unsigned int* quad0_s, int64_t q, int s,
                                            int& hint) {
    SlotRef r;
    if (!Queue) {
        const unsigned int as = static_cast<unsigned int>(q) * kPerCta + static_cast<unsigned int>(s);
        r.valid = static_cast<int64_t>(as) < a.n_ascans;
        const unsigned int asc = r.valid ? as : 0u;
        const unsigned int nx = static_cast<unsigned int>(a.nx);
        const unsigned int bt = asc / nx, x = asc - bt * nx;   // bt = segment * B + b
        const unsigned int sg = bt / static_cast<unsigned int>(a.B);
        const unsigned int b = bt - sg * static_cast<unsigned int>(a.B);
        r.row = static_cast<const RawT*>(a.seg[sg]) + ((static_cast<int64_t>(b) * a.interf + a.apod + x) * kN);
        r.apod_row = bt;
        r.as = as;
        r.tile = 0;
    } else {
        const unsigned int uq = static_cast<unsigned int>(q);
        int lo = hint;                               // last tile with quad0 <= q
        if (quad0_s[lo] > uq) {
            int hi = lo;
            lo = 0;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (quad0_s[mid] <= uq) lo = mid; else hi = mid - 1;
            }
        }
        while (lo + 1 < a.n_qt && quad0_s[lo + 1] <= uq) ++lo;
        hint = lo;
        const QueueTile& t = a.qt[lo];
        const unsigned int lq = uq - t.quad0;
        const unsigned int b = lq / static_cast<unsigned int>(t.qpb);   // quads are aligned to B-scans
        const int qb = static_cast<int>(lq - b * static_cast<unsigned int>(t.qpb));
        // the last quad of a B-scan ends on its last A-scan (it may repeat up
        // to three A-scans of the previous quad), so both edge columns find
        // their lateral neighbour in the same quad
        const int xs = (qb == t.qpb - 1 && t.nx >= kPerCta) ? t.nx - kPerCta : qb * kPerCta;
        const int64_t x = xs + s;
        // a quad outside this tile's range (only possible with a table that
        // does not match total_quads) reads and writes nothing
        r.valid = x < t.nx && lq < t.nquads;
        const int64_t xc = r.valid ? x : 0;
        const int64_t bc = r.valid ? b : 0;
        r.row = static_cast<const RawT*>(t.raw) + ((bc * t.interf + t.apod + xc) * kN);
        r.apod_row = static_cast<unsigned int>(t.apod_row0 + bc);
        r.as = static_cast<unsigned int>(bc * t.nx + xc);   // A-scan index within the tile
        r.tile = lo;
    }
    return r;
}

// One CTA (512 threads) = 4 A-scans per iteration of a persistent loop.
// Sinc: thread t owns output samples 4t..4t+3 of all four A-scans; its band
// weights live in registers for the whole kernel in a dense form over its
// window of U source samples s0_t .. s0_t + U - 1 (zero outside the band).
// Step u of the window reads the sample congruent to u (mod U) and wr[r][u]
// is that sample's weight for output 4t + r: the windows of a warp's threads
// overlap, so at one step they read the same samples or samples U apart, and
// with gcd(U, 32) = 2 those sit in distinct banks of the plain (unpadded)
// line - each A-scan costs U conflict-free shared loads and 4*U FMAs.  FFT:
// 128 threads per A-scan, radix 16,16,8 Stockham through two padded lines,
// per-group named barriers.
// Work: static grid-stride over one batch's quads, or (resample mode) quads
// taken `grab` at a time from a device work queue spanning many tiles of
// uneven size.
template <typename RawT, int Mode, int U>
__global__ void __launch_bounds__(kThreads, 1) k_spectral(const SpectralArgs a) {
    constexpr bool kQueue = Mode == kModeResample;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem<RawT>& S = *reinterpret_cast<Smem<RawT>*>(smem_raw);
    __shared__ int64_t qbuf[1];                        // queue mode: the next quad (-1: none)
    __shared__ unsigned int quad0_s[kQueue ? kMaxQueueTiles : 1];

    const int tid = threadIdx.x;
    const int g = tid / kGroup;        // A-scan slot of the iteration
    const int lt = tid % kGroup;       // thread within the A-scan group
    const int warp = tid / 32, lane = tid % 32;
    const int64_t nquads = kQueue ? static_cast<int64_t>(a.total_quads) : (a.n_ascans + kPerCta - 1) / kPerCta;
    // magnitude mode, and dB mode with a crop of a multiple of 4 rows, with
    // 16-bit raws: each A-scan's output row leaves by one bulk copy from the
    // free second FFT line (thread 0 of its group issues it)
    const bool bulk_out = (Mode == kModeMag || (Mode == kModeDb && (a.nz & 3) == 0)) && sizeof(RawT) == 2 &&
                          (reinterpret_cast<uintptr_t>(a.out) & 15u) == 0;

    // this thread's shifted sinc weights and source window base; the weights
    // of outputs 4t, 4t+1 (and 4t+2, 4t+3) at window step u form one packed
    // pair wp[0][u] (wp[1][u]): two outputs per f32x2 fma
    float2 wp[2][U];
    {
        auto set_w = [&](int r, int u, float w) {
            if (r & 1) wp[r >> 1][u].y = w; else wp[r >> 1][u].x = w;
        };
        if (U % 4 == 0) {
            const float4* src = reinterpret_cast<const float4*>(a.g.wsh + static_cast<int64_t>(tid) * 4 * U);
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int q = 0; q < U / 4; ++q) {
                    const float4 v = __ldg(src + r * (U / 4) + q);
                    set_w(r, 4 * q, v.x);
                    set_w(r, 4 * q + 1, v.y);
                    set_w(r, 4 * q + 2, v.z);
                    set_w(r, 4 * q + 3, v.w);
                }
        } else {                                      // U = 14: rows of 56 bytes, 8-byte aligned
            const float2* src = reinterpret_cast<const float2*>(a.g.wsh + static_cast<int64_t>(tid) * 4 * U);
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int q = 0; q < U / 2; ++q) {
                    const float2 v = __ldg(src + r * (U / 2) + q);
                    set_w(r, 2 * q, v.x);
                    set_w(r, 2 * q + 1, v.y);
                }
        }
    }
    const int s0 = __ldg(a.g.s0 + tid);
    const int wrot = s0 % U;                          // window samples before s0 wrap to the next period
    const int wbase = s0 - wrot;

    if (tid == 0) {
        for (int k = 0; k < kPerCta; ++k) mbar_init(&S.bar[k], kGroup);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        S.mm[0] = 0xffffffffu;
        S.mm[1] = 0u;
    }
    if (kQueue)
        for (int k = tid; k < a.n_qt; k += kThreads) quad0_s[k] = a.qt[k].quad0;
    for (int k = tid; k < kPerCta * kTail; k += kThreads) S.d[k / kTail][kN + k % kTail] = 0.f;
    for (int k = tid; k < 16 * 16; k += kThreads) {
        const int r = k / 16, j = k % 16;
        S.tw2[r][j] = __ldg(a.g.tw + (r * j * (kN / 256)) % kN);
    }
    for (int k = tid; k < 8 * 256; k += kThreads) {
        const int r = k / 256, j = k % 256;
        S.tw3[r][j] = __ldg(a.g.tw + (r * j) % kN);
    }
    S.win[0][tid] = __ldg(reinterpret_cast<const float4*>(a.g.win + 4 * tid));
    S.win[1][tid] = __ldg(reinterpret_cast<const float4*>(a.g.win + 4 * tid + 2));
    float run_min = __int_as_float(0x7f800000), run_max = -__int_as_float(0x7f800000);
    __syncthreads();

    // Rows reach shared memory by asynchronous copies issued by every thread:
    // group g copies its slot's raw row and apodisation-mean row one quad
    // ahead, and one arrival per thread on the group's barrier (kGroup a
    // phase) marks them landed.  No warp issues for the others, and the
    // CTA-wide barrier of the background doubles as the check of the bounded
    // waits.
    int64_t item_next = 0, item_end = 0;               // queue mode: current grab [next, end)
    auto next_quad = [&](int64_t cur) -> int64_t {
        if (!kQueue) {
            const int64_t n = cur < 0 ? blockIdx.x : cur + gridDim.x;
            return n < nquads ? n : -1;
        }
        if (item_next < item_end) return item_next++;
        const int64_t base = atomicAdd(a.counter, static_cast<unsigned int>(a.grab));
        if (base >= nquads) return -1;
        item_next = base + 1;
        item_end = base + a.grab < nquads ? base + a.grab : nquads;
        return base;
    };
    // queue mode: lane 0 of warp 0 owns the schedule; lanes 0-3 resolve the
    // quad's slots into S.slot (read by the groups after the next CTA barrier)
    int tile_hint = 0;                                 // queue mode, lanes 0-3: tile of the last quad resolved
    auto warp_next = [&](int64_t cur) -> int64_t {
        int64_t n = 0;
        if (lane == 0) n = next_quad(cur);
        n = static_cast<int64_t>(__shfl_sync(0xffffffffu, static_cast<long long>(n), 0));
        if (lane < kPerCta && n >= 0) S.slot[lane] = slot_ref<RawT, true>(a, quad0_s, n, lane, tile_hint);
        return n;
    };
    // static mode: this group's A-scan (position within the batch) steps by
    // gridDim.x quads a time without division (the launcher splits the
    // stride into a.step_bt B-scans + a.step_x A-scans)
    unsigned int pas = 0, px = 0, pb = 0, psg = 0;     // A-scan, column, B-scan in segment, segment
    auto static_slot = [&]() -> SlotRef {
        SlotRef r;
        r.valid = static_cast<int64_t>(pas) < a.n_ascans;
        const unsigned int sg = r.valid ? psg : 0u;
        r.row = static_cast<const RawT*>(a.seg[sg]) +
                ((static_cast<int64_t>(r.valid ? pb : 0u) * a.interf + a.apod + (r.valid ? px : 0u)) * kN);
        r.apod_row = sg * static_cast<unsigned int>(a.B) + (r.valid ? pb : 0u);
        r.as = pas;
        r.tile = 0;
        return r;
    };
    auto static_advance = [&]() {
        const unsigned int nx = static_cast<unsigned int>(a.nx), B = static_cast<unsigned int>(a.B);
        pas += static_cast<unsigned int>(gridDim.x) * kPerCta;
        px += a.step_x;
        unsigned int inc = a.step_bt;
        if (px >= nx) {
            px -= nx;
            ++inc;
        }
        pb += inc;
        if (pb >= B) {
            const unsigned int c = pb / B;
            psg += c;
            pb -= c * B;
        }
    };
    // slot r's raw row and apodisation-mean row, copied by the group in
    // 16-byte pieces through L2 only (no L1 lines: the shared memory leaves L1
    // ~28 KB), then each thread's arrival on the group's barrier (after the
    // apodisation copies); the completed phase makes both rows visible to the
    // whole group
    auto copy_raw = [&](const SlotRef& r) {
        if (!r.valid) return;
        constexpr int kPieces = kN * static_cast<int>(sizeof(RawT)) / 16;   // 256 (16-bit raws) or 512
        const char* src = static_cast<const char*>(r.row);
        char* dst = reinterpret_cast<char*>(&S.stage[g][0]);
#pragma unroll
        for (int c = lt; c < kPieces; c += kGroup) cp_async_cg16(dst + 16 * c, src + 16 * c);
    };
    auto copy_apod = [&](const SlotRef& r, bool first) {
        if (r.valid) {
            const float* src = a.apod_mean + static_cast<int64_t>(r.apod_row) * kN;
#pragma unroll
            for (int q = 0; q < 4; ++q) cp_async_cg16(&S.d[g][4 * lt + 512 * q], src + 4 * lt + 512 * q);
        }
        // self-test: the first phase of slot 0's barrier waits for bytes that never come
        if (first && tid == 0) {
            const uint32_t sb = starved_bytes(true);
            if (sb) mbar_expect_tx_only(&S.bar[0], sb);
        }
        cp_async_arrive(&S.bar[g]);
    };

    int64_t quad;
    SlotRef cur{};                                     // this group's slot of the current quad
    if (!kQueue) {
        quad = next_quad(-1);
        if (quad >= 0) {
            const unsigned int as0 = static_cast<unsigned int>(quad) * kPerCta + static_cast<unsigned int>(g);
            const unsigned int nx = static_cast<unsigned int>(a.nx), B = static_cast<unsigned int>(a.B);
            const unsigned int bt = as0 / nx;
            pas = as0;
            px = as0 - bt * nx;
            psg = bt / B;
            pb = bt - psg * B;
            cur = static_slot();
        }
    } else {
        if (warp == 0) {
            const int64_t q0 = warp_next(-1);
            if (lane == 0) qbuf[0] = q0;
        }
        __syncthreads();
        quad = qbuf[0];
        if (quad >= 0) cur = S.slot[g];
        __syncthreads();                               // read before warp 0 resolves the next quad
    }
    if (quad >= 0) {
        copy_raw(cur);
        copy_apod(cur, true);
    }

    for (int it = 0; quad >= 0; ++it) {
        const SlotRef me = cur;
        const bool valid = me.valid;
        int64_t nq = -1;
        if (!kQueue) {
            nq = next_quad(quad);
        } else {
            // the groups read S.slot / qbuf of this quad before the last CTA barrier
            if (warp == 0) {
                const int64_t n = warp_next(quad);
                if (lane == 0) qbuf[0] = n;
            }
        }
        const bool ok = mbar_wait_bounded(&S.bar[g], it & 1, a.status);

        // ---- (b) background: d = raw - apod, line mean (group g, A-scan g) ----
        // d = raw - apod stays in registers until the line mean m is known;
        // shared memory receives d - m (the float32 value the reference
        // stores, cpu_kernels.py:35-36), so the sinc reads its window as is
        float dv[16];
        float sum = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = 4 * lt + 512 * q;
            float rv[4];
            RawLoad<RawT>::load4(&S.stage[g][j], rv);
            const float4 ap = *reinterpret_cast<const float4*>(&S.d[g][j]);
            const float2 d01 = sub2(make_float2(rv[0], rv[1]), make_float2(ap.x, ap.y));
            const float2 d23 = sub2(make_float2(rv[2], rv[3]), make_float2(ap.z, ap.w));
            dv[4 * q] = d01.x;
            dv[4 * q + 1] = d01.y;
            dv[4 * q + 2] = d23.x;
            dv[4 * q + 3] = d23.y;
            sum += (dv[4 * q] + dv[4 * q + 1]) + (dv[4 * q + 2] + dv[4 * q + 3]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) S.red[g][warp & 3] = sum;
        group_sync(g);
        {
            const float m = ((S.red[g][0] + S.red[g][1]) + (S.red[g][2] + S.red[g][3])) * (1.0f / kN);
            if (lt == 0) S.mval[g] = m;
            const float2 m2 = make_float2(m, m);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float2 e01 = sub2(make_float2(dv[4 * q], dv[4 * q + 1]), m2);
                const float2 e23 = sub2(make_float2(dv[4 * q + 2], dv[4 * q + 3]), m2);
                *reinterpret_cast<float4*>(&S.d[g][4 * lt + 512 * q]) = make_float4(e01.x, e01.y, e23.x, e23.y);
            }
        }
        if (__syncthreads_or(!ok)) {
            // a wait ran out: let this thread's copies land before the CTA's
            // shared memory is released
            cp_async_wait_all();
            if (bulk_out && lt == 0) bulk_wait_all();
            __syncthreads();
            return;
        }
        // the next quad's raw samples (this thread's own have been read above)
        SlotRef nxt{};
        if (!kQueue) {
            if (nq >= 0) {
                static_advance();
                nxt = static_slot();
            }
        } else {
            nq = qbuf[0];
            if (nq >= 0) nxt = S.slot[g];
        }
        if (nq >= 0) copy_raw(nxt);
        const float4 wa = S.win[0][tid], wb = S.win[1][tid];

        // ---- (c)+(d) sinc k-linearisation and window, four A-scans ----
        {
            const int i0 = 4 * tid;
            const float wre[4] = {wa.x, wa.z, wb.x, wb.z}, wim[4] = {wa.y, wa.w, wb.y, wb.w};
            const int64_t a0 = quad * kPerCta;
#pragma unroll 1
            for (int k = 0; k < kPerCta; ++k) {
                const float mk = S.mval[k];
                // modular window order: step u reads the window sample congruent
                // to u (mod U); the weights are stored in the same order
                const float* dk = S.d[k] + wbase;
                const float* dkh = dk + U;                // samples before s0 wrap to the next period
                float win[U];
#pragma unroll
                for (int u = 0; u < U; ++u) win[u] = (u < wrot ? dkh : dk)[u];
                // acc_r = sum_u w[r][u] win[u], the fmas in window order, two
                // outputs per packed fma
                float2 acc01 = make_float2(0.f, 0.f), acc23 = make_float2(0.f, 0.f);
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const float2 wu = make_float2(win[u], win[u]);
                    acc01 = fma2(wp[0][u], wu, acc01);
                    acc23 = fma2(wp[1][u], wu, acc23);
                }
                const float2 mk2 = make_float2(mk, mk);
                const float2 v01 = add2(acc01, mk2), v23 = add2(acc23, mk2);
                const float vr[4] = {v01.x, v01.y, v23.x, v23.y};
                float lh[4], lx[4];
                bool lsafe[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const float v = vr[r];
                    const float2 sp = make_float2(v * wre[r], v * wim[r]);
                    if (Mode == kModeLinHann) {
                        // the real part of the spec output (1/N undone) times the
                        // float64 window, one rounding to float32
                        lx[r] = sp.x * kN;
                        lh[r] = mul_window(lx[r], __ldg(a.hann2 + i0 + r), lsafe[r]);
                    } else if (Mode == kModeSpec) {
                        // spec output undoes the 1/N ifft scaling folded into the window
                        if (a0 + k < a.n_ascans)
                            reinterpret_cast<float2*>(a.out)[(a0 + k) * kN + i0 + r] =
                                make_float2(sp.x * kN, sp.y * kN);
                    } else {
                        S.spec[k][pad(i0 + r)] = sp;
                    }
                }
                if (Mode == kModeLinHann) {
                    const bool all_safe = lsafe[0] && lsafe[1] && lsafe[2] && lsafe[3];
                    if (__any_sync(0xffffffffu, !all_safe)) {
#pragma unroll
                        for (int r = 0; r < 4; ++r)
                            if (!lsafe[r])
                                lh[r] = static_cast<float>(static_cast<double>(lx[r]) * __ldg(a.hann + i0 + r));
                    }
                    if (a0 + k < a.n_ascans)
                        *reinterpret_cast<float4*>(a.out + (a0 + k) * kN + i0) = make_float4(lh[0], lh[1], lh[2], lh[3]);
                }
            }
        }
        // the previous quad's magnitudes have left the second FFT line before
        // the transform below overwrites it
        if (bulk_out && lt == 0) bulk_wait_read();
        __syncthreads();
        // every line has been read: the next quad's apodisation row into d
        if (nq >= 0) copy_apod(nxt, false);
        quad = nq;
        cur = nxt;
        if (Mode == kModeSpec || Mode == kModeLinHann) continue;

        // ---- (e)+(f) inverse FFT, group g on its own line; |X[k]|, k < N/2 ----
        float2* X = S.spec[g];
        float magv[2][4];
        if (sizeof(RawT) == 2)
            ifft2048_low_mag_pp(X, S.fft_y[g], S.tw2, S.tw3, g, lt, magv);
        else
            ifft2048_low_mag(X, S.tw2, S.tw3, g, lt, magv);
        if ((Mode == kModeMag || Mode == kModeDb) && bulk_out) {
            // the last stage read only X: the second line Y is free for the
            // output row (|X[k]|, k < N/2, or dB of the crop, contiguous
            // float32), which leaves by one bulk copy
            float* M = reinterpret_cast<float*>(S.fft_y[sizeof(RawT) == 2 ? g : 0]);
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const int k = lt + 128 * h + 256 * r;
                    if (Mode == kModeMag) {
                        M[k] = magv[h][r];
                    } else {
                        const int z = k - a.z0;
                        if (z >= 0 && z < a.nz) {
                            const float db = 20.0f * log10f(magv[h][r]);
                            M[z] = db;
                            if (valid && isfinite(db)) {
                                run_min = fminf(run_min, db);
                                run_max = fmaxf(run_max, db);
                            }
                        }
                    }
                }
            fence_proxy_async();
            group_sync(g);
            const int n_row = Mode == kModeMag ? kHalf : a.nz;
            if (lt == 0 && valid)
                tma_bulk_s2g(a.out + static_cast<int64_t>(me.as) * n_row, M, static_cast<uint32_t>(n_row) * 4u);
        } else if (Mode == kModeMag || Mode == kModeDb) {
            if (valid) {
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        const int k = lt + 128 * h + 256 * r;
                        const float mag = magv[h][r];
                        if (Mode == kModeMag) {
                            a.out[static_cast<int64_t>(me.as) * kHalf + k] = mag;
                        } else {
                            const int z = k - a.z0;
                            if (z >= 0 && z < a.nz) {
                                const float db = 20.0f * log10f(mag);
                                a.out[static_cast<int64_t>(me.as) * a.nz + z] = db;
                                if (isfinite(db)) {
                                    run_min = fminf(run_min, db);
                                    run_max = fmaxf(run_max, db);
                                }
                            }
                        }
                    }
            }
        } else {
            // ---- (g) resample: the tile's depth operator and focus weight per
            // A-scan (u = Wz (a F)), then the lateral operator between the
            // quad's A-scans (num = WxT u, den likewise), as
            // TileStitcher.contribute for one tile (stitching.py:126-139), and
            // finalise (pipeline.py:296-300).  The lateral operator of a single
            // tile is the identity except for the reference's 1e-10 widening
            // of its first node, which blends A-scan 1 into column 0 with a
            // weight ~1e-7; quads are aligned to B-scans so that neighbour is
            // always in this CTA (checked on the host for every column).
            float* M = reinterpret_cast<float*>(X);        // |X[k]|, k < N/2, reuses the line
            float* Uz = M + kHalf;                          // u[zo] of this A-scan
            const QueueTile& tile = a.qt[me.tile];
            const StitchDev& p = *tile.plan;
            group_sync(g);
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int r = 0; r < 4; ++r) M[lt + 128 * h + 256 * r] = magv[h][r];
            group_sync(g);
            // per output row one 16-byte {zr, w0, w1, d} and one 8-byte {F0, F1}
            // load (F1 = 0: no second row)
            for (int zo = lt; zo < tile.nz; zo += kGroup) {
                const float4 rw = __ldg(p.zrow + zo);
                const int zr = __float_as_int(rw.x);
                float u = 0.f;
                if (zr >= 0) {
                    const float2 ff = __ldg(p.zf + zo);
                    const float a0v = M[p.r0 + zr] * ff.x;
                    const float a1v = ff.y != 0.f ? M[p.r0 + zr + 1] * ff.y : 0.f;
                    u = fmaf(a1v, rw.z, a0v * rw.y);
                }
                Uz[zo] = u;
            }
            __syncthreads();                               // every A-scan of the quad has its u
            if (valid) {
                const int64_t x = me.as % tile.nx;
                const int xq0 = static_cast<int>(x) - g;   // A-scan of slot 0
                const int xr = p.xr[x];
                const float wx0 = p.wx0[x], wx1 = p.wx1[x];
                const int s0i = xr - xq0, s1i = xr + 1 - xq0;
                const bool in0 = xr >= 0 && s0i >= 0 && s0i < kPerCta, in1 = xr >= 0 && s1i >= 0 && s1i < kPerCta;
                const float* U0 = reinterpret_cast<const float*>(S.spec[in0 ? s0i : 0]) + kHalf;
                const float* U1 = reinterpret_cast<const float*>(S.spec[in1 ? s1i : 0]) + kHalf;
                float* out = tile.out + static_cast<int64_t>(me.as) * tile.nz;
                for (int zo = lt; zo < tile.nz; zo += kGroup) {
                    const float4 rw = __ldg(p.zrow + zo);
                    const int zr = __float_as_int(rw.x);
                    float v = __int_as_float(0x7fc00000);
                    if (zr >= 0 && xr >= 0) {
                        const float d = rw.w;
                        const float u0 = in0 ? U0[zo] : 0.f, u1 = in1 ? U1[zo] : 0.f;
                        const float d0 = in0 ? d : 0.f, d1 = in1 ? d : 0.f;
                        const float num = fmaf(u1, wx1, u0 * wx0);
                        const float den = fmaf(d1, wx1, d0 * wx0);
                        if (!(den < a.thr) && !isnan(den)) v = 20.0f * log10f(__fdiv_rn(num, den));
                    }
                    out[zo] = v;
                    if (isfinite(v)) {
                        run_min = fminf(run_min, v);
                        run_max = fmaxf(run_max, v);
                    }
                }
            }
        }
    }

    if (bulk_out && lt == 0) bulk_wait_all();
    if ((Mode == kModeDb || Mode == kModeResample) && a.minmax != nullptr) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            run_min = fminf(run_min, __shfl_xor_sync(0xffffffffu, run_min, o));
            run_max = fmaxf(run_max, __shfl_xor_sync(0xffffffffu, run_max, o));
        }
        __syncthreads();
        if (lane == 0 && run_min <= run_max) {
            atomicMin(&S.mm[0], f2ord(run_min));
            atomicMax(&S.mm[1], f2ord(run_max));
        }
        __syncthreads();
        if (tid == 0 && S.mm[0] != 0xffffffffu) {
            atomicMin(&a.minmax[0], S.mm[0]);
            atomicMax(&a.minmax[1], S.mm[1]);
        }
    }
}

// apodisation mean (cpu_kernels.py:20-25): exact sum, divided in float64, stored float32
template <typename RawT>
__global__ void k_apod_mean(const SpectralArgs a, float* __restrict__ out) {
    const int bt = blockIdx.y;                  // segment * B + b
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int sg = bt / a.B, b = bt - sg * a.B;
    const int interf = a.interf, apod = a.apod;
    if (sg >= a.n_seg || j >= kN) return;
    const RawT* p = static_cast<const RawT*>(a.seg[sg]) + static_cast<int64_t>(b) * interf * kN + j;
    double s;
    if (sizeof(RawT) == 2) {
        int acc = 0;
        for (int k = 0; k < apod; ++k) acc += static_cast<int>(p[static_cast<int64_t>(k) * kN]);
        s = static_cast<double>(acc);
    } else {
        s = 0.0;
        for (int k = 0; k < apod; ++k) s += static_cast<double>(p[static_cast<int64_t>(k) * kN]);
    }
    out[static_cast<int64_t>(bt) * kN + j] = static_cast<float>(s / apod);
}

// apodisation mean of the queue tiles: block row = global B-scan row
template <typename RawT>
__global__ void k_apod_mean_tiles(const QueueTile* __restrict__ tiles, int n_tiles, float* __restrict__ out) {
    const int row = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    int lo = 0, hi = n_tiles - 1;              // last tile with apod_row0 <= row
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tiles[mid].apod_row0 <= row) lo = mid; else hi = mid - 1;
    }
    const QueueTile& t = tiles[lo];
    const int b = row - t.apod_row0;
    if (b >= t.B || j >= kN) return;
    const RawT* p = static_cast<const RawT*>(t.raw) + static_cast<int64_t>(b) * t.interf * kN + j;
    double s;
    if (sizeof(RawT) == 2) {
        int acc = 0;
        for (int k = 0; k < t.apod; ++k) acc += static_cast<int>(p[static_cast<int64_t>(k) * kN]);
        s = static_cast<double>(acc);
    } else {
        s = 0.0;
        for (int k = 0; k < t.apod; ++k) s += static_cast<double>(p[static_cast<int64_t>(k) * kN]);
    }
    out[static_cast<int64_t>(row) * kN + j] = static_cast<float>(s / t.apod);
}

template <typename RawT, int Mode, int U>
cudaError_t launch_t(const SpectralArgs& a, int grid, cudaStream_t st) {
    const size_t smem = sizeof(Smem<RawT>);
    cudaError_t e = cudaFuncSetAttribute(k_spectral<RawT, Mode, U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    // the grid stride of the static schedule in B-scans + A-scans
    SpectralArgs b = a;
    const unsigned int step = static_cast<unsigned int>(grid) * kPerCta;
    b.step_bt = a.nx > 0 ? step / static_cast<unsigned int>(a.nx) : 0u;
    b.step_x = a.nx > 0 ? step - b.step_bt * static_cast<unsigned int>(a.nx) : 0u;
    k_spectral<RawT, Mode, U><<<grid, kThreads, smem, st>>>(b);
    return cudaGetLastError();
}

template <typename RawT, int Mode>
cudaError_t launch_u(const SpectralArgs& a, int grid, cudaStream_t st) {
    switch (a.g.U) {
        case 14: return launch_t<RawT, Mode, 14>(a, grid, st);
        case 18: return launch_t<RawT, Mode, 18>(a, grid, st);
        case 22: return launch_t<RawT, Mode, 22>(a, grid, st);
        case 26: return launch_t<RawT, Mode, 26>(a, grid, st);
        default: return cudaErrorInvalidValue;
    }
}

template <typename RawT>
cudaError_t launch_mode(const SpectralArgs& a, int mode, int grid, cudaStream_t st) {
    switch (mode) {
        case kModeSpec: return launch_u<RawT, kModeSpec>(a, grid, st);
        case kModeMag: return launch_u<RawT, kModeMag>(a, grid, st);
        case kModeResample: return launch_u<RawT, kModeResample>(a, grid, st);
        case kModeLinHann: return launch_u<RawT, kModeLinHann>(a, grid, st);
        default: return launch_u<RawT, kModeDb>(a, grid, st);
    }
}

}  // namespace

cudaError_t launch_apod_mean(const SpectralArgs& a, int dtype, cudaStream_t st) {
    const dim3 grid(kN / 256, a.n_seg * a.B);
    float* out = const_cast<float*>(a.apod_mean);
    if (dtype == 0)
        k_apod_mean<uint16_t><<<grid, 256, 0, st>>>(a, out);
    else if (dtype == 1)
        k_apod_mean<int16_t><<<grid, 256, 0, st>>>(a, out);
    else
        k_apod_mean<float><<<grid, 256, 0, st>>>(a, out);
    return cudaGetLastError();
}

cudaError_t launch_apod_mean_tiles(const QueueTile* tiles_dev, int n_tiles, int total_rows, int dtype,
                                   float* apod_mean, cudaStream_t st) {
    if (total_rows == 0) return cudaSuccess;
    const dim3 grid(kN / 256, total_rows);
    if (dtype == 0)
        k_apod_mean_tiles<uint16_t><<<grid, 256, 0, st>>>(tiles_dev, n_tiles, apod_mean);
    else if (dtype == 1)
        k_apod_mean_tiles<int16_t><<<grid, 256, 0, st>>>(tiles_dev, n_tiles, apod_mean);
    else
        k_apod_mean_tiles<float><<<grid, 256, 0, st>>>(tiles_dev, n_tiles, apod_mean);
    return cudaGetLastError();
}

cudaError_t launch_spectral(const SpectralArgs& a, int dtype, int mode, int grid, cudaStream_t st) {
    // the kernel's slot arithmetic is 32-bit (q * 4 + s, quads of a tile)
    if (a.n_ascans >= (int64_t(1) << 31) || a.total_quads >= (1u << 31)) return cudaErrorInvalidValue;
    if (dtype == 0) return launch_mode<uint16_t>(a, mode, grid, st);
    if (dtype == 1) return launch_mode<int16_t>(a, mode, grid, st);
    return launch_mode<float>(a, mode, grid, st);
}

cudaError_t set_wait_test_spectral(unsigned long long limit_ns, int starve, cudaStream_t st) {
    return set_wait_test_here(limit_ns, starve, st);
}

int spectral_max_ctas_per_sm(int dtype, int mode) {
    (void)dtype;
    (void)mode;
    return 1;   // 512 threads, ~219 KB shared memory, 128 registers: one CTA per SM
}

size_t spectral_smem_bytes(int dtype) {
    return dtype == 2 ? sizeof(Smem<float>) : sizeof(Smem<uint16_t>);
}

}  // namespace octgb
