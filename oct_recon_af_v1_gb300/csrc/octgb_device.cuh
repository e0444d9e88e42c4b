// Device helpers shared by the spectral and estimation kernels: complex
// arithmetic, the inverse DFT blocks of the 2048-point shared-memory FFT,
// bulk-copy/mbarrier primitives with a bounded wait, and the FFT itself.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "octgb_internal.h"

namespace octgb {
namespace {

constexpr int kPadShift = 4;                              // one pad slot per 16 complex
constexpr int kSpecStride = kN + (kN >> kPadShift);       // padded complex line length

__device__ __forceinline__ int pad(int e) { return e + (e >> kPadShift); }

// Packed float32 pairs (sm_100 family f32x2 instructions): one instruction
// for both lanes, each lane rounded to nearest exactly as the scalar operation,
// so results are bit-identical to two scalar ops.  The explicit rounding mode
// also keeps ptxas from contracting them (as it would not contract the
// scalar forms here either).
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 x, y, z;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
        "add.rn.f32x2 z, x, y;\n\tmov.b64 {%0, %1}, z;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 x, y, z;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
        "sub.rn.f32x2 z, x, y;\n\tmov.b64 {%0, %1}, z;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
// (a.x b.x + c.x, a.y b.y + c.y), each a single-rounding fma
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 r;
    asm("{\n\t.reg .b64 x, y, z, w;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
        "mov.b64 z, {%6, %7};\n\tfma.rn.f32x2 w, x, y, z;\n\tmov.b64 {%0, %1}, w;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return add2(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return sub2(a, b); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 muli(float2 a) { return make_float2(-a.y, a.x); }

// inverse DFT-4 (omega = +i), natural order in and out; b +- i e lane-crossed
// in scalar form (a packed form would need the swapped pair of e first)
__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
    const float2 a = cadd(x0, x2), b = csub(x0, x2), c = cadd(x1, x3), e = csub(x1, x3);
    x0 = cadd(a, c);
    x2 = csub(a, c);
    x1 = make_float2(b.x - e.y, b.y + e.x);
    x3 = make_float2(b.x + e.y, b.y - e.x);
}

// cos/sin of multiples of pi/8 (float64 literals rounded to float32)
constexpr float kC1 = 0.92387953251128675613f;   // cos(pi/8)
constexpr float kS1 = 0.38268343236508977173f;   // sin(pi/8)
constexpr float kC2 = 0.70710678118654752440f;   // cos(pi/4)

// inverse DFT-16 as 4 x 4: X[4*k1 + k2] = sum_n1 w4^(n1 k1) w16^(n1 k2) sum_n2 x[n1 + 4 n2] w4^(n2 k2)
__device__ __forceinline__ void dft16(float2 (&v)[16]) {
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) dft4(v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]);
    // twiddles w16^(n1*k2) on element v[n1 + 4*k2]
    v[1 + 4] = cmul(v[1 + 4], make_float2(kC1, kS1));     // n1=1,k2=1: w^1
    v[1 + 8] = cmul(v[1 + 8], make_float2(kC2, kC2));     // n1=1,k2=2: w^2
    v[1 + 12] = cmul(v[1 + 12], make_float2(kS1, kC1));   // n1=1,k2=3: w^3
    v[2 + 4] = cmul(v[2 + 4], make_float2(kC2, kC2));     // n1=2,k2=1: w^2
    v[2 + 8] = muli(v[2 + 8]);                            // n1=2,k2=2: w^4 = i
    v[2 + 12] = cmul(v[2 + 12], make_float2(-kC2, kC2));  // n1=2,k2=3: w^6
    v[3 + 4] = cmul(v[3 + 4], make_float2(kS1, kC1));     // n1=3,k2=1: w^3
    v[3 + 8] = cmul(v[3 + 8], make_float2(-kC2, kC2));    // n1=3,k2=2: w^6
    v[3 + 12] = cmul(v[3 + 12], make_float2(-kC1, -kS1)); // n1=3,k2=3: w^9
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) dft4(v[4 * k2], v[4 * k2 + 1], v[4 * k2 + 2], v[4 * k2 + 3]);
    // X[4*k1 + k2] sits in v[k1 + 4*k2]: transpose the 4x4 block
    float2 t;
    t = v[1]; v[1] = v[4]; v[4] = t;
    t = v[2]; v[2] = v[8]; v[8] = t;
    t = v[3]; v[3] = v[12]; v[12] = t;
    t = v[6]; v[6] = v[9]; v[9] = t;
    t = v[7]; v[7] = v[13]; v[13] = t;
    t = v[11]; v[11] = v[14]; v[14] = t;
}

// inverse DFT-8 as 2 x 4, returning only X[0..3] (the last stage keeps k < N/2)
__device__ __forceinline__ void dft8_low(float2 (&v)[8], float2 (&X)[4]) {
    dft4(v[0], v[2], v[4], v[6]);
    dft4(v[1], v[3], v[5], v[7]);
    const float2 y1 = cmul(v[3], make_float2(kC2, kC2));
    const float2 y2 = muli(v[5]);
    const float2 y3 = cmul(v[7], make_float2(-kC2, kC2));
    X[0] = cadd(v[0], v[1]);
    X[1] = cadd(v[2], y1);
    X[2] = cadd(v[4], y2);
    X[3] = cadd(v[6], y3);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// one arrival on the mbarrier once every cp.async this thread issued so far
// has landed (counted against the barrier's expected arrivals)
// asynchronous global -> shared copy of 16 bytes (both addresses 16-byte
// aligned) through L2 only, no L1 line allocated; tracked per thread
__device__ __forceinline__ void cp_async_cg16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// raise the barrier's pending transaction count without arriving
__device__ __forceinline__ void mbar_expect_tx_only(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// shared -> global bulk copy (both addresses 16-byte aligned, bytes a multiple
// of 16) in this thread's bulk group; the shared source must stay unchanged
// until bulk_wait_read().  Generic-proxy writes of the source need
// fence_proxy_async() by their writers (and a barrier) before the copy.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tma_bulk_s2g(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// this thread's bulk copies have read their sources / are complete
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// try_wait suspends the thread in hardware until the phase completes or the
// hint (ns) runs out, so waiting warps issue (almost) no instructions
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity), "r"(100000u)
        : "memory");
    return done != 0;
}

// Limit of the bounded waits (ns of wall time, 2 s) and the self-test switch
// that makes each CTA's first bulk-copy barrier expect 16 bytes more than its
// copies deliver, so that wait runs out while every copy still lands.  One
// copy per translation unit, written only by its set_wait_test_* function
// (octgb_selftest_wait_expiry); the product never changes them.
__device__ unsigned long long g_wait_limit_ns = 2000000000ull;
__device__ int g_starve_first_copy = 0;

// bytes a CTA's first bulk-copy barrier expects beyond its copies (0 outside the self-test)
__device__ __forceinline__ uint32_t starved_bytes(bool first) { return first && g_starve_first_copy ? 16u : 0u; }

// Bounded wait on an mbarrier phase: gives up after g_wait_limit_ns of wall
// time and reports it through the status word (the copies and MMAs waited
// for normally complete within microseconds).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* status) {
    if (mbar_test(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    const uint64_t limit = g_wait_limit_ns;
    for (uint32_t it = 0; it < (1u << 30); ++it) {
        if (mbar_try(bar, parity)) return true;
        if (globaltimer_ns() - t0 > limit) break;
    }
    atomicExch(status, kStatusTimeout);
    return false;
}

// host side: set this translation unit's wait limit and self-test switch
inline cudaError_t set_wait_test_here(unsigned long long limit_ns, int starve, cudaStream_t st) {
    cudaError_t e = cudaMemcpyToSymbolAsync(g_wait_limit_ns, &limit_ns, sizeof(limit_ns), 0,
                                            cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyToSymbolAsync(g_starve_first_copy, &starve, sizeof(starve), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

// ---- tcgen05 (5th-generation tensor cores) helpers
// shared-memory matrix descriptor without swizzle: lbo = byte step between
// core matrices (8 rows x 16 bytes) along K, sbo = along M/N; without swizzle
// this holds for K-major operands (a core matrix row = 8 K values) and
// MN-major ones (a row = 8 M/N values) alike.  Bit 46 is the descriptor
// version of sm_100-family tensor cores.
__device__ __forceinline__ uint64_t smem_desc(const void* p, uint32_t lbo, uint32_t sbo) {
    const uint64_t a = smem_u32(p);
    return ((a >> 4) & 0x3fffull) | (static_cast<uint64_t>((lbo >> 4) & 0x3fff) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3fff) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: f16 x f16 -> f32 accumulate, K-major A and
// B, shape M x N (M = 64 or 128, N a multiple of 16 up to 256 for M = 128)
__host__ __device__ constexpr uint32_t mma_idesc_f16(int m, int n) {
    return (1u << 4) | (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16_id(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                           uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive on the mbarrier when every tcgen05 operation issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive TMEM columns of this warp's 32 lanes (one lane per thread)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void group_sync(int g) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kGroup) : "memory");
}

// Inverse FFT of one 2048-point line X (padded, see pad()) by the 128 threads
// of group g (thread lt of the group), Stockham radix 16, 16, 8 with the last
// stage pruned to the low half: on return mag[h][r] = |X[k]| for
// k = lt + 128 h + 256 r (k < N/2), the square root correctly rounded.  The
// transform is unnormalised (any 1/N is folded into the input).  X is
// overwritten.  tw2[r][j] = w^(r j N/256), tw3[r][j] = w^(r j), w = e^(2 pi i/N).
// ifft2048_low_mag_regs is the same transform with the first stage's inputs
// v[r] = x[lt + 128 r] already in registers (X is then only work space).
__device__ __forceinline__ void ifft2048_low_mag_regs(float2 (&v0)[16], float2* X, const float2 (*tw2)[16],
                                                      const float2 (*tw3)[256], int g, int lt,
                                                      float (&mag)[2][4]) {
    {
        float2 (&v)[16] = v0;
        dft16(v);
        group_sync(g);
#pragma unroll
        for (int r = 0; r < 16; ++r) X[pad(16 * lt + r)] = v[r];
        group_sync(g);
    }
    {
        float2 v[16];
        const int jm = lt & 15;
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = X[pad(lt + 128 * r)];
#pragma unroll
        for (int r = 1; r < 16; ++r) v[r] = cmul(v[r], tw2[r][jm]);
        dft16(v);
        group_sync(g);
        const int idxD = (lt >> 4) * 256 + jm;
#pragma unroll
        for (int r = 0; r < 16; ++r) X[pad(idxD + 16 * r)] = v[r];
        group_sync(g);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int j = lt + 128 * h;
        float2 v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = X[pad(j + 256 * r)];
#pragma unroll
        for (int r = 1; r < 8; ++r) v[r] = cmul(v[r], tw3[r][j]);
        float2 Xk[4];
        dft8_low(v, Xk);
#pragma unroll
        for (int r = 0; r < 4; ++r) mag[h][r] = __fsqrt_rn(fmaf(Xk[r].x, Xk[r].x, Xk[r].y * Xk[r].y));
    }
}

// The same transform with a second padded line Y: the first stage writes Y
// and the second writes X back, so a stage never overwrites the line it reads
// and only the barrier after its stores is needed (two group barriers per
// line instead of four).  X holds the input; both lines are work space.
__device__ __forceinline__ void ifft2048_low_mag_pp(float2* X, float2* Y, const float2 (*tw2)[16],
                                                    const float2 (*tw3)[256], int g, int lt, float (&mag)[2][4]) {
    {
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = X[pad(lt + 128 * r)];
        dft16(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) Y[pad(16 * lt + r)] = v[r];
        group_sync(g);
    }
    {
        float2 v[16];
        const int jm = lt & 15;
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = Y[pad(lt + 128 * r)];
#pragma unroll
        for (int r = 1; r < 16; ++r) v[r] = cmul(v[r], tw2[r][jm]);
        dft16(v);
        const int idxD = (lt >> 4) * 256 + jm;
#pragma unroll
        for (int r = 0; r < 16; ++r) X[pad(idxD + 16 * r)] = v[r];
        group_sync(g);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int j = lt + 128 * h;
        float2 v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = X[pad(j + 256 * r)];
#pragma unroll
        for (int r = 1; r < 8; ++r) v[r] = cmul(v[r], tw3[r][j]);
        float2 Xk[4];
        dft8_low(v, Xk);
#pragma unroll
        for (int r = 0; r < 4; ++r) mag[h][r] = __fsqrt_rn(fmaf(Xk[r].x, Xk[r].x, Xk[r].y * Xk[r].y));
    }
}

__device__ __forceinline__ void ifft2048_low_mag(float2* X, const float2 (*tw2)[16], const float2 (*tw3)[256],
                                                 int g, int lt, float (&mag)[2][4]) {
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = X[pad(lt + 128 * r)];
    ifft2048_low_mag_regs(v, X, tw2, tw3, g, lt, mag);
}

}  // namespace
}  // namespace octgb
