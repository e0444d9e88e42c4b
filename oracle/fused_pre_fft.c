/*
 * ORACLE — test infrastructure only. Nothing in the product path links or calls
 * this file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * use it, as the checker and as the timed CPU reference arm.
 *
 * Plain-C/OpenMP restatement of the reference CPU kernel
 *   octrecon/core/cpu_kernels.py:12-41  (fused_pre_fft, Numba parallel=True,
 *   fastmath=False)
 * with its exact numeric types:
 *   - apodisation mean: float64 sum of the raw counts (cpu_kernels.py:22-24),
 *     divided in float64, STORED as float32 (apod has w.dtype, :19,25);
 *   - d[j] = raw - apod, stored float32 (:29,32);
 *   - line mean m: float64 sum of the float32 d[j], divided by N (:30-34);
 *   - d[j] -= m, computed in float64 and stored float32 (:35-36);
 *   - acc: float64 sum of float32 products w[t,i]*d[idx[t,i]] (:38-40);
 *   - out = (acc + m) * window[i]: float64 times complex, stored complex64 (:41).
 * Build with -ffp-contract=off so no product/sum pair is fused (Numba with
 * fastmath=False does not contract either).
 *
 * raw:    (B, interf, N) of dtype code 0=uint16, 1=int16, 2=float32
 * idx:    (T, N) int64 source indices      (SpectralProcessor.idx, spectral.py:217)
 * w:      (T, N) float32 weights           (spectral.py:218)
 * window: (N, 2) float32 re/im             (spectral.py:219, complex64)
 * out:    (B, nX, N, 2) float32 re/im      (complex64)
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static inline double raw_at(const void *raw, int dtype, int64_t k)
{
    switch (dtype) {
    case 0: return (double)((const uint16_t *)raw)[k];
    case 1: return (double)((const int16_t *)raw)[k];
    default: return (double)((const float *)raw)[k];
    }
}

static inline float raw_at_f32(const void *raw, int dtype, int64_t k)
{
    switch (dtype) {
    case 0: return (float)((const uint16_t *)raw)[k];
    case 1: return (float)((const int16_t *)raw)[k];
    default: return ((const float *)raw)[k];
    }
}

int oracle_fused_pre_fft(const void *raw, int dtype, int B, int interf, int apod_size, int N, int T,
                         const int64_t *idx, const float *w, const float *window, float *out)
{
    if (B < 0 || apod_size < 1 || interf <= apod_size || N < 2 || T < 1)
        return 1;
    const int nX = interf - apod_size;
    float *apod = (float *)malloc(sizeof(float) * (size_t)B * (size_t)N);
    if (!apod)
        return 2;

    #pragma omp parallel for schedule(static)
    for (int b = 0; b < B; ++b) {
        for (int j = 0; j < N; ++j) {
            double s = 0.0;
            for (int a = 0; a < apod_size; ++a)
                s += raw_at(raw, dtype, ((int64_t)b * interf + a) * N + j);
            apod[(int64_t)b * N + j] = (float)(s / apod_size);
        }
    }

    int fail = 0;
    #pragma omp parallel
    {
        float *d = (float *)malloc(sizeof(float) * (size_t)N);
        if (!d) {
            #pragma omp atomic write
            fail = 2;
        }
        #pragma omp for schedule(static)
        for (int64_t p = 0; p < (int64_t)B * nX; ++p) {
            if (!d)
                continue;
            const int64_t b = p / nX;
            const int64_t x = p - b * nX;
            const int64_t row = (b * interf + apod_size + x) * N;
            const float *ap = apod + b * N;
            double m = 0.0;
            for (int j = 0; j < N; ++j) {
                /* float32 difference: exactly the rounding of (raw - apod) to float32 */
                d[j] = raw_at_f32(raw, dtype, row + j) - ap[j];
                m += (double)d[j];
            }
            m = m / N;
            for (int j = 0; j < N; ++j)
                d[j] = (float)((double)d[j] - m);
            float *o = out + (p * (int64_t)N) * 2;
            for (int i = 0; i < N; ++i) {
                double acc = 0.0;
                for (int t = 0; t < T; ++t) {
                    const float prod = w[(int64_t)t * N + i] * d[idx[(int64_t)t * N + i]];
                    acc += (double)prod;
                }
                const double v = acc + m;
                o[2 * i] = (float)(v * (double)window[2 * i]);
                o[2 * i + 1] = (float)(v * (double)window[2 * i + 1]);
            }
        }
        free(d);
    }
    free(apod);
    return fail;
}
