/* Oracle (test infrastructure and timed CPU baseline only): C restatement of the reference's native row kernels,
 * cpp/oblique.cpp of dsrim/adrt-pinv. Same entry points, argument meaning and results:
 *   bfly_rows   (cpp/oblique.cpp:56-70)   in-place forward / adjoint butterflies over levels m_lo..m_hi, K rows of N
 *   cheb_rows   (cpp/oblique.cpp:74-104)  fused Chebyshev semi-iteration Z_k = p_k(B^*B) Y_k per row
 *   cert_rowsum (cpp/oblique.cpp:108-130) certified row-sum bound on lambda_max(M_k)
 *   omp_max_threads (cpp/oblique.cpp:132-138)
 * Complex data are interleaved (re, im) doubles, C-contiguous rows. OpenMP over rows, one private scratch set per
 * thread. The product never links this file; bench.py times it on the host cores as the CPU baseline when the
 * reference's own library cannot be built there.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* z^t for t = 0..half by repeated multiplication (cpp/oblique.cpp:16-19) */
static void powers(cplx z, int half, cplx *pw) {
    pw[0] = 1.0;
    for (int t = 1; t <= half; ++t) pw[t] = pw[t - 1] * z;
}

/* levels m_lo..m_hi forward; ping-pong between a and b; returns the buffer holding the result
 * (cpp/oblique.cpp:22-33): o[2t] = f0[t] + z^t f1[t], o[2t+1] = f0[t] + z * (z^t f1[t]) */
static cplx *fwd_levels(int n, const cplx *pw, cplx z, cplx *a, cplx *b, int m_lo, int m_hi) {
    const int N = 1 << n;
    cplx *src = a, *dst = b;
    for (int m = m_lo; m <= m_hi; ++m) {
        const int w = 1 << (m - 1);
        for (int base = 0; base < N; base += 2 * w) {
            for (int t = 0; t < w; ++t) {
                const cplx f0 = src[base + t];
                const cplx u = pw[t] * src[base + w + t];
                dst[base + 2 * t] = f0 + u;
                dst[base + 2 * t + 1] = f0 + u * z;
            }
        }
        cplx *s = src; src = dst; dst = s;
    }
    return src;
}

/* levels m_hi..m_lo adjoint (cpp/oblique.cpp:36-51): o0[t] = g0 + g1, o1[t] = conj(z^t) (g0 + conj(z) g1) */
static cplx *adj_levels(int n, const cplx *pw, cplx z, cplx *a, cplx *b, int m_lo, int m_hi) {
    const int N = 1 << n;
    const cplx zc = conj(z);
    cplx *src = a, *dst = b;
    for (int m = m_hi; m >= m_lo; --m) {
        const int w = 1 << (m - 1);
        for (int base = 0; base < N; base += 2 * w) {
            for (int t = 0; t < w; ++t) {
                const cplx g0 = src[base + 2 * t], g1 = src[base + 2 * t + 1];
                dst[base + t] = g0 + g1;
                dst[base + w + t] = conj(pw[t]) * (g0 + zc * g1);
            }
        }
        cplx *s = src; src = dst; dst = s;
    }
    return src;
}

static int nthr(int nthreads) { return nthreads > 0 ? nthreads : 1; }

void bfly_rows(int n, int K, const cplx *z, cplx *X, int m_lo, int m_hi, int transpose, int nthreads) {
    const int N = 1 << n;
#pragma omp parallel num_threads(nthr(nthreads))
    {
        cplx *pw = malloc(sizeof(cplx) * (N / 2 + 2));
        cplx *a = malloc(sizeof(cplx) * N), *b = malloc(sizeof(cplx) * N);
#pragma omp for schedule(dynamic, 4)
        for (int k = 0; k < K; ++k) {
            powers(z[k], N / 2, pw);
            memcpy(a, X + (size_t)k * N, sizeof(cplx) * N);
            cplx *r = transpose ? adj_levels(n, pw, z[k], a, b, m_lo, m_hi) : fwd_levels(n, pw, z[k], a, b, m_lo, m_hi);
            memcpy(X + (size_t)k * N, r, sizeof(cplx) * N);
        }
        free(pw); free(a); free(b);
    }
}

void cheb_rows(int n, int K, const cplx *z, const int *deg, const double *a, const double *c, double tau,
               const cplx *Y, cplx *Z, int m_lo, int m_hi, int nthreads, long long *steps) {
    const int N = 1 << n;
    long long total = 0;
#pragma omp parallel num_threads(nthr(nthreads)) reduction(+ : total)
    {
        cplx *pw = malloc(sizeof(cplx) * (N / 2 + 2));
        cplx *cur = malloc(sizeof(cplx) * N), *prev = malloc(sizeof(cplx) * N);
        cplx *s1 = malloc(sizeof(cplx) * N), *s2 = malloc(sizeof(cplx) * N);
#pragma omp for schedule(dynamic, 4)
        for (int k = 0; k < K; ++k) {
            const cplx *y = Y + (size_t)k * N;
            const double ak = a[k], ck = c[k];
            powers(z[k], N / 2, pw);
            for (int i = 0; i < N; ++i) { cur[i] = ak * y[i]; prev[i] = 0.0; }
            double om = 1.0;
            for (int j = 1; j < deg[k]; ++j) {
                const double omj = (j == 1) ? 1.0 / (1.0 - ck * ck / 2.0) : 1.0 / (1.0 - ck * ck * om / 4.0);
                memcpy(s1, cur, sizeof(cplx) * N);
                cplx *g = fwd_levels(n, pw, z[k], s1, s2, m_lo, m_hi);
                cplx *mz = adj_levels(n, pw, z[k], g, g == s1 ? s2 : s1, m_lo, m_hi);
                for (int i = 0; i < N; ++i) {
                    const cplx r = y[i] - mz[i] - tau * cur[i];
                    const cplx nz = cur[i] + omj * (ak * r) + (omj - 1.0) * (cur[i] - prev[i]);
                    prev[i] = cur[i];
                    cur[i] = nz;
                }
                om = omj;
                total += 2 * (m_hi - m_lo + 1);
            }
            memcpy(Z + (size_t)k * N, cur, sizeof(cplx) * N);
        }
        free(pw); free(cur); free(prev); free(s1); free(s2);
    }
    if (steps) *steps += total;
}

void cert_rowsum(int n, int K, const double *omega, int m_lo, double *out, int nthreads) {
    const long A = 1L << n;
#pragma omp parallel num_threads(nthr(nthreads))
    {
        double *r = malloc(sizeof(double) * (2 * A + 1)), *rn = malloc(sizeof(double) * (2 * A + 1));
#pragma omp for schedule(static)
        for (int k = 0; k < K; ++k) {
            const double om = omega[k];
            for (long i = 0; i <= 2 * A; ++i) r[i] = 1.0;
            for (int m = m_lo; m <= n; ++m) {
                const long amax = (1L << (n - m)) - 1;
                for (long i = 0; i <= 2 * A; ++i) rn[i] = 0.0;
                for (long q = -amax; q <= amax; ++q) {
                    /* |1 + z^q| = 2 |cos(q omega / 2)| */
                    const double f0 = 2.0 * fabs(cos(0.5 * om * (double)q));
                    const double fp = 2.0 * fabs(cos(0.5 * om * (double)(q + 1)));
                    const double fm = 2.0 * fabs(cos(0.5 * om * (double)(q - 1)));
                    const double t0 = f0 * r[2 * q + A], tp = fp * r[2 * q + 1 + A], tm = fm * r[2 * q - 1 + A];
                    rn[q + A] = t0 + (tp > tm ? tp : tm);
                }
                double *s = r; r = rn; rn = s;
            }
            out[k] = r[A];
        }
        free(r); free(rn);
    }
}

int omp_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
