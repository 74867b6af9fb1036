/*
 * fft_cpu.c -- CPU complex FFTs used only by the test oracle (see fft_cpu.h).
 *
 * TEST INFRASTRUCTURE ONLY.  Written from the DFT definition; it stands in
 * for FFTW 3.3.5, which the reference links (TemsimLibrary/cfpix.cpp:140,157,
 * 225-236) but which is not installed here.
 */
#include "fft_cpu.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int n, sign;
    int *rev;      /* bit-reversal permutation (power-of-two n) */
    double *twd;   /* exp(sign*2*pi*i*k/n), k < n (interleaved) */
    float *twf;    /* the same, rounded to float */
} oc_plan;

#define OC_MAX_PLANS 64
static oc_plan g_plans[OC_MAX_PLANS];
static int g_nplans = 0;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static const oc_plan *get_plan(int n, int sign)
{
    const oc_plan *found = NULL;
    pthread_mutex_lock(&g_lock);
    for (int i = 0; i < g_nplans; i++)
        if (g_plans[i].n == n && g_plans[i].sign == sign) { found = &g_plans[i]; break; }
    if (!found && g_nplans < OC_MAX_PLANS) {
        oc_plan *p = &g_plans[g_nplans];
        p->n = n;
        p->sign = sign;
        p->twd = (double *)malloc(sizeof(double) * 2 * (size_t)n);
        p->twf = (float *)malloc(sizeof(float) * 2 * (size_t)n);
        const double twopi = 8.0 * atan(1.0);
        for (int k = 0; k < n; k++) {
            double a = sign * twopi * (double)k / (double)n;
            p->twd[2 * k] = cos(a);
            p->twd[2 * k + 1] = sin(a);
            p->twf[2 * k] = (float)p->twd[2 * k];
            p->twf[2 * k + 1] = (float)p->twd[2 * k + 1];
        }
        p->rev = NULL;
        if (is_pow2(n)) {
            int lg = 0;
            while ((1 << lg) < n) lg++;
            p->rev = (int *)malloc(sizeof(int) * (size_t)n);
            for (int i = 0; i < n; i++) {
                int r = 0;
                for (int b = 0; b < lg; b++) if (i & (1 << b)) r |= 1 << (lg - 1 - b);
                p->rev[i] = r;
            }
        }
        g_nplans++;
        found = p;
    }
    pthread_mutex_unlock(&g_lock);
    return found;
}

/* One contiguous line of n complex values, in place. */
#define OC_DEFINE_LINE(T, SUF, TW)                                                   \
    static void line_##SUF(T *a, int n, const oc_plan *p, T *tmp)                    \
    {                                                                                \
        if (p->rev) {                                                                \
            for (int i = 0; i < n; i++) {                                            \
                int r = p->rev[i];                                                   \
                if (r > i) {                                                         \
                    T t0 = a[2 * i], t1 = a[2 * i + 1];                              \
                    a[2 * i] = a[2 * r]; a[2 * i + 1] = a[2 * r + 1];                \
                    a[2 * r] = t0; a[2 * r + 1] = t1;                                \
                }                                                                    \
            }                                                                        \
            for (int len = 2; len <= n; len <<= 1) {                                 \
                int half = len >> 1, step = n / len;                                 \
                for (int j = 0; j < half; j++) {                                     \
                    T wr = p->TW[2 * j * step], wi = p->TW[2 * j * step + 1];        \
                    for (int i = j; i < n; i += len) {                               \
                        T *u = a + 2 * i, *v = a + 2 * (i + half);                   \
                        T tr = v[0] * wr - v[1] * wi;                                \
                        T ti = v[0] * wi + v[1] * wr;                                \
                        v[0] = u[0] - tr; v[1] = u[1] - ti;                          \
                        u[0] = u[0] + tr; u[1] = u[1] + ti;                          \
                    }                                                                \
                }                                                                    \
            }                                                                        \
        } else {                                                                     \
            for (int k = 0; k < n; k++) {                                            \
                double sr = 0.0, si = 0.0;                                           \
                for (int j = 0; j < n; j++) {                                        \
                    long m = ((long)j * (long)k) % n;                                \
                    double wr = p->twd[2 * m], wi = p->twd[2 * m + 1];               \
                    sr += (double)a[2 * j] * wr - (double)a[2 * j + 1] * wi;         \
                    si += (double)a[2 * j] * wi + (double)a[2 * j + 1] * wr;         \
                }                                                                    \
                tmp[2 * k] = (T)sr; tmp[2 * k + 1] = (T)si;                          \
            }                                                                        \
            memcpy(a, tmp, sizeof(T) * 2 * (size_t)n);                               \
        }                                                                            \
    }                                                                                \
                                                                                     \
    void ocfft1d_many_##SUF(T *data, int n, int howmany, int stride, int dist, int sign) \
    {                                                                                \
        const oc_plan *p = get_plan(n, sign);                                        \
        T *buf = (T *)malloc(sizeof(T) * 4 * (size_t)n);                             \
        T *tmp = buf + 2 * (size_t)n;                                                \
        for (int l = 0; l < howmany; l++) {                                          \
            T *base = data + 2 * (size_t)l * (size_t)dist;                           \
            if (stride == 1) { line_##SUF(base, n, p, tmp); continue; }              \
            for (int j = 0; j < n; j++) {                                            \
                buf[2 * j] = base[2 * (size_t)j * stride];                           \
                buf[2 * j + 1] = base[2 * (size_t)j * stride + 1];                   \
            }                                                                        \
            line_##SUF(buf, n, p, tmp);                                              \
            for (int j = 0; j < n; j++) {                                            \
                base[2 * (size_t)j * stride] = buf[2 * j];                           \
                base[2 * (size_t)j * stride + 1] = buf[2 * j + 1];                   \
            }                                                                        \
        }                                                                            \
        free(buf);                                                                   \
    }                                                                                \
                                                                                     \
    void ocfft2d_##SUF(T *data, int n0, int n1, int sign)                            \
    {                                                                                \
        /* rows: contiguous lines of length n1 */                                    \
        const oc_plan *p1 = get_plan(n1, sign);                                      \
        T *tmp = (T *)malloc(sizeof(T) * 2 * (size_t)(n0 > n1 ? n0 : n1));           \
        for (int i0 = 0; i0 < n0; i0++) line_##SUF(data + 2 * (size_t)i0 * n1, n1, p1, tmp); \
        /* columns: gather blocks of columns into contiguous lines */                \
        const oc_plan *p0 = get_plan(n0, sign);                                      \
        enum { B = 8 };                                                              \
        T *blk = (T *)malloc(sizeof(T) * 2 * (size_t)n0 * B);                        \
        for (int c0 = 0; c0 < n1; c0 += B) {                                         \
            int nb = (n1 - c0) < B ? (n1 - c0) : B;                                  \
            for (int i0 = 0; i0 < n0; i0++) {                                        \
                const T *row = data + 2 * ((size_t)i0 * n1 + c0);                    \
                for (int b = 0; b < nb; b++) {                                       \
                    blk[2 * ((size_t)b * n0 + i0)] = row[2 * b];                     \
                    blk[2 * ((size_t)b * n0 + i0) + 1] = row[2 * b + 1];             \
                }                                                                    \
            }                                                                        \
            for (int b = 0; b < nb; b++) line_##SUF(blk + 2 * (size_t)b * n0, n0, p0, tmp); \
            for (int i0 = 0; i0 < n0; i0++) {                                        \
                T *row = data + 2 * ((size_t)i0 * n1 + c0);                          \
                for (int b = 0; b < nb; b++) {                                       \
                    row[2 * b] = blk[2 * ((size_t)b * n0 + i0)];                     \
                    row[2 * b + 1] = blk[2 * ((size_t)b * n0 + i0) + 1];             \
                }                                                                    \
            }                                                                        \
        }                                                                            \
        free(blk);                                                                   \
        free(tmp);                                                                   \
    }

OC_DEFINE_LINE(float, f, twf)
OC_DEFINE_LINE(double, d, twd)
