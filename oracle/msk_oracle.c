/*
 * msk_oracle.c -- CPU restatement of the reference's multislice hot path
 * (see msk_oracle.h).  TEST INFRASTRUCTURE ONLY.
 *
 * Each function names the reference lines it restates.  The *_f32 variants
 * keep the reference's float/double mix operation by operation; built with
 * -ffp-contract=off and linked with the same FFT as oracle/_ref they give
 * the same bits as the reference build.  The *_f64 variants carry every
 * value in double.
 */
#include "msk_oracle.h"

#include <math.h>
#include <stdint.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "fft_cpu.h"

/* Kirkland's scattering-factor fit parameters (slicelib.cpp:958-2212). */
static const double kFe[104][12] = {
#include "../utr_public_gb300/csrc/kirkland_fparams.inc"
};

static int to_int(float x) { return (int)(x + 0.1F); } /* ToInt, slicelib.hpp:260 */

/* ---------------------------------------------------------------- physics */

/* slicelib.cpp:2891-2902 */
double mo_wavelength(double kev)
{
    const double emass = 510.99906, hc = 12.3984244;
    return hc / sqrt(kev * (2 * emass + kev));
}

/* slicelib.cpp:2441-2455 */
double mo_sigma(double kev)
{
    const double emass = 510.99906;
    double x = (emass + kev) / (2.0 * emass + kev);
    double wavl = mo_wavelength(kev);
    double pi = 4.0 * atan(1.0);
    return 2.0 * pi * x / (wavl * kev);
}

/* slicelib.cpp:457-474 */
void mo_freqn(float *ko, float *ko2, float *xo, int nk, double ak)
{
    int imid = (int)(nk / 2.0 + 0.5);
    for (int i = 0; i < nk; i++) {
        xo[i] = ((float)(i * ak)) / ((float)(nk - 1));
        if (i > imid) ko[i] = ((float)(i - nk)) / ((float)ak);
        else ko[i] = ((float)i) / ((float)ak);
        ko2[i] = ko[i] * ko[i];
    }
}

/* Modified Bessel I0, Abramowitz & Stegun 9.8.1-9.8.2 (slicelib.cpp:189-215). */
double mo_bessi0(double x)
{
    static const double a[] = {1.0, 3.5156229, 3.0899424, 1.2067492, 0.2659732, 0.0360768, 0.0045813};
    static const double b[] = {0.39894228, 0.01328592, 0.00225319, -0.00157565, 0.00916281,
                               -0.02057706, 0.02635537, -0.01647633, 0.00392377};
    double ax = fabs(x), sum, t;
    if (ax <= 3.75) {
        t = x / 3.75;
        t = t * t;
        sum = a[6];
        for (int i = 5; i >= 0; i--) sum = sum * t + a[i];
    } else {
        t = 3.75 / ax;
        sum = b[8];
        for (int i = 7; i >= 0; i--) sum = sum * t + b[i];
        sum = exp(ax) * sum / sqrt(ax);
    }
    return sum;
}

/* Modified Bessel K0, Abramowitz & Stegun 9.8.5-9.8.6 (slicelib.cpp:231-258). */
double mo_bessk0(double x)
{
    static const double a[] = {-0.57721566, 0.42278420, 0.23069756, 0.03488590, 0.00262698, 0.00010750, 0.00000740};
    static const double b[] = {1.25331414, -0.07832358, 0.02189568, -0.01062446, 0.00587872, -0.00251540, 0.00053208};
    double ax = fabs(x), x2, sum;
    if ((ax > 0.0) && (ax <= 2.0)) {
        x2 = ax / 2.0;
        x2 = x2 * x2;
        sum = a[6];
        for (int i = 5; i >= 0; i--) sum = sum * x2 + a[i];
        sum = -log(ax / 2.0) * mo_bessi0(x) + sum;
    } else if (ax > 2.0) {
        x2 = 2.0 / ax;
        sum = b[6];
        for (int i = 5; i >= 0; i--) sum = sum * x2 + b[i];
        sum = exp(-ax) * sum / sqrt(ax);
    } else {
        sum = 1.0e20;
    }
    return sum;
}

/* Projected atomic potential in V*Angstrom (slicelib.cpp:2759-2792). */
double mo_vzatom(int Z, double radius)
{
    const double al = 300.8242834, ag = 150.4121417, pi = 3.141592654;
    if (Z < 1 || Z > 103) return 0.0;
    double r = fabs(radius);
    if (r < 1.0e-10) r = 1.0e-10;
    double suml = 0.0, sumg = 0.0;
    double x = 2.0 * pi * r;
    for (int i = 0; i < 6; i += 2) suml += kFe[Z][i] * mo_bessk0(x * sqrt(kFe[Z][i + 1]));
    x = pi * r;
    x = x * x;
    for (int i = 6; i < 12; i += 2) sumg += kFe[Z][i] * exp(-x / kFe[Z][i + 1]) / kFe[Z][i + 1];
    return al * suml + ag * sumg;
}

/* Akima quasi-Hermite cubic spline coefficients (slicelib.cpp:2537-2603). */
void mo_splinh(const double *x, const double *y, double *b, double *c, double *d, int n)
{
    const double SMALL = 1.0e-25;
    double m1, m2, m3, m4, m5, t1, t2, m54, m43, m32, m21, x43;
    if (n < 4) return;
    m5 = (y[3] - y[2]) / (x[3] - x[2]);
    m4 = (y[2] - y[1]) / (x[2] - x[1]);
    m3 = (y[1] - y[0]) / (x[1] - x[0]);
    m2 = m3 + m3 - m4;
    m1 = m2 + m2 - m3;
    m54 = fabs(m5 - m4);
    m43 = fabs(m4 - m3);
    m32 = fabs(m3 - m2);
    m21 = fabs(m2 - m1);
    if ((m43 + m21) > SMALL) t1 = (m43 * m2 + m21 * m3) / (m43 + m21);
    else t1 = 0.5 * (m2 + m3);
    int nm1 = n - 1, nm4 = n - 4;
    for (int i = 0; i < nm1; i++) {
        if ((m54 + m32) > SMALL) t2 = (m54 * m3 + m32 * m4) / (m54 + m32);
        else t2 = 0.5 * (m3 + m4);
        x43 = x[i + 1] - x[i];
        b[i] = t1;
        c[i] = (3.0 * m3 - t1 - t1 - t2) / x43;
        d[i] = (t1 + t2 - m3 - m3) / (x43 * x43);
        m1 = m2;
        m2 = m3;
        m3 = m4;
        m4 = m5;
        if (i < nm4) m5 = (y[i + 4] - y[i + 3]) / (x[i + 4] - x[i + 3]);
        else m5 = m4 + m4 - m3;
        m21 = m32;
        m32 = m43;
        m43 = m54;
        m54 = fabs(m5 - m4);
        t1 = t2;
    }
    (void)m1;
    (void)m21;
}

/* Spline evaluation with bisection for the interval (slicelib.cpp:2402-2425). */
double mo_seval(const double *x, const double *y, const double *b, const double *c,
                const double *d, int n, double x0)
{
    int i, j, k;
    if (x0 <= x[0]) i = 0;
    else if (x0 >= x[n - 2]) i = n - 2;
    else {
        i = 0;
        j = n;
        do {
            k = (i + j) / 2;
            if (x0 < x[k]) j = k;
            else if (x0 >= x[k]) i = k;
        } while ((j - i) > 1);
    }
    double z = x0 - x[i];
    return y[i] + (b[i] + (c[i] + d[i] * z) * z) * z;
}

/* Look-up table of vzatom vs r^2 (slicelib.cpp:2812-2875): 100 knots,
 * r log-spaced from 0.01 to 5 Angstrom, then squared.  Built lazily per Z
 * under a lock so that the threaded baseline can share it. */
#define LUT_N 100
static double g_knots[LUT_N];
static double g_y[104][LUT_N], g_b[104][LUT_N], g_c[104][LUT_N], g_d[104][LUT_N];
static int g_ready[104];
static int g_knots_ready = 0;
static pthread_mutex_t g_lut_lock = PTHREAD_MUTEX_INITIALIZER;

static void lut_build(int Z)
{
    pthread_mutex_lock(&g_lut_lock);
    if (!g_knots_ready) {
        const double RMIN = 0.01, RMAX = 5.0;
        double dlnr = log(RMAX / RMIN) / (LUT_N - 1);
        for (int i = 0; i < LUT_N; i++) g_knots[i] = RMIN * exp(i * dlnr);
        for (int i = 0; i < LUT_N; i++) g_knots[i] = g_knots[i] * g_knots[i];
        g_knots_ready = 1;
    }
    if (!g_ready[Z]) {
        for (int i = 0; i < LUT_N; i++) g_y[Z][i] = mo_vzatom(Z, sqrt(g_knots[i]));
        mo_splinh(g_knots, g_y[Z], g_b[Z], g_c[Z], g_d[Z], LUT_N);
        __atomic_store_n(&g_ready[Z], 1, __ATOMIC_RELEASE);
    }
    pthread_mutex_unlock(&g_lut_lock);
}

double mo_vzatomLUT(int Z, double rsq)
{
    if (Z < 1 || Z > 103) return 0.0;
    if (!__atomic_load_n(&g_ready[Z], __ATOMIC_ACQUIRE)) lut_build(Z);
    return mo_seval(g_knots, g_y[Z], g_b[Z], g_c[Z], g_d[Z], LUT_N, rsq);
}

int mo_lut_table(int Z, double *knots, double *y, double *b, double *c, double *d)
{
    if (Z < 1 || Z > 103) return MO_EZNUM;
    if (!__atomic_load_n(&g_ready[Z], __ATOMIC_ACQUIRE)) lut_build(Z);
    memcpy(knots, g_knots, sizeof g_knots);
    memcpy(y, g_y[Z], sizeof(double) * LUT_N);
    memcpy(b, g_b[Z], sizeof(double) * LUT_N);
    memcpy(c, g_c[Z], sizeof(double) * LUT_N);
    memcpy(d, g_d[Z], sizeof(double) * LUT_N);
    return MO_OK;
}

/* ----------------------------------------------------------- host prep */

/* Shell sort by z, h = 1, 4, 13, ... (slicelib.cpp:2467-2504). */
void mo_sortByZ(float *x, float *y, float *z, float *occ, int *Znum, int natom)
{
    int i, j, h;
    for (h = 1; h <= (natom - 1) / 9; h = 3 * h + 1)
        ;
    for (; h > 0; h /= 3)
        for (i = h; i < natom; i++) {
            j = i;
            float x2 = x[i], y2 = y[i], z2 = z[i], occ2 = occ[i];
            int Z2 = Znum[i];
            while ((j >= h) && (z2 < z[j - h])) {
                x[j] = x[j - h];
                y[j] = y[j - h];
                z[j] = z[j - h];
                occ[j] = occ[j - h];
                Znum[j] = Znum[j - h];
                j -= h;
            }
            x[j] = x2;
            y[j] = y2;
            z[j] = z2;
            occ[j] = occ2;
            Znum[j] = Z2;
        }
}

/* Rotation about z, then about y' (autosliccmd.cpp:727-748), in float. */
void mo_rotate(float ctblength, double dxc, double dyc, double dzc, double angleZ,
               double angleY, int natom, float *x, float *y, float *z)
{
    float xc = (float)(ctblength / 2.0 + dxc), yc = (float)(ctblength / 2.0 + dyc),
          zc = (float)(ctblength / 2.0 + dzc);
    float sinZ = (float)sin(angleZ), cosZ = (float)cos(angleZ), sinY = (float)sin(angleY),
          cosY = (float)cos(angleY);
    for (int k = 0; k < natom; k++) {
        float xxx = xc + (x[k] - xc) * cosZ + (-y[k] + yc) * sinZ;
        float yyy = yc + (x[k] - xc) * sinZ + (y[k] - yc) * cosZ;
        x[k] = xxx;
        y[k] = yyy;
    }
    for (int k = 0; k < natom; k++) {
        float xxx = xc + (x[k] - xc) * cosY + (z[k] - zc) * sinY;
        float zzz = zc + (-x[k] + xc) * sinY + (z[k] - zc) * cosY;
        x[k] = xxx;
        z[k] = zzz;
    }
}

/* Remove atoms outside the box, keeping order: the reference's own rule in
 * its disabled block (autosliccmd.cpp:791-820), with the z bound taken as
 * the box depth.  Returns the number kept. */
int mo_drop_outside(float ctblength, float ctblengthz, int natom, float *x, float *y,
                    float *z, float *occ, int *Znum)
{
    int n = 0;
    for (int k = 0; k < natom; k++) {
        if (x[k] < 0 || x[k] > ctblength || y[k] < 0 || y[k] > ctblength || z[k] < 0 ||
            z[k] > ctblengthz)
            continue;
        x[n] = x[k];
        y[n] = y[k];
        z[n] = z[k];
        occ[n] = occ[k];
        Znum[n] = Znum[k];
        n++;
    }
    return n;
}

/* Slice loop bounds of the coherent branch (autoslic.cpp:747-756,828). */
int mo_slice_count(float deltaz_f, float zmax)
{
    double deltaz = deltaz_f, zslice = deltaz;
    int n = 0;
    while (zslice < (zmax + deltaz)) {
        n++;
        zslice += deltaz;
    }
    return n;
}

/* Slice of every atom of a z-sorted list (autoslic.cpp:756-762,828-830). */
int mo_slice_assign(float deltaz_f, float zmax, int natom, const float *z2, int *slice_of)
{
    double deltaz = deltaz_f, zslice = deltaz;
    int istart = 0, islice = 0;
    while (zslice < (zmax + deltaz)) {
        int na = 0;
        for (int i = istart; i < natom; i++)
            if (z2[i] < zslice) na++;
            else break;
        for (int i = istart; i < istart + na; i++) slice_of[i] = islice;
        zslice += deltaz;
        istart += na;
        islice++;
    }
    for (int i = istart; i < natom; i++) slice_of[i] = -1;
    return islice;
}

/* ------------------------------------------------------- multislice, FP32 */

/* cfpix::fft / cfpix::ifft (cfpix.cpp:137-193): fft is the FFTW_BACKWARD
 * (+) kernel, ifft the FFTW_FORWARD (-) kernel followed by 1/(nx*ny). */
static void cf_fft_f(float *a, int nx, int ny) { ocfft2d_f(a, nx, ny, +1); }
static void cf_ifft_f(float *a, int nx, int ny)
{
    ocfft2d_f(a, nx, ny, -1);
    float scale = 1.0F / ((float)(nx * ny));
    size_t n = (size_t)nx * ny;
    for (size_t j = 0; j < n; j++) {
        a[2 * j] *= scale;
        a[2 * j + 1] *= scale;
    }
}
static void cf_fft_d(double *a, int nx, int ny) { ocfft2d_d(a, nx, ny, +1); }
static void cf_ifft_d(double *a, int nx, int ny)
{
    ocfft2d_d(a, nx, ny, -1);
    double scale = 1.0 / ((double)nx * (double)ny);
    size_t n = (size_t)nx * ny;
    for (size_t j = 0; j < n; j++) {
        a[2 * j] *= scale;
        a[2 * j + 1] *= scale;
    }
}

/* The projected potential of one slice accumulated in float into trans[2j]
 * (autoslic.cpp:943-984, the loop trlayer and trlayerDW share). */
static void potential_f32(const float *x, const float *y, const float *occ, const int *Znum,
                          int natom, float ax, float by, float *trans, int nx, int ny)
{
    const double rmax = 3.0, rmax2 = rmax * rmax;
    double scalex = ax / nx; /* float division, as in the reference */
    double scaley = by / ny;
    double rmin = ax / ((double)nx);
    double r = by / ((double)ny);
    rmin = 0.25 * sqrt(0.5 * (rmin * rmin + r * r));
    double rminsq = rmin * rmin;
    int idx = (int)(nx * rmax / ax) + 1;
    int idy = (int)(ny * rmax / by) + 1;
    size_t n = (size_t)nx * ny;
    for (size_t j = 0; j < n; j++) trans[2 * j] = 0.0F;
    for (int i = 0; i < natom; i++) {
        int ixo = (int)(x[i] / scalex), iyo = (int)(y[i] / scaley);
        int nx1 = ixo - idx, nx2 = ixo + idx, ny1 = iyo - idy, ny2 = iyo + idy;
        for (int ix = nx1; ix <= nx2; ix++) {
            double rx2 = x[i] - ((double)ix) * scalex;
            rx2 = rx2 * rx2;
            int ixw = ix;
            while (ixw < 0) ixw = ixw + nx;
            ixw = ixw % nx;
            for (int iy = ny1; iy <= ny2; iy++) {
                double rsq = y[i] - ((double)iy) * scaley;
                rsq = rx2 + rsq * rsq;
                if (rsq <= rmax2) {
                    int iyw = iy;
                    while (iyw < 0) iyw = iyw + ny;
                    iyw = iyw % ny;
                    if (rsq < rminsq) rsq = rminsq;
                    double vz = occ[i] * mo_vzatomLUT(Znum[i], rsq);
                    trans[2 * ((size_t)iyw + (size_t)ixw * ny)] += (float)vz;
                }
            }
        }
    }
}

/* t = exp(i scale v), then the 2/3 band limit (autoslic.cpp:986-1009). */
static void phase_bandlimit_f32(float *trans, double scale, int nx, int ny, const float *kx2,
                                const float *ky2, float k2max)
{
    size_t n = (size_t)nx * ny;
    for (size_t j = 0; j < n; j++) {
        double vz = scale * trans[2 * j];
        trans[2 * j] = (float)cos(vz);
        trans[2 * j + 1] = (float)sin(vz);
    }
    cf_fft_f(trans, nx, ny);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            float k2 = ky2[iy] + kx2[ix];
            if (!(k2 < k2max)) trans[2 * ((size_t)iy + (size_t)ix * ny)] = trans[2 * ((size_t)iy + (size_t)ix * ny) + 1] = 0.0F;
        }
    cf_ifft_f(trans, nx, ny);
}

/* Transmission function of one slice (autoslic.cpp:917-1013). */
static void trlayer_f32(const float *x, const float *y, const float *occ, const int *Znum,
                        int natom, float ax, float by, float kev, float *trans, int nx, int ny,
                        const float *kx2, const float *ky2, float k2max)
{
    potential_f32(x, y, occ, Znum, natom, ax, by, trans, nx, ny);
    phase_bandlimit_f32(trans, mo_sigma(kev) / 1000.0, nx, ny, kx2, ky2, k2max);
}

/* Debye-Waller factor of one slice (autoslic.cpp:1049-1056): B averaged
 * over wobble[0 .. natom-1] -- the caller's first natom entries, as the
 * reference passes its unsorted wobble array with the slice's atom count. */
static double dw_bdw(const float *wobble, int natom, float temperature)
{
    const double twopi = 2.0 * (4.0 * atan(1.0));
    double scaleTemp2 = temperature / 300.0;
    double Bdw = 0;
    for (int i = 0; i < natom; i++) Bdw += wobble[i] * wobble[i] * scaleTemp2;
    Bdw /= natom;
    Bdw *= 2.0 * twopi * twopi;
    return Bdw;
}

/* trlayerDW (autoslic.cpp:1039-1160): the potential damped by exp(-B k^2/4)
 * (FFT, multiply, inverse FFT, real part), then as trlayer. */
static void trlayerDW_f32(const float *x, const float *y, const float *occ, const int *Znum,
                          int natom, float ax, float by, float kev, float *trans, int nx, int ny,
                          const float *kx2, const float *ky2, float k2max, const float *wobble,
                          float temperature)
{
    const double mBdw4 = -0.25 * dw_bdw(wobble, natom, temperature);
    size_t n = (size_t)nx * ny;
    potential_f32(x, y, occ, Znum, natom, ax, by, trans, nx, ny);
    for (size_t j = 0; j < n; j++) trans[2 * j + 1] = 0.0f;
    cf_fft_f(trans, nx, ny);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            float k2 = ky2[iy] + kx2[ix];
            float emM = (float)exp(mBdw4 * k2);
            trans[2 * ((size_t)iy + (size_t)ix * ny)] *= emM;
            trans[2 * ((size_t)iy + (size_t)ix * ny) + 1] *= emM;
        }
    cf_ifft_f(trans, nx, ny);
    phase_bandlimit_f32(trans, mo_sigma(kev) / 1000.0, nx, ny, kx2, ky2, k2max);
}

/* Projected potential of one slice summed in double (the accumulation of
 * trlayer, autoslic.cpp:950-984): v[(iy + ix*ny) * vstride], V*Angstrom. */
static void potential_f64(const float *x, const float *y, const float *occ, const int *Znum,
                          int natom, float ax, float by, double *v, size_t vstride, int nx,
                          int ny)
{
    const double rmax = 3.0, rmax2 = rmax * rmax;
    double rmin = ax / ((double)nx);
    double r = by / ((double)ny);
    rmin = 0.25 * sqrt(0.5 * (rmin * rmin + r * r));
    double rminsq = rmin * rmin;
    /* window and pixel centres use the reference's float-divided step so
     * that the same pixels are visited */
    double scalex_f = ax / nx, scaley_f = by / ny;
    int idx = (int)(nx * rmax / ax) + 1;
    int idy = (int)(ny * rmax / by) + 1;
    size_t n = (size_t)nx * ny;
    for (size_t j = 0; j < n; j++) v[j * vstride] = 0.0;
    for (int i = 0; i < natom; i++) {
        int ixo = (int)(x[i] / scalex_f), iyo = (int)(y[i] / scaley_f);
        for (int ix = ixo - idx; ix <= ixo + idx; ix++) {
            double rx2 = x[i] - ((double)ix) * scalex_f;
            rx2 = rx2 * rx2;
            int ixw = ix;
            while (ixw < 0) ixw += nx;
            ixw %= nx;
            for (int iy = iyo - idy; iy <= iyo + idy; iy++) {
                double rsq = y[i] - ((double)iy) * scaley_f;
                rsq = rx2 + rsq * rsq;
                if (rsq <= rmax2) {
                    int iyw = iy;
                    while (iyw < 0) iyw += ny;
                    iyw %= ny;
                    if (rsq < rminsq) rsq = rminsq;
                    v[((size_t)iyw + (size_t)ixw * ny) * vstride] +=
                        occ[i] * mo_vzatomLUT(Znum[i], rsq);
                }
            }
        }
    }
}

static void phase_bandlimit_f64(double *trans, double scale, int nx, int ny, const float *kx2,
                                const float *ky2, float k2max);

/* Same slice in double: potential summed in double, double transform. */
static void trlayer_f64(const float *x, const float *y, const float *occ, const int *Znum,
                        int natom, float ax, float by, float kev, double *trans, int nx, int ny,
                        const float *kx2, const float *ky2, float k2max)
{
    potential_f64(x, y, occ, Znum, natom, ax, by, trans, 2, nx, ny);
    phase_bandlimit_f64(trans, mo_sigma(kev) / 1000.0, nx, ny, kx2, ky2, k2max);
}

/* trlayerDW in double (same B, the multiplier exp(-B k^2/4) in double). */
static void trlayerDW_f64(const float *x, const float *y, const float *occ, const int *Znum,
                          int natom, float ax, float by, float kev, double *trans, int nx,
                          int ny, const float *kx2, const float *ky2, float k2max,
                          const float *wobble, float temperature)
{
    const double mBdw4 = -0.25 * dw_bdw(wobble, natom, temperature);
    size_t n = (size_t)nx * ny;
    potential_f64(x, y, occ, Znum, natom, ax, by, trans, 2, nx, ny);
    for (size_t j = 0; j < n; j++) trans[2 * j + 1] = 0.0;
    cf_fft_d(trans, nx, ny);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            double emM = exp(mBdw4 * (double)(ky2[iy] + kx2[ix]));
            trans[2 * ((size_t)iy + (size_t)ix * ny)] *= emM;
            trans[2 * ((size_t)iy + (size_t)ix * ny) + 1] *= emM;
        }
    cf_ifft_d(trans, nx, ny);
    phase_bandlimit_f64(trans, mo_sigma(kev) / 1000.0, nx, ny, kx2, ky2, k2max);
}

static void phase_bandlimit_f64(double *trans, double scale, int nx, int ny, const float *kx2,
                                const float *ky2, float k2max)
{
    size_t n = (size_t)nx * ny;
    for (size_t j = 0; j < n; j++) {
        double vz = scale * trans[2 * j];
        trans[2 * j] = cos(vz);
        trans[2 * j + 1] = sin(vz);
    }
    cf_fft_d(trans, nx, ny);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            float k2 = ky2[iy] + kx2[ix];
            if (!(k2 < k2max)) trans[2 * ((size_t)iy + (size_t)ix * ny)] = trans[2 * ((size_t)iy + (size_t)ix * ny) + 1] = 0.0;
        }
    cf_ifft_d(trans, nx, ny);
}

/* Fresnel propagator multiply with the 2/3 aperture (slicelib.cpp:811-849). */
static void propagate_f32(float *w, const float *pxr, const float *pxi, const float *pyr,
                          const float *pyi, const float *kx2, const float *ky2, float k2max,
                          int nx, int ny)
{
    for (int ix = 0; ix < nx; ix++) {
        float *row = w + 2 * (size_t)ix * ny;
        if (kx2[ix] < k2max) {
            float xr = pxr[ix], xi = pxi[ix];
            for (int iy = 0; iy < ny; iy++) {
                if ((kx2[ix] + ky2[iy]) < k2max) {
                    float yr = pyr[iy], yi = pyi[iy];
                    float wr = row[2 * iy], wi = row[2 * iy + 1];
                    float tr = wr * yr - wi * yi;
                    float ti = wr * yi + wi * yr;
                    row[2 * iy] = tr * xr - ti * xi;
                    row[2 * iy + 1] = tr * xi + ti * xr;
                } else {
                    row[2 * iy] = 0.0F;
                    row[2 * iy + 1] = 0.0F;
                }
            }
        } else {
            for (int iy = 0; iy < ny; iy++) row[2 * iy] = row[2 * iy + 1] = 0.0F;
        }
    }
}

static void propagate_f64(double *w, const double *pxr, const double *pxi, const double *pyr,
                          const double *pyi, const float *kx2, const float *ky2, float k2max,
                          int nx, int ny)
{
    for (int ix = 0; ix < nx; ix++) {
        double *row = w + 2 * (size_t)ix * ny;
        for (int iy = 0; iy < ny; iy++) {
            if (kx2[ix] < k2max && (kx2[ix] + ky2[iy]) < k2max) {
                double wr = row[2 * iy], wi = row[2 * iy + 1];
                double tr = wr * pyr[iy] - wi * pyi[iy];
                double ti = wr * pyi[iy] + wi * pyr[iy];
                row[2 * iy] = tr * pxr[ix] - ti * pxi[ix];
                row[2 * iy + 1] = tr * pxi[ix] + ti * pxr[ix];
            } else {
                row[2 * iy] = row[2 * iy + 1] = 0.0;
            }
        }
    }
}

typedef struct {
    int nx, ny;
    float ax, by, v0, wavlen, k2max, tctx, tcty;
    double deltaz;
    float *kx, *kx2, *xpos, *ky, *ky2, *ypos;
} calc_setup;

static void setup_free(calc_setup *s)
{
    free(s->kx);
    free(s->kx2);
    free(s->xpos);
    free(s->ky);
    free(s->ky2);
    free(s->ypos);
}

/* Parameter read, checks and frequency grids (autoslic.cpp:238-393). */
static int calc_setup_init(calc_setup *s, const float *param, int natom, const int *Znum,
                           const float *x, const float *y, const float *z, float ctblength,
                           float ctblengthz)
{
    memset(s, 0, sizeof *s);
    s->ax = param[MO_pAX];
    s->by = param[MO_pBY];
    s->nx = to_int(param[MO_pNX]);
    s->ny = to_int(param[MO_pNY]);
    s->v0 = param[MO_pENERGY];
    s->deltaz = param[MO_pDELTAZ];
    if ((s->nx < 1) || (s->ny < 1) || (s->ax < 0.0) || (s->by < 0.0)) return MO_EBADSIZE;
    s->wavlen = (float)mo_wavelength(s->v0);
    if (natom > 0) {
        float xmin = x[0], xmax = x[0], ymin = y[0], ymax = y[0], zmin = z[0], zmax = z[0];
        for (int i = 0; i < natom; i++) {
            if (x[i] < xmin) xmin = x[i];
            if (x[i] > xmax) xmax = x[i];
            if (y[i] < ymin) ymin = y[i];
            if (y[i] > ymax) ymax = y[i];
            if (z[i] < zmin) zmin = z[i];
            if (z[i] > zmax) zmax = z[i];
            if (Znum[i] < 1 || Znum[i] > 103) return MO_EZNUM;
        }
        if (xmin < 0 || ymin < 0 || zmin < 0) return MO_EBOX;
        if (xmax > ctblength || ymax > ctblength || zmax > ctblengthz) return MO_EBOX;
    }
    int nx = s->nx, ny = s->ny;
    s->kx = (float *)malloc(sizeof(float) * nx);
    s->kx2 = (float *)malloc(sizeof(float) * nx);
    s->xpos = (float *)malloc(sizeof(float) * nx);
    s->ky = (float *)malloc(sizeof(float) * ny);
    s->ky2 = (float *)malloc(sizeof(float) * ny);
    s->ypos = (float *)malloc(sizeof(float) * ny);
    mo_freqn(s->kx, s->kx2, s->xpos, nx, s->ax);
    mo_freqn(s->ky, s->ky2, s->ypos, ny, s->by);
    const float BW = (2.0F / 3.0F);
    float k2max = nx / (2.0F * s->ax);
    float tctx = ny / (2.0F * s->by);
    if (tctx < k2max) k2max = tctx;
    k2max = BW * k2max;
    s->k2max = k2max * k2max;
    s->tctx = (float)(2.0 * tan(param[MO_pXCTILT]));
    s->tcty = (float)(2.0 * tan(param[MO_pYCTILT]));
    return MO_OK;
}

/* The Gaussian deviate the thermal wobble draws (autoslic.cpp:707-709 calls
 * gasdev from the XArrayLibrary, which is not part of the reference): this
 * project's definition, shared with oracle/ref_driver.cpp (the harness of
 * the reference build) --
 * two steps of the 64-bit LCG (6364136223846793005, 1442695040888963407) on
 * the seed, Box-Muller from the top 53 bits. */
double mo_gasdev(long *idum)
{
    uint64_t s = (uint64_t)(*idum) * 6364136223846793005ULL + 1442695040888963407ULL;
    uint64_t s2 = s * 6364136223846793005ULL + 1442695040888963407ULL;
    *idum = (long)s2;
    double u1 = ((s >> 11) + 1.0) / 9007199254740993.0;
    double u2 = (s2 >> 11) / 9007199254740992.0;
    return sqrt(-2.0 * log(u1)) * cos(8.0 * atan(1.0) * u2);
}

/* Sorted working copies of the atoms (autoslic.cpp:689-739), with the random
 * thermal displacement of lwobble == 1, nwobble > 1 (autoslic.cpp:701-713). */
static int sorted_copy_th(int natom, const int *Znum, const float *x, const float *y,
                          const float *z, const float *occ, float ctblengthz, float **x2,
                          float **y2, float **z2, float **occ2, int **Z2, const mo_thermal *th)
{
    size_t n = natom > 0 ? (size_t)natom : 1;
    *x2 = (float *)malloc(sizeof(float) * n);
    *y2 = (float *)malloc(sizeof(float) * n);
    *z2 = (float *)malloc(sizeof(float) * n);
    *occ2 = (float *)malloc(sizeof(float) * n);
    *Z2 = (int *)malloc(sizeof(int) * n);
    if (natom > 0) {
        memcpy(*x2, x, sizeof(float) * natom);
        memcpy(*y2, y, sizeof(float) * natom);
        memcpy(*z2, z, sizeof(float) * natom);
        memcpy(*occ2, occ, sizeof(float) * natom);
        memcpy(*Z2, Znum, sizeof(int) * natom);
        if (th && th->lwobble == 1 && th->nwobble > 1) {
            const float scale = (float)sqrt(th->temperature / 300.0);
            for (int i = 0; i < natom; i++) {
                (*x2)[i] = x[i] + (float)(th->wobble[i] * mo_gasdev(th->iseed) * scale);
                (*y2)[i] = y[i] + (float)(th->wobble[i] * mo_gasdev(th->iseed) * scale);
                (*z2)[i] = z[i] + (float)(th->wobble[i] * mo_gasdev(th->iseed) * scale);
            }
        }
        mo_sortByZ(*x2, *y2, *z2, *occ2, *Z2, natom);
        if ((*z2)[0] < 0 || (*z2)[natom - 1] > ctblengthz) return MO_EZSORT;
    }
    return MO_OK;
}

static int sorted_copy(int natom, const int *Znum, const float *x, const float *y,
                       const float *z, const float *occ, float ctblengthz, float **x2,
                       float **y2, float **z2, float **occ2, int **Z2)
{
    return sorted_copy_th(natom, Znum, x, y, z, occ, ctblengthz, x2, y2, z2, occ2, Z2, NULL);
}

/* autoslic::calculate coherent branch (autoslic.cpp:209-869, 666-837). */
int mo_calculate_f32(float *pix, const float *wave0, const float *param, int natom,
                     const int *Znum, const float *x, const float *y, const float *z,
                     const float *occ, float ctblength, float ctblengthz, int nmode,
                     int max_slices)
{
    return mo_calculate_sample_f32(pix, wave0, param, natom, Znum, x, y, z, occ, ctblength,
                                   ctblengthz, nmode, 0, max_slices);
}

static int calculate_f32(float *pix, const float *wave0, const float *param, int natom,
                         const int *Znum, const float *x, const float *y, const float *z,
                         const float *occ, float ctblength, float ctblengthz, int nmode,
                         int min_slice, int max_slices, const mo_thermal *th);

int mo_calculate_sample_f32(float *pix, const float *wave0, const float *param, int natom,
                            const int *Znum, const float *x, const float *y, const float *z,
                            const float *occ, float ctblength, float ctblengthz, int nmode,
                            int min_slice, int max_slices)
{
    return calculate_f32(pix, wave0, param, natom, Znum, x, y, z, occ, ctblength, ctblengthz,
                         nmode, min_slice, max_slices, NULL);
}

int mo_calculate_thermal_f32(float *pix, const float *wave0, const float *param, int natom,
                             const int *Znum, const float *x, const float *y, const float *z,
                             const float *occ, const float *wobble, float ctblength,
                             float ctblengthz, int nmode, int lwobble, long *iseed)
{
    mo_thermal th = {wobble, lwobble != 0, 0, param[MO_pTEMPER], iseed};
    th.nwobble = to_int(param[MO_pNWOBBLE]);
    if (th.nwobble < 1) th.nwobble = 1;
    return calculate_f32(pix, wave0, param, natom, Znum, x, y, z, occ, ctblength, ctblengthz,
                         nmode, 0, -1, &th);
}

static int calculate_f32(float *pix, const float *wave0, const float *param, int natom,
                         const int *Znum, const float *x, const float *y, const float *z,
                         const float *occ, float ctblength, float ctblengthz, int nmode,
                         int min_slice, int max_slices, const mo_thermal *th)
{
    calc_setup s;
    int st = calc_setup_init(&s, param, natom, Znum, x, y, z, ctblength, ctblengthz);
    if (st) { setup_free(&s); return st; }
    const int nx = s.nx, ny = s.ny;
    const size_t n = (size_t)nx * ny;
    const float pi = (float)(4.0 * atan(1.0));
    float *pxr = (float *)malloc(sizeof(float) * nx), *pxi = (float *)malloc(sizeof(float) * nx);
    float *pyr = (float *)malloc(sizeof(float) * ny), *pyi = (float *)malloc(sizeof(float) * ny);
    float scale = pi * ((float)s.deltaz);
    for (int ix = 0; ix < nx; ix++) {
        double t = scale * (s.kx2[ix] * s.wavlen - s.kx[ix] * s.tctx);
        pxr[ix] = (float)cos(t);
        pxi[ix] = (float)-sin(t);
    }
    for (int iy = 0; iy < ny; iy++) {
        double t = scale * (s.ky2[iy] * s.wavlen - s.ky[iy] * s.tcty);
        pyr[iy] = (float)cos(t);
        pyi[iy] = (float)-sin(t);
    }
    float *x2, *y2, *z2, *occ2;
    int *Z2;
    st = sorted_copy_th(natom, Znum, x, y, z, occ, ctblengthz, &x2, &y2, &z2, &occ2, &Z2, th);
    float *wave = (float *)malloc(sizeof(float) * 2 * n);
    float *trans = (float *)malloc(sizeof(float) * 2 * n);
    if (st == MO_OK) {
        memcpy(wave, wave0, sizeof(float) * 2 * n);
        const float zmax = ctblengthz;
        double zslice = s.deltaz;
        int istart = 0, islice = 1;
        while (zslice < (zmax + s.deltaz)) {
            int na = 0;
            for (int i = istart; i < natom; i++)
                if (z2[i] < zslice) na++;
                else break;
            if (islice <= min_slice) {  /* skipped (timing samples only) */
                zslice += s.deltaz;
                istart += na;
                islice++;
                continue;
            }
            if (na > 0) {
                if (th && th->lwobble == 1 && th->nwobble == 1)  /* autoslic.cpp:766-774 */
                    trlayerDW_f32(&x2[istart], &y2[istart], &occ2[istart], &Z2[istart], na, s.ax,
                                  s.by, s.v0, trans, nx, ny, s.kx2, s.ky2, s.k2max, th->wobble,
                                  th->temperature);
                else
                    trlayer_f32(&x2[istart], &y2[istart], &occ2[istart], &Z2[istart], na, s.ax,
                                s.by, s.v0, trans, nx, ny, s.kx2, s.ky2, s.k2max);
                for (size_t j = 0; j < n; j++) { /* cfpix::operator*= (cfpix.cpp:349-372) */
                    float wr = wave[2 * j], wi = wave[2 * j + 1];
                    float tr = trans[2 * j], ti = trans[2 * j + 1];
                    wave[2 * j] = wr * tr - wi * ti;
                    wave[2 * j + 1] = wr * ti + wi * tr;
                }
            }
            if (nmode == 0) {
                cf_fft_f(wave, nx, ny);
                propagate_f32(wave, pxr, pxi, pyr, pyi, s.kx2, s.ky2, s.k2max, nx, ny);
                cf_ifft_f(wave, nx, ny);
            }
            zslice += s.deltaz;
            istart += na;
            islice++;
            if (max_slices >= 0 && islice > max_slices) break;
        }
        memcpy(pix, wave, sizeof(float) * 2 * n);
    }
    free(wave);
    free(trans);
    free(x2);
    free(y2);
    free(z2);
    free(occ2);
    free(Z2);
    free(pxr);
    free(pxi);
    free(pyr);
    free(pyi);
    setup_free(&s);
    return st;
}

static int calculate_f64(double *pix, const double *wave0, const float *param, int natom,
                         const int *Znum, const float *x, const float *y, const float *z,
                         const float *occ, float ctblength, float ctblengthz, int nmode,
                         int max_slices, const mo_thermal *th);

int mo_calculate_f64(double *pix, const double *wave0, const float *param, int natom,
                     const int *Znum, const float *x, const float *y, const float *z,
                     const float *occ, float ctblength, float ctblengthz, int nmode,
                     int max_slices)
{
    return calculate_f64(pix, wave0, param, natom, Znum, x, y, z, occ, ctblength, ctblengthz,
                         nmode, max_slices, NULL);
}

int mo_calculate_thermal_f64(double *pix, const double *wave0, const float *param, int natom,
                             const int *Znum, const float *x, const float *y, const float *z,
                             const float *occ, const float *wobble, float ctblength,
                             float ctblengthz, int nmode, int lwobble, long *iseed)
{
    mo_thermal th = {wobble, lwobble != 0, 0, param[MO_pTEMPER], iseed};
    th.nwobble = to_int(param[MO_pNWOBBLE]);
    if (th.nwobble < 1) th.nwobble = 1;
    return calculate_f64(pix, wave0, param, natom, Znum, x, y, z, occ, ctblength, ctblengthz,
                         nmode, -1, &th);
}

static int calculate_f64(double *pix, const double *wave0, const float *param, int natom,
                         const int *Znum, const float *x, const float *y, const float *z,
                         const float *occ, float ctblength, float ctblengthz, int nmode,
                         int max_slices, const mo_thermal *th)
{
    calc_setup s;
    int st = calc_setup_init(&s, param, natom, Znum, x, y, z, ctblength, ctblengthz);
    if (st) { setup_free(&s); return st; }
    const int nx = s.nx, ny = s.ny;
    const size_t n = (size_t)nx * ny;
    const double pi = 4.0 * atan(1.0);
    double *pxr = (double *)malloc(sizeof(double) * nx), *pxi = (double *)malloc(sizeof(double) * nx);
    double *pyr = (double *)malloc(sizeof(double) * ny), *pyi = (double *)malloc(sizeof(double) * ny);
    for (int ix = 0; ix < nx; ix++) {
        double t = pi * s.deltaz * ((double)s.kx2[ix] * s.wavlen - (double)s.kx[ix] * s.tctx);
        pxr[ix] = cos(t);
        pxi[ix] = -sin(t);
    }
    for (int iy = 0; iy < ny; iy++) {
        double t = pi * s.deltaz * ((double)s.ky2[iy] * s.wavlen - (double)s.ky[iy] * s.tcty);
        pyr[iy] = cos(t);
        pyi[iy] = -sin(t);
    }
    float *x2, *y2, *z2, *occ2;
    int *Z2;
    st = sorted_copy_th(natom, Znum, x, y, z, occ, ctblengthz, &x2, &y2, &z2, &occ2, &Z2, th);
    double *wave = (double *)malloc(sizeof(double) * 2 * n);
    double *trans = (double *)malloc(sizeof(double) * 2 * n);
    if (st == MO_OK) {
        memcpy(wave, wave0, sizeof(double) * 2 * n);
        const float zmax = ctblengthz;
        double zslice = s.deltaz;
        int istart = 0, islice = 1;
        while (zslice < (zmax + s.deltaz)) {
            int na = 0;
            for (int i = istart; i < natom; i++)
                if (z2[i] < zslice) na++;
                else break;
            if (na > 0) {
                if (th && th->lwobble == 1 && th->nwobble == 1)
                    trlayerDW_f64(&x2[istart], &y2[istart], &occ2[istart], &Z2[istart], na, s.ax,
                                  s.by, s.v0, trans, nx, ny, s.kx2, s.ky2, s.k2max, th->wobble,
                                  th->temperature);
                else
                    trlayer_f64(&x2[istart], &y2[istart], &occ2[istart], &Z2[istart], na, s.ax,
                                s.by, s.v0, trans, nx, ny, s.kx2, s.ky2, s.k2max);
                for (size_t j = 0; j < n; j++) {
                    double wr = wave[2 * j], wi = wave[2 * j + 1];
                    double tr = trans[2 * j], ti = trans[2 * j + 1];
                    wave[2 * j] = wr * tr - wi * ti;
                    wave[2 * j + 1] = wr * ti + wi * tr;
                }
            }
            if (nmode == 0) {
                cf_fft_d(wave, nx, ny);
                propagate_f64(wave, pxr, pxi, pyr, pyi, s.kx2, s.ky2, s.k2max, nx, ny);
                cf_ifft_d(wave, nx, ny);
            }
            zslice += s.deltaz;
            istart += na;
            islice++;
            if (max_slices >= 0 && islice > max_slices) break;
        }
        memcpy(pix, wave, sizeof(double) * 2 * n);
    }
    free(wave);
    free(trans);
    free(x2);
    free(y2);
    free(z2);
    free(occ2);
    free(Z2);
    free(pxr);
    free(pxi);
    free(pyr);
    free(pyi);
    setup_free(&s);
    return st;
}

/* ------------------------------------------------------ free space step */

static double chi_phase(double kx, double ky, double wavlen, double rprime, double cs3,
                        double cs5, double astig, double astig_angle)
{
    const double pi = 4.0 * atan(1.0);
    double k2 = kx * kx + ky * ky;
    double l3 = wavlen * wavlen * wavlen;
    double chi = pi * wavlen * rprime * k2 + (pi / 2.0) * cs3 * l3 * k2 * k2 +
                 (pi / 3.0) * cs5 * l3 * wavlen * wavlen * k2 * k2 * k2;
    if (astig != 0.0)
        chi += (pi / 2.0) * wavlen * astig *
               ((kx * kx - ky * ky) * cos(2.0 * astig_angle) + 2.0 * kx * ky * sin(2.0 * astig_angle));
    double twopi = 2.0 * pi;
    chi = fmod(chi, twopi);
    return chi;
}

int mo_defocus_f32(const float *pix, int nx, int ny, float ax, float by, double wavlen,
                   double rprime, float k2maxo, double cs3, double cs5, double astig,
                   double astig_angle, float *inten_out)
{
    size_t n = (size_t)nx * ny;
    float *kx = (float *)malloc(sizeof(float) * 3 * nx), *ky = (float *)malloc(sizeof(float) * 3 * ny);
    mo_freqn(kx, kx + nx, kx + 2 * nx, nx, ax);
    mo_freqn(ky, ky + ny, ky + 2 * ny, ny, by);
    float *w = (float *)malloc(sizeof(float) * 2 * n);
    memcpy(w, pix, sizeof(float) * 2 * n);
    cf_fft_f(w, nx, ny);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            float *e = w + 2 * ((size_t)iy + (size_t)ix * ny);
            float k2 = kx[nx + ix] + ky[ny + iy];
            if (k2maxo > 0.0F && !(k2 < k2maxo)) {
                e[0] = e[1] = 0.0F;
                continue;
            }
            double chi = chi_phase(kx[ix], ky[iy], wavlen, rprime, cs3, cs5, astig, astig_angle);
            float c = (float)cos(chi), sn = (float)sin(chi);
            float re = e[0], im = e[1];
            e[0] = re * c + im * sn;
            e[1] = im * c - re * sn;
        }
    cf_ifft_f(w, nx, ny);
    for (size_t j = 0; j < n; j++) inten_out[j] = w[2 * j] * w[2 * j] + w[2 * j + 1] * w[2 * j + 1];
    free(w);
    free(kx);
    free(ky);
    return MO_OK;
}

int mo_defocus_f64(const double *pix, int nx, int ny, float ax, float by, double wavlen,
                   double rprime, float k2maxo, double cs3, double cs5, double astig,
                   double astig_angle, double *inten_out)
{
    size_t n = (size_t)nx * ny;
    float *kx = (float *)malloc(sizeof(float) * 3 * nx), *ky = (float *)malloc(sizeof(float) * 3 * ny);
    mo_freqn(kx, kx + nx, kx + 2 * nx, nx, ax);
    mo_freqn(ky, ky + ny, ky + 2 * ny, ny, by);
    double *w = (double *)malloc(sizeof(double) * 2 * n);
    memcpy(w, pix, sizeof(double) * 2 * n);
    cf_fft_d(w, nx, ny);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            double *e = w + 2 * ((size_t)iy + (size_t)ix * ny);
            float k2 = kx[nx + ix] + ky[ny + iy];
            if (k2maxo > 0.0F && !(k2 < k2maxo)) {
                e[0] = e[1] = 0.0;
                continue;
            }
            double chi = chi_phase(kx[ix], ky[iy], wavlen, rprime, cs3, cs5, astig, astig_angle);
            double c = cos(chi), sn = sin(chi);
            double re = e[0], im = e[1];
            e[0] = re * c + im * sn;
            e[1] = im * c - re * sn;
        }
    cf_ifft_d(w, nx, ny);
    for (size_t j = 0; j < n; j++) inten_out[j] = w[2 * j] * w[2 * j] + w[2 * j + 1] * w[2 * j + 1];
    free(w);
    free(kx);
    free(ky);
    return MO_OK;
}

/* The image-plane rotation and shift of autosliccmd.cpp:1119-1143 with this
 * project's definitions of the missing XArrayLibrary calls (NormAverEdge(5),
 * XArray2DSpln::Rotate, XArray2DMove::Move): fill = the mean of each part over
 * the 5-pixel border; out(p) = in(c + R(-theta)(p - c)) by Catmull-Rom bicubic
 * interpolation, grid points outside reading the fill; then out(ix, iy) =
 * in(ix - sx, iy - sy), fill outside.  amp: complex [nx][ny], in place. */
static double cr_weight(double t, int k)
{
    double t2 = t * t, t3 = t2 * t;
    switch (k) {
    case 0: return 0.5 * (-t3 + 2.0 * t2 - t);
    case 1: return 0.5 * (3.0 * t3 - 5.0 * t2 + 2.0);
    case 2: return 0.5 * (-3.0 * t3 + 4.0 * t2 + t);
    default: return 0.5 * (t3 - t2);
    }
}

void mo_image_plane_f64(double *amp, int nx, int ny, double xst, double yst, double xc,
                        double yc, double theta, int sx, int sy)
{
    size_t n = (size_t)nx * ny;
    double fr = 0.0, fi = 0.0;
    long cnt = 0;
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++)
            if (ix < 5 || ix >= nx - 5 || iy < 5 || iy >= ny - 5) {
                fr += amp[2 * ((size_t)ix * ny + iy)];
                fi += amp[2 * ((size_t)ix * ny + iy) + 1];
                cnt++;
            }
    if (cnt) {
        fr /= cnt;
        fi /= cnt;
    }
    double *rot = (double *)malloc(sizeof(double) * 2 * n);
    const double c = cos(theta), sn = sin(theta);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            double *o = rot + 2 * ((size_t)ix * ny + iy);
            if (theta == 0.0) {
                o[0] = amp[2 * ((size_t)ix * ny + iy)];
                o[1] = amp[2 * ((size_t)ix * ny + iy) + 1];
                continue;
            }
            double dx = ix * xst - xc, dy = iy * yst - yc;
            double fx = (xc + c * dx + sn * dy) / xst, fy = (yc - sn * dx + c * dy) / yst;
            int x0 = (int)floor(fx), y0 = (int)floor(fy);
            double tx = fx - x0, ty = fy - y0, ar = 0.0, ai = 0.0;
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 4; b++) {
                    int xx = x0 - 1 + a, yy = y0 - 1 + b;
                    double w = cr_weight(tx, a) * cr_weight(ty, b);
                    int in = xx >= 0 && xx < nx && yy >= 0 && yy < ny;
                    ar += w * (in ? amp[2 * ((size_t)xx * ny + yy)] : fr);
                    ai += w * (in ? amp[2 * ((size_t)xx * ny + yy) + 1] : fi);
                }
            o[0] = ar;
            o[1] = ai;
        }
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            int jx = ix - sx, jy = iy - sy;
            double *o = amp + 2 * ((size_t)ix * ny + iy);
            if (jx >= 0 && jx < nx && jy >= 0 && jy < ny) {
                o[0] = rot[2 * ((size_t)jx * ny + jy)];
                o[1] = rot[2 * ((size_t)jx * ny + jy) + 1];
            } else {
                o[0] = fr;
                o[1] = fi;
            }
        }
    free(rot);
}

/* mo_defocus_f64's free-space step, returning the complex amplitude. */
int mo_defocus_amp_f64(const double *pix, int nx, int ny, float ax, float by, double wavlen,
                       double rprime, float k2maxo, double cs3, double cs5, double *amp)
{
    size_t n = (size_t)nx * ny;
    float *kx = (float *)malloc(sizeof(float) * 3 * nx), *ky = (float *)malloc(sizeof(float) * 3 * ny);
    mo_freqn(kx, kx + nx, kx + 2 * nx, nx, ax);
    mo_freqn(ky, ky + ny, ky + 2 * ny, ny, by);
    memcpy(amp, pix, sizeof(double) * 2 * n);
    cf_fft_d(amp, nx, ny);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            double *e = amp + 2 * ((size_t)iy + (size_t)ix * ny);
            float k2 = kx[nx + ix] + ky[ny + iy];
            if (k2maxo > 0.0F && !(k2 < k2maxo)) {
                e[0] = e[1] = 0.0;
                continue;
            }
            double chi = chi_phase(kx[ix], ky[iy], wavlen, rprime, cs3, cs5, 0.0, 0.0);
            double cc = cos(chi), sn = sin(chi);
            double re = e[0], im = e[1];
            e[0] = re * cc + im * sn;
            e[1] = im * cc - re * sn;
        }
    cf_ifft_d(amp, nx, ny);
    free(kx);
    free(ky);
    return MO_OK;
}

/* --------------------------------------------------- per-orientation worker */

static void fill_param(const mo_series_params *sp, float *param)
{
    memset(param, 0, sizeof(float) * MO_NPARAM);
    param[MO_pAX] = sp->ax;
    param[MO_pBY] = sp->ax;
    param[MO_pNX] = (float)sp->nx;
    param[MO_pNY] = (float)sp->ny;
    param[MO_pENERGY] = sp->v0;
    param[MO_pDELTAZ] = sp->deltaz;
    param[MO_pOAPERT] = sp->aobj;
}

/* Rotate and drop atoms for one orientation; returns malloc'ed copies. */
static int prep_orientation(const mo_series_params *sp, int natom, const int *Znum,
                            const float *x, const float *y, const float *z, const float *occ,
                            double angleZ, double angleY, const float *disp, float **xo,
                            float **yo, float **zo, float **oo, int **Zo)
{
    size_t n = natom > 0 ? (size_t)natom : 1;
    *xo = (float *)malloc(sizeof(float) * n);
    *yo = (float *)malloc(sizeof(float) * n);
    *zo = (float *)malloc(sizeof(float) * n);
    *oo = (float *)malloc(sizeof(float) * n);
    *Zo = (int *)malloc(sizeof(int) * n);
    if (natom > 0) {
        memcpy(*xo, x, sizeof(float) * natom);
        memcpy(*yo, y, sizeof(float) * natom);
        memcpy(*zo, z, sizeof(float) * natom);
        memcpy(*oo, occ, sizeof(float) * natom);
        memcpy(*Zo, Znum, sizeof(int) * natom);
    }
    mo_rotate(sp->ax, sp->dxc, sp->dyc, sp->dzc, angleZ, angleY, natom, *xo, *yo, *zo);
    if (disp) /* thermal displacement of the rotated atoms (autoslic.cpp:701-713) */
        for (int k = 0; k < natom; k++) {
            (*xo)[k] += disp[k];
            (*yo)[k] += disp[natom + k];
            (*zo)[k] += disp[2 * natom + k];
        }
    return mo_drop_outside(sp->ax, sp->ctblengthz, natom, *xo, *yo, *zo, *oo, *Zo);
}

int mo_orientation_f32(const mo_series_params *sp, int natom, const int *Znum,
                       const float *x, const float *y, const float *z, const float *occ,
                       double angleZ, double angleY, const float *disp, int ndef,
                       const double *defocus,
                       float *images, float *exitwave)
{
    float *xo, *yo, *zo, *oo;
    int *Zo;
    int kept = prep_orientation(sp, natom, Znum, x, y, z, occ, angleZ, angleY, disp, &xo, &yo, &zo, &oo, &Zo);
    float param[MO_NPARAM];
    fill_param(sp, param);
    size_t n = (size_t)sp->nx * sp->ny;
    float *wave0 = (float *)malloc(sizeof(float) * 2 * n);
    float *pix = (float *)malloc(sizeof(float) * 2 * n);
    for (size_t j = 0; j < n; j++) { wave0[2 * j] = 1.0f; wave0[2 * j + 1] = 0.0f; }
    int st = mo_calculate_sample_f32(pix, wave0, param, kept, Zo, xo, yo, zo, oo, sp->ax,
                                     sp->ctblengthz, sp->nmode, sp->min_slice, sp->max_slices);
    if (st == MO_OK) {
        float wavlen = (float)mo_wavelength(sp->v0);
        float k2maxo = sp->aobj / wavlen;
        k2maxo = k2maxo * k2maxo;
        for (int d = 0; d < ndef; d++) {
            double rprime = defocus[d] - 0.5 * sp->ctblengthz;
            mo_defocus_f32(pix, sp->nx, sp->ny, sp->ax, sp->ax, wavlen, rprime, k2maxo, sp->cs3,
                           sp->cs5, 0.0, 0.0, images + (size_t)d * n);
        }
        if (exitwave) memcpy(exitwave, pix, sizeof(float) * 2 * n);
    }
    free(wave0);
    free(pix);
    free(xo);
    free(yo);
    free(zo);
    free(oo);
    free(Zo);
    return st == MO_OK ? kept : st;
}

int mo_orientation_f64(const mo_series_params *sp, int natom, const int *Znum,
                       const float *x, const float *y, const float *z, const float *occ,
                       double angleZ, double angleY, const float *disp, int ndef,
                       const double *defocus,
                       double *images, double *exitwave)
{
    float *xo, *yo, *zo, *oo;
    int *Zo;
    int kept = prep_orientation(sp, natom, Znum, x, y, z, occ, angleZ, angleY, disp, &xo, &yo, &zo, &oo, &Zo);
    float param[MO_NPARAM];
    fill_param(sp, param);
    size_t n = (size_t)sp->nx * sp->ny;
    double *wave0 = (double *)malloc(sizeof(double) * 2 * n);
    double *pix = (double *)malloc(sizeof(double) * 2 * n);
    for (size_t j = 0; j < n; j++) { wave0[2 * j] = 1.0; wave0[2 * j + 1] = 0.0; }
    int st = mo_calculate_f64(pix, wave0, param, kept, Zo, xo, yo, zo, oo, sp->ax, sp->ctblengthz,
                              sp->nmode, sp->max_slices);
    if (st == MO_OK) {
        float wavlen = (float)mo_wavelength(sp->v0);
        float k2maxo = sp->aobj / wavlen;
        k2maxo = k2maxo * k2maxo;
        for (int d = 0; d < ndef; d++) {
            double rprime = defocus[d] - 0.5 * sp->ctblengthz;
            mo_defocus_f64(pix, sp->nx, sp->ny, sp->ax, sp->ax, wavlen, rprime, k2maxo, sp->cs3,
                           sp->cs5, 0.0, 0.0, images + (size_t)d * n);
        }
        if (exitwave) memcpy(exitwave, pix, sizeof(double) * 2 * n);
    }
    free(wave0);
    free(pix);
    free(xo);
    free(yo);
    free(zo);
    free(oo);
    free(Zo);
    return st == MO_OK ? kept : st;
}

typedef struct {
    const mo_series_params *sp;
    int nunits, natom, ndef;
    long stride;
    const int *Znum;
    const float *x, *y, *z, *occ;
    const double *angZ, *angY, *defocus;
    float *images;
    int next, status;
} many_job;

static void *many_worker(void *arg)
{
    many_job *j = (many_job *)arg;
    size_t img = (size_t)j->sp->nx * j->sp->ny * j->ndef;
    for (;;) {
        int u = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
        if (u >= j->nunits) break;
        long o = (long)u * j->stride;
        int st = mo_orientation_f32(j->sp, j->natom, j->Znum + o, j->x + o, j->y + o, j->z + o,
                                    j->occ + o, j->angZ[u], j->angY[u], NULL, j->ndef, j->defocus,
                                    j->images + img * u, NULL);
        if (st < 0) __atomic_store_n(&j->status, st, __ATOMIC_RELAXED);
    }
    return NULL;
}

int mo_orientations_f32(const mo_series_params *sp, int nunits, int nthreads, int natom,
                        long coord_stride, const int *Znum, const float *x, const float *y,
                        const float *z, const float *occ, const double *angZ,
                        const double *angY, int ndef, const double *defocus, float *images)
{
    many_job j = {sp, nunits, natom, ndef, coord_stride, Znum, x, y, z, occ, angZ, angY,
                  defocus, images, 0, MO_OK};
    /* build the spline tables before the threads start */
    for (int i = 0; i < natom; i++) mo_vzatomLUT(Znum[i], 0.5);
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, many_worker, &j);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
    return j.status;
}

/* ------------------------------------------------ potential stacks and adjoint */

/* Per-slice projected potentials of one orientation (FP64 sums): the
 * atoms rotated and dropped as mo_orientation_*, sorted, and split into the
 * slices of calculate() (autoslic.cpp:747-830); v[k][ix][iy] for
 * k < mo_slice_count(deltaz, ctblengthz).  Returns atoms kept or a status. */
int mo_orientation_potential_f64(const mo_series_params *sp, int natom, const int *Znum,
                                 const float *x, const float *y, const float *z,
                                 const float *occ, double angleZ, double angleY, double *v)
{
    float *xo, *yo, *zo, *oo;
    int *Zo;
    int kept = prep_orientation(sp, natom, Znum, x, y, z, occ, angleZ, angleY, NULL, &xo, &yo,
                                &zo, &oo, &Zo);
    float param[MO_NPARAM];
    fill_param(sp, param);
    calc_setup s;
    int st = calc_setup_init(&s, param, kept, Zo, xo, yo, zo, sp->ax, sp->ctblengthz);
    float *x2 = NULL, *y2 = NULL, *z2 = NULL, *occ2 = NULL;
    int *Z2 = NULL;
    if (st == MO_OK)
        st = sorted_copy(kept, Zo, xo, yo, zo, oo, sp->ctblengthz, &x2, &y2, &z2, &occ2, &Z2);
    if (st == MO_OK) {
        const int nsl = mo_slice_count(sp->deltaz, sp->ctblengthz);
        const size_t n = (size_t)sp->nx * sp->ny;
        double zslice = s.deltaz;
        int istart = 0;
        for (int k = 0; k < nsl; k++) {
            int na = 0;
            for (int i = istart; i < kept; i++)
                if (z2[i] < zslice) na++;
                else break;
            potential_f64(&x2[istart], &y2[istart], &occ2[istart], &Z2[istart], na, s.ax, s.by,
                          v + (size_t)k * n, 1, s.nx, s.ny);
            zslice += s.deltaz;
            istart += na;
        }
    }
    free(x2);
    free(y2);
    free(z2);
    free(occ2);
    free(Z2);
    free(xo);
    free(yo);
    free(zo);
    free(oo);
    free(Zo);
    setup_free(&s);
    return st == MO_OK ? kept : st;
}

typedef struct {
    int nx, ny;
    size_t n;
    double sigma;
    double *M;        /* band limit 0/1 */
    double *p;        /* propagator (complex) with the 2/3 aperture */
    double *X;        /* ndef free-space multipliers (complex) */
} stack_ops;

static int stack_setup(const mo_stack_params *sp, int ndef, const double *rprime, stack_ops *o)
{
    float param[MO_NPARAM];
    memset(param, 0, sizeof param);
    param[MO_pAX] = sp->ax;
    param[MO_pBY] = sp->by;
    param[MO_pNX] = (float)sp->nx;
    param[MO_pNY] = (float)sp->ny;
    param[MO_pENERGY] = sp->v0;
    param[MO_pDELTAZ] = sp->deltaz;
    param[MO_pXCTILT] = sp->ctiltx;
    param[MO_pYCTILT] = sp->ctilty;
    calc_setup s;
    int st = calc_setup_init(&s, param, 0, NULL, NULL, NULL, NULL, sp->ax, 1.0f);
    if (st) { setup_free(&s); return st; }
    const int nx = s.nx, ny = s.ny;
    const size_t n = (size_t)nx * ny;
    o->nx = nx;
    o->ny = ny;
    o->n = n;
    o->sigma = mo_sigma(sp->v0) / 1000.0;
    o->M = (double *)malloc(sizeof(double) * n);
    o->p = (double *)malloc(sizeof(double) * 2 * n);
    o->X = (double *)malloc(sizeof(double) * 2 * n * (ndef > 0 ? ndef : 1));
    const double pi = 4.0 * atan(1.0);
    float k2maxo = sp->aobj / s.wavlen;
    k2maxo = k2maxo * k2maxo;
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            const size_t i = (size_t)ix * ny + iy;
            const int keep = (s.ky2[iy] + s.kx2[ix]) < s.k2max;
            o->M[i] = keep ? 1.0 : 0.0;
            double tx = pi * s.deltaz * ((double)s.kx2[ix] * s.wavlen - (double)s.kx[ix] * s.tctx);
            double ty = pi * s.deltaz * ((double)s.ky2[iy] * s.wavlen - (double)s.ky[iy] * s.tcty);
            /* (cos ty - i sin ty)(cos tx - i sin tx) = exp(-i (tx + ty)) */
            o->p[2 * i] = keep ? cos(tx + ty) : 0.0;
            o->p[2 * i + 1] = keep ? -sin(tx + ty) : 0.0;
            for (int d = 0; d < ndef; d++) {
                double *x = o->X + 2 * ((size_t)d * n + i);
                float k2 = s.kx2[ix] + s.ky2[iy];
                if (k2maxo > 0.0F && !(k2 < k2maxo)) {
                    x[0] = x[1] = 0.0;
                } else {
                    double chi = chi_phase(s.kx[ix], s.ky[iy], s.wavlen, rprime[d], sp->cs3,
                                           sp->cs5, 0.0, 0.0);
                    x[0] = cos(chi);
                    x[1] = -sin(chi);
                }
            }
        }
    setup_free(&s);
    return MO_OK;
}

static void stack_free(stack_ops *o)
{
    free(o->M);
    free(o->p);
    free(o->X);
}

/* f <- K[m] f;  m complex (mc) or real (mr), conjugated if conj */
static void kmul(const stack_ops *o, double *f, const double *mc, const double *mr, int conj)
{
    cf_fft_d(f, o->nx, o->ny);
    for (size_t i = 0; i < o->n; i++) {
        double a = f[2 * i], b = f[2 * i + 1];
        if (mr) {
            f[2 * i] = a * mr[i];
            f[2 * i + 1] = b * mr[i];
        } else {
            double c = mc[2 * i], s = conj ? -mc[2 * i + 1] : mc[2 * i + 1];
            f[2 * i] = a * c - b * s;
            f[2 * i + 1] = a * s + b * c;
        }
    }
    cf_ifft_d(f, o->nx, o->ny);
}

/* Forward through all slices; keeps psi_0..psi_S (psi[k]) and t_k (t[k-1]). */
static void stack_forward(const stack_ops *o, int S, const double *v, double *psi, double *t)
{
    const size_t n = o->n;
    for (size_t i = 0; i < n; i++) { psi[2 * i] = 1.0; psi[2 * i + 1] = 0.0; }
    for (int k = 1; k <= S; k++) {
        double *tk = t + 2 * n * (size_t)(k - 1);
        const double *vk = v + n * (size_t)(k - 1);
        for (size_t i = 0; i < n; i++) {
            tk[2 * i] = cos(o->sigma * vk[i]);
            tk[2 * i + 1] = sin(o->sigma * vk[i]);
        }
        kmul(o, tk, NULL, o->M, 0);
        const double *pp = psi + 2 * n * (size_t)(k - 1);
        double *pk = psi + 2 * n * (size_t)k;
        for (size_t i = 0; i < n; i++) {
            double a = pp[2 * i], b = pp[2 * i + 1], c = tk[2 * i], d = tk[2 * i + 1];
            pk[2 * i] = a * c - b * d;
            pk[2 * i + 1] = a * d + b * c;
        }
        kmul(o, pk, o->p, NULL, 0);
    }
}

int mo_stack_images_f64(const mo_stack_params *sp, const double *v, int ndef,
                        const double *rprime, double *images)
{
    stack_ops o;
    int st = stack_setup(sp, ndef, rprime, &o);
    if (st) return st;
    const int S = sp->nslices;
    const size_t n = o.n;
    double *psi = (double *)malloc(sizeof(double) * 2 * n * (S + 1));
    double *t = (double *)malloc(sizeof(double) * 2 * n * (S > 0 ? S : 1));
    double *phi = (double *)malloc(sizeof(double) * 2 * n);
    stack_forward(&o, S, v, psi, t);
    for (int d = 0; d < ndef; d++) {
        memcpy(phi, psi + 2 * n * (size_t)S, sizeof(double) * 2 * n);
        kmul(&o, phi, o.X + 2 * n * (size_t)d, NULL, 0);
        for (size_t i = 0; i < n; i++)
            images[(size_t)d * n + i] = phi[2 * i] * phi[2 * i] + phi[2 * i + 1] * phi[2 * i + 1];
    }
    free(psi);
    free(t);
    free(phi);
    stack_free(&o);
    return MO_OK;
}

double mo_stack_loss_f64(const mo_stack_params *sp, const double *v, int ndef,
                         const double *rprime, const float *target)
{
    const size_t n = (size_t)sp->nx * sp->ny;
    double *img = (double *)malloc(sizeof(double) * n * (ndef > 0 ? ndef : 1));
    mo_stack_images_f64(sp, v, ndef, rprime, img);
    double L = 0.0;
    for (size_t i = 0; i < n * ndef; i++) {
        double r = img[i] - target[i];
        L += r * r;
    }
    free(img);
    return L;
}

int mo_stack_adjoint_f64(const mo_stack_params *sp, const double *v, int ndef,
                         const double *rprime, const float *target, double *grad, double *loss)
{
    stack_ops o;
    int st = stack_setup(sp, ndef, rprime, &o);
    if (st) return st;
    const int S = sp->nslices;
    const size_t n = o.n;
    double *psi = (double *)malloc(sizeof(double) * 2 * n * (S + 1));
    double *t = (double *)malloc(sizeof(double) * 2 * n * (S > 0 ? S : 1));
    double *phi = (double *)malloc(sizeof(double) * 2 * n);
    double *g = (double *)calloc(2 * n, sizeof(double));   /* dL/d conj(psi_k) */
    double *gu = (double *)malloc(sizeof(double) * 2 * n);
    stack_forward(&o, S, v, psi, t);
    double L = 0.0;
    for (int d = 0; d < ndef; d++) {
        memcpy(phi, psi + 2 * n * (size_t)S, sizeof(double) * 2 * n);
        kmul(&o, phi, o.X + 2 * n * (size_t)d, NULL, 0);
        for (size_t i = 0; i < n; i++) {
            double I = phi[2 * i] * phi[2 * i] + phi[2 * i + 1] * phi[2 * i + 1];
            double r = I - target[(size_t)d * n + i];
            L += r * r;
            phi[2 * i] *= 2.0 * r;    /* dL/d conj(phi) = 2 (I - T) phi */
            phi[2 * i + 1] *= 2.0 * r;
        }
        kmul(&o, phi, o.X + 2 * n * (size_t)d, NULL, 1);  /* K[X]^H = K[conj X] */
        for (size_t i = 0; i < 2 * n; i++) g[i] += phi[i];
    }
    for (int k = S; k >= 1; k--) {
        memcpy(gu, g, sizeof(double) * 2 * n);
        kmul(&o, gu, o.p, NULL, 1);                       /* g_u = K[conj p] g_psi */
        const double *tk = t + 2 * n * (size_t)(k - 1);
        const double *pp = psi + 2 * n * (size_t)(k - 1);
        for (size_t i = 0; i < n; i++) {
            double ar = gu[2 * i], ai = gu[2 * i + 1];
            double tr = tk[2 * i], ti = tk[2 * i + 1], pr = pp[2 * i], pi_ = pp[2 * i + 1];
            g[2 * i] = ar * tr + ai * ti;                 /* conj(t) g_u */
            g[2 * i + 1] = ai * tr - ar * ti;
            gu[2 * i] = ar * pr + ai * pi_;               /* conj(psi_{k-1}) g_u */
            gu[2 * i + 1] = ai * pr - ar * pi_;
        }
        kmul(&o, gu, NULL, o.M, 0);                       /* g_e = K[M] g_t */
        const double *vk = v + n * (size_t)(k - 1);
        double *gk = grad + n * (size_t)(k - 1);
        for (size_t i = 0; i < n; i++) {
            double er = cos(o.sigma * vk[i]), ei = sin(o.sigma * vk[i]);
            /* dL/dv = 2 sigma Im(g_e conj(e)) */
            gk[i] = 2.0 * o.sigma * (gu[2 * i + 1] * er - gu[2 * i] * ei);
        }
    }
    if (loss) *loss = L;
    free(psi);
    free(t);
    free(phi);
    free(g);
    free(gu);
    stack_free(&o);
    return MO_OK;
}

/* Central finite differences of mo_stack_loss_f64 at chosen voxels.
 * Perturbing v_k at one pixel changes e_k there only, so the band-limited
 * transmission becomes t_k + c h(. - pixel) with h = K[M] delta (computed
 * once) and c the exact change of exp(i sigma v).  For fixed transmissions
 * the slice loop is linear in the wave, so the perturbed wave is psi + d
 * with d_k = K[p](psi_{k-1} c h(. - pixel)) and d_m = K[p](d_{m-1} t_m)
 * exactly, and each image changes by dI = 2 Re(conj(phi) dphi) + |dphi|^2.
 * L(v + h) - L(v - h) = sum (dI+ - dI-) (2 r + dI+ + dI-), r = I - T: the
 * same central difference as two full evaluations, without the cancellation
 * of two large sums.  Voxels run on nthreads threads; fd[i] = that difference
 * / (2 h_i), h_i = h_rel * max(1, |v|). */
typedef struct {
    const stack_ops *o;
    int S, ndef;
    const double *v, *psi, *t, *hk;
    const double *phi;  /* base free-space waves [ndef][n] (complex) */
    const double *res;  /* base residuals I - T [ndef][n] */
    const int *vox;
    int nvox;
    double h_rel;
    double *fd;
    int next;
    pthread_mutex_t lock;
} fd_job;

/* dI[d][px] for the change dv of v_k at (ix, iy). */
static void fd_delta(fd_job *J, int k, int ix, int iy, double dv, double *w, double *dphi,
                     double *dI)
{
    const stack_ops *o = J->o;
    const size_t n = o->n;
    const int nx = o->nx, ny = o->ny;
    const double vk = J->v[(size_t)(k - 1) * n + (size_t)ix * ny + iy];
    const double c_r = cos(o->sigma * (vk + dv)) - cos(o->sigma * vk);
    const double c_i = sin(o->sigma * (vk + dv)) - sin(o->sigma * vk);
    const double *pp = J->psi + 2 * n * (size_t)(k - 1);
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) {
            const size_t i = (size_t)x * ny + y;
            /* h shifted to the pixel: h[(x - ix) mod nx][(y - iy) mod ny] */
            const size_t hi = (size_t)((x - ix + nx) % nx) * ny + (size_t)((y - iy + ny) % ny);
            const double hr = J->hk[2 * hi], him = J->hk[2 * hi + 1];
            const double tr = c_r * hr - c_i * him, ti = c_r * him + c_i * hr;
            const double a = pp[2 * i], b = pp[2 * i + 1];
            w[2 * i] = a * tr - b * ti;
            w[2 * i + 1] = a * ti + b * tr;
        }
    kmul(o, w, o->p, NULL, 0);
    for (int m = k + 1; m <= J->S; m++) {
        const double *tm = J->t + 2 * n * (size_t)(m - 1);
        for (size_t i = 0; i < n; i++) {
            const double a = w[2 * i], b = w[2 * i + 1], c = tm[2 * i], d = tm[2 * i + 1];
            w[2 * i] = a * c - b * d;
            w[2 * i + 1] = a * d + b * c;
        }
        kmul(o, w, o->p, NULL, 0);
    }
    for (int d = 0; d < J->ndef; d++) {
        memcpy(dphi, w, sizeof(double) * 2 * n);
        kmul(o, dphi, o->X + 2 * n * (size_t)d, NULL, 0);
        const double *ph = J->phi + 2 * n * (size_t)d;
        double *di = dI + n * (size_t)d;
        for (size_t i = 0; i < n; i++) {
            const double pr = ph[2 * i], pi_ = ph[2 * i + 1];
            const double qr = dphi[2 * i], qi = dphi[2 * i + 1];
            di[i] = 2.0 * (pr * qr + pi_ * qi) + (qr * qr + qi * qi);
        }
    }
}

static void *fd_worker(void *arg)
{
    fd_job *J = (fd_job *)arg;
    const size_t n = J->o->n;
    const size_t nd = n * (size_t)J->ndef;
    double *w = (double *)malloc(sizeof(double) * 2 * n);
    double *dphi = (double *)malloc(sizeof(double) * 2 * n);
    double *dIp = (double *)malloc(sizeof(double) * (nd > 0 ? nd : 1));
    double *dIm = (double *)malloc(sizeof(double) * (nd > 0 ? nd : 1));
    for (;;) {
        pthread_mutex_lock(&J->lock);
        const int q = J->next++;
        pthread_mutex_unlock(&J->lock);
        if (q >= J->nvox) break;
        const int k = J->vox[3 * q] + 1, ix = J->vox[3 * q + 1], iy = J->vox[3 * q + 2];
        const double vk = J->v[(size_t)(k - 1) * n + (size_t)ix * J->o->ny + iy];
        const double h = J->h_rel * (fabs(vk) > 1.0 ? fabs(vk) : 1.0);
        fd_delta(J, k, ix, iy, h, w, dphi, dIp);
        fd_delta(J, k, ix, iy, -h, w, dphi, dIm);
        double dL = 0.0;
        for (size_t i = 0; i < nd; i++) dL += (dIp[i] - dIm[i]) * (2.0 * J->res[i] + dIp[i] + dIm[i]);
        J->fd[q] = dL / (2.0 * h);
    }
    free(w);
    free(dphi);
    free(dIp);
    free(dIm);
    return NULL;
}

int mo_stack_fd_f64(const mo_stack_params *sp, const double *v, int ndef, const double *rprime,
                    const float *target, int nvox, const int *vox, double h_rel, int nthreads,
                    double *fd)
{
    stack_ops o;
    int st = stack_setup(sp, ndef, rprime, &o);
    if (st) return st;
    const int S = sp->nslices;
    const size_t n = o.n;
    for (int q = 0; q < nvox; q++)
        if (vox[3 * q] < 0 || vox[3 * q] >= S || vox[3 * q + 1] < 0 || vox[3 * q + 1] >= o.nx ||
            vox[3 * q + 2] < 0 || vox[3 * q + 2] >= o.ny) {
            stack_free(&o);
            return MO_EBADSIZE;
        }
    double *psi = (double *)malloc(sizeof(double) * 2 * n * (S + 1));
    double *t = (double *)malloc(sizeof(double) * 2 * n * (S > 0 ? S : 1));
    double *hk = (double *)calloc(2 * n, sizeof(double));
    double *phi = (double *)malloc(sizeof(double) * 2 * n * (ndef > 0 ? ndef : 1));
    double *res = (double *)malloc(sizeof(double) * n * (ndef > 0 ? ndef : 1));
    stack_forward(&o, S, v, psi, t);
    hk[0] = 1.0;
    kmul(&o, hk, NULL, o.M, 0);
    for (int d = 0; d < ndef; d++) {
        double *ph = phi + 2 * n * (size_t)d;
        memcpy(ph, psi + 2 * n * (size_t)S, sizeof(double) * 2 * n);
        kmul(&o, ph, o.X + 2 * n * (size_t)d, NULL, 0);
        for (size_t i = 0; i < n; i++)
            res[(size_t)d * n + i] = ph[2 * i] * ph[2 * i] + ph[2 * i + 1] * ph[2 * i + 1] -
                                     target[(size_t)d * n + i];
    }
    fd_job J;
    J.o = &o;
    J.S = S;
    J.ndef = ndef;
    J.v = v;
    J.psi = psi;
    J.t = t;
    J.hk = hk;
    J.phi = phi;
    J.res = res;
    J.vox = vox;
    J.nvox = nvox;
    J.h_rel = h_rel;
    J.fd = fd;
    J.next = 0;
    pthread_mutex_init(&J.lock, NULL);
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, fd_worker, &J);
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&J.lock);
    free(psi);
    free(t);
    free(hk);
    free(phi);
    free(res);
    stack_free(&o);
    return MO_OK;
}
