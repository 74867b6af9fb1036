/*
 * utr_oracle.c -- CPU restatement of UTR.exe's reconstruction core.
 *
 * TEST INFRASTRUCTURE ONLY (see utr_oracle.h).  Every function cites the
 * reference lines it follows (MultisliceCppTest/PhaseRetrieval/UTR.cpp and
 * UTR.h).  The float mirrors reproduce the reference's float expressions in
 * the same order (this file is compiled with -ffp-contract=off) and are
 * pinned against the reference's own UTR.h templates (oracle/_ref).
 *
 * The steps that run through XArrayLibrary in the reference, which is not
 * part of the reference tree, follow this definition (parity unpinned):
 *   - Log0: ln(x) for x > 0, else 0;
 *   - Shuffle: the half-size circular shift of each dimension (even sizes),
 *     so Shuffle, forward FFT, Shuffle = the centred DFT with FFTW's forward
 *     sign exp(-2 pi i ...), unnormalised;
 *   - Fftwd3frc inverse: FFTW's complex-to-real 3D transform of the half
 *     spectrum kx = 0 .. nx/2 (centred indices nx/2 .. nx-1 and 0): complex
 *     inverse transforms along z and y, then a real inverse along x that
 *     reads the real parts of its kx = 0 and kx = nx/2 terms; GetRealXArray3D
 *     shuffles back and divides by nx*ny*nz (UTR.cpp:1266-1272);
 *   - NormAverEdge(5), XArray2DMove::Move and XArray2DSpln::Rotate of the
 *     input images (UTR.cpp:920-940): the mean over the pixels within 5 of any
 *     edge; out(j, i) = in(j - dy, i - dx); out(p) = in(c + R(-t)(p - c)) by
 *     Catmull-Rom bicubic interpolation, R(t) = [[cos t, -sin t], [sin t,
 *     cos t]] on (x, y) = (i, j), both reading the edge mean outside the
 *     image (the definitions this library uses for MsctKirkland's image plane).
 */
#include "utr_oracle.h"

#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fft_cpu.h"

static const double kPi = 3.14159265358979323846;

/* ------------------------------------------------------------------ geometry */

int mo_utr_geom_make(const msk_utr *p, int nangles, const double *angles, const double *defocus,
                     mo_utr_geom *g)
{
    if (!p || nangles < 1 || !angles || !defocus || p->xst <= 0.0 || p->wl <= 0.0) return -1;
    memset(g, 0, sizeof(*g));
    const int nx = p->nx, ny = p->ny;
    g->nx = nx;
    g->ny = ny;
    g->xst = p->xst;
    /* UTR.cpp:296-330 */
    g->xlo = -0.5 * p->xst * nx;
    g->xhi = g->xlo + p->xst * nx;
    g->ylo = -0.5 * p->xst * ny;
    g->yhi = g->ylo + p->xst * ny;
    g->fxst = 1.0 / (g->xhi - g->xlo);
    g->fyst = 1.0 / (g->yhi - g->ylo);
    g->fxlo = -g->fxst * (nx / 2);
    g->fylo = -g->fyst * (ny / 2);
    double zlo = p->zlo, zhi = p->zhi;
    if (p->modality == 1 && zlo == 0.0 && zhi == 0.0) { /* the .xri default: zlo = xlo, zhi = xhi */
        zlo = g->xlo;
        zhi = g->xhi;
    }
    if (zlo > zhi) {
        const double t = zlo;
        zlo = zhi;
        zhi = t;
    }
    g->zlo = zlo;
    g->zhi = zhi;
    g->nz = (int)((zhi - zlo) / p->xst + 0.5);
    if (g->nz <= 0) return -1;
    g->fzst = 1.0 / (zhi - zlo);
    g->fzlo = -g->fzst * (g->nz / 2);
    /* UTR.cpp:341-345 (index_t = size_t in XArrayLibrary) */
    g->xc = (g->xhi + g->xlo) / 2.0 + p->dxc;
    g->yc = (g->yhi + g->ylo) / 2.0 + p->dyc;
    g->zc = (g->zhi + g->zlo) / 2.0 + p->dzc;
    g->ic = (long)(size_t)((g->xc - g->xlo) / p->xst + 0.5);
    g->jc = (long)(size_t)((g->yc - g->ylo) / p->xst + 0.5);
    g->kc = (long)(size_t)((g->zc - g->zlo) / p->xst + 0.5);
    g->wl = p->wl;
    /* UTR.cpp:353-370: electron energy from the wavelength (long double) */
    if (p->modality == 0) {
        const double hp = 6.62607004e-34, cc = 299792458, ee = 1.602176634e-19,
                     m0 = 9.1093837015e-31;
        const long double mc2 = m0 * cc * cc;
        const long double chl2 = (long double)(cc * cc * hp * hp) / (long double)(p->wl * p->wl * 1.e-20);
        const long double abra = sqrtl(mc2 * mc2 + chl2);
        g->ee = (double)((-mc2 + abra) / (long double)(ee));
    } else {
        g->ee = 0.001239841662513396 / p->wl;
    }
    g->k2maxo = pow(p->aobj * 0.001f / p->wl, 2.0); /* UTR.cpp:388 (a float literal) */
    g->cs3 = p->cs3 * 1.e+7;                        /* UTR.cpp:398-399, mm -> length unit */
    g->cs5 = p->cs5 * 1.e+7;
    /* UTR.cpp:211-238: rotation flags (from the second orientation on, as
     * the reference loops) and the mean defocus */
    g->rot_z_only = g->rot_y_only = g->rot_z2_only = 1;
    double zav = defocus[0];
    for (int i = 1; i < nangles; i++) {
        if (angles[2 * i] != 0) {
            g->rot_y_only = 0;
            g->rot_z2_only = 0;
        }
        if (angles[2 * i + 1] != 0) {
            g->rot_z_only = 0;
            g->rot_z2_only = 0;
        }
        zav += defocus[i];
    }
    zav /= nangles;
    g->zout_aver = zav - p->dzextra; /* UTR.cpp:330 */
    return 0;
}

/* ------------------------------------------------------------------ spectra */

/* the half-size circular shift of both dimensions of a complex [ny][nx] array */
static void shuffle2_d(double *a, int nx, int ny)
{
    double *t = (double *)malloc(sizeof(double) * 2 * (size_t)nx * ny);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const size_t s = (size_t)((j + ny / 2) % ny) * nx + (i + nx / 2) % nx;
            t[2 * ((size_t)j * nx + i)] = a[2 * s];
            t[2 * ((size_t)j * nx + i) + 1] = a[2 * s + 1];
        }
    memcpy(a, t, sizeof(double) * 2 * (size_t)nx * ny);
    free(t);
}

static double cr_w(double t, int k)
{
    const double t2 = t * t, t3 = t2 * t;
    switch (k) {
    case 0: return 0.5 * (-t3 + 2.0 * t2 - t);
    case 1: return 0.5 * (3.0 * t3 - 5.0 * t2 + 2.0);
    case 2: return 0.5 * (-3.0 * t3 + 4.0 * t2 + t);
    default: return 0.5 * (t3 - t2);
    }
}

/* UTR.cpp:920-940 on a normalised image [ny][nx] in place: the edge mean,
 * the shift (dx, dy) pixels, then the rotation by `t` about (cx, cy) (pixels),
 * as defined in the file header (UTR rotates by -Z'': t = -Z'') */
void mo_utr_image_plane_f64(double *img, int nx, int ny, double cx, double cy, double t,
                            long dx, long dy)
{
    const size_t n = (size_t)nx * ny;
    double f = 0.0;
    long cnt = 0;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
            if (i < 5 || i >= nx - 5 || j < 5 || j >= ny - 5) {
                f += img[(size_t)j * nx + i];
                cnt++;
            }
    if (cnt) f /= cnt;
    double *s1 = (double *)malloc(sizeof(double) * n);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const long jj = j - dy, ii = i - dx;
            s1[(size_t)j * nx + i] =
                (jj >= 0 && jj < ny && ii >= 0 && ii < nx) ? img[(size_t)jj * nx + ii] : f;
        }
    if (t == 0.0) {
        memcpy(img, s1, sizeof(double) * n);
        free(s1);
        return;
    }
    const double c = cos(t), sn = sin(t);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const double ddx = i - cx, ddy = j - cy;
            const double fx = cx + c * ddx + sn * ddy, fy = cy - sn * ddx + c * ddy;  /* R(-t) */
            const int x0 = (int)floor(fx), y0 = (int)floor(fy);
            const double tx = fx - x0, ty = fy - y0;
            double acc = 0.0;
            for (int b = 0; b < 4; b++)
                for (int a = 0; a < 4; a++) {
                    const int xx = x0 - 1 + a, yy = y0 - 1 + b;
                    const double w = cr_w(tx, a) * cr_w(ty, b);
                    acc += w * ((xx >= 0 && xx < nx && yy >= 0 && yy < ny) ? s1[(size_t)yy * nx + xx] : f);
                }
            img[(size_t)j * nx + i] = acc;
        }
    free(s1);
}

/* the log-FFT of a normalised double image (UTR.cpp:989-996) */
static void k2four_from_norm(double *k2, const double *v, int nx, int ny)
{
    const size_t n = (size_t)nx * ny;
    for (size_t q = 0; q < n; q++) {
        k2[2 * q] = v[q] > 0.0 ? log(v[q]) : 0.0;
        k2[2 * q + 1] = 0.0;
    }
    shuffle2_d(k2, nx, ny);
    ocfft2d_d(k2, ny, nx, -1);
    shuffle2_d(k2, nx, ny);
}

/* UTR.cpp:940-950 (normalisation, threshold) and 989-996 (Log0, complex,
 * Shuffle, FFT, Shuffle), with the normalised image kept in float */
void mo_utr_k2four_f32(const float *img, int nx, int ny, double f1, double f2, float *k2)
{
    const size_t n = (size_t)nx * ny;
    double *a = (double *)malloc(sizeof(double) * 2 * n);
    for (size_t q = 0; q < n; q++) {
        float v = img[q];
        if (f1 != 1.0) v /= (float)f1;
        if (f2 != 0.0) v += (float)f2;
        if (v < 0.0f) v = 0.0f;
        a[2 * q] = v > 0.0f ? (double)logf(v) : 0.0;
        a[2 * q + 1] = 0.0;
    }
    shuffle2_d(a, nx, ny);
    ocfft2d_d(a, ny, nx, -1);
    shuffle2_d(a, nx, ny);
    for (size_t q = 0; q < 2 * n; q++) k2[q] = (float)a[q];
    free(a);
}

void mo_utr_k2four_f64(const float *img, int nx, int ny, double f1, double f2, double *k2)
{
    const size_t n = (size_t)nx * ny;
    for (size_t q = 0; q < n; q++) {
        double v = img[q];
        if (f1 != 1.0) v /= f1;
        if (f2 != 0.0) v += f2;
        if (v < 0.0) v = 0.0;
        k2[2 * q] = v > 0.0 ? log(v) : 0.0;
        k2[2 * q + 1] = 0.0;
    }
    shuffle2_d(k2, nx, ny);
    ocfft2d_d(k2, ny, nx, -1);
    shuffle2_d(k2, nx, ny);
}

/* ------------------------------------------------------------------ gridding */

/* The per-image coordinate tables of CT_3Dgridding (UTR.h:214-236): the
 * frequency coordinate of column i in double from float steps, then the
 * products with the float sines in double, rounded to float. */
typedef struct {
    float *xxx2, *xsy, *xcy, *yyy2, *ysz, *ycz;
    float sinY, cosY, sinZ, cosZ;
} GridTabs;

static void grid_tabs(GridTabs *t, int nx, int ny, double angleY, double angleZ, float fxlo,
                      float fxst, float fylo, float fyst, double wl)
{
    const double wl2 = 0.5 * wl;
    t->sinY = (float)sin(angleY);
    t->cosY = (float)cos(angleY);
    t->sinZ = (float)sin(angleZ);
    t->cosZ = (float)cos(angleZ);
    t->xxx2 = (float *)malloc(sizeof(float) * 3 * nx);
    t->xsy = t->xxx2 + nx;
    t->xcy = t->xsy + nx;
    t->yyy2 = (float *)malloc(sizeof(float) * 3 * ny);
    t->ysz = t->yyy2 + ny;
    t->ycz = t->ysz + ny;
    for (int i = 0; i < nx; i++) {
        const float fs = fxst * (float)i;
        const double x = (double)(fxlo + fs);
        t->xxx2[i] = (float)(-wl2 * x * x);
        t->xsy[i] = (float)(x * (double)t->sinY);
        t->xcy[i] = (float)(x * (double)t->cosY);
    }
    for (int j = 0; j < ny; j++) {
        const float fs = fyst * (float)j;
        const double y = (double)(fylo + fs);
        t->yyy2[j] = (float)(-wl2 * y * y);
        t->ysz[j] = (float)(y * (double)t->sinZ);
        t->ycz[j] = (float)(y * (double)t->cosZ);
    }
}

static void grid_tabs_free(GridTabs *t)
{
    free(t->xxx2);
    free(t->yyy2);
}

/* One pixel's cell in the volume: the lower corner (ii, jj, nn), the float
 * fractions, and the frequency coordinates (UTR.h:248-269).  Returns 0 when
 * the reference's `continue` skips the pixel. */
typedef struct {
    int ii, jj, nn;
    float dx0, dx1, dy0, dy1, dz0, dz1;
    float qx, qy, qz;
} Cell;

static int grid_cell(const GridTabs *t, int i, int j, int nx, int ny, int nz, float fxlo,
                     float fxst, float fylo, float fyst, float fzlo, float fzst, int escc,
                     Cell *c)
{
    float zz = 0.0f;
    if (escc) zz = t->xxx2[i] + t->yyy2[j];
    const float zs = zz * t->sinY;
    const float xx = t->xcy[i] - zs;  /* qx after the inverse rotation about Y' */
    const float zc = zz * t->cosY;
    const float zzz = t->xsy[i] + zc; /* qz */
    float dz1 = (zzz - fzlo) / fzst;
    const int nn = (int)floorf(dz1);
    if (nn < 0 || nn > nz - 2) return 0;
    const float xcz = xx * t->cosZ;
    const float xxx = xcz + t->ysz[j]; /* qx after the inverse rotation about Z */
    float dx1 = (xxx - fxlo) / fxst;
    const int ii = (int)floorf(dx1);
    if (ii < 0 || ii > nx - 2) return 0;
    const float mxs = -xx * t->sinZ;
    const float yyy = mxs + t->ycz[j]; /* qy */
    float dy1 = (yyy - fylo) / fyst;
    const int jj = (int)floorf(dy1);
    if (jj < 0 || jj > ny - 2) return 0;
    dx1 -= (float)ii;
    dy1 -= (float)jj;
    dz1 -= (float)nn;
    c->ii = ii;
    c->jj = jj;
    c->nn = nn;
    c->dx1 = dx1;
    c->dx0 = 1.0f - dx1;
    c->dy1 = dy1;
    c->dy0 = 1.0f - dy1;
    c->dz1 = dz1;
    c->dz0 = 1.0f - dz1;
    c->qx = xxx;
    c->qy = yyy;
    c->qz = zzz;
    return 1;
}

/* the value cd of a pixel, times the centre-of-rotation phase factor
 * exp(Fxc qx + Fyc qy + Fzc qz) in complex float (UTR.h:271-273) */
static void pixel_value_f(const float *k2, const float *fc, int rotshift, const Cell *c,
                          float *re, float *im)
{
    float a = k2[0], b = k2[1];
    if (rotshift) {
        const float ex = fc[0] * c->qx, ey = fc[1] * c->qx;
        const float fx = fc[2] * c->qy, fy = fc[3] * c->qy;
        const float gx = fc[4] * c->qz, gy = fc[5] * c->qz;
        const float sx = (ex + fx) + gx, sy = (ey + fy) + gy;
        const float complex e = cexpf(sx + sy * I);
        const float er = crealf(e), ei = cimagf(e);
        const float r = a * er - b * ei, q = a * ei + b * er;
        a = r;
        b = q;
    }
    *re = a;
    *im = b;
}

/* weights of the eight corners in the reference's order, (dx, dy, dz) */
static void corner_weights(const Cell *c, float w[8], int off[8][3])
{
    const float dx[2] = {c->dx0, c->dx1}, dy[2] = {c->dy0, c->dy1}, dz[2] = {c->dz0, c->dz1};
    int n = 0;
    for (int b = 0; b < 2; b++)      /* y */
        for (int a = 0; a < 2; a++)  /* z */
            for (int e = 0; e < 2; e++) { /* x */
                w[n] = dx[e] * dy[b] * dz[a];
                off[n][0] = e;
                off[n][1] = b;
                off[n][2] = a;
                n++;
            }
}

void mo_utr_grid_f32(const float *k2four, int nx, int ny, int nz, double angleY, double angleZ,
                     float fxlo, float fxst, float fylo, float fyst, float fzlo, float fzst,
                     const float *fc, double wl, int rotshift, int escc, float *v3, float *samp3)
{
    GridTabs t;
    grid_tabs(&t, nx, ny, angleY, angleZ, fxlo, fxst, fylo, fyst, wl);
    const size_t nxny = (size_t)nx * ny;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            Cell c;
            if (!grid_cell(&t, i, j, nx, ny, nz, fxlo, fxst, fylo, fyst, fzlo, fzst, escc, &c))
                continue;
            float re, im;
            pixel_value_f(k2four + 2 * ((size_t)j * nx + i), fc, rotshift, &c, &re, &im);
            float w[8];
            int off[8][3];
            corner_weights(&c, w, off);
            for (int n = 0; n < 8; n++) {
                const size_t v = (size_t)(c.nn + off[n][2]) * nxny + (size_t)(c.jj + off[n][1]) * nx +
                                 (size_t)(c.ii + off[n][0]);
                samp3[v] += w[n];
                v3[2 * v] += re * w[n];
                v3[2 * v + 1] += im * w[n];
            }
        }
    grid_tabs_free(&t);
}

void mo_utr_grid_acc64(const float *k2four, int nx, int ny, int nz, double angleY,
                       double angleZ, float fxlo, float fxst, float fylo, float fyst, float fzlo,
                       float fzst, const float *fc, double wl, int rotshift, int escc,
                       double *v3, double *samp3)
{
    GridTabs t;
    grid_tabs(&t, nx, ny, angleY, angleZ, fxlo, fxst, fylo, fyst, wl);
    const size_t nxny = (size_t)nx * ny;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            Cell c;
            if (!grid_cell(&t, i, j, nx, ny, nz, fxlo, fxst, fylo, fyst, fzlo, fzst, escc, &c))
                continue;
            float re, im;
            pixel_value_f(k2four + 2 * ((size_t)j * nx + i), fc, rotshift, &c, &re, &im);
            float w[8];
            int off[8][3];
            corner_weights(&c, w, off);
            for (int n = 0; n < 8; n++) {
                const size_t v = (size_t)(c.nn + off[n][2]) * nxny + (size_t)(c.jj + off[n][1]) * nx +
                                 (size_t)(c.ii + off[n][0]);
                samp3[v] += (double)w[n];
                v3[2 * v] += (double)(re * w[n]);
                v3[2 * v + 1] += (double)(im * w[n]);
            }
        }
    grid_tabs_free(&t);
}

void mo_utr_grid_f64(const double *k2four, int nx, int ny, int nz, double angleY,
                     double angleZ, float fxlo, float fxst, float fylo, float fyst, float fzlo,
                     float fzst, const double *fcd, double wl, int rotshift, int escc,
                     double *v3, double *samp3)
{
    GridTabs t;
    grid_tabs(&t, nx, ny, angleY, angleZ, fxlo, fxst, fylo, fyst, wl);
    const size_t nxny = (size_t)nx * ny;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            Cell c;
            if (!grid_cell(&t, i, j, nx, ny, nz, fxlo, fxst, fylo, fyst, fzlo, fzst, escc, &c))
                continue;
            const double *k = k2four + 2 * ((size_t)j * nx + i);
            double re = k[0], im = k[1];
            if (rotshift) { /* fcd: the imaginary parts of Fxc, Fyc, Fzc */
                const double th = fcd[0] * c.qx + fcd[1] * c.qy + fcd[2] * c.qz;
                const double cr = cos(th), ci = sin(th);
                const double r = re * cr - im * ci, q = re * ci + im * cr;
                re = r;
                im = q;
            }
            float w[8];
            int off[8][3];
            corner_weights(&c, w, off);
            for (int n = 0; n < 8; n++) {
                const size_t v = (size_t)(c.nn + off[n][2]) * nxny + (size_t)(c.jj + off[n][1]) * nx +
                                 (size_t)(c.ii + off[n][0]);
                samp3[v] += (double)w[n];
                v3[2 * v] += re * (double)w[n];
                v3[2 * v + 1] += im * (double)w[n];
            }
        }
    grid_tabs_free(&t);
}

/* ------------------------------------------------------------------ 3D filters */

/* The CTF-correction factor (sinreg, -cosreg) of voxel (k, j, i) with the
 * reference's double expressions (UTR.h:54-121); 0 where the aperture
 * excludes it (the voxel is then left unchanged: returns 0). */
typedef struct {
    double fac2, fac3, fac5, omega, epsilon, dksi2, deta2, dzeta2, q2max;
    int aper, c35, escc, nxd2, nyd2, nzd2;
} CtfPar;

static int ctf_par(CtfPar *c, int nx, int ny, int nz, double wl, double zlo, double zhi, double ylo,
                   double yhi, double xlo, double xhi, double defocdist, double q2max, double cs3,
                   double cs5, double sigma, double epsilon, int escc)
{
    if ((nx & 1) || (ny & 1) || (nz & 1)) return -1;
    const double xst = (xhi - xlo) / nx, yst = (yhi - ylo) / ny,
                 zst = (zhi - zlo) / ny; /* GetZStep(ny), as UTR.h:48 asks */
    const double xap2 = (xhi - xlo) * (xhi - xlo), yap2 = (yhi - ylo) * (yhi - ylo),
                 zap2 = (zhi - zlo) * (zhi - zlo);
    const double srad = sqrt(0.25 / (xst * xst) + 0.25 / (yst * yst) + 0.25 / (zst * zst));
    if (srad * wl > 1.0) return -1;
    c->aper = q2max > 0;
    c->q2max = q2max;
    c->omega = atan(sigma);
    c->c35 = (cs3 != 0) || (cs5 != 0);
    c->dksi2 = 1.0 / xap2;
    c->deta2 = 1.0 / yap2;
    c->dzeta2 = 1.0 / zap2;
    c->fac2 = kPi * wl * defocdist;
    double mn = c->deta2 < c->dzeta2 ? c->deta2 : c->dzeta2;
    mn = c->dksi2 < mn ? c->dksi2 : mn;
    c->epsilon = epsilon <= 0 ? 0.1 * pow(fabs(c->fac2) * mn, 2) : epsilon;
    c->fac3 = kPi * pow(wl, 3) / 2.0 * cs3;
    c->fac5 = kPi * pow(wl, 5) / 3.0 * cs5;
    c->escc = escc;
    c->nxd2 = nx / 2;
    c->nyd2 = ny / 2;
    c->nzd2 = nz / 2;
    return 0;
}

static int ctf_factor(const CtfPar *c, int k, int j, int i, double *sinreg, double *cosreg)
{
    const int k1 = k - c->nzd2, j1 = j - c->nyd2, i1 = i - c->nxd2;
    const double zeta2 = c->dzeta2 * k1 * k1;
    const double zeta2fac2 = c->fac2 * zeta2 - c->omega;
    double eta2 = c->deta2 * j1 * j1;
    const double eta2fac2 = c->fac2 * eta2 + zeta2fac2;
    eta2 += zeta2;
    double ksi2 = c->dksi2 * i1 * i1;
    const double ksi2fac2 = c->fac2 * ksi2 + eta2fac2;
    ksi2 += eta2;
    if (c->aper && !(ksi2 < c->q2max)) return 0;
    double cst = 0;
    if (c->c35) cst = c->fac3 * ksi2 * ksi2 + c->fac5 * pow(ksi2, 3);
    const double dtemp = ksi2fac2 + cst;
    const double s = sin(dtemp);
    *sinreg = s / (s * s + c->epsilon);
    *cosreg = 0.0;
    if (c->escc) {
        const double co = cos(dtemp);
        *cosreg = co / (co * co + c->epsilon);
    }
    return 1;
}

int mo_utr_ctf3d_f32(float *v3, int nx, int ny, int nz, double wl, double zlo, double zhi,
                     double ylo, double yhi, double xlo, double xhi, double defocdist,
                     double q2max, double cs3, double cs5, double sigma, double epsilon, int escc)
{
    CtfPar c;
    if (ctf_par(&c, nx, ny, nz, wl, zlo, zhi, ylo, yhi, xlo, xhi, defocdist, q2max, cs3, cs5,
                sigma, epsilon, escc))
        return -1;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                double sr, cr;
                if (!ctf_factor(&c, k, j, i, &sr, &cr)) continue;
                const float fs = (float)sr, fc = -(float)cr;
                float *v = v3 + 2 * (((size_t)k * ny + j) * nx + i);
                const float a = v[0], b = v[1];
                v[0] = a * fs - b * fc;
                v[1] = a * fc + b * fs;
            }
    return 0;
}

int mo_utr_ctf3d_f64(double *v3, int nx, int ny, int nz, double wl, double zlo, double zhi,
                     double ylo, double yhi, double xlo, double xhi, double defocdist,
                     double q2max, double cs3, double cs5, double sigma, double epsilon, int escc)
{
    CtfPar c;
    if (ctf_par(&c, nx, ny, nz, wl, zlo, zhi, ylo, yhi, xlo, xhi, defocdist, q2max, cs3, cs5,
                sigma, epsilon, escc))
        return -1;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                double sr, cr;
                if (!ctf_factor(&c, k, j, i, &sr, &cr)) continue;
                double *v = v3 + 2 * (((size_t)k * ny + j) * nx + i);
                const double a = v[0], b = v[1];
                v[0] = a * sr + b * cr;
                v[1] = -a * cr + b * sr;
            }
    return 0;
}

/* UTR.h:126-175: multiply by norm / (alpha + 4 pi^2 (ksi^2 + eta^2 + zeta^2)) */
static int invlap_check(int nx, int ny, int nz, double zaper, double yaper, double xaper,
                        double alpha)
{
    if (alpha <= 0 || xaper == 0 || yaper == 0 || zaper == 0) return -1;
    if ((nx & 1) || (ny & 1) || (nz & 1)) return -1;
    return 0;
}

static double invlap_den(int k, int j, int i, int nx, int ny, int nz, double zaper, double yaper,
                         double xaper, double alpha)
{
    const double fact = 4.0 * kPi * kPi;
    const double dksi2 = fact / (xaper * xaper), deta2 = fact / (yaper * yaper),
                 dzeta2 = fact / (zaper * zaper);
    const int k1 = k - nz / 2, j1 = j - ny / 2, i1 = i - nx / 2;
    const double zeta2 = k1 * k1 * dzeta2 + alpha;
    const double eta2 = j1 * j1 * deta2 + zeta2;
    return dksi2 * i1 * i1 + eta2;
}

int mo_utr_invlap3d_f32(float *v3, int nx, int ny, int nz, double zaper, double yaper,
                        double xaper, double alpha, double norm)
{
    if (invlap_check(nx, ny, nz, zaper, yaper, xaper, alpha)) return -1;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const float s = (float)(norm / invlap_den(k, j, i, nx, ny, nz, zaper, yaper, xaper, alpha));
                float *v = v3 + 2 * (((size_t)k * ny + j) * nx + i);
                v[0] *= s;
                v[1] *= s;
            }
    return 0;
}

int mo_utr_invlap3d_f64(double *v3, int nx, int ny, int nz, double zaper, double yaper,
                        double xaper, double alpha, double norm)
{
    if (invlap_check(nx, ny, nz, zaper, yaper, xaper, alpha)) return -1;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const double s = norm / invlap_den(k, j, i, nx, ny, nz, zaper, yaper, xaper, alpha);
                double *v = v3 + 2 * (((size_t)k * ny + j) * nx + i);
                v[0] *= s;
                v[1] *= s;
            }
    return 0;
}

/* ------------------------------------------------------------------ pipeline */

/* Fxc, Fyc, Fzc of one orientation (UTR.cpp:893-898): the imaginary parts
 * (the real parts are 0), in double and as the reference's float values */
static void centre_phase(const msk_utr *p, double angleY, double angleZ, double fd[3], float ff[6])
{
    const double tpi = 2.0 * kPi;
    const double cy = cos(angleY), sy = sin(angleY), cz = cos(angleZ), sz = sin(angleZ);
    const double ax = tpi * (p->dxc * (1.0 - cy * cz) - p->dyc * sz + p->dzc * sy * cz);
    const double ay = tpi * (p->dxc * cy * sz + p->dyc * (1.0 - cz) - p->dzc * sy * sz);
    const double az = tpi * (-p->dxc * sy + p->dzc * (1.0 - cy));
    fd[0] = -ax;
    fd[1] = -ay;
    fd[2] = -az;
    /* fcomplex(0, -1) * float(a): (0 * a, -1 * a) */
    const float fa[3] = {(float)ax, (float)ay, (float)az};
    for (int q = 0; q < 3; q++) {
        ff[2 * q] = 0.0f * fa[q];
        ff[2 * q + 1] = -1.0f * fa[q];
    }
}

typedef struct {
    const msk_utr *p;
    const mo_utr_geom *g;
    const double *angles, *zrot, *shifts;
    const float *images;
    int a0, a1;
    double *v3, *samp3;
} GridJob;

static void *grid_worker(void *arg)
{
    GridJob *J = (GridJob *)arg;
    const mo_utr_geom *g = J->g;
    const int nx = g->nx, ny = g->ny;
    double *k2 = (double *)malloc(sizeof(double) * 2 * (size_t)nx * ny);
    double *nv = (double *)malloc(sizeof(double) * (size_t)nx * ny);
    const int rotshift = J->p->dxc != 0 || J->p->dyc != 0 || J->p->dzc != 0;
    const double cx = (g->xc - g->xlo) / g->xst, cy = (g->yc - g->ylo) / g->xst;
    for (int a = J->a0; a < J->a1; a++) {
        const double angleZ = J->angles[2 * a] * kPi / 180.0, angleY = J->angles[2 * a + 1] * kPi / 180.0;
        const double z2 = J->zrot ? J->zrot[a] : 0.0;
        const double shx = J->shifts ? J->shifts[2 * a] : 0.0, shy = J->shifts ? J->shifts[2 * a + 1] : 0.0;
        if (z2 != 0.0 || shx != 0.0 || shy != 0.0) {
            /* UTR.cpp:940-948 then 920-940: normalise, shift and rotate back */
            const float *im = J->images + (size_t)a * nx * ny;
            for (size_t q = 0; q < (size_t)nx * ny; q++) {
                double v = im[q];
                if (J->p->f1 != 1.0) v /= J->p->f1;
                if (J->p->f2 != 0.0) v += J->p->f2;
                nv[q] = v < 0.0 ? 0.0 : v;
            }
            mo_utr_image_plane_f64(nv, nx, ny, cx, cy, -z2 * kPi / 180.0,
                                   (long)floor(-shx / g->xst + 0.5), (long)floor(-shy / g->xst + 0.5));
            k2four_from_norm(k2, nv, nx, ny);
        } else {
            mo_utr_k2four_f64(J->images + (size_t)a * nx * ny, nx, ny, J->p->f1, J->p->f2, k2);
        }
        double fd[3];
        float ff[6];
        centre_phase(J->p, angleY, angleZ, fd, ff);
        mo_utr_grid_f64(k2, nx, ny, g->nz, angleY, angleZ, (float)g->fxlo, (float)g->fxst,
                        (float)g->fylo, (float)g->fyst, (float)g->fzlo, (float)g->fzst, fd, g->wl,
                        rotshift, J->p->escc, J->v3, J->samp3);
    }
    free(nv);
    free(k2);
    return NULL;
}

/* UTR.cpp:1052-1093: sampling normalisation and the SNR filter (modes 0, 2,
 * 3, 4), in double */
static void normalise_f64(const msk_utr *p, const mo_utr_geom *g, double *v3, const double *samp3)
{
    const size_t nv = (size_t)g->nx * g->ny * g->nz;
    const double nsr = p->nsr * sqrt((double)g->nx * g->ny);
    for (size_t q = 0; q < nv; q++) {
        const double x = samp3[q];
        double *v = v3 + 2 * q;
        if (x == 0) {
            v[0] = v[1] = 0.0;
            continue;
        }
        double s = 1.0 / x;
        if (nsr != 0) {
            const double y = hypot(v[0], v[1]) / (nsr * sqrt(x));
            s *= 0.5 + atan(100.0 * (y - 1.414213562373)) / kPi;
        }
        v[0] *= s;
        v[1] *= s;
    }
}

/* UTR.cpp:1203-1217, in the reference's loop order */
static void hermitian_f64(double *v3, int nx, int ny, int nz)
{
    for (int k = 0; k < nz; k++) {
        const int ka = k == 0 ? 0 : nz - k;
        for (int j = 0; j < ny; j++) {
            const int ja = j == 0 ? 0 : ny - j;
            for (int i = 0; i < nx / 2; i++) {
                const int ia = i == 0 ? 0 : nx - i;
                double *d = v3 + 2 * (((size_t)k * ny + j) * nx + ia);
                const double *s = v3 + 2 * (((size_t)ka * ny + ja) * nx + i);
                const double re = 0.5 * (d[0] + s[0]), im = 0.5 * (d[1] - s[1]);
                d[0] = re;
                d[1] = im;
            }
        }
    }
}

/* Complex-to-real inverse 3D FFT of the half spectrum of a centred volume,
 * shuffled back to centred real space and divided by nx*ny*nz (see the file
 * header for the definition). */
static void c2r3_f64(const double *v3, int nx, int ny, int nz, double *out)
{
    const int h = nx / 2 + 1;
    /* the half spectrum in wrapped order: kx = 0..nx/2 <- centred x index
     * (kx + nx/2) mod nx; ky, kz wrapped likewise */
    double *hs = (double *)malloc(sizeof(double) * 2 * (size_t)h * ny * nz);
    for (int kz = 0; kz < nz; kz++)
        for (int ky = 0; ky < ny; ky++)
            for (int kx = 0; kx < h; kx++) {
                const int k = (kz + nz / 2) % nz, j = (ky + ny / 2) % ny, i = (kx + nx / 2) % nx;
                const double *s = v3 + 2 * (((size_t)k * ny + j) * nx + i);
                double *d = hs + 2 * (((size_t)kz * ny + ky) * h + kx);
                d[0] = s[0];
                d[1] = s[1];
            }
    /* complex inverse along z, then y */
    ocfft1d_many_d(hs, nz, ny * h, ny * h, 1, +1);
    for (int kz = 0; kz < nz; kz++) ocfft1d_many_d(hs + 2 * (size_t)kz * ny * h, ny, h, h, 1, +1);
    /* real inverse along x: Hermitian extension with the real parts of the
     * kx = 0 and kx = nx/2 terms */
    double *line = (double *)malloc(sizeof(double) * 2 * nx);
    const double sc = 1.0 / ((double)nx * ny * nz);
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++) {
            const double *s = hs + 2 * (((size_t)z * ny + y) * h);
            for (int kx = 0; kx < nx; kx++) {
                if (kx == 0 || kx == nx / 2) {
                    line[2 * kx] = s[2 * kx];
                    line[2 * kx + 1] = 0.0;
                } else if (kx < nx / 2) {
                    line[2 * kx] = s[2 * kx];
                    line[2 * kx + 1] = s[2 * kx + 1];
                } else {
                    line[2 * kx] = s[2 * (nx - kx)];
                    line[2 * kx + 1] = -s[2 * (nx - kx) + 1];
                }
            }
            ocfft1d_many_d(line, nx, 1, 1, nx, +1);
            /* centred output: real-space index (x + n/2) mod n */
            const int zc = (z + nz / 2) % nz, yc = (y + ny / 2) % ny;
            for (int x = 0; x < nx; x++)
                out[((size_t)zc * ny + yc) * nx + (x + nx / 2) % nx] = line[2 * x] * sc;
        }
    free(line);
    free(hs);
}

static int utr_finish_geom(const msk_utr *p, const mo_utr_geom *gp, double *v3,
                           const double *samp3, double *volume)
{
    const mo_utr_geom g = *gp;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    normalise_f64(p, &g, v3, samp3);
    /* UTR.cpp:1177-1201 */
    if (g.zout_aver != 0) {
        if (p->ctf_mode == 2) {
            const double alpha = -4.0 * kPi * p->asigma / (g.zout_aver * g.wl);
            const double norm = -alpha * sqrt(1.0 + p->asigma * p->asigma) / p->asigma;
            if (mo_utr_invlap3d_f64(v3, nx, ny, nz, g.zhi - g.zlo, g.yhi - g.ylo, g.xhi - g.ylo,
                                    alpha, norm))
                return -1;
        } else if (p->ctf_mode == 4) {
            if (mo_utr_ctf3d_f64(v3, nx, ny, nz, g.wl, g.zlo, g.zhi, g.ylo, g.yhi, g.xlo, g.xhi,
                                 g.zout_aver, g.k2maxo, g.cs3, g.cs5, p->asigma, p->epsilon,
                                 p->escc))
                return -1;
        }
    }
    if (p->inv_laplace && p->ctf_mode != 1 && p->ctf_mode != 2)
        if (mo_utr_invlap3d_f64(v3, nx, ny, nz, g.zhi - g.zlo, g.yhi - g.ylo, g.xhi - g.ylo,
                                p->epsilon, p->epsilon))
            return -1;
    hermitian_f64(v3, nx, ny, nz);
    c2r3_f64(v3, nx, ny, nz, volume);
    /* UTR.cpp:1235-1262: outside the reconstruction sphere (or cylinder) 0,
     * inside times exp(2 r^2 / (kc^2 + jc^2 + ic^2)) */
    const long ic = g.ic, jc = g.jc, kc = g.kc;
    const long nxd2 = nx / 2, nyd2 = ny / 2, nzd2 = nz / 2;
    const long nxR2 = ic <= nxd2 ? ic * ic : (nx - ic) * (nx - ic);
    const long nyR2 = jc <= nyd2 ? jc * jc : (ny - jc) * (ny - jc);
    const long nzR2 = kc <= nzd2 ? kc * kc : (nz - kc) * (nz - kc);
    long nR2;
    if (g.rot_y_only) nR2 = nxR2 < nzR2 ? nxR2 : nzR2;
    else if (g.rot_z_only || g.rot_z2_only) nR2 = nxR2 < nyR2 ? nxR2 : nyR2;
    else {
        nR2 = nxR2 < nyR2 ? nxR2 : nyR2;
        nR2 = nR2 < nzR2 ? nR2 : nzR2;
    }
    const double dtemp = 2.0 / (double)(kc * kc + jc * jc + ic * ic);
    double fnorm;
    if (p->modality == 0)
        fnorm = g.ee * g.wl / (2.0 * kPi * sqrt(1.0 + p->asigma * p->asigma) * g.xst);
    else
        fnorm = p->asigma * g.wl / (4.0 * kPi * sqrt(1.0 + p->asigma * p->asigma) * g.xst);
    for (int k = 0; k < nz; k++) {
        long kk2 = 0;
        if (!g.rot_z_only && !g.rot_z2_only) kk2 = (k - kc) * (k - kc);
        for (int j = 0; j < ny; j++) {
            const long jj2 = !g.rot_y_only ? (j - jc) * (j - jc) + kk2 : kk2;
            for (int i = 0; i < nx; i++) {
                const long ii2 = (i - ic) * (i - ic) + jj2;
                double *o = volume + ((size_t)k * ny + j) * nx + i;
                *o = ii2 > nR2 ? 0.0 : *o * exp(dtemp * (double)ii2) * fnorm;
            }
        }
    }
    return 0;
}

int mo_utr_finish_f64(const msk_utr *p, int nangles, const double *angles,
                      const double *defocus, double *v3, const double *samp3, double *volume)
{
    mo_utr_geom g;
    if (mo_utr_geom_make(p, nangles, angles, defocus, &g)) return -1;
    return utr_finish_geom(p, &g, v3, samp3, volume);
}

int mo_utr_reconstruct_f64(const msk_utr *p, int nangles, const double *angles,
                           const double *defocus, const double *zrot, const double *shifts,
                           const float *images, double *volume, int nthreads)
{
    mo_utr_geom g;
    if (mo_utr_geom_make(p, nangles, angles, defocus, &g)) return -1;
    if (zrot) /* UTR.cpp:221: a Z'' rotation (from the second orientation on) */
        for (int i = 1; i < nangles; i++)
            if (zrot[i] != 0) g.rot_y_only = g.rot_z_only = 0;
    if (p->ctf_mode == 1 || p->ctf_mode == 3) return -1; /* XArrayLibrary's 2D filters */
    const size_t nv = (size_t)g.nx * g.ny * g.nz;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > nangles) nthreads = nangles;
    GridJob *jobs = (GridJob *)calloc(nthreads, sizeof(GridJob));
    pthread_t *th = (pthread_t *)calloc(nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        jobs[t].p = p;
        jobs[t].g = &g;
        jobs[t].angles = angles;
        jobs[t].zrot = zrot;
        jobs[t].shifts = shifts;
        jobs[t].images = images;
        jobs[t].a0 = (int)((long)nangles * t / nthreads);
        jobs[t].a1 = (int)((long)nangles * (t + 1) / nthreads);
        jobs[t].v3 = (double *)calloc(2 * nv, sizeof(double));
        jobs[t].samp3 = (double *)calloc(nv, sizeof(double));
        pthread_create(&th[t], NULL, grid_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    double *v3 = jobs[0].v3, *samp3 = jobs[0].samp3;
    for (int t = 1; t < nthreads; t++) {
        for (size_t q = 0; q < 2 * nv; q++) v3[q] += jobs[t].v3[q];
        for (size_t q = 0; q < nv; q++) samp3[q] += jobs[t].samp3[q];
        free(jobs[t].v3);
        free(jobs[t].samp3);
    }
    const int st = utr_finish_geom(p, &g, v3, samp3, volume);
    free(v3);
    free(samp3);
    free(jobs);
    free(th);
    return st;
}
