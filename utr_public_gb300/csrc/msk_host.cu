// msk_host.cu -- host side of libmsk: the C ABI (include/msk.h), the
// reference-exact host preparation (rotation, Shell sort, slice assignment),
// the potential tables, and the schedule of passes over a batch of waves.
//
// Host arithmetic that must round like the reference (rotation, slice
// boundaries, frequency grids, propagator tables) is compiled with
// -ffp-contract=off so that x86-64 and aarch64 give the same bits.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cudaTypedefs.h>
#include <cufft.h>
#include <dlfcn.h>

#include "msk.h"
#include "msk_ctx.h"
#include "msk_launch.cuh"

namespace msk {

const SizeOps *size_ops_16();
const SizeOps *size_ops_32();
const SizeOps *size_ops_64();
const SizeOps *size_ops_128();
const SizeOps *size_ops_256();
const SizeOps *size_ops_512();
const SizeOps *size_ops_1024();
const SizeOps *size_ops_2048();
const SizeOps *size_ops_4096();

const SizeOps *size_ops(int n)
{
    switch (n) {
    case 16: return size_ops_16();
    case 32: return size_ops_32();
    case 64: return size_ops_64();
    case 128: return size_ops_128();
    case 256: return size_ops_256();
    case 512: return size_ops_512();
    case 1024: return size_ops_1024();
    case 2048: return size_ops_2048();
    case 4096: return size_ops_4096();
    default: return nullptr;
    }
}

__global__ void k_plane_init(float2 *psi, const int *__restrict__ units, int nunits, int nx, int ny)
{
    const size_t plane = (size_t)nx * ny;
    const size_t total = plane * nunits;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t ui = i / plane, r = i % plane;
        const int u = units ? units[ui] : (int)ui;
        psi[(size_t)u * plane + r] = make_float2((r % ny) == 0 ? (float)ny : 0.0f, 0.0f);
    }
}

// rows x width floats between device memory and page-locked host memory the
// GPU addresses (mapped; row r at src + r * spitch, dst + r * dpitch): the SMs'
// loads and stores cross NVLink-C2C several times faster than a copy-engine
// transfer between the same buffers does on the Grace hosts.  Run on a stream
// of its own beside the slice kernels, with a small grid (a CTA of it takes
// registers a CTA of those kernels would use on its SM) and four 16-byte
// accesses in flight a thread.
constexpr int kCopyCtas = 38;
__global__ void __launch_bounds__(256) k_copy_rows(const float *__restrict__ src, size_t spitch,
                                                   float *dst, size_t dpitch, size_t width, int rows)
{
    const size_t nt = (size_t)gridDim.x * blockDim.x, tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const bool v4 = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) |
                      spitch | dpitch | width) & 3) == 0 &&
                    ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0;
    for (int r = 0; r < rows; r++) {
        const float *sr = src + (size_t)r * spitch;
        float *dr = dst + (size_t)r * dpitch;
        size_t done = 0;
        if (v4) {
            const float4 *s4 = reinterpret_cast<const float4 *>(sr);
            float4 *d4 = reinterpret_cast<float4 *>(dr);
            const size_t n4 = width / 4;
            size_t i = tid;
            for (; i + 3 * nt < n4; i += 4 * nt) {
                float4 v[4];
#pragma unroll
                for (int k = 0; k < 4; k++) v[k] = __ldcs(&s4[i + k * nt]);
#pragma unroll
                for (int k = 0; k < 4; k++) d4[i + k * nt] = v[k];
            }
            for (; i < n4; i += nt) d4[i] = __ldcs(&s4[i]);
            done = n4 * 4;
        }
        for (size_t i = done + tid; i < width; i += nt) dr[i] = sr[i];
    }
}

__global__ void k_fresnel_table(const Geom g, const Fresnel fr, float scale, float2 *table)
{
    const size_t n = (size_t)g.nx * g.ny;
    const double twopi = 6.283185307179586;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i / g.ny), iy = (int)(i % g.ny);
        const float k2f = __fadd_rn(g.kx2[ix], g.ky2[iy]);
        if (fr.k2maxo > 0.0f && !(k2f < fr.k2maxo)) {
            table[i] = make_float2(0.0f, 0.0f);
            continue;
        }
        const double kx = (double)fr.kx[ix], ky = (double)fr.ky[iy];
        const double k2 = kx * kx + ky * ky;
        double chi = fr.a1 * k2 + fr.a3 * k2 * k2 + fr.a5 * k2 * k2 * k2 +
                     fr.a2c * (kx * kx - ky * ky) + fr.a2s * (2.0 * kx * ky);
        chi -= twopi * rint(chi / twopi);
        float s, c;
        sincosf((float)chi, &s, &c);
        table[i] = make_float2(c * scale, -s * scale);
    }
}

// ------------------------------------------------------------------ image plane
// The rotation about the optic axis and the XY shift MsctKirkland applies to
// the propagated amplitude of a detector plane (autosliccmd.cpp:1119-1143,
// XArray2DSpln::Rotate, XArray2DMove::Move and NormAverEdge(5) from the
// XArrayLibrary, which is not part of the reference).  This library's
// definitions, per component (real, imaginary):
//   fill   = the mean over the pixels within 5 of any edge;
//   rotate = out(p) = in(c + R(-theta)(p - c)), p = (ix*xst, iy*yst), c the
//            rotation centre, R(t) = [[cos t, -sin t], [sin t, cos t]] (the atom
//            rotation of autosliccmd.cpp:734-736), Catmull-Rom bicubic
//            interpolation on the pixel grid, grid points outside the image
//            reading the fill value;
//   shift  = out(ix, iy) = in(ix - sx, iy - sy), fill outside, (sx, sy) the shift
//            rounded to whole pixels.

// Per unit: the edge means of the real and imaginary parts, in double.
__global__ void k_edge_mean(const float2 *__restrict__ phi, const int *__restrict__ units, int nx,
                            int ny, int border, float2 *__restrict__ mean)
{
    const int u = units ? units[blockIdx.x] : (int)blockIdx.x;
    const float2 *p = phi + (size_t)u * nx * ny;
    double sr = 0.0, si = 0.0;
    long long cnt = 0;
    for (int i = threadIdx.x; i < nx * ny; i += blockDim.x) {
        const int ix = i / ny, iy = i % ny;
        if (ix < border || ix >= nx - border || iy < border || iy >= ny - border) {
            sr += p[i].x;
            si += p[i].y;
            cnt++;
        }
    }
    __shared__ double s_r[256], s_i[256];
    __shared__ long long s_c[256];
    s_r[threadIdx.x] = sr;
    s_i[threadIdx.x] = si;
    s_c[threadIdx.x] = cnt;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s_r[threadIdx.x] += s_r[threadIdx.x + w];
            s_i[threadIdx.x] += s_i[threadIdx.x + w];
            s_c[threadIdx.x] += s_c[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        mean[u] = s_c[0] ? make_float2((float)(s_r[0] / s_c[0]), (float)(s_i[0] / s_c[0]))
                         : make_float2(0.0f, 0.0f);
}

__device__ __forceinline__ float catmull_rom(float t, int k)
{
    // weights of the samples at -1, 0, 1, 2 for a fractional position t
    const float t2 = t * t, t3 = t2 * t;
    switch (k) {
    case 0: return 0.5f * (-t3 + 2.0f * t2 - t);
    case 1: return 0.5f * (3.0f * t3 - 5.0f * t2 + 2.0f);
    case 2: return 0.5f * (-3.0f * t3 + 4.0f * t2 + t);
    default: return 0.5f * (t3 - t2);
    }
}

__global__ void k_rotate_shift(const float2 *__restrict__ in, float2 *__restrict__ out,
                               const int *__restrict__ units, int nunits, int nx, int ny,
                               double xst, double yst, double xc, double yc, double cth,
                               double sth, int rotate, int sx, int sy,
                               const float2 *__restrict__ fill)
{
    const size_t plane = (size_t)nx * ny;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane * nunits;
         i += (size_t)gridDim.x * blockDim.x) {
        const int ui = (int)(i / plane), r = (int)(i % plane);
        const int u = units ? units[ui] : ui;
        const int ix = r / ny - sx, iy = r % ny - sy;
        const float2 f = fill[u];
        const float2 *src = in + (size_t)u * plane;
        float2 v = f;
        if (ix >= 0 && ix < nx && iy >= 0 && iy < ny) {
            if (!rotate) {
                v = src[(size_t)ix * ny + iy];
            } else {
                const double dx = ix * xst - xc, dy = iy * yst - yc;
                const double fx = (xc + cth * dx + sth * dy) / xst;  // R(-theta)
                const double fy = (yc - sth * dx + cth * dy) / yst;
                const int x0 = (int)floor(fx), y0 = (int)floor(fy);
                const float tx = (float)(fx - x0), ty = (float)(fy - y0);
                float ar = 0.0f, ai = 0.0f;
                for (int a = 0; a < 4; a++) {
                    const int xx = x0 - 1 + a;
                    const float wx = catmull_rom(tx, a);
                    for (int b = 0; b < 4; b++) {
                        const int yy = y0 - 1 + b;
                        const float w = wx * catmull_rom(ty, b);
                        const float2 q = (xx >= 0 && xx < nx && yy >= 0 && yy < ny)
                                             ? src[(size_t)xx * ny + yy]
                                             : f;
                        ar += w * q.x;
                        ai += w * q.y;
                    }
                }
                v = make_float2(ar, ai);
            }
        }
        out[(size_t)u * plane + r] = v;
    }
}

// Images from real-space amplitudes: images[dst[i]] (+)= sum over the units
// img_units[img_off[i] .. img_off[i+1]) of |a|^2, divided by nconf when
// flags & 2 (the bookkeeping of k_row_intensity).
__global__ void k_intensity_direct(int nimg, const int *__restrict__ img_off,
                                   const int *__restrict__ img_units,
                                   const int *__restrict__ img_dst,
                                   const int *__restrict__ img_flags,
                                   const float2 *__restrict__ amp, float *__restrict__ images,
                                   size_t plane, float nconf)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane * nimg;
         i += (size_t)gridDim.x * blockDim.x) {
        const int img = (int)(i / plane);
        const size_t r = i % plane;
        float *dst = images + (size_t)img_dst[img] * plane + r;
        const int fl = img_flags[img];
        float acc = (fl & 1) ? *dst : 0.0f;
        for (int k = img_off[img]; k < img_off[img + 1]; k++) {
            const float2 a = amp[(size_t)img_units[k] * plane + r];
            acc += a.x * a.x + a.y * a.y;
        }
        *dst = (fl & 2) ? __fdiv_rn(acc, nconf) : acc;
    }
}

// ------------------------------------------------------------------ physics
// Restatements of the reference's slicelib routines used to build tables.
namespace phys {

static const double kFe[104][12] = {
#include "kirkland_fparams.inc"
};

// slicelib.cpp:2891-2902
double wavelength(double kev)
{
    const double emass = 510.99906, hc = 12.3984244;
    return hc / sqrt(kev * (2 * emass + kev));
}

// slicelib.cpp:2441-2455
double sigma(double kev)
{
    const double emass = 510.99906;
    double x = (emass + kev) / (2.0 * emass + kev);
    double wavl = wavelength(kev);
    double pi = 4.0 * atan(1.0);
    return 2.0 * pi * x / (wavl * kev);
}

// slicelib.cpp:457-474
void freqn(float *ko, float *ko2, float *xo, int nk, double ak)
{
    int imid = (int)(nk / 2.0 + 0.5);
    for (int i = 0; i < nk; i++) {
        xo[i] = ((float)(i * ak)) / ((float)(nk - 1));
        ko[i] = (i > imid) ? ((float)(i - nk)) / ((float)ak) : ((float)i) / ((float)ak);
        ko2[i] = ko[i] * ko[i];
    }
}

// Abramowitz & Stegun 9.8.1-9.8.6 polynomial fits (slicelib.cpp:189-258)
double bessi0(double x)
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

double bessk0(double x)
{
    static const double a[] = {-0.57721566, 0.42278420, 0.23069756, 0.03488590, 0.00262698, 0.00010750, 0.00000740};
    static const double b[] = {1.25331414, -0.07832358, 0.02189568, -0.01062446, 0.00587872, -0.00251540, 0.00053208};
    double ax = fabs(x), x2, sum;
    if ((ax > 0.0) && (ax <= 2.0)) {
        x2 = ax / 2.0;
        x2 = x2 * x2;
        sum = a[6];
        for (int i = 5; i >= 0; i--) sum = sum * x2 + a[i];
        sum = -log(ax / 2.0) * bessi0(x) + sum;
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

// Projected potential, 3 Lorentzians + 3 Gaussians (slicelib.cpp:2759-2792)
double vzatom(int Z, double radius)
{
    const double al = 300.8242834, ag = 150.4121417, pi = 3.141592654;
    if (Z < 1 || Z > 103) return 0.0;
    double r = fabs(radius);
    if (r < 1.0e-10) r = 1.0e-10;
    double suml = 0.0, sumg = 0.0;
    double x = 2.0 * pi * r;
    for (int i = 0; i < 6; i += 2) suml += kFe[Z][i] * bessk0(x * sqrt(kFe[Z][i + 1]));
    x = pi * r;
    x = x * x;
    for (int i = 6; i < 12; i += 2) sumg += kFe[Z][i] * exp(-x / kFe[Z][i + 1]) / kFe[Z][i + 1];
    return al * suml + ag * sumg;
}

// Akima quasi-Hermite spline (slicelib.cpp:2537-2603)
void splinh(const double *x, const double *y, double *b, double *c, double *d, int n)
{
    const double SMALL = 1.0e-25;
    if (n < 4) return;
    double m5 = (y[3] - y[2]) / (x[3] - x[2]);
    double m4 = (y[2] - y[1]) / (x[2] - x[1]);
    double m3 = (y[1] - y[0]) / (x[1] - x[0]);
    double m2 = m3 + m3 - m4;
    double m1 = m2 + m2 - m3;
    double m54 = fabs(m5 - m4), m43 = fabs(m4 - m3), m32 = fabs(m3 - m2), m21 = fabs(m2 - m1);
    double t1 = ((m43 + m21) > SMALL) ? (m43 * m2 + m21 * m3) / (m43 + m21) : 0.5 * (m2 + m3);
    for (int i = 0; i < n - 1; i++) {
        double t2 = ((m54 + m32) > SMALL) ? (m54 * m3 + m32 * m4) / (m54 + m32) : 0.5 * (m3 + m4);
        double x43 = x[i + 1] - x[i];
        b[i] = t1;
        c[i] = (3.0 * m3 - t1 - t1 - t2) / x43;
        d[i] = (t1 + t2 - m3 - m3) / (x43 * x43);
        m1 = m2;
        m2 = m3;
        m3 = m4;
        m4 = m5;
        m5 = (i < n - 4) ? (y[i + 4] - y[i + 3]) / (x[i + 4] - x[i + 3]) : m4 + m4 - m3;
        m21 = m32;
        m32 = m43;
        m43 = m54;
        m54 = fabs(m5 - m4);
        t1 = t2;
    }
    (void)m1;
    (void)m21;
}

constexpr int kN = 100;

// vzatomLUT tables (slicelib.cpp:2812-2875): knots r^2 with r log-spaced in
// [0.01, 5] Angstrom; coefficients per Z built once and kept.
struct Lut {
    double knots[kN];
    double y[104][kN], b[104][kN], c[104][kN], d[104][kN];
    bool ready[104];
    std::mutex mu;
    Lut()
    {
        const double RMIN = 0.01, RMAX = 5.0;
        double dlnr = log(RMAX / RMIN) / (kN - 1);
        for (int i = 0; i < kN; i++) knots[i] = RMIN * exp(i * dlnr);
        for (int i = 0; i < kN; i++) knots[i] = knots[i] * knots[i];
        for (int z = 0; z < 104; z++) ready[z] = false;
    }
    void build(int Z)
    {
        std::lock_guard<std::mutex> g(mu);
        if (ready[Z]) return;
        for (int i = 0; i < kN; i++) y[Z][i] = vzatom(Z, sqrt(knots[i]));
        splinh(knots, y[Z], b[Z], c[Z], d[Z], kN);
        ready[Z] = true;
    }
};

Lut &lut()
{
    static Lut L;
    return L;
}

}  // namespace phys

// ------------------------------------------------------------------ host prep

// Shell sort by z (slicelib.cpp:2467-2504); same comparisons and moves, so
// the same permutation.
static void sort_by_z(float *x, float *y, float *z, float *occ, int *Znum, int natom)
{
    int h;
    for (h = 1; h <= (natom - 1) / 9; h = 3 * h + 1)
        ;
    for (; h > 0; h /= 3)
        for (int i = h; i < natom; i++) {
            int j = i;
            const float x2 = x[i], y2 = y[i], z2 = z[i], occ2 = occ[i];
            const int Z2 = Znum[i];
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

// Rotation about z then y' (autosliccmd.cpp:727-748), float arithmetic.
static void rotate(float ctblength, double dxc, double dyc, double dzc, double angleZ,
                   double angleY, int natom, float *x, float *y, float *z)
{
    const float xc = (float)(ctblength / 2.0 + dxc), yc = (float)(ctblength / 2.0 + dyc),
                zc = (float)(ctblength / 2.0 + dzc);
    const float sinZ = (float)sin(angleZ), cosZ = (float)cos(angleZ);
    const float sinY = (float)sin(angleY), cosY = (float)cos(angleY);
    for (int k = 0; k < natom; k++) {
        const float xxx = xc + (x[k] - xc) * cosZ + (-y[k] + yc) * sinZ;
        const float yyy = yc + (x[k] - xc) * sinZ + (y[k] - yc) * cosZ;
        x[k] = xxx;
        y[k] = yyy;
    }
    for (int k = 0; k < natom; k++) {
        const float xxx = xc + (x[k] - xc) * cosY + (z[k] - zc) * sinY;
        const float zzz = zc + (-x[k] + xc) * sinY + (z[k] - zc) * cosY;
        x[k] = xxx;
        z[k] = zzz;
    }
}

// Slice boundaries of the coherent branch (autoslic.cpp:747-756, 828):
// zslice = dz, 2dz, ... accumulated in double while < zmax + dz.
static int slice_count(float deltaz_f, float zmax)
{
    const double deltaz = deltaz_f;
    double zslice = deltaz;
    int n = 0;
    while (zslice < (zmax + deltaz)) {
        n++;
        zslice += deltaz;
    }
    return n;
}

// Atoms per slice of a z-sorted list (autoslic.cpp:756-762, 828-830).
static void slice_counts(float deltaz_f, float zmax, int natom, const float *z2, int nslices,
                         int *counts)
{
    const double deltaz = deltaz_f;
    double zslice = deltaz;
    int istart = 0;
    for (int s = 0; s < nslices; s++) {
        int na = 0;
        for (int i = istart; i < natom; i++)
            if (z2[i] < zslice) na++;
            else break;
        counts[s] = na;
        zslice += deltaz;
        istart += na;
    }
}

// Plan-wide geometry computed on the host exactly as the reference does.
struct GridPre {
    std::vector<int2> kband;  // per column iy: kx2 + ky2 < k2max <=> ix <= A or ix >= B
    int nx, ny;
    float ax, by, v0, wavlen, k2max;
    double scalex, scaley;  // float-divided pixel pitch, promoted
    double sigma;
    Geom g;                 // device pointers filled at upload
    const float *d_kx = nullptr, *d_ky = nullptr;  // device kx, ky (free-space step)
    std::vector<float> kx, kx2, ky, ky2;
    std::vector<float2> propx, propy;
    int band_p = 0, band_q = 0;  // in-band columns: iy <= band_p or iy >= band_q
};

// msk_calculate's last grid and the atomic numbers of its tables.
struct CalcCache {
    std::vector<float> key;
    std::vector<int> zlist;
    GridPre gp;
    const void *tables = nullptr;
};

static bool grid_pre(GridPre &gp, int nx, int ny, float ax, float by, float v0, float deltaz,
                     float ctiltx, float ctilty)
{
    gp.nx = nx;
    gp.ny = ny;
    gp.ax = ax;
    gp.by = by;
    gp.v0 = v0;
    gp.wavlen = (float)phys::wavelength(v0);
    gp.kx.resize(nx);
    gp.kx2.resize(nx);
    gp.ky.resize(ny);
    gp.ky2.resize(ny);
    std::vector<float> xp(std::max(nx, ny));
    phys::freqn(gp.kx.data(), gp.kx2.data(), xp.data(), nx, ax);
    phys::freqn(gp.ky.data(), gp.ky2.data(), xp.data(), ny, by);
    // autoslic.cpp:383-393
    const float BW = 2.0F / 3.0F;
    float k2max = nx / (2.0F * ax);
    float tctx = ny / (2.0F * by);
    if (tctx < k2max) k2max = tctx;
    k2max = BW * k2max;
    gp.k2max = k2max * k2max;
    // autoslic.cpp:395-414
    tctx = (float)(2.0 * tan(ctiltx));
    const float tcty = (float)(2.0 * tan(ctilty));
    const float pi = (float)(4.0 * atan(1.0));
    const float scale = pi * deltaz;
    gp.propx.resize(nx);
    gp.propy.resize(ny);
    for (int ix = 0; ix < nx; ix++) {
        const double t = scale * (gp.kx2[ix] * gp.wavlen - gp.kx[ix] * tctx);
        // with the propagator pass's 1/nx (a power of two: exact)
        gp.propx[ix] = make_float2((float)cos(t) / (float)nx, (float)-sin(t) / (float)nx);
    }
    for (int iy = 0; iy < ny; iy++) {
        const double t = scale * (gp.ky2[iy] * gp.wavlen - gp.ky[iy] * tcty);
        gp.propy[iy] = make_float2((float)cos(t), (float)-sin(t));
    }
    // Band limit as index ranges per column: freqn's kx2 rises on [0, imid]
    // and falls on (imid, nx), and a float sum is monotone in each term, so
    // the pixels kept by kx2[ix] + ky2[iy] < k2max (autoslic.cpp:1004,
    // slicelib.cpp:827-829) are ix <= A or ix >= B.  Checked element by element.
    gp.kband.resize(ny);
    for (int iy = 0; iy < ny; iy++) {
        int A = -1, B = nx;
        for (int ix = 0; ix < nx; ix++)
            if (gp.ky2[iy] + gp.kx2[ix] < gp.k2max) {
                if (B == nx && (A == ix - 1)) A = ix;
            }
        for (int ix = nx - 1; ix > A; ix--)
            if (gp.ky2[iy] + gp.kx2[ix] < gp.k2max) B = ix;
            else break;
        for (int ix = 0; ix < nx; ix++) {
            const bool keep = gp.ky2[iy] + gp.kx2[ix] < gp.k2max;
            const bool prop = gp.kx2[ix] < gp.k2max && (gp.kx2[ix] + gp.ky2[iy]) < gp.k2max;
            if (keep != (ix <= A || ix >= B) || prop != keep) return false;
        }
        gp.kband[iy] = make_int2(A, B);
    }
    // whole columns outside the band (ky2 >= k2max): iy in (band_p, band_q)
    {
        int p = -1, q = ny;
        while (p + 1 < ny && gp.kband[p + 1].x >= 0) p++;
        while (q - 1 > p && gp.kband[q - 1].x >= 0) q--;
        for (int iy = p + 1; iy < q; iy++)
            if (gp.kband[iy].x >= 0) {  // in-band columns not of that shape: no skipping
                p = ny - 1;
                q = ny;
                break;
            }
        gp.band_p = p;
        gp.band_q = q;
    }
    // trlayer constants (autoslic.cpp:927-941)
    gp.sigma = phys::sigma(v0) / 1000.0;
    gp.scalex = ax / nx;  // float division, as the reference
    gp.scaley = by / ny;
    double rmin = ax / ((double)nx);
    const double r = by / ((double)ny);
    rmin = 0.25 * sqrt(0.5 * (rmin * rmin + r * r));
    Geom &g = gp.g;
    g = Geom{};
    g.nx = nx;
    g.ny = ny;
    g.k2max = gp.k2max;
    g.inv_n = 1.0f / ((float)nx * (float)ny);
    g.sigma_f = (float)gp.sigma;
    g.scalex_f = (float)gp.scalex;
    g.scaley_f = (float)gp.scaley;
    g.rminsq = (float)(rmin * rmin);
    g.idx = (int)(nx * 3.0 / ax) + 1;
    g.idy = (int)(ny * 3.0 / by) + 1;
    // column blocks of the column passes (C columns each) holding in-band columns
    g.band_p = gp.band_p;
    g.band_q = gp.band_q;
    for (int v = 0; v < kColVariants; v++) {
        const int C = size_ops(nx)->col_c[v], nblk = ny / C;
        g.cb_lo[v] = std::min(nblk, (gp.band_p + 1 + C - 1) / C);
        g.cb_hi0[v] = std::max(g.cb_lo[v], gp.band_q / C);
        g.cb_n[v] = g.cb_lo[v] + (nblk - g.cb_hi0[v]);
    }
    g.seg_e1 = std::min(ny, (gp.band_p + 2) & ~1);
    g.seg_s2 = std::max(g.seg_e1, gp.band_q & ~1);
    return true;
}

// Stockham stage twiddles for line length n, matching FftPlan<n, ev>: per
// stage of radix R entered by sub-transforms of size NS, w(r, j) = exp(2 pi i
// r j / (NS R)) for r = 1..R-1, stored in pairs -- float2 index 2 (p NS + j) +
// q holds w(2p + 1 + q, j), so one 16-byte load fetches the twiddles of r =
// 2p+1 and 2p+2 (the pair of r = R-1 is padded with 1).  Computed in double.
template <int N, int EV>
static void twiddles_n(std::vector<float2> &out)
{
    using P = FftPlan<N, EV>;
    out.assign(std::max(P::TWN, 2), make_float2(1.0f, 0.0f));
    const double twopi = 8.0 * atan(1.0);
    auto fill = [&](int off, int ns, int r_) {
        for (int r = 1; r < r_; r++)
            for (int j = 0; j < ns; j++) {
                const double a = twopi * (double)r * (double)j / (double)(ns * r_);
                const int pr = (r - 1) / 2, q = (r - 1) % 2;
                out[off + 2 * (pr * ns + j) + q] = make_float2((float)cos(a), (float)sin(a));
            }
    };
    if (P::S >= 2) fill(0, P::NS2, P::R2);
    if (P::S == 3) fill(P::TW2, P::NS3, P::R3);
}

bool twiddles(int n, std::vector<float2> &out, int ev)
{
    if (ev == 16) {
        switch (n) {
        case 16: twiddles_n<16, 16>(out); return true;
        case 32: twiddles_n<32, 16>(out); return true;
        case 64: twiddles_n<64, 16>(out); return true;
        case 128: twiddles_n<128, 16>(out); return true;
        case 256: twiddles_n<256, 16>(out); return true;
        case 512: twiddles_n<512, 16>(out); return true;
        case 1024: twiddles_n<1024, 16>(out); return true;
        case 2048: twiddles_n<2048, 16>(out); return true;
        default: return false;
        }
    }
    switch (n) {
    case 16: twiddles_n<16, 0>(out); return true;
    case 32: twiddles_n<32, 0>(out); return true;
    case 64: twiddles_n<64, 0>(out); return true;
    case 128: twiddles_n<128, 0>(out); return true;
    case 256: twiddles_n<256, 0>(out); return true;
    case 512: twiddles_n<512, 0>(out); return true;
    case 1024: twiddles_n<1024, 0>(out); return true;
    case 2048: twiddles_n<2048, 0>(out); return true;
    case 4096: twiddles_n<4096, 0>(out); return true;
    default: return false;
    }
}

// One orientation/configuration ready for the splat: atoms inside the box,
// sorted by z, grouped by slice, positions relative to their pixel.
struct UnitAtoms {
    std::vector<SplatAtom> atoms;
    std::vector<int> counts;  // per slice
    std::vector<float> dw;    // Debye-Waller branch: -B/4 per slice
    int kept = 0;
    int status = MSK_OK;
};

// This library's gasdev: the reference draws its thermal displacements with
// gasdev from the XArrayLibrary (autoslic.cpp:707-709), which is not part of
// the reference.  Two steps of the 64-bit LCG (6364136223846793005,
// 1442695040888963407) on the seed, Box-Muller from the top 53 bits.
static double gasdev(long *idum)
{
    uint64_t s = (uint64_t)(*idum) * 6364136223846793005ULL + 1442695040888963407ULL;
    uint64_t s2 = s * 6364136223846793005ULL + 1442695040888963407ULL;
    *idum = (long)s2;
    double u1 = ((s >> 11) + 1.0) / 9007199254740993.0;
    double u2 = (s2 >> 11) / 9007199254740992.0;
    return sqrt(-2.0 * log(u1)) * cos(8.0 * atan(1.0) * u2);
}

enum { kThermNone = 0, kThermDW = 1, kThermRandom = 2 };

struct PrepSpec {
    int natom;
    const int *Znum;
    const float *x, *y, *z, *occ;
    float ctblength, ctblengthz, deltaz;
    int nslices;
    bool rotate;
    double angZ, angY, dxc, dyc, dzc;
    const float *disp;  // [3][natom] or null
    bool drop_outside;
    const int *zmap;    // Z -> compact index
    // thermal branches of calculate (lwobble = 1): kThermDW (nwobble 1) or
    // kThermRandom (nwobble > 1, displacements drawn from *iseed)
    int thermal = kThermNone;
    const float *wobble = nullptr;  // rms displacement at 300 K per atom
    float temperature = 0.0f;
    long *iseed = nullptr;
};

static void prep_unit(const GridPre &gp, const PrepSpec &ps, UnitAtoms &out)
{
    const int n0 = ps.natom;
    std::vector<float> x(ps.x, ps.x + n0), y(ps.y, ps.y + n0), z(ps.z, ps.z + n0),
        occ(ps.occ, ps.occ + n0);
    std::vector<int> Z(ps.Znum, ps.Znum + n0);
    std::vector<float> wob;
    if (ps.thermal != kThermNone) wob.assign(ps.wobble, ps.wobble + n0);
    if (ps.rotate)
        rotate(ps.ctblength, ps.dxc, ps.dyc, ps.dzc, ps.angZ, ps.angY, n0, x.data(), y.data(),
               z.data());
    if (ps.disp) {
        for (int k = 0; k < n0; k++) {
            x[k] += ps.disp[k];
            y[k] += ps.disp[n0 + k];
            z[k] += ps.disp[2 * n0 + k];
        }
    }
    int n = n0;
    if (ps.drop_outside) {
        n = 0;
        for (int k = 0; k < n0; k++) {
            if (x[k] < 0 || x[k] > ps.ctblength || y[k] < 0 || y[k] > ps.ctblength || z[k] < 0 ||
                z[k] > ps.ctblengthz)
                continue;
            x[n] = x[k];
            y[n] = y[k];
            z[n] = z[k];
            occ[n] = occ[k];
            Z[n] = Z[k];
            if (!wob.empty()) wob[n] = wob[k];  // autosliccmd.cpp:806-818 keeps wobble along
            n++;
        }
    } else if (n > 0) {
        // the reference's range checks (autoslic.cpp:270-299)
        float xmin = x[0], xmax = x[0], ymin = y[0], ymax = y[0], zmin = z[0], zmax = z[0];
        for (int i = 0; i < n; i++) {
            xmin = std::min(xmin, x[i]);
            xmax = std::max(xmax, x[i]);
            ymin = std::min(ymin, y[i]);
            ymax = std::max(ymax, y[i]);
            zmin = std::min(zmin, z[i]);
            zmax = std::max(zmax, z[i]);
        }
        if (xmin < 0 || ymin < 0 || zmin < 0 || xmax > ps.ctblength || ymax > ps.ctblength ||
            zmax > ps.ctblengthz) {
            out.status = MSK_EBOX;
            return;
        }
    }
    for (int i = 0; i < n; i++)
        if (Z[i] < 1 || Z[i] > 103) {
            out.status = MSK_EZNUM;
            return;
        }
    if (ps.thermal == kThermRandom) {  // autoslic.cpp:701-713, before the sort
        const float scale = (float)sqrt(ps.temperature / 300.0);
        for (int i = 0; i < n; i++) {
            x[i] = x[i] + (float)(wob[i] * gasdev(ps.iseed) * scale);
            y[i] = y[i] + (float)(wob[i] * gasdev(ps.iseed) * scale);
            z[i] = z[i] + (float)(wob[i] * gasdev(ps.iseed) * scale);
        }
    }
    sort_by_z(x.data(), y.data(), z.data(), occ.data(), Z.data(), n);
    if (n > 0 && (z[0] < 0 || z[n - 1] > ps.ctblengthz)) {  // autoslic.cpp:734-739
        out.status = MSK_EZSORT;
        return;
    }
    out.counts.assign(ps.nslices, 0);
    slice_counts(ps.deltaz, ps.ctblengthz, n, z.data(), ps.nslices, out.counts.data());
    int used = 0;
    for (int s = 0; s < ps.nslices; s++) used += out.counts[s];
    if (ps.thermal == kThermDW) {
        // trlayerDW's B for a slice of na atoms (autoslic.cpp:1049-1056): the
        // mean over wobble[0 .. na-1] of the caller's (unsorted) order
        const double twopi = 2.0 * (4.0 * atan(1.0));
        const double scaleTemp2 = ps.temperature / 300.0;
        std::vector<double> pre(n + 1, 0.0);
        for (int i = 0; i < n; i++) pre[i + 1] = pre[i] + wob[i] * wob[i] * scaleTemp2;
        out.dw.assign(ps.nslices, 0.0f);
        for (int s = 0; s < ps.nslices; s++) {
            const int na = out.counts[s];
            if (na == 0) continue;
            double Bdw = pre[na];
            Bdw /= na;
            Bdw *= 2.0 * twopi * twopi;
            out.dw[s] = (float)(-0.25 * Bdw);
        }
    }
    out.atoms.resize(used);
    for (int i = 0; i < used; i++) {
        // trlayer's pixel of the atom (autoslic.cpp:952-953) and the offset
        // of the atom from it, in double
        const int ixo = (int)(x[i] / gp.scalex), iyo = (int)(y[i] / gp.scaley);
        SplatAtom a;
        a.fx = (float)((double)x[i] - (double)ixo * gp.scalex);
        a.fy = (float)((double)y[i] - (double)iyo * gp.scaley);
        a.occ = occ[i];
        a.meta = (uint32_t)ixo | ((uint32_t)iyo << kMetaBits) |
                 ((uint32_t)ps.zmap[Z[i]] << (2 * kMetaBits));
        out.atoms[i] = a;
    }
    out.kept = n;
    out.status = MSK_OK;
}

static void parallel_for(int n, int nthreads, const std::function<void(int)> &fn)
{
    nthreads = std::max(1, std::min(nthreads, n));
    if (nthreads == 1) {
        for (int i = 0; i < n; i++) fn(i);
        return;
    }
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&] {
            for (;;) {
                const int i = next.fetch_add(1);
                if (i >= n) break;
                fn(i);
            }
        });
    for (auto &t : th) t.join();
}

static int host_threads()
{
    const unsigned hc = std::thread::hardware_concurrency();
    return hc ? (int)hc : 4;
}

}  // namespace msk

// Spherical incident wave of MsctKirkland (autosliccmd.cpp:650-689): a point
// source R1 before the box centre, defined on the entrance surface (R1in =
// R1 - ctblength/2): amplitude 1/sqrt(1 + r^2/R1in^2), phase
// 2 pi/lambda sqrt(r^2 + R1in^2) - the phase at the grid corner, r measured
// from pixel (nx/2, ny/2); values computed in double, stored as float.
static void spherical_wave(int nx, int ny, float ctblength, float v0, double R1,
                           std::vector<float2> &w)
{
    const double pi = 4.0 * atan(1.0);
    const double R1in = R1 - 0.5 * ctblength;
    const double R12 = R1in * R1in, aR12 = 1.0 / R12;
    const double tPIdlambda = 2.0 * pi / msk::phys::wavelength(v0);
    const double xst = ctblength / nx, yst = ctblength / ny;  // float divisions
    const int nx2 = nx / 2, ny2 = ny / 2;
    const double phamax =
        tPIdlambda * sqrt(xst * xst * nx2 * nx2 + yst * yst * ny2 * ny2 + R12);
    w.resize((size_t)nx * ny);
    for (int j = 0; j < ny; j++) {
        double yy = double(j - ny2) * yst;
        yy *= yy;
        const double yyR12 = yy + R12;
        for (int i = 0; i < nx; i++) {
            double xx = double(i - nx2) * xst;
            xx *= xx;
            const float amp = float(1.0 / sqrt(1.0 + (xx + yy) * aR12));
            xx += yyR12;
            const float pha = float(tPIdlambda * sqrt(xx) - phamax);
            w[(size_t)i * ny + j] = make_float2(float(amp * cos((double)pha)),
                                                float(amp * sin((double)pha)));
        }
    }
}

// ------------------------------------------------------------------ context

using namespace msk;

namespace msk {
std::atomic<long long> g_device_allocs{0};
thread_local bool t_no_alloc = false;

const char *const kKindName[kKinds] = {
    "row_splat", "col_bandlimit", "row_transmit", "col_propagate", "col_fresnel",
    "row_intensity", "row_exit", "row_init", "plane_init", "fresnel_table",
    "row_expv", "row_adj_transmit", "row_grad", "row_imgrad", "accumulate", "col_debye_waller",
    "row_dw_phase", "image_rotate_shift",
    "utr_image_rows", "utr_image_cols", "utr_grid", "utr_fourier_rows", "utr_volume_cols",
    "utr_final_cols", "utr_pointwise", "copy_images_d2h", "small_slices"};
}  // namespace msk

namespace msk {

int fail(msk_context *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->err = msg;
    return code;
}

bool pow2_supported(int n) { return size_ops(n) != nullptr; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// 2D view of a wave buffer for the column passes of tile variant v: rows =
// units * nx, each row ny complex64 = 2*ny floats; box = the variant's
// column tile.
int column_map(msk_context *ctx, ColView *view, void *base, int nx, int ny, size_t units,
               const SizeOps *cop, int v)
{
    if (v < 0 || v >= cop->col_nv) return fail(ctx, MSK_EINVAL, "no column-pass variant " + std::to_string(v));
    auto enc = tensor_map_encoder();
    if (!enc) return fail(ctx, MSK_ECUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[2] = {(cuuint64_t)2 * ny, (cuuint64_t)units * nx};
    const cuuint64_t strides[1] = {(cuuint64_t)ny * 8};
    const cuuint32_t box[2] = {(cuuint32_t)(2 * cop->col_c[v]), (cuuint32_t)cop->col_box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&view->map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box,
                     estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(ctx, MSK_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    view->v = v;
    return MSK_OK;
}

// Device error flags: cleared at the start of a call, read after its last
// synchronisation (a bounded wait in a kernel that gave up sets a bit).
// The same buffer holds, after 256 bytes, kZeroBytes of zeros: the source
// the row passes fill out-of-band row segments from.
constexpr size_t kZeroBytes = 4096 * sizeof(float2);
constexpr size_t kFlagBytes = 256 + kZeroBytes;

int flags_reset(msk_context *ctx, Geom &g)
{
    if (ctx->flags.cap < kFlagBytes) {
        MSK_CUDA(ctx, ctx->flags.reserve(kFlagBytes));
        MSK_CUDA(ctx, cudaMemsetAsync(ctx->flags.p, 0, kFlagBytes, ctx->stream));
    }
    MSK_CUDA(ctx, cudaMemsetAsync(ctx->flags.p, 0, sizeof(int), ctx->stream));
    g.err = ctx->flags.as<int>();
    g.zeros = reinterpret_cast<const float2 *>(ctx->flags.as<unsigned char>() + 256);
    return MSK_OK;
}

int flags_check(msk_context *ctx)
{
    int h = 0;
    MSK_CUDA(ctx, cudaMemcpyAsync(&h, ctx->flags.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h) return fail(ctx, MSK_ECUDA, "a kernel's bounded wait for its copies timed out");
    return MSK_OK;
}

// Host<->device copy accounting (dir 0: to the device, 1: to the host).
void count_copy(msk_context *ctx, int dir, double bytes)
{
    if (!ctx->prof_on) return;
    ctx->copies[dir] += 1;
    ctx->copy_bytes[dir] += bytes;
}

// After a stream synchronisation: fold the recorded events into the totals.
void prof_collect(msk_context *ctx)
{
    for (const ProfRec &r : ctx->prof_pending) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            ctx->prof_ms[r.kind] += ms;
            ctx->prof_launches[r.kind] += 1;
            ctx->prof_bytes[r.kind] += r.bytes;
        }
        ctx->prof_pool.push_back(r.a);
        ctx->prof_pool.push_back(r.b);
    }
    ctx->prof_pending.clear();
}

}  // namespace msk

namespace {

// Times launch(v) for the variants v in [0, nv): two warm-up launches of every
// variant, then kTuneRounds rounds in which every variant runs once between two
// events, the order rotating from round to round; ms[v] = the variant's fastest
// launch.  Interleaving the variants keeps a clock that is still rising (the
// first launches of a process) from favouring whichever variant runs last.
template <typename F>
bool time_variants(cudaStream_t s, int nv, F launch, float *ms)
{
    constexpr int kTuneRounds = 5;
    std::vector<cudaEvent_t> ev((size_t)2 * nv * kTuneRounds, nullptr);
    bool ok = true;
    for (auto &e : ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    for (int w = 0; w < 2 && ok; w++)
        for (int v = 0; v < nv; v++) launch(v);
    for (int r = 0; r < kTuneRounds && ok; r++)
        for (int i = 0; i < nv && ok; i++) {
            const int v = (i + r) % nv;
            cudaEvent_t *e = &ev[(size_t)2 * (r * nv + v)];
            ok = cudaEventRecord(e[0], s) == cudaSuccess;
            launch(v);
            ok = ok && cudaEventRecord(e[1], s) == cudaSuccess;
        }
    ok = ok && cudaStreamSynchronize(s) == cudaSuccess && cudaGetLastError() == cudaSuccess;
    for (int v = 0; v < nv; v++) {
        ms[v] = 3.0e38f;
        for (int r = 0; r < kTuneRounds && ok; r++) {
            float t = 0.0f;
            ok = cudaEventElapsedTime(&t, ev[(size_t)2 * (r * nv + v)],
                                      ev[(size_t)2 * (r * nv + v) + 1]) == cudaSuccess;
            ms[v] = std::min(ms[v], t);
        }
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    return ok;
}

// The schedule of each column pass (ColCfg variant: FFT plan and tile width),
// per device, grid and pass, in the manner of FFTW_MEASURE planning
// (TemsimLibrary/cfpix.cpp:225-228): the first time a pass runs on a grid,
// every variant with kernels for the line length -- 32 and (64 to 2048 points)
// 16 points a thread, each at two tile widths -- runs on a scratch grid
// (time_variants) and the fastest is kept for the life of the process (the
// default unless another gains 3%).  Tile widths compute
// every column identically; the plans differ by FP32 rounding.  MSK_COL_TILE=
// 0..3 in the environment fixes the variant (0, 1: 32 points, 2, 3: 16).
struct ColChoices {
    std::mutex m;
    std::map<std::array<int, 4>, int> v;  // (device, nx, ny, pass) -> variant
};
ColChoices &col_choices()
{
    static ColChoices c;
    return c;
}

int col_variant(msk_context *ctx, const GridPre &gp, int mode)
{
    if (ctx->no_tune) return 0;
    const SizeOps *cop = size_ops(gp.nx);
    const std::array<int, 4> key = {ctx->device, gp.nx, gp.ny, mode};
    ColChoices &cc = col_choices();
    std::lock_guard<std::mutex> lock(cc.m);
    const char *forced = getenv("MSK_COL_TILE");
    if (forced && forced[0] >= '0' && forced[0] < '0' + cop->col_nv && forced[1] == 0)
        return cc.v[key] = forced[0] - '0';  // recorded, so msk_column_plan reports it
    auto it = cc.v.find(key);
    if (it != cc.v.end()) return it->second;
    const size_t plane = (size_t)gp.nx * gp.ny;
    const int U = (int)std::max<size_t>(2, std::min<size_t>(64, ((size_t)256 << 20) / (plane * 8)));
    int choice = 0;
    float ms[kColVariants] = {};
    bool ok = ctx->tune.reserve((size_t)(U + 1) * plane * sizeof(float2)) == cudaSuccess &&
              cudaMemsetAsync(ctx->tune.p, 0, (size_t)(U + 1) * plane * sizeof(float2),
                              ctx->stream) == cudaSuccess;
    float2 *grid = ctx->tune.as<float2>();
    Fresnel fr{};
    fr.table = grid + (size_t)U * plane;  // zeros
    fr.dw = reinterpret_cast<const float *>(grid + (size_t)U * plane);
    fr.dw_stride = 1;
    const Geom &g = gp.g;
    ColView views[kColVariants];
    for (int v = 0; v < cop->col_nv && ok; v++)
        ok = column_map(ctx, &views[v], grid, gp.nx, gp.ny, U, cop, v) == MSK_OK;
    auto launch = [&](int v) {
        const ColView &view = views[v];
        switch (mode) {
        case kColMask: cop->col_mask(g, view, view, nullptr, U, 1, 1.0f, ctx->stream); break;
        case kColProp: cop->col_prop(g, view, view, nullptr, U, 1, ctx->stream); break;
        case kColFresnel: cop->col_fresnel(g, view, view, nullptr, U, fr, 1.0f, ctx->stream); break;
        default: cop->col_dw(g, view, nullptr, U, fr.dw, 1, ctx->stream); break;
        }
    };
    ok = ok && time_variants(ctx->stream, cop->col_nv, launch, ms);
    // the fastest variant, unless it gains less than 3% on the default
    for (int v = 1; ok && v < cop->col_nv; v++)
        if (ms[v] < 0.97f * ms[0] && ms[v] < ms[choice]) choice = v;
    if (!ok) cudaGetLastError();
    cc.v[key] = choice;
    return choice;
}

// The transmit's schedule (TrCfg: the FFT plan, 32 or, for 64 to 2048 points,
// 16 points a thread, and the CTA width), chosen per device and grid the way
// the column passes' is: the first time the transmit runs on a grid every
// schedule runs on a scratch grid (time_variants) and the fastest is kept for
// the process (the default unless another gains 3%).  The two widths of one plan compute every row
// identically; the plans differ by FP32 rounding (another radix split of the
// same transforms).  MSK_ROW_PLAN=0..2 in the environment fixes it.  The wave
// and scattered forms share it.
struct RowChoices {
    std::mutex m;
    std::map<std::array<int, 3>, int> v;  // (device, nx, ny) -> variant
};
RowChoices &row_choices()
{
    static RowChoices c;
    return c;
}

int row_variant(msk_context *ctx, const GridPre &gp)
{
    if (ctx->no_tune) return 0;
    const SizeOps *rop = size_ops(gp.ny);
    const std::array<int, 3> key = {ctx->device, gp.nx, gp.ny};
    RowChoices &rc = row_choices();
    std::lock_guard<std::mutex> lock(rc.m);
    const char *forced = getenv("MSK_ROW_PLAN");
    if (forced && forced[0] >= '0' && forced[0] < '0' + rop->row_nv && forced[1] == 0)
        return rc.v[key] = forced[0] - '0';  // recorded, so msk_row_plan reports it
    auto it = rc.v.find(key);
    if (it != rc.v.end()) return it->second;
    if (rop->row_nv < 2) return rc.v[key] = 0;
    const size_t plane = (size_t)gp.nx * gp.ny;
    const int U = (int)std::max<size_t>(2, std::min<size_t>(32, ((size_t)128 << 20) / (plane * 8)));
    int choice = 0;
    float ms[kRowVariants] = {};
    bool ok = ctx->tune.reserve((size_t)2 * U * plane * sizeof(float2)) == cudaSuccess &&
              cudaMemsetAsync(ctx->tune.p, 0, (size_t)2 * U * plane * sizeof(float2),
                              ctx->stream) == cudaSuccess;
    float2 *tb = ctx->tune.as<float2>(), *psi = tb + (size_t)U * plane;
    auto launch = [&](int v) {
        rop->row_transmit(gp.g, nullptr, U, tb, psi, psi, 1.0f, 1, v, ctx->stream);
    };
    ok = ok && time_variants(ctx->stream, rop->row_nv, launch, ms);
    for (int v = 1; ok && v < rop->row_nv; v++)
        if (ms[v] < 0.97f * ms[0] && ms[v] < ms[choice]) choice = v;
    if (!ok) cudaGetLastError();
    rc.v[key] = choice;
    return choice;
}

// Device tables of one grid (frequency grids, propagator, twiddles, potential
// spline, band-limit ranges) laid out in one block of 256-byte aligned pieces.
struct TableLayout {
    size_t kx2, ky2, kx, ky, px, py, twr, twc, twr16, twc16, kn, cf, kb, bytes;
    size_t n_twr, n_twc, n_twr16, n_twc16;  // twiddle counts (float2)
};

// Offsets (256-byte aligned pieces) of the grid tables of an nx x ny grid with
// nz compact atomic numbers; the 16-point-plan twiddles only for lines of
// <= 2048 points.  The one formula behind the table upload and the fixed
// scratch of msk_calculate_static.
TableLayout layout_tables(int nx, int ny, int nz)
{
    TableLayout o{};
    std::vector<float2> t;
    twiddles(ny, t);
    o.n_twr = t.size();
    twiddles(nx, t);
    o.n_twc = t.size();
    o.n_twr16 = twiddles(ny, t, 16) ? t.size() : 0;
    o.n_twc16 = twiddles(nx, t, 16) ? t.size() : 0;
    size_t off = 0;
    auto piece = [&](size_t bytes) {
        size_t q = off;
        off += (bytes + 255) & ~size_t(255);
        return q;
    };
    o.kx2 = piece(4 * (size_t)nx);
    o.ky2 = piece(4 * (size_t)ny);
    o.kx = piece(4 * (size_t)nx);
    o.ky = piece(4 * (size_t)ny);
    o.px = piece(8 * (size_t)nx);
    o.py = piece(8 * (size_t)ny);
    o.twr = piece(8 * o.n_twr);
    o.twc = piece(8 * o.n_twc);
    o.twr16 = piece(8 * o.n_twr16);
    o.twc16 = piece(8 * o.n_twc16);
    o.kn = piece(4 * (size_t)kKnotWords);
    o.cf = piece(16 * (size_t)std::max(nz, 1) * phys::kN);
    o.kb = piece(8 * (size_t)ny);
    o.bytes = off;
    return o;
}

static void build_tables(const GridPre &gp, const std::vector<int> &zlist,
                         std::vector<unsigned char> &host, TableLayout &o)
{
    std::vector<float2> twr, twc, twr16, twc16;
    twiddles(gp.ny, twr);
    twiddles(gp.nx, twc);
    twiddles(gp.ny, twr16, 16);
    twiddles(gp.nx, twc16, 16);
    const int nz = (int)zlist.size();
    auto &L = phys::lut();
    for (int Z : zlist) L.build(Z);
    // the knot piece: the knots, then spline_vz's interval per bucket of r^2
    std::vector<float> knots(kKnotWords, 0.0f);
    for (int i = 0; i < phys::kN; i++) knots[i] = (float)L.knots[i];
    unsigned char *bucket = reinterpret_cast<unsigned char *>(knots.data() + 128);
    for (int bi = 0; bi < kKnotBuckets; bi++) {
        // the last knot at or below the bucket's start; the knots being 13%
        // apart, the bucket holds at most the next one
        float lo;
        const uint32_t blo = (uint32_t)(kKnotBucketBase + bi) << kKnotBucketShift;
        std::memcpy(&lo, &blo, 4);
        int i0 = 0;
        while (i0 < phys::kN - 2 && knots[i0 + 1] <= lo) i0++;
        bucket[bi] = (unsigned char)i0;
    }
    std::vector<float4> coef((size_t)std::max(nz, 1) * phys::kN);
    for (int zi = 0; zi < nz; zi++) {
        const int Z = zlist[zi];
        for (int i = 0; i < phys::kN; i++)
            coef[(size_t)zi * phys::kN + i] = make_float4((float)L.y[Z][i], (float)L.b[Z][i],
                                                          (float)L.c[Z][i], (float)L.d[Z][i]);
    }
    o = layout_tables(gp.nx, gp.ny, nz);
    host.assign(o.bytes, 0);
    std::memcpy(&host[o.kx2], gp.kx2.data(), 4 * gp.nx);
    std::memcpy(&host[o.ky2], gp.ky2.data(), 4 * gp.ny);
    std::memcpy(&host[o.kx], gp.kx.data(), 4 * gp.nx);
    std::memcpy(&host[o.ky], gp.ky.data(), 4 * gp.ny);
    std::memcpy(&host[o.px], gp.propx.data(), 8 * gp.nx);
    std::memcpy(&host[o.py], gp.propy.data(), 8 * gp.ny);
    std::memcpy(&host[o.twr], twr.data(), 8 * twr.size());
    std::memcpy(&host[o.twc], twc.data(), 8 * twc.size());
    if (o.n_twr16) std::memcpy(&host[o.twr16], twr16.data(), 8 * twr16.size());
    if (o.n_twc16) std::memcpy(&host[o.twc16], twc16.data(), 8 * twc16.size());
    std::memcpy(&host[o.kn], knots.data(), 4 * knots.size());
    std::memcpy(&host[o.cf], coef.data(), 16 * coef.size());
    std::memcpy(&host[o.kb], gp.kband.data(), 8 * gp.ny);
}

// Point the grid's Geom (and kx, ky for the free-space step) at a device copy
// of its table block.
static void bind_tables(GridPre &gp, const unsigned char *b, const TableLayout &o)
{
    Geom &g = gp.g;
    g.kx2 = reinterpret_cast<const float *>(b + o.kx2);
    g.ky2 = reinterpret_cast<const float *>(b + o.ky2);
    g.propx = reinterpret_cast<const float2 *>(b + o.px);
    g.propy = reinterpret_cast<const float2 *>(b + o.py);
    g.tw_row = reinterpret_cast<const float2 *>(b + o.twr);
    g.tw_col = reinterpret_cast<const float2 *>(b + o.twc);
    g.tw_row16 = o.n_twr16 ? reinterpret_cast<const float2 *>(b + o.twr16) : nullptr;
    g.tw_col16 = o.n_twc16 ? reinterpret_cast<const float2 *>(b + o.twc16) : nullptr;
    g.knots = reinterpret_cast<const float *>(b + o.kn);
    g.coef = reinterpret_cast<const float4 *>(b + o.cf);
    g.kband = reinterpret_cast<const int2 *>(b + o.kb);
    gp.d_kx = reinterpret_cast<const float *>(b + o.kx);
    gp.d_ky = reinterpret_cast<const float *>(b + o.ky);
}

// Tables of one grid into the context's table buffer.
int upload_tables(msk_context *ctx, GridPre &gp, const std::vector<int> &zlist)
{
    ctx->calc_cache.reset();  // the tables msk_calculate cached are replaced
    std::vector<unsigned char> host;
    TableLayout o;
    build_tables(gp, zlist, host, o);
    MSK_CUDA(ctx, ctx->tables.reserve(o.bytes));
    MSK_CUDA(ctx, cudaMemcpyAsync(ctx->tables.p, host.data(), o.bytes, cudaMemcpyHostToDevice,
                                  ctx->stream));
    count_copy(ctx, 0, (double)o.bytes);
    // the host staging vector must outlive the copy
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    bind_tables(gp, ctx->tables.as<unsigned char>(), o);
    return MSK_OK;
}

// The grid of the previous call (msk_calculate, a tilt series or a potential
// stack), when it was made for the same grid parameters `key` and its tables
// are still the context's: gp from it, and the record (else null, gp untouched).
std::shared_ptr<CalcCache> grid_cached(msk_context *ctx, const std::vector<float> &key, GridPre &gp)
{
    auto cache = std::static_pointer_cast<CalcCache>(ctx->calc_cache);
    if (!cache || cache->key != key || cache->tables != ctx->tables.p) return nullptr;
    gp = cache->gp;
    return cache;
}

// The grid's tables on the device for the atomic numbers zlist: kept when `hit`
// (grid_cached) holds them for the same numbers -- no host build, upload or
// synchronisation -- else built, uploaded and recorded for the next call.
int grid_tables(msk_context *ctx, GridPre &gp, const std::vector<float> &key,
                const std::shared_ptr<CalcCache> &hit, const std::vector<int> &zlist)
{
    if (hit && hit->zlist == zlist) return MSK_OK;
    const int st = upload_tables(ctx, gp, zlist);
    if (st) return st;
    auto c = std::make_shared<CalcCache>();
    c->key = key;
    c->zlist = zlist;
    c->gp = gp;
    c->tables = ctx->tables.p;
    ctx->calc_cache = c;
    return MSK_OK;
}

const float *tables_kx(msk_context *, const GridPre &gp) { return gp.d_kx; }
const float *tables_ky(msk_context *, const GridPre &gp) { return gp.d_ky; }

}  // namespace

namespace msk {
bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked host memory (cudaHostAlloc / cudaHostRegister): a copy to it
// may be captured into a graph and runs asynchronously.
// The device address of page-locked host memory the GPU can address directly
// (mapped: over NVLink-C2C on a Grace host, PCIe elsewhere), or null.
void *mapped_host(void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

bool is_pinned_host(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}
}  // namespace msk

namespace {

// A batch of units (waves) with their atoms uploaded: the slice loop.
struct Batch {
    int nunits = 0, nslices = 0;
    // units of the whole call (0: this batch's): whether the small-grid path
    // runs is decided for the call, so a unit's result does not depend on
    // where the batches of the call are cut
    int call_units = 0;
    std::vector<int> slice_off;   // [nunits][nslices+1] absolute atom offsets
    std::vector<int> act_off;     // [nslices+1]
    std::vector<int> act;         // active units per slice
    std::vector<float> dw;        // Debye-Waller branch: [nunits][nslices] -B/4 (else empty)
};

// Per-slice atom offsets and active units per slice of units u0 ..
// u0+nunits-1 (and their Debye-Waller factors); returns the atom count.
size_t pack_batch_meta(const std::vector<UnitAtoms> &ua, int u0, int nunits, int nslices, Batch &b)
{
    b.nunits = nunits;
    b.nslices = nslices;
    const int nsl1 = nslices + 1;
    b.slice_off.assign((size_t)nunits * nsl1, 0);
    size_t total = 0;
    for (int i = 0; i < nunits; i++) {
        const UnitAtoms &u = ua[u0 + i];
        int o = (int)total;
        for (int s = 0; s < nslices; s++) {
            b.slice_off[(size_t)i * nsl1 + s] = o;
            o += u.counts[s];
        }
        b.slice_off[(size_t)i * nsl1 + nslices] = o;
        total = (size_t)o;
    }
    b.act_off.assign(nsl1, 0);
    b.act.clear();
    for (int s = 0; s < nslices; s++) {
        b.act_off[s] = (int)b.act.size();
        for (int i = 0; i < nunits; i++)
            if (ua[u0 + i].counts[s] > 0) b.act.push_back(i);
    }
    b.act_off[nslices] = (int)b.act.size();
    b.dw.clear();
    if (nunits > 0 && !ua[u0].dw.empty()) {
        b.dw.assign((size_t)nunits * nslices, 0.0f);
        for (int i = 0; i < nunits; i++)
            std::copy(ua[u0 + i].dw.begin(), ua[u0 + i].dw.end(), b.dw.begin() + (size_t)i * nslices);
    }
    return total;
}

// The packed atoms of the batch b describes (pack_batch_meta) into dst
// (max(total, 1) records), a unit at a time on `threads` host threads.
void pack_atoms(const std::vector<UnitAtoms> &ua, int u0, const Batch &b, SplatAtom *dst,
                int threads)
{
    const int nsl1 = b.nslices + 1;
    dst[0] = SplatAtom{};
    parallel_for(b.nunits, threads, [&](int i) {
        const auto &a = ua[u0 + i].atoms;
        std::copy(a.begin(), a.end(), dst + b.slice_off[(size_t)i * nsl1]);
    });
}

void pack_batch(const std::vector<UnitAtoms> &ua, int u0, int nunits, int nslices, Batch &b,
                std::vector<SplatAtom> &atoms)
{
    atoms.assign(std::max<size_t>(pack_batch_meta(ua, u0, nunits, nslices, b), 1), SplatAtom{});
    pack_atoms(ua, u0, b, atoms.data(), 1);  // (callers run one batch per host thread)
}

// Page-locked staging of at least `bytes` (grown by cudaHostAlloc; the copies
// out of the old one have finished when it is replaced: every upload ends
// with a stream synchronisation).  Null where the context allocates nothing.
void *host_stage(msk_context *ctx, size_t bytes)
{
    if (ctx->no_host_stage) return nullptr;
    if (ctx->h_stage_cap < bytes) {
        if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
        ctx->h_stage = nullptr;
        ctx->h_stage_cap = 0;
        const size_t cap = bytes + bytes / 4;
        if (cudaHostAlloc(&ctx->h_stage, cap, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            ctx->h_stage = nullptr;
            return nullptr;
        }
        ctx->h_stage_cap = cap;
    }
    return ctx->h_stage;
}

int upload_batch(msk_context *ctx, const std::vector<UnitAtoms> &ua, int u0, int nunits,
                 int nslices, Batch &b)
{
    const size_t na = std::max<size_t>(pack_batch_meta(ua, u0, nunits, nslices, b), 1);
    const size_t ab = na * sizeof(SplatAtom), ob = b.slice_off.size() * sizeof(int),
                 cb = b.act.size() * sizeof(int);
    MSK_CUDA(ctx, ctx->atoms.reserve(ab));
    MSK_CUDA(ctx, ctx->slice_off.reserve(ob));
    MSK_CUDA(ctx, ctx->act.reserve(std::max<size_t>(cb, sizeof(int))));
    // from page-locked staging when the context has it (the copies then run at
    // the link's rate right after the previous batch, instead of through the
    // driver's pageable bounce buffers with the GPU idle), else from vectors
    std::vector<SplatAtom> atoms;
    const SplatAtom *src_atoms;
    const int *src_off = b.slice_off.data(), *src_act = b.act.data();
    if (unsigned char *st = static_cast<unsigned char *>(host_stage(ctx, ab + ob + cb))) {
        SplatAtom *dst = reinterpret_cast<SplatAtom *>(st);
        pack_atoms(ua, u0, b, dst, host_threads());
        std::memcpy(st + ab, b.slice_off.data(), ob);
        if (cb) std::memcpy(st + ab + ob, b.act.data(), cb);
        src_atoms = dst;
        src_off = reinterpret_cast<const int *>(st + ab);
        src_act = reinterpret_cast<const int *>(st + ab + ob);
    } else {
        atoms.assign(na, SplatAtom{});
        pack_atoms(ua, u0, b, atoms.data(), host_threads());
        src_atoms = atoms.data();
    }
    MSK_CUDA(ctx, cudaMemcpyAsync(ctx->atoms.p, src_atoms, ab, cudaMemcpyHostToDevice, ctx->stream));
    count_copy(ctx, 0, (double)(ab + ob + cb));
    MSK_CUDA(ctx, cudaMemcpyAsync(ctx->slice_off.p, src_off, ob, cudaMemcpyHostToDevice, ctx->stream));
    if (cb)
        MSK_CUDA(ctx, cudaMemcpyAsync(ctx->act.p, src_act, cb, cudaMemcpyHostToDevice, ctx->stream));
    if (!b.dw.empty()) {
        MSK_CUDA(ctx, ctx->dwbuf.reserve(b.dw.size() * sizeof(float)));
        MSK_CUDA(ctx, cudaMemcpyAsync(ctx->dwbuf.p, b.dw.data(), b.dw.size() * sizeof(float),
                                      cudaMemcpyHostToDevice, ctx->stream));
        count_copy(ctx, 0, (double)(b.dw.size() * sizeof(float)));
    }
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MSK_OK;
}

// The slice loop over a batch: the psi buffer holds W0 = S(wave0) on entry
// and W = S(exit wave) on return.
//
// Two chains per slice: the transmission chain (P1 splat, P2 band limit) and
// the wave chain (P3 transmit, P4 propagate).  With two transmission buffers
// the transmission chain of the next non-empty slice runs on the context's
// stream while the wave chain of the current one runs on the second stream,
// so the compute-bound splat overlaps the memory-bound wave passes.  Events
// order P3 after its P2 and the reuse of a transmission buffer after the P3
// that read it.  With per-kernel profiling on, everything runs in order on
// one stream so that each launch is timed alone.
// Whether the slice loop of this grid runs as one cluster launch (msk_small.cuh):
// square grids of 64^2 to 256^2 in the coherent branch with two transmission
// buffers, on a device that fits the clusters.  MSK_SMALL_GRID=0 in the
// environment keeps the launch-per-pass loop (=1: the default).
// Only when the units fit in one wave of clusters: with more, the launch-per-pass
// loop keeps the whole GPU busy and is faster (64 orientations of a 256^2 specimen:
// 116k slice-steps/s in clusters against 188k in the loop), while a few units leave
// the loop's launches latency-bound (C1, one unit: 0.52 ms against ~1 ms).
static bool small_grid_ok(msk_context *ctx, const GridPre &gp, bool dw, int nmode, int nunits)
{
    const char *forced = getenv("MSK_SMALL_GRID");
    if (forced && forced[0] == '0') return false;
    const SizeOps *op = size_ops(gp.nx);
    return nmode == 0 && !dw && gp.nx == gp.ny && op && op->small_slices &&
           nunits <= op->small_ok(ctx->device);
}

static bool small_path(msk_context *ctx, const GridPre &gp, const Batch &b, int nmode)
{
    return ctx->tbuf2.cap >= ctx->tbuf.cap && ctx->tbuf.cap > 0 &&
           small_grid_ok(ctx, gp, !b.dw.empty(), nmode, std::max(b.nunits, b.call_units));
}

int run_slices(msk_context *ctx, const GridPre &gp, const Batch &b, int nmode, bool w_in_band)
{
    const SizeOps *rop = size_ops(gp.ny), *cop = size_ops(gp.nx);
    const Geom &g = gp.g;
    if (small_path(ctx, gp, b, nmode)) {
        // every slice of every unit in one launch; algorithmic bytes as the
        // passes count them (64 N per slice-step with atoms, 16 N without)
        const double plane = (double)gp.nx * gp.ny;
        const double ne = b.act_off[b.nslices], all = (double)b.nunits * b.nslices;
        Prof p(ctx, kSmall, plane * (64.0 * ne + 16.0 * (all - ne)));
        MSK_CUDA(ctx, cop->small_slices(g, b.nunits, b.nslices, b.nslices + 1,
                                        ctx->slice_off.as<int>(), ctx->atoms.as<SplatAtom>(),
                                        ctx->psi.as<float2>(), ctx->tbuf.as<float2>(),
                                        ctx->tbuf2.as<float2>(), ctx->stream));
        return MSK_OK;
    }
    // Debye-Waller branch: the second transmission buffer holds the potential's
    // spectrum, so the two slice chains run in order on one stream
    const bool dw = !b.dw.empty();
    if (dw && ctx->tbuf2.cap < ctx->tbuf.cap)
        return fail(ctx, MSK_EUNSUPPORTED, "the Debye-Waller branch needs a second buffer");
    const bool overlap = !dw && !ctx->prof_on && ctx->tbuf2.cap >= ctx->tbuf.cap;
    cudaStream_t sA = ctx->stream, sB = overlap ? ctx->aux : ctx->stream;
    float2 *psi = ctx->psi.as<float2>();
    float2 *tbs[2] = {ctx->tbuf.as<float2>(), overlap ? ctx->tbuf2.as<float2>() : ctx->tbuf.as<float2>()};
    const int *act = ctx->act.as<int>();
    const int nsl1 = b.nslices + 1;
    ColView tmaps[2], pmap;
    const int vm = col_variant(ctx, gp, kColMask), vp = col_variant(ctx, gp, kColProp);
    const int rv = row_variant(ctx, gp);
    int st = column_map(ctx, &tmaps[0], tbs[0], gp.nx, gp.ny, ctx->units_alloc, cop, vm);
    if (st) return st;
    st = column_map(ctx, &tmaps[1], tbs[1], gp.nx, gp.ny, ctx->units_alloc, cop, vm);
    if (st) return st;
    st = column_map(ctx, &pmap, psi, gp.nx, gp.ny, ctx->units_alloc, cop, vp);
    if (st) return st;
    ColView smap;
    if (dw) {
        st = column_map(ctx, &smap, ctx->tbuf2.p, gp.nx, gp.ny, ctx->units_alloc, cop,
                        col_variant(ctx, gp, kColDW));
        if (st) return st;
    }
    const double plane = (double)gp.nx * gp.ny;
    if (overlap) {
        MSK_CUDA(ctx, cudaEventRecord(ctx->ev_fork, sA));
        MSK_CUDA(ctx, cudaStreamWaitEvent(sB, ctx->ev_fork, 0));
    }
    bool pending_free[2] = {false, false};
    int uses = 0;
    for (int sl = 0; sl < b.nslices; sl++) {
        const int na = b.act_off[sl + 1] - b.act_off[sl];
        const int *units = act + b.act_off[sl];
        if (na > 0) {
            const int k = overlap ? (uses++ & 1) : 0;
            float2 *tb = tbs[k];
            if (overlap && pending_free[k]) MSK_CUDA(ctx, cudaStreamWaitEvent(sA, ctx->ev_free[k], 0));
            if (dw) {  // trlayerDW: S(v), damping, then A = S(exp(i sigma v'))
                float2 *spec = ctx->tbuf2.as<float2>();
                {
                    Prof p(ctx, kSplat, 8.0 * plane * na, sA);
                    rop->splat_spec(g, units, na, sl, nsl1, ctx->slice_off.as<int>(),
                                    ctx->atoms.as<SplatAtom>(), spec, sA);
                }
                {
                    Prof p(ctx, kDW, 16.0 * plane * na, sA);
                    cop->col_dw(g, smap, units, na, ctx->dwbuf.as<float>() + sl, b.nslices, sA);
                }
                Prof p(ctx, kDWExp, 16.0 * plane * na, sA);
                rop->row_dwexp(g, units, na, spec, tb, sA);
            } else {
                Prof p(ctx, kSplat, 8.0 * plane * na, sA);
                rop->splat(g, units, na, sl, nsl1, ctx->slice_off.as<int>(),
                           ctx->atoms.as<SplatAtom>(), tb, sA);
            }
            {
                Prof p(ctx, kKColMask, 16.0 * plane * na, sA);
                // B = S(t_bl) / ny^2: the transmit's 1/ny^2, exact, carried here
                cop->col_mask(g, tmaps[k], tmaps[k], units, na, 1,
                              1.0f / ((float)gp.ny * (float)gp.ny), sA);
            }
            if (overlap) {
                MSK_CUDA(ctx, cudaEventRecord(ctx->ev_t[k], sA));
                MSK_CUDA(ctx, cudaStreamWaitEvent(sB, ctx->ev_t[k], 0));
            }
            {
                Prof p(ctx, kTransmit, 24.0 * plane * na, sB);
                rop->row_transmit(g, units, na, tb, psi, psi, 1.0f, nmode == 0 && w_in_band, rv,
                                  sB);
            }
            if (overlap) {
                MSK_CUDA(ctx, cudaEventRecord(ctx->ev_free[k], sB));
                pending_free[k] = true;
            }
        }
        if (nmode == 0) {
            Prof p(ctx, kKColProp, 16.0 * plane * b.nunits, sB);
            // band mode once every wave is zero out of band: from the start for
            // a plane wave, else after one full pass (the transmit leaves zeros
            // there, but units without atoms in a slice keep their wave)
            cop->col_prop(g, pmap, pmap, nullptr, b.nunits, w_in_band ? 1 : 0, sB);
            w_in_band = true;
        }
    }
    if (overlap) {
        MSK_CUDA(ctx, cudaEventRecord(ctx->ev_join, sB));
        MSK_CUDA(ctx, cudaStreamWaitEvent(sA, ctx->ev_join, 0));
    }
    MSK_CUDA(ctx, cudaGetLastError());
    return MSK_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" {

int msk_create(int device, msk_context **out)
{
    if (!out) return MSK_EINVAL;
    *out = nullptr;
    msk_context *ctx = new (std::nothrow) msk_context();
    if (!ctx) return MSK_ENOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux2, cudaStreamNonBlocking);
    for (cudaEvent_t *ev : {&ctx->ev_fork, &ctx->ev_join, &ctx->ev_t[0], &ctx->ev_t[1],
                            &ctx->ev_free[0], &ctx->ev_free[1]})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    ctx->stream = ctx->own_stream;
    if (e != cudaSuccess) {
        delete ctx;
        return MSK_ECUDA;
    }
    *out = ctx;
    return MSK_OK;
}

void msk_destroy(msk_context *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    prof_collect(ctx);
    for (cudaEvent_t e : ctx->prof_pool) cudaEventDestroy(e);
    for (DevBuf *b : {&ctx->psi, &ctx->tbuf, &ctx->tbuf2, &ctx->atoms, &ctx->slice_off, &ctx->act, &ctx->tables,
                      &ctx->imgmeta, &ctx->wave0, &ctx->images, &ctx->exitw, &ctx->fresnel,
                      &ctx->flags, &ctx->pa_v, &ctx->pa_t, &ctx->pa_psi, &ctx->pa_e, &ctx->stk,
                      &ctx->stk_v, &ctx->stk_g, &ctx->stk_t, &ctx->stk_img, &ctx->stk_part,
                      &ctx->adjtab, &ctx->arena, &ctx->dwbuf, &ctx->imgfill, &ctx->tune,
                      &ctx->utr_img, &ctx->utr_k2, &ctx->utr_acc, &ctx->utr_vol, &ctx->utr_out,
                      &ctx->utr_tab, &ctx->utr_stage})
        b->release();
    for (cudaEvent_t e : {ctx->ev_fork, ctx->ev_join, ctx->ev_t[0], ctx->ev_t[1], ctx->ev_free[0],
                          ctx->ev_free[1]})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->stk_ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->stk_sev) cudaEventDestroy(e);
    for (cudaStream_t l : ctx->lanes) cudaStreamDestroy(l);
    for (cudaEvent_t e : ctx->lane_ev) cudaEventDestroy(e);
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    if (ctx->aux2) cudaStreamDestroy(ctx->aux2);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    delete ctx;
}

const char *msk_last_error(const msk_context *ctx) { return ctx ? ctx->err.c_str() : ""; }

const char *msk_status_string(int st)
{
    switch (st) {
    case MSK_OK: return "ok";
    case MSK_EBADSIZE: return "bad size parameters";
    case MSK_EBOX: return "atom outside the box";
    case MSK_EZSORT: return "sorted z outside [0, ctblengthz]";
    case MSK_EZNUM: return "atomic number outside 1..103";
    case MSK_ENOMEM: return "out of memory";
    case MSK_EUNSUPPORTED: return "unsupported grid size or mode";
    case MSK_ECUDA: return "CUDA error";
    case MSK_EINVAL: return "invalid argument";
    case MSK_ETOOLARGE: return "beyond the fixed scratch limits of msk_calculate_static";
    default: return "unknown status";
    }
}

int msk_set_stream(msk_context *ctx, void *stream)
{
    if (!ctx) return MSK_EINVAL;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return MSK_OK;
}

int msk_profile(msk_context *ctx, int enable)
{
    if (!ctx) return MSK_EINVAL;
    if (enable) {
        cudaStreamSynchronize(ctx->stream);
        prof_collect(ctx);
        for (int k = 0; k < kKinds; k++) {
            ctx->prof_launches[k] = 0;
            ctx->prof_ms[k] = 0.0;
            ctx->prof_bytes[k] = 0.0;
        }
        ctx->copies[0] = ctx->copies[1] = 0;
        ctx->copy_bytes[0] = ctx->copy_bytes[1] = 0.0;
    }
    ctx->prof_on = enable != 0;
    return MSK_OK;
}

int msk_profile_read(msk_context *ctx, msk_kernel_stat *out, int max)
{
    if (!ctx || (max > 0 && !out)) return MSK_EINVAL;
    cudaStreamSynchronize(ctx->stream);
    prof_collect(ctx);
    int n = 0;
    for (int k = 0; k < kKinds; k++) {
        if (!ctx->prof_launches[k]) continue;
        if (n < max) {
            std::snprintf(out[n].name, sizeof out[n].name, "%s", kKindName[k]);
            out[n].launches = ctx->prof_launches[k];
            out[n].ms = ctx->prof_ms[k];
            out[n].bytes = ctx->prof_bytes[k];
        }
        n++;
    }
    for (int d = 0; d < 2; d++) {
        if (!ctx->copies[d]) continue;
        if (n < max) {
            std::snprintf(out[n].name, sizeof out[n].name, "%s", d ? "copy_d2h" : "copy_h2d");
            out[n].launches = ctx->copies[d];
            out[n].ms = 0.0;
            out[n].bytes = ctx->copy_bytes[d];
        }
        n++;
    }
    return n;
}

int msk_slice_count(float deltaz, float ctblengthz) { return slice_count(deltaz, ctblengthz); }

int msk_slice_assign(float deltaz_f, float zmax, int natom, const float *z2, int *slice_of)
{
    const int n = slice_count(deltaz_f, zmax);
    std::vector<int> counts(n);
    slice_counts(deltaz_f, zmax, natom, z2, n, counts.data());
    int i = 0;
    for (int s = 0; s < n; s++)
        for (int k = 0; k < counts[s]; k++) slice_of[i++] = s;
    for (; i < natom; i++) slice_of[i] = -1;
    return n;
}

void msk_sort_by_z(float *x, float *y, float *z, float *occ, int *Znum, int natom)
{
    sort_by_z(x, y, z, occ, Znum, natom);
}

void msk_rotate(float ctblength, double dxc, double dyc, double dzc, double angleZ,
                double angleY, int natom, float *x, float *y, float *z)
{
    rotate(ctblength, dxc, dyc, dzc, angleZ, angleY, natom, x, y, z);
}

int msk_potential_table(int Z, double *knots, double *coef)
{
    if (Z < 1 || Z > 103) return MSK_EZNUM;
    auto &L = phys::lut();
    L.build(Z);
    for (int i = 0; i < phys::kN; i++) {
        knots[i] = L.knots[i];
        coef[4 * i] = L.y[Z][i];
        coef[4 * i + 1] = L.b[Z][i];
        coef[4 * i + 2] = L.c[Z][i];
        coef[4 * i + 3] = L.d[Z][i];
    }
    return MSK_OK;
}


static int build_zmap(msk_context *ctx, int natom, const int *Znum, std::vector<int> &zlist)
{
    std::vector<int> &zmap = ctx->zmap;
    std::fill(zmap.begin(), zmap.end(), -1);
    zlist.clear();
    for (int i = 0; i < natom; i++) {
        const int Z = Znum[i];
        if (Z < 1 || Z > 103) return fail(ctx, MSK_EZNUM, "atomic number " + std::to_string(Z));
        if (zmap[Z] < 0) {
            if ((int)zlist.size() >= kMaxZidx)
                return fail(ctx, MSK_EUNSUPPORTED, "more than 64 distinct atomic numbers");
            zmap[Z] = (int)zlist.size();
            zlist.push_back(Z);
        }
    }
    return MSK_OK;
}

int msk_calculate(msk_context *ctx, float *pix, const float *wave0, const float *param,
                  int natom, const int *Znum, const float *x, const float *y, const float *z,
                  const float *occ, const float *wobble, float ctblength, float ctblengthz,
                  int nmode, int lwobble, long *iseed)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!pix || !wave0 || !param || natom < 0 ||
        (natom > 0 && (!Znum || !x || !y || !z || !occ)))
        return fail(ctx, MSK_EINVAL, "null pointer or negative atom count");
    // thermal branches (autoslic.cpp:250-254, 701-713, 766-774)
    int nwobble = (int)(param[MSK_pNWOBBLE] + 0.1F);
    if (nwobble < 1) nwobble = 1;
    const int thermal = !lwobble ? kThermNone : (nwobble == 1 ? kThermDW : kThermRandom);
    if (thermal != kThermNone && natom > 0 && !wobble)
        return fail(ctx, MSK_EINVAL, "lwobble needs the wobble array");
    if (thermal == kThermRandom && !iseed)
        return fail(ctx, MSK_EINVAL, "random thermal displacements need iseed");
    const float ax = param[MSK_pAX], by = param[MSK_pBY];
    const int nx = (int)(param[MSK_pNX] + 0.1F), ny = (int)(param[MSK_pNY] + 0.1F);
    if (nx < 1 || ny < 1 || ax < 0.0 || by < 0.0)
        return fail(ctx, MSK_EBADSIZE, "bad size parameters");
    if (!pow2_supported(nx) || !pow2_supported(ny))
        return fail(ctx, MSK_EUNSUPPORTED, "grid must be a power of two from 16 to 4096");
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    // the grid of the previous call, when its parameters are the same (the
    // reference's per-orientation loop calls calculate() on one grid)
    const std::vector<float> key = {(float)nx, (float)ny, ax, by, param[MSK_pENERGY],
                                    param[MSK_pDELTAZ], param[MSK_pXCTILT], param[MSK_pYCTILT]};
    GridPre gp;
    const auto hit = grid_cached(ctx, key, gp);
    if (!hit && !grid_pre(gp, nx, ny, ax, by, param[MSK_pENERGY], param[MSK_pDELTAZ],
                          param[MSK_pXCTILT], param[MSK_pYCTILT]))
        return fail(ctx, MSK_EUNSUPPORTED, "band limit is not two index ranges per column");
    const int nslices = slice_count(param[MSK_pDELTAZ], ctblengthz);
    std::vector<int> zlist;
    // the reference's range check comes before any atomic-number check
    // (autoslic.cpp:270-299 before vzatomLUT)
    if (natom > 0) {
        float xmin = x[0], xmax = x[0], ymin = y[0], ymax = y[0], zmin = z[0], zmax = z[0];
        for (int i = 0; i < natom; i++) {
            xmin = std::min(xmin, x[i]);
            xmax = std::max(xmax, x[i]);
            ymin = std::min(ymin, y[i]);
            ymax = std::max(ymax, y[i]);
            zmin = std::min(zmin, z[i]);
            zmax = std::max(zmax, z[i]);
        }
        if (xmin < 0 || ymin < 0 || zmin < 0 || xmax > ctblength || ymax > ctblength ||
            zmax > ctblengthz)
            return fail(ctx, MSK_EBOX, "atom outside the box");
    }
    {
        int st = build_zmap(ctx, natom, Znum, zlist);
        if (st) return st;
    }
    std::vector<UnitAtoms> ua(1);
    PrepSpec ps{natom, Znum, x, y, z, occ, ctblength, ctblengthz, param[MSK_pDELTAZ], nslices,
                false, 0, 0, 0, 0, 0, nullptr, false, ctx->zmap.data()};
    ps.thermal = thermal;
    ps.wobble = wobble;
    ps.temperature = param[MSK_pTEMPER];
    ps.iseed = iseed;
    prep_unit(gp, ps, ua[0]);
    if (ua[0].status) return fail(ctx, ua[0].status, msk_status_string(ua[0].status));
    int st = grid_tables(ctx, gp, key, hit, zlist);
    if (st) return st;
    Batch b;
    st = upload_batch(ctx, ua, 0, 1, nslices, b);
    if (st) return st;
    const size_t plane = (size_t)nx * ny;
    MSK_CUDA(ctx, ctx->psi.reserve(plane * sizeof(float2)));
    MSK_CUDA(ctx, ctx->tbuf.reserve(plane * sizeof(float2)));
    MSK_CUDA(ctx, ctx->tbuf2.reserve(plane * sizeof(float2)));
    // the splat stores in-band row segments only: the rest must read as zeros
    MSK_CUDA(ctx, cudaMemsetAsync(ctx->tbuf.p, 0, plane * sizeof(float2), ctx->stream));
    MSK_CUDA(ctx, cudaMemsetAsync(ctx->tbuf2.p, 0, plane * sizeof(float2), ctx->stream));
    ctx->units_alloc = 1;
    MSK_CUDA(ctx, ctx->wave0.reserve(plane * sizeof(float2)));
    st = flags_reset(ctx, gp.g);
    if (st) return st;
    // the incident wave of the previous call when it is the same (the
    // reference's per-orientation loop passes one plane wave to every call):
    // compared on the host, not uploaded again
    const size_t wbytes = plane * sizeof(float2);
    if (!(ctx->w0_valid && ctx->w0_dev == ctx->wave0.p && ctx->w0_host.size() * sizeof(float) == wbytes &&
          std::memcmp(ctx->w0_host.data(), wave0, wbytes) == 0)) {
        ctx->w0_valid = false;
        MSK_CUDA(ctx, cudaMemcpyAsync(ctx->wave0.p, wave0, wbytes, cudaMemcpyHostToDevice, ctx->stream));
        count_copy(ctx, 0, (double)wbytes);
        ctx->w0_host.assign(wave0, wave0 + 2 * plane);
        ctx->w0_dev = ctx->wave0.p;
        ctx->w0_valid = true;
    }
    const SizeOps *rop = size_ops(ny);
    {
        Prof p(ctx, kInit, 16.0 * plane);
        rop->row_init(gp.g, nullptr, 1, ctx->wave0.as<float2>(), ctx->psi.as<float2>(), 1.0f,
                      ctx->stream);
    }
    st = run_slices(ctx, gp, b, nmode, false);  // any incident wave
    if (st) return st;
    {
        Prof p(ctx, kExit, 16.0 * plane);
        rop->row_exit(gp.g, nullptr, 1, ctx->psi.as<float2>(), ctx->tbuf.as<float2>(), ctx->stream);
    }
    MSK_CUDA(ctx, cudaGetLastError());
    MSK_CUDA(ctx, cudaMemcpyAsync(pix, ctx->tbuf.p, plane * sizeof(float2),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    count_copy(ctx, 1, (double)(plane * sizeof(float2)));
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    return flags_check(ctx);
}

}  // extern "C"

namespace {

// Detector planes per orientation: orientation a images planes
// [off[a], off[a+1]) of `p`, shifted by shift[2a], shift[2a+1] Angstrom;
// images[k] is the image of plane k.
struct PlaneDesc {
    double defocus, rotation, astig, astig_angle;
};
struct PlaneList {
    int total = 0;
    std::vector<int> off;
    std::vector<PlaneDesc> p;
    std::vector<double> shift;
};

int tilt_series_impl(msk_context *ctx, const msk_series *s, int natom, const int *Znum,
                     const float *x, const float *y, const float *z, const float *occ,
                     int nangles, const double *angleZ, const double *angleY,
                     const PlaneList &pl, int nconfig, const float *displacements,
                     float *images, float *exitwaves, int *kept)
{
    if (!s || natom < 0 || nangles < 1 || nconfig < 1 || !angleZ || !angleY ||
        (pl.total > 0 && !images) || (natom > 0 && (!Znum || !x || !y || !z || !occ)) ||
        (nconfig > 1 && !displacements && !s->lwobble))
        return fail(ctx, MSK_EINVAL, "bad tilt-series arguments");
    const int ndefocus = pl.total;  // images in all
    const int nx = s->nx, ny = s->ny;
    if (nx < 1 || ny < 1 || s->ctblength < 0.0f) return fail(ctx, MSK_EBADSIZE, "bad size parameters");
    if (!pow2_supported(nx) || !pow2_supported(ny))
        return fail(ctx, MSK_EUNSUPPORTED, "grid must be a power of two from 16 to 4096");
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    GridPre gp;
    // MsctKirkland passes a zero crystal tilt (autosliccmd.cpp:435-437); the
    // grid tables of the previous call (this or msk_calculate) when they match
    const std::vector<float> key = {(float)nx, (float)ny, s->ctblength, s->ctblength, s->v0,
                                    s->deltaz, 0.0f, 0.0f};
    const auto hit = grid_cached(ctx, key, gp);
    if (!hit && !grid_pre(gp, nx, ny, s->ctblength, s->ctblength, s->v0, s->deltaz, 0.0f, 0.0f))
        return fail(ctx, MSK_EUNSUPPORTED, "band limit is not two index ranges per column");
    const int nslices = slice_count(s->deltaz, s->ctblengthz);
    std::vector<int> zlist;
    int st = build_zmap(ctx, natom, Znum, zlist);
    if (st) return st;
    if ((st = grid_tables(ctx, gp, key, hit, zlist))) return st;

    const size_t plane = (size_t)nx * ny;
    const int nunits = nangles * nconfig;
    size_t free_b = 0, total_b = 0;
    MSK_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
    // psi + t per unit; the image and exit-wave outputs are held separately
    const bool img_dev = ndefocus > 0 && is_device_ptr(images);
    // page-locked host images the GPU can address: the image pass writes them
    // in place (no staging buffer, no copy after the last batch)
    float *img_mapped =
        ndefocus > 0 && !img_dev ? static_cast<float *>(mapped_host(images)) : nullptr;
    const bool img_direct = img_dev || img_mapped;
    const bool ew_dev = exitwaves && is_device_ptr(exitwaves);
    const size_t img_bytes = (size_t)ndefocus * plane * sizeof(float);
    size_t budget = free_b - std::min(free_b, (size_t)(img_direct ? 0 : img_bytes));
    budget = std::min<size_t>(budget / 2, (size_t)64 << 30);
    // psi and two transmission buffers per unit in flight
    int B = (int)std::max<size_t>(1, std::min<size_t>(nunits, budget / (3 * plane * sizeof(float2))));
    if (s->max_batch > 0) B = std::min(B, s->max_batch);
    if (nconfig > 1 && B > nconfig) B = (B / nconfig) * nconfig;  // whole angles per batch
    // batch bounds: a large call starts with a small batch (~1/16 of the
    // units) so that only its host preparation is exposed; each later batch is
    // prepared on the host while the GPU runs the one before
    std::vector<int> bounds = {0};
    {
        int first = B;
        if (s->max_batch <= 0 && nunits >= 32) {
            first = std::min(B, std::max(8, (nunits + 15) / 16));
            if (nconfig > 1) first = std::max(nconfig, (first / nconfig) * nconfig);
            first = std::min(first, B);
        }
        bounds.push_back(std::min(first, nunits));
        while (bounds.back() < nunits) bounds.push_back(std::min(nunits, bounds.back() + B));
        // images bound for page-locked host memory leave a batch at a time,
        // beside the next batch's kernels: end with a small batch too, so that
        // little of the copy is left after the last kernel
        const int nb_last = bounds.back() - bounds[bounds.size() - 2];
        if (img_mapped && s->max_batch <= 0 && nunits >= 32 && nb_last >= 3 * first)
            bounds.insert(bounds.end() - 1, bounds.back() - first);
    }
    // page-locked host images: each batch's images are made in a device buffer
    // and written out (k_copy_rows, through the mapped address) on the third
    // stream while the next batch runs -- when no orientation's configurations
    // span two batches (a configuration average is completed within its
    // batch); else the image pass writes them in place
    bool img_stage = img_mapped != nullptr;
    size_t stage_planes = 0;
    for (size_t bi = 0; img_stage && bi + 1 < bounds.size(); bi++) {
        img_stage = bounds[bi] % nconfig == 0 && bounds[bi + 1] % nconfig == 0;
        const int a0 = bounds[bi] / nconfig, a1 = (bounds[bi + 1] - 1) / nconfig;
        stage_planes = std::max<size_t>(stage_planes, (size_t)(pl.off[a1 + 1] - pl.off[a0]));
    }
    float *d_images = img_mapped ? img_mapped : images;
    if (ndefocus > 0 && !img_direct) {
        MSK_CUDA(ctx, ctx->images.reserve(img_bytes));
        d_images = ctx->images.as<float>();
    }
    cudaEvent_t ev_ready = nullptr, ev_copied = nullptr;
    if (img_stage) {
        MSK_CUDA(ctx, ctx->images.reserve(stage_planes * plane * sizeof(float)));
        d_images = ctx->images.as<float>();
        if (!ctx->stk_ev[0])
            for (cudaEvent_t &e : ctx->stk_ev)
                MSK_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ev_ready = ctx->stk_ev[0];
        ev_copied = ctx->stk_ev[1];
    }
    MSK_CUDA(ctx, ctx->psi.reserve((size_t)B * plane * sizeof(float2)));
    MSK_CUDA(ctx, ctx->tbuf.reserve((size_t)B * plane * sizeof(float2)));
    MSK_CUDA(ctx, ctx->tbuf2.reserve((size_t)B * plane * sizeof(float2)));
    // the splat stores in-band row segments only: the rest must read as zeros
    MSK_CUDA(ctx, cudaMemsetAsync(ctx->tbuf.p, 0, (size_t)B * plane * sizeof(float2), ctx->stream));
    MSK_CUDA(ctx, cudaMemsetAsync(ctx->tbuf2.p, 0, (size_t)B * plane * sizeof(float2), ctx->stream));
    ctx->units_alloc = B;
    st = flags_reset(ctx, gp.g);
    if (st) return st;
    ColView pmap, tmap;  // the free-space pass's views
    const int vf = col_variant(ctx, gp, kColFresnel);
    st = column_map(ctx, &pmap, ctx->psi.p, nx, ny, B, size_ops(nx), vf);
    if (st) return st;
    st = column_map(ctx, &tmap, ctx->tbuf.p, nx, ny, B, size_ops(nx), vf);
    if (st) return st;

    // thermal branches: Debye-Waller with one configuration, displacements
    // drawn in the engine with several (when the caller gives none)
    const int thermal = !s->lwobble ? kThermNone
                        : nconfig == 1 ? kThermDW
                        : displacements ? kThermNone : kThermRandom;
    if (thermal != kThermNone && natom > 0 && !s->wobble)
        return fail(ctx, MSK_EINVAL, "lwobble needs the wobble array");
    std::vector<long> seeds;
    if (thermal == kThermRandom)
        for (int a = 0; a < nangles; a++) seeds.push_back(s->seed - a);
    // incident wave: a plane wave, or MsctKirkland's spherical wave
    const bool spherical = s->R1 != 0.0;
    if (spherical) {
        std::vector<float2> w0;
        spherical_wave(nx, ny, s->ctblength, s->v0, s->R1, w0);
        MSK_CUDA(ctx, ctx->wave0.reserve(plane * sizeof(float2)));
        ctx->w0_valid = false;  // msk_calculate's incident wave is overwritten
        MSK_CUDA(ctx, cudaMemcpyAsync(ctx->wave0.p, w0.data(), plane * sizeof(float2),
                                      cudaMemcpyHostToDevice, ctx->stream));
        count_copy(ctx, 0, (double)(plane * sizeof(float2)));
        MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }

    // image plane: rotation centre and shift (autosliccmd.cpp:1046, 1137-1141)
    const double xst = s->ctblength / nx, yst = s->ctblength / ny;  // float divisions
    const double xcen = 0.5 * (0.0 + s->ctblength) + s->dxc, ycen = 0.5 * (0.0 + s->ctblength) + s->dyc;

    const float wavlen = gp.wavlen;
    float k2maxo = s->aobj / wavlen;  // autosliccmd.cpp:1042-1043
    k2maxo = k2maxo * k2maxo;
    const double pi = 4.0 * atan(1.0);
    const double l = wavlen;

    std::vector<UnitAtoms> ua(nunits);
    const SizeOps *rop = size_ops(ny), *cop = size_ops(nx);
    auto prep_batch = [&](int u0, int nb) {
        auto prep = [&](int u) {
            const int a = u / nconfig, c = u % nconfig;
            PrepSpec ps{natom, Znum, x, y, z, occ, s->ctblength, s->ctblengthz, s->deltaz,
                        nslices, true, angleZ[a], angleY[a], s->dxc, s->dyc, s->dzc,
                        displacements ? displacements + (size_t)c * 3 * natom : nullptr, true,
                        ctx->zmap.data()};
            ps.thermal = thermal;
            ps.wobble = s->wobble;
            ps.temperature = s->temperature;
            ps.iseed = thermal == kThermRandom ? &seeds[a] : nullptr;
            prep_unit(gp, ps, ua[u]);
        };
        if (thermal == kThermRandom) {
            // one orientation's configurations in order (they draw from one sequence)
            const int a0 = u0 / nconfig, a1 = (u0 + nb - 1) / nconfig;
            parallel_for(a1 - a0 + 1, host_threads(), [&](int k) {
                const int a = a0 + k;
                for (int u = std::max(u0, a * nconfig); u < std::min(u0 + nb, (a + 1) * nconfig); u++)
                    prep(u);
            });
        } else {
            parallel_for(nb, host_threads(), [&](int i) { prep(u0 + i); });
        }
    };
    prep_batch(0, bounds[1]);
    for (size_t bi = 0; bi + 1 < bounds.size(); bi++) {
        const int u0 = bounds[bi], nb = bounds[bi + 1] - bounds[bi];
        for (int i = 0; i < nb; i++)
            if (ua[u0 + i].status)
                return fail(ctx, ua[u0 + i].status, msk_status_string(ua[u0 + i].status));
        Batch b;
        st = upload_batch(ctx, ua, u0, nb, nslices, b);
        if (st) return st;
        b.call_units = nunits;
        float2 *psi = ctx->psi.as<float2>(), *tb = ctx->tbuf.as<float2>();
        if (spherical) {
            Prof p(ctx, kInit, 8.0 * plane * (nb + 1));
            rop->row_init(gp.g, nullptr, nb, ctx->wave0.as<float2>(), psi, 1.0f, ctx->stream);
        } else {
            Prof p(ctx, kPlane, 8.0 * plane * nb);
            k_plane_init<<<1024, 256, 0, ctx->stream>>>(psi, nullptr, nb, nx, ny);
        }
        st = run_slices(ctx, gp, b, s->nmode, !spherical);  // a plane wave is in band
        if (st) return st;
        if (exitwaves) {
            {
                Prof p(ctx, kExit, 16.0 * plane * nb);
                rop->row_exit(gp.g, nullptr, nb, psi, tb, ctx->stream);
            }
            MSK_CUDA(ctx, cudaMemcpyAsync(exitwaves + (size_t)u0 * plane * 2, tb,
                                          (size_t)nb * plane * sizeof(float2),
                                          ew_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                          ctx->stream));
            if (!ew_dev) count_copy(ctx, 1, (double)nb * plane * sizeof(float2));
        }
        if (ndefocus > 0) {
            // this batch's orientations: their units (configurations in order) and
            // whether their images continue or finish a configuration average
            const int a_first = u0 / nconfig, a_last = (u0 + nb - 1) / nconfig;
            const int na_b = a_last - a_first + 1;
            std::vector<std::vector<int>> aunits(na_b);
            std::vector<int> aflags(na_b);
            int kmax = 0;
            for (int a = a_first; a <= a_last; a++) {
                const int c0 = std::max(u0, a * nconfig), c1 = std::min(u0 + nb, (a + 1) * nconfig);
                for (int u = c0; u < c1; u++) aunits[a - a_first].push_back(u - u0);
                int f = 0;
                if (c0 > a * nconfig) f |= 1;                        // continue a partial sum
                if (c1 == (a + 1) * nconfig && nconfig > 1) f |= 2;   // last configuration
                aflags[a - a_first] = f;
                kmax = std::max(kmax, pl.off[a + 1] - pl.off[a]);
            }
            MSK_CUDA(ctx, ctx->fresnel.reserve(plane * sizeof(float2)));
            MSK_CUDA(ctx, ctx->imgfill.reserve((size_t)B * sizeof(float2)));
            // staged: this batch's planes from the start of the device buffer,
            // once the previous batch's copy out of it has finished
            const int dst_base = img_stage ? pl.off[a_first] : 0;
            if (img_stage && bi > 0) MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev_copied, 0));
            for (int k = 0; k < kmax; k++) {
                // the k-th plane of every orientation, grouped by equal free-space
                // and image-plane parameters: one table and one pass per group
                struct Group {
                    std::array<double, 6> key;
                    std::vector<int> ori;  // orientation indices within the batch
                    size_t o_units, o_off, o_dst, o_flags;
                    int n_units;
                };
                std::vector<Group> groups;
                for (int a = a_first; a <= a_last; a++) {
                    if (pl.off[a + 1] - pl.off[a] <= k) continue;
                    const PlaneDesc &q = pl.p[pl.off[a] + k];
                    const std::array<double, 6> key = {
                        q.defocus, q.astig, q.astig_angle, q.rotation,
                        floor(pl.shift[2 * a] / xst + 0.5), floor(pl.shift[2 * a + 1] / yst + 0.5)};
                    size_t gi = 0;
                    while (gi < groups.size() && groups[gi].key != key) gi++;
                    if (gi == groups.size()) groups.push_back(Group{key, {}, 0, 0, 0, 0, 0});
                    groups[gi].ori.push_back(a - a_first);
                }
                // per group: img_off[n+1] | img_units | img_dst[n] | img_flags[n]
                std::vector<int> meta;
                for (Group &gr : groups) {
                    const int n = (int)gr.ori.size();
                    gr.o_off = meta.size();
                    int cnt = 0;
                    for (int oa : gr.ori) {
                        meta.push_back(cnt);
                        cnt += (int)aunits[oa].size();
                    }
                    meta.push_back(cnt);
                    gr.o_units = meta.size();
                    gr.n_units = cnt;
                    for (int oa : gr.ori) meta.insert(meta.end(), aunits[oa].begin(), aunits[oa].end());
                    gr.o_dst = meta.size();
                    for (int oa : gr.ori) meta.push_back(pl.off[a_first + oa] + k - dst_base);
                    gr.o_flags = meta.size();
                    for (int oa : gr.ori) meta.push_back(aflags[oa]);
                    (void)n;
                }
                MSK_CUDA(ctx, ctx->imgmeta.reserve(meta.size() * sizeof(int)));
                MSK_CUDA(ctx, cudaMemcpyAsync(ctx->imgmeta.p, meta.data(), meta.size() * sizeof(int),
                                              cudaMemcpyHostToDevice, ctx->stream));
                count_copy(ctx, 0, (double)(meta.size() * sizeof(int)));
                const int *dm = ctx->imgmeta.as<int>();
                for (const Group &gr : groups) {
                    const int nimg = (int)gr.ori.size(), nu = gr.n_units;
                    const int *d_off = dm + gr.o_off, *d_units = dm + gr.o_units,
                              *d_dst = dm + gr.o_dst, *d_flags = dm + gr.o_flags;
                    const double rprime = gr.key[0] - 0.5 * s->ctblengthz;  // autosliccmd.cpp:1060
                    Fresnel fr{};
                    fr.a1 = pi * l * rprime;
                    fr.a3 = (pi / 2.0) * s->cs3 * l * l * l;
                    fr.a5 = (pi / 3.0) * s->cs5 * l * l * l * l * l;
                    fr.a2c = (pi / 2.0) * l * gr.key[1] * cos(2.0 * gr.key[2]);
                    fr.a2s = (pi / 2.0) * l * gr.key[1] * sin(2.0 * gr.key[2]);
                    fr.k2maxo = k2maxo;
                    fr.kx = tables_kx(ctx, gp);
                    fr.ky = tables_ky(ctx, gp);
                    // psi_d = iS(iF(exp(-i chi) F(W)))/N: the multiplier (with 1/N)
                    // once per group, then one column pass over its waves
                    fr.table = ctx->fresnel.as<float2>();
                    {
                        Prof p(ctx, kFresTab, 8.0 * plane);
                        k_fresnel_table<<<4 * 152, 256, 0, ctx->stream>>>(
                            gp.g, fr, 1.0f / ((float)nx * (float)ny), ctx->fresnel.as<float2>());
                    }
                    {
                        Prof p(ctx, kFresnel, 16.0 * plane * nu);
                        cop->col_fresnel(gp.g, pmap, tmap, d_units, nu, fr, 1.0f, ctx->stream);
                    }
                    const double rot = gr.key[3];
                    const int sxp = (int)gr.key[4], syp = (int)gr.key[5];
                    if (rot != 0.0 || sxp != 0 || syp != 0) {
                        // the amplitude in real space, rotated and shifted, then |.|^2
                        float2 *phi = ctx->tbuf2.as<float2>();
                        {
                            Prof p(ctx, kExit, 16.0 * plane * nu);
                            rop->row_inverse(gp.g, d_units, nu, tb, phi, 1.0f, ctx->stream);
                        }
                        k_edge_mean<<<nu, 256, 0, ctx->stream>>>(phi, d_units, nx, ny, 5,
                                                                 ctx->imgfill.as<float2>());
                        {
                            Prof p(ctx, kRotShift, 16.0 * plane * nu);
                            k_rotate_shift<<<8 * 152, 256, 0, ctx->stream>>>(
                                phi, tb, d_units, nu, nx, ny, xst, yst, xcen, ycen, cos(rot),
                                sin(rot), rot != 0.0, sxp, syp, ctx->imgfill.as<float2>());
                        }
                        Prof p(ctx, kIntensity, 8.0 * plane * nu + 4.0 * plane * nimg);
                        k_intensity_direct<<<8 * 152, 256, 0, ctx->stream>>>(
                            nimg, d_off, d_units, d_dst, d_flags, tb, d_images, plane,
                            (float)nconfig);
                    } else {
                        Prof p(ctx, kIntensity, 8.0 * plane * nu + 4.0 * plane * nimg);
                        rop->row_intensity(gp.g, nimg, d_off, d_units, d_dst, d_flags, tb,
                                           d_images, (float)nconfig, ctx->stream);
                    }
                }
            }
            if (img_stage) {
                const size_t bytes = (size_t)(pl.off[a_last + 1] - dst_base) * plane * sizeof(float);
                MSK_CUDA(ctx, cudaEventRecord(ev_ready, ctx->stream));
                MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->aux2, ev_ready, 0));
                {
                    Prof p(ctx, kCopyImages, (double)bytes, ctx->aux2);
                    k_copy_rows<<<kCopyCtas, 256, 0, ctx->aux2>>>(
                        d_images, 0, img_mapped + (size_t)dst_base * plane, 0, bytes / sizeof(float), 1);
                }
                MSK_CUDA(ctx, cudaEventRecord(ev_copied, ctx->aux2));
                count_copy(ctx, 1, (double)bytes);
            }
        }
        MSK_CUDA(ctx, cudaGetLastError());
        // the next batch's atoms while this one runs (its upload waits for it)
        if (bi + 2 < bounds.size()) prep_batch(bounds[bi + 1], bounds[bi + 2] - bounds[bi + 1]);
    }
    if (img_stage) MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev_copied, 0));
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    if (ndefocus > 0 && img_mapped && !img_stage) count_copy(ctx, 1, (double)img_bytes);  // in place
    if (ndefocus > 0 && !img_direct) {
        Prof p(ctx, kCopyImages, (double)img_bytes);
        MSK_CUDA(ctx, cudaMemcpyAsync(images, d_images, img_bytes, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        count_copy(ctx, 1, (double)img_bytes);
    }
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (kept)
        for (int u = 0; u < nunits; u++) kept[u] = ua[u].kept;
    return flags_check(ctx);
}

}  // namespace

extern "C" {

int msk_tilt_series(msk_context *ctx, const msk_series *s, int natom, const int *Znum,
                    const float *x, const float *y, const float *z, const float *occ,
                    int nangles, const double *angleZ, const double *angleY, int ndefocus,
                    const double *defocus, int nconfig, const float *displacements,
                    float *images, float *exitwaves, int *kept)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!s || nangles < 1 || ndefocus < 0 || (ndefocus > 0 && (!defocus || !images)))
        return fail(ctx, MSK_EINVAL, "bad tilt-series arguments");
    // the same planes for every orientation: image [a][d] is plane a * ndefocus + d
    PlaneList pl;
    pl.total = nangles * ndefocus;
    for (int a = 0; a <= nangles; a++) pl.off.push_back(a * ndefocus);
    for (int a = 0; a < nangles; a++) {
        for (int d = 0; d < ndefocus; d++)
            pl.p.push_back(PlaneDesc{defocus[d], s->rotation ? s->rotation[d] : 0.0, s->astig,
                                     s->astig_angle});
        pl.shift.push_back(s->xshift);
        pl.shift.push_back(s->yshift);
    }
    return tilt_series_impl(ctx, s, natom, Znum, x, y, z, occ, nangles, angleZ, angleY, pl,
                            nconfig, displacements, images, exitwaves, kept);
}

int msk_tilt_series_planes(msk_context *ctx, const msk_series *s, int natom, const int *Znum,
                           const float *x, const float *y, const float *z, const float *occ,
                           int nangles, const double *angleZ, const double *angleY,
                           const int *plane_off, const msk_plane *planes, const double *shifts,
                           int nconfig, const float *displacements, float *images,
                           float *exitwaves, int *kept)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!s || nangles < 1 || !plane_off || plane_off[0] != 0)
        return fail(ctx, MSK_EINVAL, "bad plane lists");
    PlaneList pl;
    for (int a = 0; a <= nangles; a++) {
        if (a > 0 && plane_off[a] < plane_off[a - 1])
            return fail(ctx, MSK_EINVAL, "plane_off must not decrease");
        pl.off.push_back(plane_off[a]);
    }
    pl.total = plane_off[nangles];
    if (pl.total > 0 && (!planes || !images)) return fail(ctx, MSK_EINVAL, "bad plane lists");
    for (int k = 0; k < pl.total; k++)
        pl.p.push_back(PlaneDesc{planes[k].defocus, planes[k].rotation, planes[k].astig,
                                 planes[k].astig_angle});
    for (int a = 0; a < nangles; a++) {
        pl.shift.push_back(shifts ? shifts[2 * a] : 0.0);
        pl.shift.push_back(shifts ? shifts[2 * a + 1] : 0.0);
    }
    return tilt_series_impl(ctx, s, natom, Znum, x, y, z, occ, nangles, angleZ, angleY, pl,
                            nconfig, displacements, images, exitwaves, kept);
}

}  // extern "C"

// ------------------------------------------------------------------ potential stacks
// The multislice of calculate() (autoslic.cpp:838-861) driven by given
// per-slice projected potentials v_k instead of atoms, from a plane wave, with
// the free-space step of msk_tilt_series to each detector plane; and the
// adjoint of an image misfit through it.  Kernels: P1 is k_row_expv (no
// splat), P2-P4 as in the atom path; the backward pass runs the adjoint of
// every step in W-states with conjugated propagator and free-space tables
// (the 2/3 band limit is real and symmetric: its own adjoint).  Waves and
// transmissions are carried in the scattered form (phi = psi - 1, tau = t - 1;
// k_row_transmit<N, true>), which keeps the FP32 rounding of the images ~10x
// below that of psi and t themselves: the adjoint's residuals I - T are a few
// 1e-4 of I.

namespace {

__global__ void k_add_waves(float2 *__restrict__ dst, const float2 *__restrict__ src, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float2 a = dst[i], b = src[i];
        dst[i] = make_float2(a.x + b.x, a.y + b.y);
    }
}

struct StackJob {
    const msk_stack *s;
    int nunits, ndef;
    const float *v;
    const double *defocus;
    const float *target;  // adjoint only
    float *images;        // forward only (may be NULL)
    float *grad;          // adjoint only
    double *loss;
};

Fresnel stack_fresnel(msk_context *ctx, const GridPre &gp, const msk_stack *s, double rprime,
                      double sign)
{
    const double pi = 4.0 * atan(1.0), l = gp.wavlen;
    float k2maxo = s->aobj / gp.wavlen;
    k2maxo = k2maxo * k2maxo;
    Fresnel fr{};
    fr.a1 = sign * pi * l * rprime;
    fr.a3 = sign * (pi / 2.0) * s->cs3 * l * l * l;
    fr.a5 = sign * (pi / 3.0) * s->cs5 * l * l * l * l * l;
    fr.k2maxo = k2maxo;
    fr.kx = tables_kx(ctx, gp);
    fr.ky = tables_ky(ctx, gp);
    return fr;
}

int stack_run(msk_context *ctx, const StackJob &J)
{
    const msk_stack *s = J.s;
    const bool adjoint = J.grad != nullptr;
    if (!s || J.nunits < 1 || J.ndef < 0 || !J.v || (J.ndef > 0 && !J.defocus) ||
        (adjoint && (J.ndef < 1 || !J.target)) || (!adjoint && J.ndef > 0 && !J.images) ||
        s->nslices < 1 || s->checkpoint < 0)
        return fail(ctx, MSK_EINVAL, "bad potential-stack arguments");
    const int nx = s->nx, ny = s->ny, S = s->nslices, ndef = J.ndef;
    if (nx < 1 || ny < 1 || s->ax < 0.0f || s->by < 0.0f)
        return fail(ctx, MSK_EBADSIZE, "bad size parameters");
    if (!pow2_supported(nx) || !pow2_supported(ny))
        return fail(ctx, MSK_EUNSUPPORTED, "grid must be a power of two from 16 to 4096");
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    GridPre gp;
    const std::vector<float> key = {(float)nx, (float)ny, s->ax, s->by, s->v0, s->deltaz,
                                    s->ctiltx, s->ctilty};
    const auto hit = grid_cached(ctx, key, gp);
    if (!hit && !grid_pre(gp, nx, ny, s->ax, s->by, s->v0, s->deltaz, s->ctiltx, s->ctilty))
        return fail(ctx, MSK_EUNSUPPORTED, "band limit is not two index ranges per column");
    int st = grid_tables(ctx, gp, key, hit, std::vector<int>());
    if (st) return st;
    Geom &g = gp.g;
    st = flags_reset(ctx, g);
    if (st) return st;
    // conjugated propagator for the backward pass
    Geom gc = g;
    if (adjoint) {
        std::vector<float2> pc(nx + ny);
        for (int i = 0; i < nx; i++) pc[i] = make_float2(gp.propx[i].x, -gp.propx[i].y);
        for (int i = 0; i < ny; i++) pc[nx + i] = make_float2(gp.propy[i].x, -gp.propy[i].y);
        MSK_CUDA(ctx, ctx->adjtab.reserve(pc.size() * sizeof(float2)));
        MSK_CUDA(ctx, cudaMemcpyAsync(ctx->adjtab.p, pc.data(), pc.size() * sizeof(float2),
                                      cudaMemcpyHostToDevice, ctx->stream));
        count_copy(ctx, 0, (double)(pc.size() * sizeof(float2)));
        MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        gc.propx = ctx->adjtab.as<float2>();
        gc.propy = ctx->adjtab.as<float2>() + nx;
    }

    const size_t plane = (size_t)nx * ny;
    const size_t pb = plane * sizeof(float2);
    const bool v_dev = is_device_ptr(J.v);
    const bool g_dev = adjoint && is_device_ptr(J.grad);
    // page-locked host stacks the GPU addresses: their slices move by
    // k_copy_rows through the mapped addresses (else by 2D copies)
    const float *v_map = v_dev ? nullptr : static_cast<const float *>(mapped_host(const_cast<float *>(J.v)));
    float *g_map = adjoint && !g_dev ? static_cast<float *>(mapped_host(J.grad)) : nullptr;
    const float *t_map = adjoint && !is_device_ptr(J.target)
                             ? static_cast<const float *>(mapped_host(const_cast<float *>(J.target)))
                             : nullptr;
    const bool t_dev = adjoint && is_device_ptr(J.target);
    const bool i_dev = !adjoint && ndef > 0 && is_device_ptr(J.images);
    const size_t vb = (size_t)S * plane * sizeof(float);      // one unit's stack
    const size_t ib = (size_t)ndef * plane * sizeof(float);   // one unit's images
    const size_t staged = (v_dev ? 0 : vb) + (adjoint && !g_dev ? vb : 0) +
                          (adjoint && !t_dev ? ib : 0) + (!adjoint && !i_dev ? ib : 0);
    // Host buffers: the copies in and out run on two more streams, slice by
    // slice -- slice k of every unit of a batch (one 2D copy) goes in ahead of
    // the forward pass's slice k, and dL/dv_k goes out as soon as the backward
    // pass has written it -- so the kernels wait only for the first slice and
    // the host only for the last.  Several batches (when memory is short) use
    // two sets of staging buffers.
    const bool host_io = staged > 0;
    const int nslot_max = host_io ? 2 : 1;
    size_t free_b = 0, total_b = 0;
    MSK_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = std::min<size_t>(free_b / 2, (size_t)64 << 30);
    // Adjoint with checkpoint 0: keep every wave and every transmission of the
    // forward pass (2S + 4 planes a unit) when memory holds at least 32 units
    // (or all of them) at once -- the backward pass then recomputes nothing;
    // otherwise a checkpoint every K slices (8 by default) with the waves and
    // transmissions of a block recomputed from its checkpoint.
    const size_t keep_unit = (size_t)(2 * S + 4) * pb + nslot_max * staged;
    const bool keep = adjoint && s->checkpoint == 0 &&
                      budget / keep_unit >= (size_t)std::min(J.nunits, 32) &&
                      (s->max_batch <= 0 || s->max_batch >= std::min(J.nunits, 32));
    const int K = !adjoint ? 1 : keep ? 1 : (s->checkpoint > 0 ? std::min(s->checkpoint, S) : std::min(8, S));
    const int nblk = adjoint ? (S + K - 1) / K : 1;
    // planes per unit: forward W, transmission B, free-space E (+ adjoint:
    // checkpoints, the block's transmissions and waves, the wave gradient G;
    // keeping everything: the S + 1 waves and the S transmissions, G)
    const int planes = keep ? 2 * S + 4 : adjoint ? 3 + nblk + K + (K - 1) : 3;
    const size_t per_unit = planes * pb + nslot_max * staged;
    int B = (int)std::max<size_t>(1, std::min<size_t>(J.nunits, budget / per_unit));
    if (s->max_batch > 0) B = std::min(B, s->max_batch);
    const int nbat = (J.nunits + B - 1) / B;
    const int nslot = nbat > 1 ? nslot_max : 1;

    MSK_CUDA(ctx, ctx->stk.reserve((size_t)planes * B * pb));
    float2 *base = ctx->stk.as<float2>();
    auto grid_at = [&](int i) { return base + (size_t)i * B * plane; };
    float2 *W = grid_at(0), *E = grid_at(1), *Bt = grid_at(2), *G = nullptr;
    std::vector<float2 *> ck, Bb, Wb, waves, trans;
    if (keep) {
        G = grid_at(2);
        for (int k = 0; k <= S; k++) waves.push_back(grid_at(3 + k));          // W_0 .. W_S
        for (int k = 1; k <= S; k++) trans.push_back(grid_at(3 + S + k));      // B_1 .. B_S
        W = waves[S];  // the exit wave the free-space step reads
    } else if (adjoint) {
        G = grid_at(2);
        for (int i = 0; i < nblk; i++) ck.push_back(grid_at(3 + i));
        for (int i = 0; i < K; i++) Bb.push_back(grid_at(3 + nblk + i));
        for (int i = 0; i < K - 1; i++) Wb.push_back(grid_at(3 + nblk + K + i));
        Bt = Bb[0];  // the forward pass's transmission: a block buffer, free until the backward
    }
    if (!v_dev) MSK_CUDA(ctx, ctx->stk_v.reserve((size_t)nslot * B * vb));
    if (adjoint && !g_dev) MSK_CUDA(ctx, ctx->stk_g.reserve((size_t)nslot * B * vb));
    if (adjoint && !t_dev) MSK_CUDA(ctx, ctx->stk_t.reserve((size_t)nslot * B * ib));
    if (!adjoint && ndef > 0 && !i_dev) MSK_CUDA(ctx, ctx->stk_img.reserve((size_t)nslot * B * ib));
    // staging of batch b: slot b % nslot
    auto slot_of = [&](const DevBuf &buf, size_t per, int b) {
        return reinterpret_cast<float *>(buf.as<char>() + (size_t)(b % nslot) * B * per);
    };
    if (host_io && !ctx->stk_ev[0])
        for (cudaEvent_t &e : ctx->stk_ev)
            MSK_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    while (host_io && ctx->stk_sev.size() < (size_t)2 * S) {
        cudaEvent_t e = nullptr;
        MSK_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->stk_sev.push_back(e);
    }
    cudaEvent_t *ev_sin = host_io ? ctx->stk_sev.data() : nullptr;    // slice k of v is in
    cudaEvent_t *ev_sout = host_io ? ctx->stk_sev.data() + S : nullptr;  // dL/dv_k is written
    cudaEvent_t *ev_in = ctx->stk_ev, *ev_done = ctx->stk_ev + 2, *ev_out = ctx->stk_ev + 4;
    cudaStream_t cin = host_io ? ctx->aux : ctx->stream, cout = host_io ? ctx->aux2 : ctx->stream;
    // slice-by-slice copies are 2D copies with a unit's stack as the pitch;
    // beyond the device's largest pitch whole batches go in and out instead
    int max_pitch = 0;
    MSK_CUDA(ctx, cudaDeviceGetAttribute(&max_pitch, cudaDevAttrMaxPitch, ctx->device));
    const bool by_slice = vb <= (size_t)max_pitch;
    MSK_CUDA(ctx, ctx->fresnel.reserve((adjoint ? 2 : 1) * pb));

    const SizeOps *rop = size_ops(ny), *cop = size_ops(nx);
    // one view per grid buffer the column passes touch and tile variant
    const int vmask = col_variant(ctx, gp, kColMask), vprop = col_variant(ctx, gp, kColProp),
              vfres = col_variant(ctx, gp, kColFresnel), rv = row_variant(ctx, gp);
    // (views of every variant the tuner chose for these passes; indexed by variant)
    std::vector<ColView> maps[kColVariants];
    for (int v : {vmask, vprop, vfres}) {
        if (v < 0 || v >= cop->col_nv) return fail(ctx, MSK_ECUDA, "column variant out of range");
        if (!maps[v].empty()) continue;
        maps[v].resize(planes);
        for (int i = 0; i < planes; i++) {
            st = column_map(ctx, &maps[v][i], grid_at(i), nx, ny, B, cop, v);
            if (st) return st;
        }
    }
    auto map_of = [&](const float2 *p, int v) -> const ColView & {
        return maps[v][(size_t)(p - base) / ((size_t)B * plane)];
    };
    const double P = (double)plane;
    const float tscale = 1.0f / (float)ny;  // scattered-form transmit: S(n phi') / ny
    // loss partials: one per row-pass CTA (at most one per row) and defocus
    // (every batch's, kept on the device and summed on the host at the end)
    if (adjoint)
        MSK_CUDA(ctx, ctx->stk_part.reserve((size_t)ndef * J.nunits * nx * sizeof(double)));
    std::vector<double> partial_host;
    double loss = 0.0;
    int part_off = 0;

    // the host inputs of batch b into its staging slot, on the copy-in stream
    // once the kernels of batch b - nslot (the slot's last reader) are done;
    // v slice by slice, each slice of every unit of the batch one 2D copy
    // (rows: the units, S planes apart)
    auto upload = [&](int b) -> int {
        const int u0 = b * B, nb = std::min(B, J.nunits - u0);
        if (host_io && b >= nslot) MSK_CUDA(ctx, cudaStreamWaitEvent(cin, ev_done[b % nslot], 0));
        if (!v_dev) {
            float *dst = slot_of(ctx->stk_v, vb, b);
            if (!by_slice)
                MSK_CUDA(ctx, cudaMemcpyAsync(dst, J.v + (size_t)u0 * S * plane, nb * vb,
                                              cudaMemcpyHostToDevice, cin));
            for (int k = 0; k < S; k++) {
                if (by_slice && v_map)
                    k_copy_rows<<<kCopyCtas, 256, 0, cin>>>(v_map + ((size_t)u0 * S + k) * plane,
                                                            (size_t)S * plane, dst + (size_t)k * plane,
                                                            (size_t)S * plane, plane, nb);
                else if (by_slice)
                    MSK_CUDA(ctx, cudaMemcpy2DAsync(dst + (size_t)k * plane, vb,
                                                    J.v + ((size_t)u0 * S + k) * plane, vb,
                                                    plane * sizeof(float), nb,
                                                    cudaMemcpyHostToDevice, cin));
                MSK_CUDA(ctx, cudaEventRecord(ev_sin[k], cin));
            }
            count_copy(ctx, 0, (double)nb * vb);
        }
        if (adjoint && !t_dev) {
            if (t_map)
                k_copy_rows<<<kCopyCtas, 256, 0, cin>>>(t_map + (size_t)u0 * ndef * plane, 0,
                                                        slot_of(ctx->stk_t, ib, b), 0,
                                                        (size_t)nb * ib / sizeof(float), 1);
            else
                MSK_CUDA(ctx, cudaMemcpyAsync(slot_of(ctx->stk_t, ib, b),
                                              J.target + (size_t)u0 * ndef * plane, nb * ib,
                                              cudaMemcpyHostToDevice, cin));
            count_copy(ctx, 0, (double)nb * ib);
        }
        if (host_io) MSK_CUDA(ctx, cudaEventRecord(ev_in[b % nslot], cin));
        return MSK_OK;
    };
    if (host_io) {  // the copies start after the work already queued on the library's stream
        MSK_CUDA(ctx, cudaEventRecord(ctx->stk_ev[6], ctx->stream));
        MSK_CUDA(ctx, cudaStreamWaitEvent(cin, ctx->stk_ev[6], 0));
        MSK_CUDA(ctx, cudaStreamWaitEvent(cout, ctx->stk_ev[6], 0));
    }
    if ((st = upload(0))) return st;

    for (int b = 0; b < nbat; b++) {
        const int u0 = b * B, nb = std::min(B, J.nunits - u0), sl = b % nslot;
        // the slot's outputs of batch b - nslot copied out before they are overwritten
        if (host_io && b >= nslot) MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev_out[sl], 0));
        const float *vd = v_dev ? J.v + (size_t)u0 * S * plane : slot_of(ctx->stk_v, vb, b);
        const size_t ustride = (size_t)S * plane;
        auto vslice = [&](int k) { return vd + (size_t)(k - 1) * plane; };  // k = 1..S
        // P1 + P2 of slice k into buffer `dst`
        auto transmission = [&](int k, float2 *dst) {
            {
                Prof p(ctx, kExpv, 12.0 * P * nb);
                rop->row_expv(g, nb, vslice(k), ustride, dst, ctx->stream);
            }
            Prof p(ctx, kKColMask, 16.0 * P * nb);
            cop->col_mask(g, map_of(dst, vmask), map_of(dst, vmask), nullptr, nb, 1, 1.0f,
                          ctx->stream);
        };
        // P3 + P4 of one slice: out = W(K[p](iS(in) t))
        auto step = [&](const float2 *tb, const float2 *in, float2 *out) {
            {
                Prof p(ctx, kTransmit, 24.0 * P * nb);
                rop->row_transmit_scat(g, nullptr, nb, tb, in, out, tscale, 1, rv, ctx->stream);
            }
            Prof p(ctx, kKColProp, 16.0 * P * nb);
            cop->col_prop(g, map_of(out, vprop), map_of(out, vprop), nullptr, nb, 1,
                          ctx->stream);  // W0 in band
        };

        // the wave buffers start as zeros: the band-mode transmit stores only
        // in-band row segments, and W_0 = S(phi_0) = 0 (psi_0 = 1, the
        // scattered form); checkpoints W_{bK} (or every wave and
        // transmission) kept for the backward pass.  Keeping everything, only
        // the S + 1 wave planes (the transmissions' row pass writes whole rows).
        if (keep)
            MSK_CUDA(ctx, cudaMemsetAsync(waves[0], 0, (size_t)(S + 1) * B * pb, ctx->stream));
        else
            MSK_CUDA(ctx, cudaMemsetAsync(base, 0, (size_t)planes * B * pb, ctx->stream));
        for (int k = 1; k <= S; k++) {
            if (!v_dev) MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev_sin[k - 1], 0));
            if (keep) {
                transmission(k, trans[k - 1]);
                step(trans[k - 1], waves[k - 1], waves[k]);
                continue;
            }
            const float2 *in = (adjoint && (k - 1) % K == 0) ? ck[(k - 1) / K] : W;
            float2 *out = (adjoint && k % K == 0 && k < S) ? ck[k / K] : W;
            transmission(k, Bt);
            step(Bt, in, out);
        }
        // the next batch's inputs go in while this one runs (after this batch's
        // waits on the per-slice events are queued)
        if (b + 1 < nbat && (st = upload(b + 1))) return st;
        if (host_io) MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev_in[sl], 0));  // the target

        // free space to every detector plane; images or the loss and its gradient
        float *img_d = nullptr;
        if (!adjoint && ndef > 0)
            img_d = i_dev ? J.images + (size_t)u0 * ndef * plane : slot_of(ctx->stk_img, ib, b);
        const float *tgt = nullptr;
        if (adjoint) tgt = t_dev ? J.target + (size_t)u0 * ndef * plane : slot_of(ctx->stk_t, ib, b);
        int nparts = 0;
        for (int d = 0; d < ndef; d++) {
            float2 *tab = ctx->fresnel.as<float2>();
            Fresnel fr = stack_fresnel(ctx, gp, s, J.defocus[d], 1.0);
            fr.table = tab;
            {
                Prof p(ctx, kFresTab, 8.0 * P);
                k_fresnel_table<<<4 * 152, 256, 0, ctx->stream>>>(
                    g, fr, 1.0f / ((float)nx * (float)ny), tab);
            }
            {
                Prof p(ctx, kFresnel, 16.0 * P * nb);
                cop->col_fresnel(g, map_of(W, vfres), map_of(E, vfres), nullptr, nb, fr, 1.0f,
                                 ctx->stream);
            }
            if (!adjoint) {
                // images[u][d] = |1 + iS(E)|^2: one image per unit, no averaging
                std::vector<int> meta;
                for (int i = 0; i <= nb; i++) meta.push_back(i);          // img_off
                for (int i = 0; i < nb; i++) meta.push_back(i);           // img_units
                for (int i = 0; i < nb; i++) meta.push_back(i * ndef + d);  // img_dst
                for (int i = 0; i < nb; i++) meta.push_back(0);           // img_flags
                MSK_CUDA(ctx, ctx->imgmeta.reserve(meta.size() * sizeof(int) * ndef));
                int *dm = ctx->imgmeta.as<int>() + (size_t)d * meta.size();
                MSK_CUDA(ctx, cudaMemcpyAsync(dm, meta.data(), meta.size() * sizeof(int),
                                              cudaMemcpyHostToDevice, ctx->stream));
                count_copy(ctx, 0, (double)(meta.size() * sizeof(int)));
                Prof p(ctx, kIntensity, 12.0 * P * nb);
                rop->row_intensity_scat(g, nb, dm, dm + nb + 1, dm + 2 * nb + 1, dm + 3 * nb + 1,
                                        E, img_d, 1.0f, ctx->stream);
                continue;
            }
            // G_d = W(2 (I - T) psi), in place in E; partial sums of the loss
            int np = 0;
            {
                Prof p(ctx, kImGrad, 20.0 * P * nb);
                np = rop->row_imgrad(g, nb, E, tgt + (size_t)d * plane, (size_t)ndef * plane, E,
                                     ctx->stk_part.as<double>() + part_off + nparts, ctx->stream);
            }
            nparts += np;
            // g_psiS += K[conj X] g_phi: conjugate table with the column 1/nx
            Fresnel fc = stack_fresnel(ctx, gp, s, J.defocus[d], -1.0);
            fc.table = tab + plane;
            {
                Prof p(ctx, kFresTab, 8.0 * P);
                k_fresnel_table<<<4 * 152, 256, 0, ctx->stream>>>(g, fc, 1.0f / (float)nx,
                                                                   tab + plane);
            }
            {
                Prof p(ctx, kFresnel, 16.0 * P * nb);
                cop->col_fresnel(g, map_of(E, vfres), map_of(d == 0 ? G : E, vfres), nullptr, nb, fc, 1.0f,
                                 ctx->stream);
            }
            if (d > 0) {
                Prof p(ctx, kAccum, 24.0 * P * nb);
                k_add_waves<<<8 * 152, 256, 0, ctx->stream>>>(G, E, (size_t)nb * plane);
            }
        }

        if (adjoint) {
            float *gd = g_dev ? J.grad + (size_t)u0 * S * plane : slot_of(ctx->stk_g, vb, b);
            // dL/dv_k of every unit of the batch to the host (one 2D copy) once written
            auto grad_out = [&](int k) -> int {
                if (g_dev || !by_slice) return MSK_OK;
                MSK_CUDA(ctx, cudaEventRecord(ev_sout[k - 1], ctx->stream));
                MSK_CUDA(ctx, cudaStreamWaitEvent(cout, ev_sout[k - 1], 0));
                if (g_map)
                    k_copy_rows<<<kCopyCtas, 256, 0, cout>>>(gd + (size_t)(k - 1) * plane,
                                                             (size_t)S * plane,
                                                             g_map + ((size_t)u0 * S + (k - 1)) * plane,
                                                             (size_t)S * plane, plane, nb);
                else
                    MSK_CUDA(ctx, cudaMemcpy2DAsync(J.grad + ((size_t)u0 * S + (k - 1)) * plane, vb,
                                                    gd + (size_t)(k - 1) * plane, vb,
                                                    plane * sizeof(float), nb, cudaMemcpyDeviceToHost,
                                                    cout));
                return MSK_OK;
            };
            // backward with every wave and transmission kept: slice by slice
            for (int k = keep ? S : 0; k >= 1; k--) {
                {
                    Prof p(ctx, kKColProp, 16.0 * P * nb);  // g_u = K[conj p] g_psi
                    cop->col_prop(gc, map_of(G, vprop), map_of(G, vprop), nullptr, nb, 0,
                                  ctx->stream);
                }
                {
                    Prof p(ctx, kAdjTransmit, 40.0 * P * nb);
                    rop->row_adj_transmit(g, nb, G, trans[k - 1], waves[k - 1], ctx->stream);
                }
                {
                    Prof p(ctx, kKColMask, 16.0 * P * nb);  // g_e = K[M] g_t
                    cop->col_mask(g, map_of(trans[k - 1], vmask), map_of(trans[k - 1], vmask),
                                  nullptr, nb, 0, 1.0f, ctx->stream);
                }
                {
                    Prof p(ctx, kGrad, 16.0 * P * nb);
                    rop->row_grad(g, nb, trans[k - 1], vslice(k), ustride,
                                  gd + (size_t)(k - 1) * plane, ctx->stream);
                }
                if ((st = grad_out(k))) return st;
            }
            // backward, one checkpoint block at a time from the last
            for (int blk = keep ? -1 : nblk - 1; blk >= 0; blk--) {
                const int k0 = blk * K, nj = std::min(S, k0 + K) - k0;
                for (int j = 1; j <= nj; j++) {  // recompute the block's t_k and psi_k
                    transmission(k0 + j, Bb[j - 1]);
                    if (j < nj) step(Bb[j - 1], j == 1 ? ck[blk] : Wb[j - 2], Wb[j - 1]);
                }
                for (int j = nj; j >= 1; j--) {
                    const int k = k0 + j;
                    {
                        Prof p(ctx, kKColProp, 16.0 * P * nb);  // g_u = K[conj p] g_psi
                        cop->col_prop(gc, map_of(G, vprop), map_of(G, vprop), nullptr, nb, 0,
                                      ctx->stream);
                    }
                    {
                        Prof p(ctx, kAdjTransmit, 40.0 * P * nb);
                        rop->row_adj_transmit(g, nb, G, Bb[j - 1], j == 1 ? ck[blk] : Wb[j - 2],
                                              ctx->stream);
                    }
                    {
                        Prof p(ctx, kKColMask, 16.0 * P * nb);  // g_e = K[M] g_t
                        cop->col_mask(g, map_of(Bb[j - 1], vmask), map_of(Bb[j - 1], vmask), nullptr, nb, 0,
                                      1.0f, ctx->stream);
                    }
                    {
                        Prof p(ctx, kGrad, 16.0 * P * nb);
                        rop->row_grad(g, nb, Bb[j - 1], vslice(k), ustride,
                                      gd + (size_t)(k - 1) * plane, ctx->stream);
                    }
                    if ((st = grad_out(k))) return st;
                }
            }
        }
        part_off += nparts;
        // the host outputs of batch b, on the copy-out stream once its kernels are done
        if (host_io) {
            MSK_CUDA(ctx, cudaEventRecord(ev_done[sl], ctx->stream));
            MSK_CUDA(ctx, cudaStreamWaitEvent(cout, ev_done[sl], 0));
            if (adjoint && !g_dev) {
                if (!by_slice)
                    MSK_CUDA(ctx, cudaMemcpyAsync(J.grad + (size_t)u0 * S * plane,
                                                  slot_of(ctx->stk_g, vb, b), nb * vb,
                                                  cudaMemcpyDeviceToHost, cout));
                count_copy(ctx, 1, (double)nb * vb);  // (by slice: copied as written)
            }
            if (!adjoint && ndef > 0 && !i_dev) {
                MSK_CUDA(ctx, cudaMemcpyAsync(J.images + (size_t)u0 * ndef * plane, img_d, nb * ib,
                                              cudaMemcpyDeviceToHost, cout));
                count_copy(ctx, 1, (double)nb * ib);
            }
            MSK_CUDA(ctx, cudaEventRecord(ev_out[sl], cout));
        }
        MSK_CUDA(ctx, cudaGetLastError());
    }
    if (host_io) {
        MSK_CUDA(ctx, cudaStreamSynchronize(cin));
        MSK_CUDA(ctx, cudaStreamSynchronize(cout));
    }
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    if (adjoint) {
        partial_host.resize(part_off);
        MSK_CUDA(ctx, cudaMemcpy(partial_host.data(), ctx->stk_part.p, part_off * sizeof(double),
                                 cudaMemcpyDeviceToHost));
        count_copy(ctx, 1, (double)part_off * sizeof(double));
        for (int i = 0; i < part_off; i++) loss += partial_host[i];  // fixed order
    }
    if (J.loss) *J.loss = loss;
    return flags_check(ctx);
}

}  // namespace

extern "C" {

int msk_stack_images(msk_context *ctx, const msk_stack *s, int nunits, const float *v,
                     int ndefocus, const double *defocus, float *images)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    StackJob J{s, nunits, ndefocus, v, defocus, nullptr, images, nullptr, nullptr};
    return stack_run(ctx, J);
}

int msk_adjoint(msk_context *ctx, const msk_stack *s, int nunits, const float *v,
                      int ndefocus, const double *defocus, const float *target, float *grad,
                      double *loss)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!grad) return fail(ctx, MSK_EINVAL, "grad is required");
    StackJob J{s, nunits, ndefocus, v, defocus, target, nullptr, grad, loss};
    return stack_run(ctx, J);
}

int msk_potential_stack(msk_context *ctx, const msk_series *s, int natom, const int *Znum,
                        const float *x, const float *y, const float *z, const float *occ,
                        int nangles, const double *angleZ, const double *angleY, float *v,
                        int *kept)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!s || natom < 0 || nangles < 1 || !angleZ || !angleY || !v ||
        (natom > 0 && (!Znum || !x || !y || !z || !occ)))
        return fail(ctx, MSK_EINVAL, "bad potential-stack arguments");
    const int nx = s->nx, ny = s->ny;
    if (nx < 1 || ny < 1 || s->ctblength < 0.0f) return fail(ctx, MSK_EBADSIZE, "bad size parameters");
    if (!pow2_supported(nx) || !pow2_supported(ny))
        return fail(ctx, MSK_EUNSUPPORTED, "grid must be a power of two from 16 to 4096");
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    GridPre gp;
    if (!grid_pre(gp, nx, ny, s->ctblength, s->ctblength, s->v0, s->deltaz, 0.0f, 0.0f))
        return fail(ctx, MSK_EUNSUPPORTED, "band limit is not two index ranges per column");
    const int nslices = slice_count(s->deltaz, s->ctblengthz);
    std::vector<int> zlist;
    int st = build_zmap(ctx, natom, Znum, zlist);
    if (st) return st;
    st = upload_tables(ctx, gp, zlist);
    if (st) return st;
    st = flags_reset(ctx, gp.g);
    if (st) return st;
    const size_t plane = (size_t)nx * ny;
    const size_t ub = (size_t)nslices * plane * sizeof(float);  // one orientation's stack
    const bool v_dev = is_device_ptr(v);
    int B = nangles;
    if (!v_dev) {
        size_t free_b = 0, total_b = 0;
        MSK_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
        const size_t budget = std::min<size_t>(free_b / 2, (size_t)64 << 30);
        B = (int)std::max<size_t>(1, std::min<size_t>(nangles, budget / ub));
        if (s->max_batch > 0) B = std::min(B, s->max_batch);
        MSK_CUDA(ctx, ctx->stk_v.reserve((size_t)B * ub));
    }
    const SizeOps *rop = size_ops(ny);
    std::vector<UnitAtoms> ua(nangles);
    for (int u0 = 0; u0 < nangles; u0 += B) {
        const int nb = std::min(B, nangles - u0);
        parallel_for(nb, host_threads(), [&](int i) {
            const int a = u0 + i;
            PrepSpec ps{natom, Znum, x, y, z, occ, s->ctblength, s->ctblengthz, s->deltaz,
                        nslices, true, angleZ[a], angleY[a], s->dxc, s->dyc, s->dzc, nullptr,
                        true, ctx->zmap.data()};
            prep_unit(gp, ps, ua[a]);
        });
        for (int i = 0; i < nb; i++)
            if (ua[u0 + i].status)
                return fail(ctx, ua[u0 + i].status, msk_status_string(ua[u0 + i].status));
        Batch b;
        st = upload_batch(ctx, ua, u0, nb, nslices, b);
        if (st) return st;
        float *vd = v_dev ? v + (size_t)u0 * nslices * plane : ctx->stk_v.as<float>();
        MSK_CUDA(ctx, cudaMemsetAsync(vd, 0, nb * ub, ctx->stream));
        for (int sl = 0; sl < nslices; sl++) {
            const int na = b.act_off[sl + 1] - b.act_off[sl];
            if (na == 0) continue;
            Prof p(ctx, kSplat, 4.0 * plane * na);
            rop->splat_potential(gp.g, ctx->act.as<int>() + b.act_off[sl], na, sl, nslices + 1,
                                 ctx->slice_off.as<int>(), ctx->atoms.as<SplatAtom>(),
                                 vd + (size_t)sl * plane, (size_t)nslices * plane, ctx->stream);
        }
        if (!v_dev) {
            MSK_CUDA(ctx, cudaMemcpyAsync(v + (size_t)u0 * nslices * plane, vd, nb * ub,
                                          cudaMemcpyDeviceToHost, ctx->stream));
            count_copy(ctx, 1, (double)nb * ub);
        }
        MSK_CUDA(ctx, cudaGetLastError());
        MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        prof_collect(ctx);
    }
    if (kept)
        for (int a = 0; a < nangles; a++) kept[a] = ua[a].kept;
    return flags_check(ctx);
}

}  // extern "C"

// ------------------------------------------------------------------ specimen batches
// msk_tilt_series_batch: many specimens -- each with its own atoms, box, grid
// and orientations -- in one call.  Every specimen keeps its own tables,
// atoms, waves and images in one device arena; specimens are spread over
// concurrent streams (longest first onto the least-loaded stream) and, with
// MSK_BATCH_GRAPH, the whole launch sequence is captured into one CUDA graph
// and launched once.

namespace {

constexpr int kLanes = 8;

// Detector planes of one specimen that share their free-space and image-plane
// parameters: one multiplier table and one pass over the group's units.
struct ImgGroup {
    double defocus, astig, astig_angle, rotation;
    int sxp, syp;   // whole-pixel image shift
    int nimg, nu;   // images (orientations) and units of the group
    bool all;       // every unit of the specimen, in order: passes take no unit list
    size_t o_meta;  // in the meta: img_off[nimg + 1] | img_units[nu] | img_dst[nimg] | img_flags[nimg]
};

bool same_plane(const ImgGroup &a, const ImgGroup &b)
{
    return a.defocus == b.defocus && a.astig == b.astig && a.astig_angle == b.astig_angle &&
           a.rotation == b.rotation && a.sxp == b.sxp && a.syp == b.syp;
}

// The detector planes of one specimen's units (u = a * nc + c), grouped as
// msk_tilt_series groups them: the k-th plane of every orientation that has
// one, by equal parameters.
void group_planes(const PlaneList &pl, int na, int nc, double xst, double yst,
                  std::vector<ImgGroup> &groups, std::vector<int> &meta)
{
    groups.clear();
    meta.clear();
    int kmax = 0;
    for (int a = 0; a < na; a++) kmax = std::max(kmax, pl.off[a + 1] - pl.off[a]);
    for (int k = 0; k < kmax; k++) {
        const size_t g0 = groups.size();
        std::vector<std::vector<int>> ori;
        for (int a = 0; a < na; a++) {
            if (pl.off[a + 1] - pl.off[a] <= k) continue;
            const PlaneDesc &d = pl.p[pl.off[a] + k];
            ImgGroup key{};
            key.defocus = d.defocus;
            key.astig = d.astig;
            key.astig_angle = d.astig_angle;
            key.rotation = d.rotation;
            key.sxp = (int)floor(pl.shift[2 * a] / xst + 0.5);
            key.syp = (int)floor(pl.shift[2 * a + 1] / yst + 0.5);
            size_t gi = g0;
            while (gi < groups.size() && !same_plane(groups[gi], key)) gi++;
            if (gi == groups.size()) {
                groups.push_back(key);
                ori.emplace_back();
            }
            ori[gi - g0].push_back(a);
        }
        for (size_t j = 0; j < ori.size(); j++) {
            ImgGroup &gr = groups[g0 + j];
            gr.nimg = (int)ori[j].size();
            gr.nu = gr.nimg * nc;
            gr.all = gr.nimg == na;
            gr.o_meta = meta.size();
            for (int i = 0; i <= gr.nimg; i++) meta.push_back(i * nc);           // img_off
            for (int a : ori[j])
                for (int c = 0; c < nc; c++) meta.push_back(a * nc + c);          // img_units
            for (int a : ori[j]) meta.push_back(pl.off[a] + k);                   // img_dst
            for (size_t i = 0; i < ori[j].size(); i++) meta.push_back(nc > 1 ? 2 : 0);  // mean
        }
    }
}

struct SpecPlan {
    GridPre gp;
    int nslices = 0, nangles = 0;
    int nconf = 1, nunits = 0;  // thermal configurations per orientation; units = both
    std::vector<UnitAtoms> ua;
    Batch b;
    std::vector<SplatAtom> atoms;
    std::vector<unsigned char> tables;
    TableLayout tl;
    std::vector<ImgGroup> groups;  // detector planes
    std::vector<int> meta;         // the groups' image lists
    int nimages = 0;               // images of the specimen
    bool image_plane = false;      // some plane rotated or shifted
    float ctblength = 0.0f, ctblengthz = 0.0f;
    std::vector<float2> wave0;  // spherical incident wave (empty: a plane wave)
    size_t o_tab = 0, o_atoms = 0, o_soff = 0, o_act = 0, o_meta = 0, o_w0 = 0;  // upload region
    size_t o_fres = 0, o_psi = 0, o_tbuf = 0, o_img = 0, o_phi = 0, o_fill = 0;  // work region
    size_t o_dw = 0, o_spec = 0;  // Debye-Waller branch: -B/4 per (unit, slice); S(v) grids
    bool small = false;      // the slice loop as one cluster launch (msk_small.cuh)
    size_t o_tbuf2 = 0;      // its second transmission buffer
    bool img_dev = false;
    bool img_pinned = false;  // host images in page-locked memory: copied on the lane
    float *ew = nullptr;      // exit waves out (may be null)
    bool ew_dev = false, ew_pinned = false;
    size_t o_ew = 0;          // work region: pageable-host exit waves, staged
    double work = 0.0;
    int lane = 0;
};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int ensure_lanes(msk_context *ctx)
{
    while ((int)ctx->lanes.size() < kLanes) {
        cudaStream_t l = nullptr;
        MSK_CUDA(ctx, cudaStreamCreateWithFlags(&l, cudaStreamNonBlocking));
        ctx->lanes.push_back(l);
    }
    while ((int)ctx->lane_ev.size() < kLanes + 1) {
        cudaEvent_t e = nullptr;
        MSK_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->lane_ev.push_back(e);
    }
    return MSK_OK;
}

// The launches of one specimen on one stream: plane wave, slice loop, then
// per group of detector planes the free-space step and the intensity.
int enqueue_specimen(msk_context *ctx, SpecPlan &P, unsigned char *arena, const msk_series *s,
                     float *d_images, cudaStream_t st)
{
    const GridPre &gp = P.gp;
    const Geom &g = gp.g;
    // units u = a * nconf + c (orientation a, configuration c); images per orientation
    const int nx = gp.nx, ny = gp.ny, na = P.nunits, nconf = P.nconf;
    const size_t plane = (size_t)nx * ny;
    const SizeOps *rop = size_ops(ny), *cop = size_ops(nx);
    float2 *psi = reinterpret_cast<float2 *>(arena + P.o_psi);
    float2 *tb = reinterpret_cast<float2 *>(arena + P.o_tbuf);
    const int *act = reinterpret_cast<const int *>(arena + P.o_act);
    const int *soff = reinterpret_cast<const int *>(arena + P.o_soff);
    const SplatAtom *atoms = reinterpret_cast<const SplatAtom *>(arena + P.o_atoms);
    // views for each pass's tile variant (chosen before any capture begins)
    const int vm = col_variant(ctx, gp, kColMask), vp = col_variant(ctx, gp, kColProp),
              vf = col_variant(ctx, gp, kColFresnel), rv = row_variant(ctx, gp);
    ColView pmap, tmap, pmapf, tmapf, smap;
    int rc = column_map(ctx, &pmap, psi, nx, ny, na, cop, vp);
    if (rc) return rc;
    rc = column_map(ctx, &tmap, tb, nx, ny, na, cop, vm);
    if (rc) return rc;
    rc = column_map(ctx, &pmapf, psi, nx, ny, na, cop, vf);
    if (rc) return rc;
    rc = column_map(ctx, &tmapf, tb, nx, ny, na, cop, vf);
    if (rc) return rc;
    // Debye-Waller branch (trlayerDW): S(v) of each unit in its own grid
    const bool dw = !P.b.dw.empty();
    float2 *spec = reinterpret_cast<float2 *>(arena + P.o_spec);
    const float *dwf = reinterpret_cast<const float *>(arena + P.o_dw);
    if (dw && (rc = column_map(ctx, &smap, spec, nx, ny, na, cop, col_variant(ctx, gp, kColDW))))
        return rc;
    const double pl = (double)plane;
    // incident wave: a plane wave (in band from the start) or the specimen's
    // spherical wave (in band after the first propagator pass), as msk_tilt_series
    bool w_in_band = P.wave0.empty();
    if (w_in_band) {
        Prof p(ctx, kPlane, 8.0 * pl * na, st);
        k_plane_init<<<1024, 256, 0, st>>>(psi, nullptr, na, nx, ny);
    } else {
        Prof p(ctx, kInit, 8.0 * pl * (na + 1), st);
        rop->row_init(g, nullptr, na, reinterpret_cast<const float2 *>(arena + P.o_w0), psi, 1.0f,
                      st);
    }
    const int nsl1 = P.nslices + 1;
    if (P.small) {  // every slice of every unit in one cluster launch, as run_slices
        const double ne = P.b.act_off[P.nslices], all = (double)na * P.nslices;
        Prof p(ctx, kSmall, pl * (64.0 * ne + 16.0 * (all - ne)), st);
        MSK_CUDA(ctx, cop->small_slices(g, na, P.nslices, nsl1, soff, atoms, psi, tb,
                                        reinterpret_cast<float2 *>(arena + P.o_tbuf2), st));
    }
    for (int sl = 0; sl < (P.small ? 0 : P.nslices); sl++) {
        const int nact = P.b.act_off[sl + 1] - P.b.act_off[sl];
        const int *units = act + P.b.act_off[sl];
        if (nact > 0) {
            if (dw) {  // S(v), the damping, then A = S(exp(i sigma v')), as run_slices
                {
                    Prof p(ctx, kSplat, 8.0 * pl * nact, st);
                    rop->splat_spec(g, units, nact, sl, nsl1, soff, atoms, spec, st);
                }
                {
                    Prof p(ctx, kDW, 16.0 * pl * nact, st);
                    cop->col_dw(g, smap, units, nact, dwf + sl, P.nslices, st);
                }
                Prof p(ctx, kDWExp, 16.0 * pl * nact, st);
                rop->row_dwexp(g, units, nact, spec, tb, st);
            } else {
                Prof p(ctx, kSplat, 8.0 * pl * nact, st);
                rop->splat(g, units, nact, sl, nsl1, soff, atoms, tb, st);
            }
            {
                Prof p(ctx, kKColMask, 16.0 * pl * nact, st);
                // B = S(t_bl) / ny^2: the transmit's 1/ny^2, exact, carried here
                cop->col_mask(g, tmap, tmap, units, nact, 1, 1.0f / ((float)ny * (float)ny), st);
            }
            Prof p(ctx, kTransmit, 24.0 * pl * nact, st);
            rop->row_transmit(g, units, nact, tb, psi, psi, 1.0f, s->nmode == 0 && w_in_band, rv,
                              st);
        }
        if (s->nmode == 0) {
            Prof p(ctx, kKColProp, 16.0 * pl * na, st);
            cop->col_prop(g, pmap, pmap, nullptr, na, w_in_band ? 1 : 0, st);
            w_in_band = true;
        }
    }
    // exit waves (psi = iS(W)/ny): into a device destination directly, else
    // through the transmission buffer (free until the free-space step) to
    // page-locked host memory on this stream or to the arena for a later copy
    if (P.ew) {
        const size_t ewb = (size_t)na * plane * sizeof(float2);
        float2 *dst = P.ew_dev ? reinterpret_cast<float2 *>(P.ew) : tb;
        {
            Prof p(ctx, kExit, 16.0 * pl * na, st);
            rop->row_exit(g, nullptr, na, psi, dst, st);
        }
        if (P.ew_pinned) {
            MSK_CUDA(ctx, cudaMemcpyAsync(P.ew, tb, ewb, cudaMemcpyDeviceToHost, st));
            count_copy(ctx, 1, (double)ewb);
        } else if (!P.ew_dev) {
            MSK_CUDA(ctx, cudaMemcpyAsync(arena + P.o_ew, tb, ewb, cudaMemcpyDeviceToDevice, st));
        }
    }
    // image plane (autosliccmd.cpp:1119-1143): rotation centre
    const double xst = P.ctblength / nx, yst = P.ctblength / ny;  // float divisions
    const double xcen = 0.5 * P.ctblength + s->dxc, ycen = 0.5 * P.ctblength + s->dyc;
    const double pi = 4.0 * atan(1.0), l = gp.wavlen;
    float k2maxo = s->aobj / gp.wavlen;
    k2maxo = k2maxo * k2maxo;
    const int *meta = reinterpret_cast<const int *>(arena + P.o_meta);
    for (size_t gi = 0; gi < P.groups.size(); gi++) {
        const ImgGroup &gr = P.groups[gi];
        const int ni = gr.nimg, nu = gr.nu;
        Fresnel fr{};
        const double rprime = gr.defocus - 0.5 * P.ctblengthz;  // autosliccmd.cpp:1060
        fr.a1 = pi * l * rprime;
        fr.a3 = (pi / 2.0) * s->cs3 * l * l * l;
        fr.a5 = (pi / 3.0) * s->cs5 * l * l * l * l * l;
        fr.a2c = (pi / 2.0) * l * gr.astig * cos(2.0 * gr.astig_angle);
        fr.a2s = (pi / 2.0) * l * gr.astig * sin(2.0 * gr.astig_angle);
        fr.k2maxo = k2maxo;
        fr.kx = gp.d_kx;
        fr.ky = gp.d_ky;
        float2 *tab = reinterpret_cast<float2 *>(arena + P.o_fres) + gi * plane;
        fr.table = tab;
        // a group of every unit in order takes no unit list
        const int *d_off = meta + gr.o_meta, *d_units = d_off + ni + 1,
                  *d_dst = d_units + nu, *d_flags = d_dst + ni;
        const int *ulist = gr.all ? nullptr : d_units;
        {
            Prof p(ctx, kFresTab, 8.0 * pl, st);
            k_fresnel_table<<<4 * 152, 256, 0, st>>>(g, fr, 1.0f / ((float)nx * (float)ny), tab);
        }
        {
            Prof p(ctx, kFresnel, 16.0 * pl * nu, st);
            cop->col_fresnel(g, pmapf, tmapf, ulist, nu, fr, 1.0f, st);
        }
        const double rot = gr.rotation;
        if (rot != 0.0 || gr.sxp != 0 || gr.syp != 0) {
            // the amplitude in real space, rotated and shifted, then |.|^2
            float2 *phi = reinterpret_cast<float2 *>(arena + P.o_phi);
            float2 *fill = reinterpret_cast<float2 *>(arena + P.o_fill);
            {
                Prof p(ctx, kExit, 16.0 * pl * nu, st);
                rop->row_inverse(g, ulist, nu, tb, phi, 1.0f, st);
            }
            k_edge_mean<<<nu, 256, 0, st>>>(phi, ulist, nx, ny, 5, fill);
            {
                Prof p(ctx, kRotShift, 16.0 * pl * nu, st);
                k_rotate_shift<<<8 * 152, 256, 0, st>>>(phi, tb, ulist, nu, nx, ny, xst, yst, xcen,
                                                        ycen, cos(rot), sin(rot), rot != 0.0,
                                                        gr.sxp, gr.syp, fill);
            }
            Prof p(ctx, kIntensity, 8.0 * pl * nu + 4.0 * pl * ni, st);
            k_intensity_direct<<<8 * 152, 256, 0, st>>>(ni, d_off, d_units, d_dst, d_flags, tb,
                                                        d_images, plane, (float)nconf);
            continue;
        }
        Prof p(ctx, kIntensity, 8.0 * pl * nu + 4.0 * pl * ni, st);
        rop->row_intensity(g, ni, d_off, d_units, d_dst, d_flags, tb, d_images, (float)nconf, st);
    }
    MSK_CUDA(ctx, cudaGetLastError());
    return MSK_OK;
}

}  // namespace

extern "C" int msk_tilt_series_batch(msk_context *ctx, const msk_series *s, int nspec,
                                     const msk_specimen *spec, int ndefocus,
                                     const double *defocus, int flags)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!s || nspec < 1 || !spec || ndefocus < 0 || (ndefocus > 0 && !defocus))
        return fail(ctx, MSK_EINVAL, "bad batch arguments");
    for (int i = 0; i < nspec; i++) {
        const msk_specimen &q = spec[i];
        if (s->lwobble && !(q.nconfig > 1 && q.displacements) && q.natom > 0 && !q.wobble)
            return fail(ctx, MSK_EINVAL, "lwobble needs each specimen's wobble array");
        if (q.nconfig < 0 || (q.nconfig > 1 && !s->lwobble && !q.displacements))
            return fail(ctx, MSK_EINVAL, "several configurations need lwobble = 1 (bad specimen " +
                                             std::to_string(i) + ")");
        if (q.natom < 0 || q.nangles < 1 || !q.angleZ || !q.angleY ||
            (q.natom > 0 && (!q.Znum || !q.x || !q.y || !q.z || !q.occ)))
            return fail(ctx, MSK_EINVAL, "bad specimen " + std::to_string(i));
        int nimg = q.nangles * ndefocus;
        if (q.plane_off) {
            bool ok = q.plane_off[0] == 0;
            for (int a = 0; a < q.nangles && ok; a++) ok = q.plane_off[a + 1] >= q.plane_off[a];
            if (!ok) return fail(ctx, MSK_EINVAL, "bad plane lists of specimen " + std::to_string(i));
            nimg = q.plane_off[q.nangles];
            if (nimg > 0 && !q.planes)
                return fail(ctx, MSK_EINVAL, "bad plane lists of specimen " + std::to_string(i));
        }
        if (nimg > 0 && !q.images) return fail(ctx, MSK_EINVAL, "bad specimen " + std::to_string(i));
        if (q.nx < 1 || q.ny < 1 || q.ctblength < 0.0f)
            return fail(ctx, MSK_EBADSIZE, "bad size parameters of specimen " + std::to_string(i));
        if (!pow2_supported(q.nx) || !pow2_supported(q.ny))
            return fail(ctx, MSK_EUNSUPPORTED, "grid must be a power of two from 16 to 4096");
    }
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = ensure_lanes(ctx);
    if (st) return st;

    // one compact Z map over every specimen
    std::vector<int> allZ;
    for (int i = 0; i < nspec; i++) allZ.insert(allZ.end(), spec[i].Znum, spec[i].Znum + spec[i].natom);
    std::vector<int> zlist;
    st = build_zmap(ctx, (int)allZ.size(), allZ.data(), zlist);
    if (st) return st;

    // host preparation: grids, then every (specimen, orientation) unit in parallel
    std::vector<SpecPlan> P(nspec);
    std::vector<std::pair<int, int>> units;
    for (int i = 0; i < nspec; i++) {
        const msk_specimen &q = spec[i];
        if (!grid_pre(P[i].gp, q.nx, q.ny, q.ctblength, q.ctblength, s->v0, s->deltaz, 0.0f, 0.0f))
            return fail(ctx, MSK_EUNSUPPORTED, "band limit is not two index ranges per column");
        P[i].nslices = slice_count(s->deltaz, q.ctblengthz);
        P[i].nangles = q.nangles;
        P[i].nconf = std::max(1, q.nconfig);
        P[i].nunits = q.nangles * P[i].nconf;
        P[i].ctblength = q.ctblength;
        P[i].ctblengthz = q.ctblengthz;
        P[i].ua.resize(P[i].nunits);
        for (int a = 0; a < q.nangles; a++) units.push_back({i, a});
    }
    parallel_for((int)units.size(), host_threads(), [&](int k) {
        const int i = units[k].first, a = units[k].second;
        const msk_specimen &q = spec[i];
        // the thermal branch as msk_tilt_series chooses it: none without lwobble,
        // Debye-Waller with one configuration, none with given displacements, else
        // random displacements, orientation a's configurations in order from seed - a
        long seed = s->seed - a;
        const int nc = P[i].nconf;
        const int thermal = !s->lwobble ? kThermNone
                            : nc == 1 ? kThermDW
                            : q.displacements ? kThermNone : kThermRandom;
        for (int c = 0; c < nc; c++) {
            const float *disp =
                q.displacements ? q.displacements + (size_t)c * 3 * q.natom : nullptr;
            PrepSpec ps{q.natom, q.Znum, q.x, q.y, q.z, q.occ, q.ctblength, q.ctblengthz,
                        s->deltaz, P[i].nslices, true, q.angleZ[a], q.angleY[a], s->dxc, s->dyc,
                        s->dzc, disp, true, ctx->zmap.data()};
            if (thermal != kThermNone) {
                ps.thermal = thermal;
                ps.wobble = q.wobble;
                ps.temperature = s->temperature;
                ps.iseed = thermal == kThermRandom ? &seed : nullptr;
            }
            prep_unit(P[i].gp, ps, P[i].ua[(size_t)a * P[i].nconf + c]);
        }
    });
    for (int i = 0; i < nspec; i++)
        for (int u = 0; u < P[i].nunits; u++)
            if (P[i].ua[u].status)
                return fail(ctx, P[i].ua[u].status, "specimen " + std::to_string(i) + ": " +
                                                         msk_status_string(P[i].ua[u].status));
    parallel_for(nspec, host_threads(), [&](int i) {
        SpecPlan &q = P[i];
        build_tables(q.gp, zlist, q.tables, q.tl);
        pack_batch(q.ua, 0, q.nunits, q.nslices, q.b, q.atoms);
        // detector planes: the specimen's own lists, else the call's defoci with
        // s's image plane for every orientation (as msk_tilt_series builds them)
        const msk_specimen &sp = spec[i];
        const int na = q.nangles, nc = q.nconf;
        PlaneList pl;
        for (int a = 0; a <= na; a++) pl.off.push_back(sp.plane_off ? sp.plane_off[a] : a * ndefocus);
        pl.total = pl.off[na];
        for (int a = 0; a < na; a++) {
            if (sp.plane_off) {
                for (int k = pl.off[a]; k < pl.off[a + 1]; k++)
                    pl.p.push_back(PlaneDesc{sp.planes[k].defocus, sp.planes[k].rotation,
                                             sp.planes[k].astig, sp.planes[k].astig_angle});
                pl.shift.push_back(sp.shifts ? sp.shifts[2 * a] : 0.0);
                pl.shift.push_back(sp.shifts ? sp.shifts[2 * a + 1] : 0.0);
            } else {
                for (int d = 0; d < ndefocus; d++)
                    pl.p.push_back(PlaneDesc{defocus[d], s->rotation ? s->rotation[d] : 0.0,
                                             s->astig, s->astig_angle});
                pl.shift.push_back(s->xshift);
                pl.shift.push_back(s->yshift);
            }
        }
        group_planes(pl, na, nc, q.ctblength / q.gp.nx, q.ctblength / q.gp.ny, q.groups, q.meta);
        q.nimages = pl.total;
        q.image_plane = false;
        for (const ImgGroup &gr : q.groups)
            q.image_plane |= gr.rotation != 0.0 || gr.sxp != 0 || gr.syp != 0;
        q.work = (double)q.nunits * q.nslices * q.gp.nx * q.gp.ny;
        q.img_dev = q.nimages > 0 && is_device_ptr(spec[i].images);
        q.img_pinned = q.nimages > 0 && !q.img_dev && is_pinned_host(spec[i].images);
        q.ew = spec[i].exitwaves;
        q.ew_dev = q.ew && is_device_ptr(q.ew);
        q.ew_pinned = q.ew && !q.ew_dev && is_pinned_host(q.ew);
        if (s->R1 != 0.0) spherical_wave(q.gp.nx, q.gp.ny, q.ctblength, s->v0, s->R1, q.wave0);
    });
    // waves of specimens whose arena fits the memory budget
    size_t free_b = 0, total_b = 0;
    MSK_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = (size_t)((double)(free_b + ctx->arena.cap) * 0.8);
    auto arena_of = [&](SpecPlan &q, size_t &up, size_t &work) {
        const size_t plane = (size_t)q.gp.nx * q.gp.ny;
        q.o_tab = up;
        up += align256(q.tables.size());
        q.o_atoms = up;
        up += align256(q.atoms.size() * sizeof(SplatAtom));
        q.o_soff = up;
        up += align256(q.b.slice_off.size() * sizeof(int));
        q.o_act = up;
        up += align256(std::max<size_t>(q.b.act.size(), 1) * sizeof(int));
        q.o_meta = up;
        up += align256(std::max<size_t>(q.meta.size(), 1) * sizeof(int));
        q.o_w0 = up;
        up += align256(q.wave0.size() * sizeof(float2));
        q.o_dw = up;
        up += align256(q.b.dw.size() * sizeof(float));
        q.o_fres = work;
        work += align256(std::max<size_t>(q.groups.size(), 1) * plane * sizeof(float2));
        q.o_psi = work;
        work += align256((size_t)q.nunits * plane * sizeof(float2));
        q.o_tbuf = work;
        work += align256((size_t)q.nunits * plane * sizeof(float2));
        q.small = small_grid_ok(ctx, q.gp, !q.b.dw.empty(), s->nmode, q.nunits);
        q.o_tbuf2 = work;
        if (q.small) work += align256((size_t)q.nunits * plane * sizeof(float2));
        q.o_img = work;
        if (!q.img_dev) work += align256((size_t)q.nimages * plane * sizeof(float));
        // a rotated or shifted image plane: a real-space scratch grid per unit and
        // the edge means
        q.o_phi = work;
        if (q.image_plane) work += align256((size_t)q.nunits * plane * sizeof(float2));
        q.o_fill = work;
        if (q.image_plane) work += align256((size_t)q.nunits * sizeof(float2));
        q.o_spec = work;
        if (!q.b.dw.empty()) work += align256((size_t)q.nunits * plane * sizeof(float2));
        q.o_ew = work;
        if (q.ew && !q.ew_dev && !q.ew_pinned)
            work += align256((size_t)q.nunits * plane * sizeof(float2));
    };
    const bool graph = (flags & MSK_BATCH_GRAPH) && !ctx->prof_on;
    int first = 0;
    while (first < nspec) {
        // the next wave: as many specimens (in order) as fit
        int last = first;
        size_t up = 0, work = 0;
        for (; last < nspec; last++) {
            size_t up2 = up, work2 = work;
            arena_of(P[last], up2, work2);
            if (last > first && up2 + work2 > budget) break;
            up = up2;
            work = work2;
        }
        // offsets of the work region follow the upload region
        for (int i = first; i < last; i++) {
            P[i].o_fres += align256(up);
            P[i].o_psi += align256(up);
            P[i].o_tbuf += align256(up);
            P[i].o_tbuf2 += align256(up);
            P[i].o_img += align256(up);
            P[i].o_phi += align256(up);
            P[i].o_fill += align256(up);
            P[i].o_spec += align256(up);
            P[i].o_ew += align256(up);
        }
        const size_t total = align256(up) + work;
        MSK_CUDA(ctx, ctx->arena.reserve(total));
        unsigned char *arena = ctx->arena.as<unsigned char>();
        std::vector<unsigned char> host(up);
        for (int i = first; i < last; i++) {
            SpecPlan &q = P[i];
            std::memcpy(&host[q.o_tab], q.tables.data(), q.tables.size());
            if (!q.atoms.empty())
                std::memcpy(&host[q.o_atoms], q.atoms.data(), q.atoms.size() * sizeof(SplatAtom));
            std::memcpy(&host[q.o_soff], q.b.slice_off.data(), q.b.slice_off.size() * sizeof(int));
            if (!q.b.act.empty())
                std::memcpy(&host[q.o_act], q.b.act.data(), q.b.act.size() * sizeof(int));
            if (!q.meta.empty())
                std::memcpy(&host[q.o_meta], q.meta.data(), q.meta.size() * sizeof(int));
            if (!q.wave0.empty())
                std::memcpy(&host[q.o_w0], q.wave0.data(), q.wave0.size() * sizeof(float2));
            if (!q.b.dw.empty())
                std::memcpy(&host[q.o_dw], q.b.dw.data(), q.b.dw.size() * sizeof(float));
            bind_tables(q.gp, arena + q.o_tab, q.tl);
        }
        MSK_CUDA(ctx, cudaMemcpyAsync(arena, host.data(), up, cudaMemcpyHostToDevice, ctx->stream));
        count_copy(ctx, 0, (double)up);
        Geom gflag{};
        st = flags_reset(ctx, gflag);
        if (st) return st;
        for (int i = first; i < last; i++) {
            P[i].gp.g.err = gflag.err;
            P[i].gp.g.zeros = gflag.zeros;
            // the splat stores in-band row segments only: the rest reads as zeros
            MSK_CUDA(ctx, cudaMemsetAsync(arena + P[i].o_tbuf, 0,
                                          (size_t)P[i].nunits * P[i].gp.nx * P[i].gp.ny *
                                              sizeof(float2),
                                          ctx->stream));
        }
        MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));

        // longest specimen first onto the least-loaded lane
        std::vector<int> order;
        for (int i = first; i < last; i++) order.push_back(i);
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return P[a].work > P[b].work; });
        const int nl = ctx->prof_on ? 1 : kLanes;
        std::vector<double> load(nl, 0.0);
        std::vector<std::vector<int>> lane_of(nl);
        for (int i : order) {
            const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            load[l] += P[i].work;
            lane_of[l].push_back(i);
        }
        // the tuners run launches of their own: settle every choice first
        for (int i = first; i < last; i++) {
            for (int mode : {(int)kColMask, (int)kColProp, (int)kColFresnel, (int)kColDW})
                (void)col_variant(ctx, P[i].gp, mode);
            (void)row_variant(ctx, P[i].gp);
        }
        cudaGraph_t gr = nullptr;
        if (graph)
            MSK_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
        int rc = MSK_OK;
        // a specimen's images to page-locked host memory on its own lane, as
        // soon as they are made (beside the other lanes' kernels)
        auto images_out = [&](int i, cudaStream_t st_) -> int {
            if (P[i].nimages == 0 || !P[i].img_pinned) return MSK_OK;
            const size_t bytes = (size_t)P[i].nimages * P[i].gp.nx * P[i].gp.ny * sizeof(float);
            if (cudaMemcpyAsync(spec[i].images, arena + P[i].o_img, bytes, cudaMemcpyDeviceToHost,
                                st_) != cudaSuccess)
                return fail(ctx, MSK_ECUDA, "image copy");
            count_copy(ctx, 1, (double)bytes);
            return MSK_OK;
        };
        if (nl == 1) {
            for (int i : lane_of[0]) {
                float *dimg = P[i].img_dev ? spec[i].images : reinterpret_cast<float *>(arena + P[i].o_img);
                if ((rc = enqueue_specimen(ctx, P[i], arena, s, dimg, ctx->stream)))
                    break;
                if ((rc = images_out(i, ctx->stream))) break;
            }
        } else {
            cudaEvent_t fork = ctx->lane_ev[kLanes];
            if (cudaEventRecord(fork, ctx->stream) != cudaSuccess) rc = fail(ctx, MSK_ECUDA, "fork");
            for (int l = 0; l < nl && !rc; l++) {
                if (cudaStreamWaitEvent(ctx->lanes[l], fork, 0) != cudaSuccess) {
                    rc = fail(ctx, MSK_ECUDA, "lane wait");
                    break;
                }
                for (int i : lane_of[l]) {
                    float *dimg = P[i].img_dev ? spec[i].images : reinterpret_cast<float *>(arena + P[i].o_img);
                    if ((rc = enqueue_specimen(ctx, P[i], arena, s, dimg, ctx->lanes[l])))
                        break;
                    if ((rc = images_out(i, ctx->lanes[l]))) break;
                }
                if (!rc && cudaEventRecord(ctx->lane_ev[l], ctx->lanes[l]) != cudaSuccess)
                    rc = fail(ctx, MSK_ECUDA, "lane join");
            }
            for (int l = 0; l < nl && !rc; l++)
                if (cudaStreamWaitEvent(ctx->stream, ctx->lane_ev[l], 0) != cudaSuccess)
                    rc = fail(ctx, MSK_ECUDA, "join wait");
        }
        if (graph) {
            cudaError_t e = cudaStreamEndCapture(ctx->stream, &gr);
            if (!rc && e != cudaSuccess)
                rc = fail(ctx, MSK_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
            if (!rc) {
                cudaGraphExec_t ex = nullptr;
                e = cudaGraphInstantiate(&ex, gr, 0);
                if (e == cudaSuccess) e = cudaGraphLaunch(ex, ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                if (ex) cudaGraphExecDestroy(ex);
                if (e != cudaSuccess)
                    rc = fail(ctx, MSK_ECUDA, std::string("graph launch: ") + cudaGetErrorString(e));
            }
            if (gr) cudaGraphDestroy(gr);
        }
        if (rc) {  // nothing of this wave may still run when the arena is reused
            for (cudaStream_t l : ctx->lanes) cudaStreamSynchronize(l);
            cudaStreamSynchronize(ctx->stream);
            return rc;
        }
        // images and exit waves to pageable host buffers
        for (int i = first; i < last; i++) {
            if (P[i].ew && !P[i].ew_dev && !P[i].ew_pinned) {
                const size_t ewb = (size_t)P[i].nunits * P[i].gp.nx * P[i].gp.ny * sizeof(float2);
                MSK_CUDA(ctx, cudaMemcpyAsync(P[i].ew, arena + P[i].o_ew, ewb,
                                              cudaMemcpyDeviceToHost, ctx->stream));
                count_copy(ctx, 1, (double)ewb);
            }
            if (P[i].nimages == 0 || P[i].img_dev || P[i].img_pinned) continue;
            const size_t bytes = (size_t)P[i].nimages * P[i].gp.nx * P[i].gp.ny * sizeof(float);
            MSK_CUDA(ctx, cudaMemcpyAsync(spec[i].images, arena + P[i].o_img, bytes,
                                          cudaMemcpyDeviceToHost, ctx->stream));
            count_copy(ctx, 1, (double)bytes);
        }
        MSK_CUDA(ctx, cudaGetLastError());
        MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        prof_collect(ctx);
        st = flags_check(ctx);
        if (st) return st;
        first = last;
    }
    for (int i = 0; i < nspec; i++)
        if (spec[i].kept)
            for (int u = 0; u < P[i].nunits; u++) spec[i].kept[u] = P[i].ua[u].kept;
    return MSK_OK;
}

// ------------------------------------------------------------------ allocation-free calculate()
//
// msk_calculate_static: calculate() for callers that cannot allocate device
// memory -- a plug-in whose host framework owns all device memory through
// its own pool, or a latency-critical loop where a cudaMalloc (and the
// synchronisation it implies) is not acceptable.  It creates no context, no
// stream, no event and no device buffer: its device scratch is one fixed
// array compiled into this library, which every GPU that loads the library
// holds until the process exits.  Limits (MSK_ETOOLARGE beyond them):
// nx*ny <= 512*512 pixels, natom <= 65536, at most 4096 slices.
namespace {

constexpr size_t kStaticPixels = 512 * 512;
constexpr int kStaticAtoms = 65536;
constexpr int kStaticSlices = 4096;
// regions of the scratch, 256-byte aligned
constexpr size_t kSGrid = kStaticPixels * sizeof(float2);          // 2 MiB
constexpr size_t kSTables = (size_t)1 << 20;                          // 1 MiB
constexpr size_t kSAtoms = (size_t)kStaticAtoms * sizeof(SplatAtom);  // 1 MiB
constexpr size_t kSSliceOff = 20 << 10;
constexpr size_t kSAct = 20 << 10;
constexpr size_t kSFlags = kFlagBytes;  // error flag + zero source
constexpr size_t kOffPsi = 0, kOffTbuf = kOffPsi + kSGrid, kOffWave0 = kOffTbuf + kSGrid,
                 kOffTables = kOffWave0 + kSGrid, kOffAtoms = kOffTables + kSTables,
                 kOffSliceOff = kOffAtoms + kSAtoms, kOffAct = kOffSliceOff + kSSliceOff,
                 kOffFlags = kOffAct + kSAct, kStaticBytes = kOffFlags + kSFlags;

}  // namespace

// The scratch of msk_calculate_static.  Host code cannot use this name as a
// device address: its address comes from cudaGetSymbolAddress, per device.
static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

namespace {

// The array's device address per device, looked up on the first call that
// succeeds on that device (a failed lookup is retried by the next call).
struct StaticScratch {
    std::mutex m;
    void *ptr = nullptr;
};
constexpr int kStaticDevices = 64;
StaticScratch g_static[kStaticDevices];

// Marks the calling host thread as one whose library calls must not allocate
// device memory, for the guard's lifetime.
struct NoAllocScope {
    bool prev;
    NoAllocScope() : prev(t_no_alloc) { t_no_alloc = true; }
    ~NoAllocScope() { t_no_alloc = prev; }
};

// Bytes upload_tables() needs for this grid.
size_t static_table_bytes(int nx, int ny, int nz) { return layout_tables(nx, ny, nz).bytes; }

}  // namespace

extern "C" int msk_calculate_static(void *stream, float *pix, const float *wave0,
                                    const float *param, int natom, const int *Znum,
                                    const float *x, const float *y, const float *z,
                                    const float *occ, float ctblength, float ctblengthz, int nmode)
{
    if (!pix || !wave0 || !param || natom < 0 || (natom > 0 && (!Znum || !x || !y || !z || !occ)))
        return MSK_EINVAL;
    const float ax = param[MSK_pAX], by = param[MSK_pBY];
    const int nx = (int)(param[MSK_pNX] + 0.1F), ny = (int)(param[MSK_pNY] + 0.1F);
    if (nx < 1 || ny < 1 || ax < 0.0 || by < 0.0) return MSK_EBADSIZE;
    if (!pow2_supported(nx) || !pow2_supported(ny)) return MSK_EUNSUPPORTED;
    const int nslices = slice_count(param[MSK_pDELTAZ], ctblengthz);
    if ((size_t)nx * ny > kStaticPixels || natom > kStaticAtoms || nslices > kStaticSlices)
        return MSK_ETOOLARGE;

    // once per device, with that device current: the array's device address
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kStaticDevices) return MSK_ECUDA;
    StaticScratch &sc = g_static[dev];
    void *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(sc.m);
        if (!sc.ptr) {
            void *q = nullptr;
            if (cudaGetSymbolAddress(&q, g_static_scratch) != cudaSuccess || !q) {
                cudaGetLastError();  // not sticky: the next call tries again
                return MSK_ECUDA;
            }
            sc.ptr = q;
        }
        scratch = sc.ptr;
    }

    // A context on the stack whose buffers are borrowed views of the scratch.
    // A view never grows, and while this call runs no other buffer of this
    // thread may allocate either: a size beyond a view fails the call
    // (MSK_ENOMEM) instead of calling cudaMalloc.
    NoAllocScope no_alloc;
    msk_context ctx;
    ctx.device = dev;
    ctx.stream = (cudaStream_t)stream;
    ctx.no_tune = true;  // the tuners would allocate: the default schedules
    ctx.no_host_stage = true;
    unsigned char *base = static_cast<unsigned char *>(scratch);
    auto view = [&](DevBuf &b, size_t off, size_t bytes) { b.borrow(base + off, bytes); };
    view(ctx.psi, kOffPsi, kSGrid);
    view(ctx.tbuf, kOffTbuf, kSGrid);
    view(ctx.wave0, kOffWave0, kSGrid);
    view(ctx.tables, kOffTables, kSTables);
    view(ctx.atoms, kOffAtoms, kSAtoms);
    view(ctx.slice_off, kOffSliceOff, kSSliceOff);
    view(ctx.act, kOffAct, kSAct);
    view(ctx.flags, kOffFlags, kSFlags);
    // the zero source and the transmission buffer's out-of-band columns must
    // read as zeros; the scratch holds whatever the last call left
    if (cudaMemsetAsync(ctx.flags.p, 0, kSFlags, ctx.stream) != cudaSuccess ||
        cudaMemsetAsync(ctx.tbuf.p, 0, (size_t)nx * ny * sizeof(float2), ctx.stream) != cudaSuccess)
        return MSK_ECUDA;
    // ctx.tbuf2 stays empty: the slice loop then runs in order on `stream`

    GridPre gp;
    if (!grid_pre(gp, nx, ny, ax, by, param[MSK_pENERGY], param[MSK_pDELTAZ], param[MSK_pXCTILT],
                  param[MSK_pYCTILT]))
        return MSK_EUNSUPPORTED;
    if (natom > 0) {  // the reference's range check first (autoslic.cpp:270-299)
        float xmin = x[0], xmax = x[0], ymin = y[0], ymax = y[0], zmin = z[0], zmax = z[0];
        for (int i = 0; i < natom; i++) {
            xmin = std::min(xmin, x[i]);
            xmax = std::max(xmax, x[i]);
            ymin = std::min(ymin, y[i]);
            ymax = std::max(ymax, y[i]);
            zmin = std::min(zmin, z[i]);
            zmax = std::max(zmax, z[i]);
        }
        if (xmin < 0 || ymin < 0 || zmin < 0 || xmax > ctblength || ymax > ctblength ||
            zmax > ctblengthz)
            return MSK_EBOX;
    }
    std::vector<int> zlist;
    int st = build_zmap(&ctx, natom, Znum, zlist);
    if (st) return st;
    if (static_table_bytes(nx, ny, (int)zlist.size()) > kSTables) return MSK_ETOOLARGE;
    std::vector<UnitAtoms> ua(1);
    PrepSpec ps{natom, Znum, x, y, z, occ, ctblength, ctblengthz, param[MSK_pDELTAZ], nslices,
                false, 0, 0, 0, 0, 0, nullptr, false, ctx.zmap.data()};
    prep_unit(gp, ps, ua[0]);
    if (ua[0].status) return ua[0].status;
    if ((st = upload_tables(&ctx, gp, zlist))) return st;
    Batch b;
    if ((st = upload_batch(&ctx, ua, 0, 1, nslices, b))) return st;
    ctx.units_alloc = 1;
    // the device error flag is the only scratch a call reads before writing
    if ((st = flags_reset(&ctx, gp.g))) return st;
    const size_t plane = (size_t)nx * ny;
    if (cudaMemcpyAsync(ctx.wave0.p, wave0, plane * sizeof(float2), cudaMemcpyHostToDevice,
                        ctx.stream) != cudaSuccess)
        return MSK_ECUDA;
    const SizeOps *rop = size_ops(ny);
    rop->row_init(gp.g, nullptr, 1, ctx.wave0.as<float2>(), ctx.psi.as<float2>(), 1.0f, ctx.stream);
    if ((st = run_slices(&ctx, gp, b, nmode, false))) return st;
    rop->row_exit(gp.g, nullptr, 1, ctx.psi.as<float2>(), ctx.tbuf.as<float2>(), ctx.stream);
    if (cudaGetLastError() != cudaSuccess) return MSK_ECUDA;
    if (cudaMemcpyAsync(pix, ctx.tbuf.p, plane * sizeof(float2), cudaMemcpyDeviceToHost,
                        ctx.stream) != cudaSuccess)
        return MSK_ECUDA;
    return flags_check(&ctx);
}

extern "C" int msk_column_plan(int device, int nx, int ny, int pass, int *info)
{
    if (!info || pass < 0 || pass > 3 || !size_ops(nx)) return MSK_EINVAL;
    const int modes[4] = {kColMask, kColProp, kColFresnel, kColDW};
    ColChoices &cc = col_choices();
    std::lock_guard<std::mutex> lock(cc.m);
    auto it = cc.v.find(std::array<int, 4>{device, nx, ny, modes[pass]});
    if (it == cc.v.end()) return MSK_EINVAL;
    const int v = it->second;
    info[0] = v;
    info[1] = v >= 2 ? 16 : std::min(nx, 32);
    info[2] = size_ops(nx)->col_c[v];
    return MSK_OK;
}

extern "C" int msk_row_plan(int device, int nx, int ny, int pass, int *info)
{
    if (!info || pass != 0 || !size_ops(ny)) return MSK_EINVAL;
    RowChoices &rc = row_choices();
    std::lock_guard<std::mutex> lock(rc.m);
    auto it = rc.v.find(std::array<int, 3>{device, nx, ny});
    if (it == rc.v.end()) return MSK_EINVAL;
    const int v = it->second;
    info[0] = v;
    info[1] = v == 2 ? 16 : std::min(ny, 32);
    info[2] = std::max(1, (v == 0 ? 64 : 128) / (ny / info[1]));
    return MSK_OK;
}

extern "C" long long msk_device_allocations(void)
{
    return g_device_allocs.load(std::memory_order_relaxed);
}

// ------------------------------------------------------------------ per-orientation form
//
// msk_tilt_series_per_angle: the same tilt series computed the way a direct GPU
// port of the reference would compute it -- one orientation at a time, one
// launch sequence per slice with unfused kernels and library 2D FFTs (cuFFT,
// loaded at run time), an atomic scatter for the potential, and a
// synchronisation after every orientation (MultisliceT.cpp:403-448 runs one
// host thread per orientation).  It is the comparison form for the batched
// path; the batched path never uses cuFFT.
namespace {

struct CufftApi {
    bool ok = false;
    cufftResult (*plan2d)(cufftHandle *, int, int, cufftType) = nullptr;
    cufftResult (*set_stream)(cufftHandle, cudaStream_t) = nullptr;
    cufftResult (*exec_c2c)(cufftHandle, cufftComplex *, cufftComplex *, int) = nullptr;
    cufftResult (*destroy)(cufftHandle) = nullptr;
};

const CufftApi &cufft_api()
{
    static CufftApi api;
    static std::once_flag once;
    std::call_once(once, [] {
        const char *names[] = {getenv("MSK_CUFFT_LIBRARY"), "libcufft.so.12", "libcufft.so",
                               "/usr/local/cuda/lib64/libcufft.so.12",
                               "/usr/local/cuda/targets/sbsa-linux/lib/libcufft.so.12",
                               "/usr/local/cuda/targets/x86_64-linux/lib/libcufft.so.12"};
        void *h = nullptr;
        for (const char *n : names)
            if (n && (h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) return;
        api.plan2d = reinterpret_cast<decltype(api.plan2d)>(dlsym(h, "cufftPlan2d"));
        api.set_stream = reinterpret_cast<decltype(api.set_stream)>(dlsym(h, "cufftSetStream"));
        api.exec_c2c = reinterpret_cast<decltype(api.exec_c2c)>(dlsym(h, "cufftExecC2C"));
        api.destroy = reinterpret_cast<decltype(api.destroy)>(dlsym(h, "cufftDestroy"));
        api.ok = api.plan2d && api.set_stream && api.exec_c2c && api.destroy;
    });
    return api;
}

}  // namespace

namespace msk {

// One thread per (atom, window pixel), atomically added: the reference's
// trlayer loop (autoslic.cpp:950-984) run in parallel as written.
__global__ void k_plain_splat(const Geom g, const SplatAtom *__restrict__ atoms, int a0, int na,
                              float *v)
{
    const int W = 2 * g.idx + 1, H = 2 * g.idy + 1;
    const long total = (long)na * W * H;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int a = (int)(i / (W * H)), r = (int)(i % (W * H));
        const int dxw = r / H - g.idx, dyw = r % H - g.idy;
        const SplatAtom at = atoms[a0 + a];
        const int ixo = (int)(at.meta & kMetaMask), iyo = (int)((at.meta >> kMetaBits) & kMetaMask);
        const float dx = at.fx - (float)dxw * g.scalex_f, dy = at.fy - (float)dyw * g.scaley_f;
        float rsq = dx * dx + dy * dy;
        if (rsq <= 9.0f) {
            rsq = fmaxf(rsq, g.rminsq);
            const float4 *coef = g.coef + (at.meta >> (2 * kMetaBits)) * kKnots;
            const int ix = (ixo + dxw) & (g.nx - 1), iy = (iyo + dyw) & (g.ny - 1);
            atomicAdd(&v[(size_t)ix * g.ny + iy], at.occ * spline_vz(g.knots, coef, rsq));
        }
    }
}

__global__ void k_plain_exp(const float *__restrict__ v, float sigma, size_t n, float2 *t)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float s, c;
        sincosf(v[i] * sigma, &s, &c);
        t[i] = make_float2(c, s);
    }
}

// MODE 0: 2/3 band limit; MODE 1: propagator with the 2/3 aperture
template <int MODE>
__global__ void k_plain_kmul(const Geom g, float scale, float2 *w)
{
    const size_t n = (size_t)g.nx * g.ny;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i / g.ny), iy = (int)(i % g.ny);
        const int2 ab = g.kband[iy];
        if (ix <= ab.x || ix >= ab.y) {
            float2 x = w[i];
            if (MODE == 1) x = cmul(cmul(x, g.propy[iy]), g.propx[ix]);
            w[i] = cscale(x, scale);
        } else {
            w[i] = make_float2(0.0f, 0.0f);
        }
    }
}

__global__ void k_plain_mul(float2 *a, const float2 *__restrict__ b, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        a[i] = cmul(a[i], b[i]);
}

__global__ void k_plain_fill(float2 *a, float2 val, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        a[i] = val;
}

// image += |e|^2; after the last configuration, / nconf
__global__ void k_plain_accum(const float2 *__restrict__ e, size_t n, int first, int last, float nconf,
                              float *img)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 x = e[i];
        float acc = x.x * x.x + x.y * x.y;
        if (!first) acc = img[i] + acc;
        img[i] = last ? __fdiv_rn(acc, nconf) : acc;
    }
}

}  // namespace msk

extern "C" int msk_tilt_series_per_angle(msk_context *ctx, const msk_series *s, int natom,
                                         const int *Znum, const float *x, const float *y,
                                         const float *z, const float *occ, int nangles,
                                         const double *angleZ, const double *angleY,
                                         int ndefocus, const double *defocus, int nconfig,
                                         const float *displacements, float *images, int *kept)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!s || natom < 0 || nangles < 1 || ndefocus < 0 || nconfig < 1 || !angleZ || !angleY ||
        (ndefocus > 0 && (!defocus || !images)) ||
        (natom > 0 && (!Znum || !x || !y || !z || !occ)) || (nconfig > 1 && !displacements))
        return fail(ctx, MSK_EINVAL, "bad tilt-series arguments");
    if (s->lwobble || s->R1 != 0.0 || s->rotation || s->xshift != 0.0 || s->yshift != 0.0)
        return fail(ctx, MSK_EUNSUPPORTED,
                    "the comparison form takes plane waves without thermal branches or image rotation");
    const int nx = s->nx, ny = s->ny;
    if (!pow2_supported(nx) || !pow2_supported(ny))
        return fail(ctx, MSK_EUNSUPPORTED, "grid must be a power of two from 16 to 4096");
    const CufftApi &fft = cufft_api();
    if (!fft.ok) return fail(ctx, MSK_EUNSUPPORTED, "cuFFT could not be loaded");
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    GridPre gp;
    if (!grid_pre(gp, nx, ny, s->ctblength, s->ctblength, s->v0, s->deltaz, 0.0f, 0.0f))
        return fail(ctx, MSK_EUNSUPPORTED, "band limit is not two index ranges per column");
    const int nslices = slice_count(s->deltaz, s->ctblengthz);
    std::vector<int> zlist;
    int st = build_zmap(ctx, natom, Znum, zlist);
    if (st) return st;
    if ((st = upload_tables(ctx, gp, zlist))) return st;
    const size_t plane = (size_t)nx * ny;
    const Geom &g = gp.g;
    cudaStream_t sm = ctx->stream;
    MSK_CUDA(ctx, ctx->pa_v.reserve(plane * sizeof(float)));
    MSK_CUDA(ctx, ctx->pa_t.reserve(plane * sizeof(float2)));
    MSK_CUDA(ctx, ctx->pa_psi.reserve(plane * sizeof(float2)));
    MSK_CUDA(ctx, ctx->pa_e.reserve(plane * sizeof(float2)));
    MSK_CUDA(ctx, ctx->fresnel.reserve(plane * sizeof(float2) * std::max(ndefocus, 1)));
    const bool img_dev = ndefocus > 0 && is_device_ptr(images);
    const size_t img_bytes = (size_t)nangles * ndefocus * plane * sizeof(float);
    float *d_images = images;
    if (ndefocus > 0 && !img_dev) {
        MSK_CUDA(ctx, ctx->images.reserve(img_bytes));
        d_images = ctx->images.as<float>();
    }
    float *v = ctx->pa_v.as<float>();
    float2 *t = ctx->pa_t.as<float2>(), *psi = ctx->pa_psi.as<float2>(), *e = ctx->pa_e.as<float2>();
    // free-space multipliers (with 1/N) for every plane, once
    const double pi = 4.0 * atan(1.0), l = gp.wavlen;
    float k2maxo = s->aobj / gp.wavlen;
    k2maxo = k2maxo * k2maxo;
    for (int d = 0; d < ndefocus; d++) {
        Fresnel fr{};
        const double rprime = defocus[d] - 0.5 * s->ctblengthz;
        fr.a1 = pi * l * rprime;
        fr.a3 = (pi / 2.0) * s->cs3 * l * l * l;
        fr.a5 = (pi / 3.0) * s->cs5 * l * l * l * l * l;
        fr.a2c = (pi / 2.0) * l * s->astig * cos(2.0 * s->astig_angle);
        fr.a2s = (pi / 2.0) * l * s->astig * sin(2.0 * s->astig_angle);
        fr.k2maxo = k2maxo;
        fr.kx = tables_kx(ctx, gp);
        fr.ky = tables_ky(ctx, gp);
        k_fresnel_table<<<4 * 152, 256, 0, sm>>>(g, fr, 1.0f / ((float)nx * (float)ny),
                                                  ctx->fresnel.as<float2>() + (size_t)d * plane);
    }
    cufftHandle plan;
    if (fft.plan2d(&plan, nx, ny, CUFFT_C2C) != CUFFT_SUCCESS)
        return fail(ctx, MSK_ECUDA, "cufftPlan2d failed");
    fft.set_stream(plan, sm);
    auto FFT = [&](float2 *a, int dir) {  // cfpix::fft is the +1 kernel, ifft the -1 kernel
        fft.exec_c2c(plan, reinterpret_cast<cufftComplex *>(a), reinterpret_cast<cufftComplex *>(a), dir);
    };
    const int G = 4 * 152, TB = 256;
    const float invN = 1.0f / ((float)nx * (float)ny);
    std::vector<UnitAtoms> ua(1);
    int status = MSK_OK;
    for (int u = 0; u < nangles * nconfig && status == MSK_OK; u++) {
        const int a = u / nconfig, c = u % nconfig;
        PrepSpec ps{natom, Znum, x, y, z, occ, s->ctblength, s->ctblengthz, s->deltaz, nslices, true,
                    angleZ[a], angleY[a], s->dxc, s->dyc, s->dzc,
                    displacements ? displacements + (size_t)c * 3 * natom : nullptr, true,
                    ctx->zmap.data()};
        prep_unit(gp, ps, ua[0]);
        if (ua[0].status) {
            status = fail(ctx, ua[0].status, msk_status_string(ua[0].status));
            break;
        }
        if (kept) kept[u] = ua[0].kept;
        Batch b;
        if ((status = upload_batch(ctx, ua, 0, 1, nslices, b))) break;
        k_plain_fill<<<G, TB, 0, sm>>>(psi, make_float2(1.0f, 0.0f), plane);
        for (int sl = 0; sl < nslices; sl++) {
            const int a0 = b.slice_off[sl], na = b.slice_off[sl + 1] - a0;
            if (na > 0) {
                cudaMemsetAsync(v, 0, plane * sizeof(float), sm);
                k_plain_splat<<<G, TB, 0, sm>>>(g, ctx->atoms.as<SplatAtom>(), a0, na, v);
                k_plain_exp<<<G, TB, 0, sm>>>(v, g.sigma_f, plane, t);
                FFT(t, CUFFT_INVERSE);
                k_plain_kmul<0><<<G, TB, 0, sm>>>(g, invN, t);
                FFT(t, CUFFT_FORWARD);
                k_plain_mul<<<G, TB, 0, sm>>>(psi, t, plane);
            }
            if (s->nmode == 0) {
                FFT(psi, CUFFT_INVERSE);
                k_plain_kmul<1><<<G, TB, 0, sm>>>(g, invN * (float)nx, psi);  // propx holds 1/nx
                FFT(psi, CUFFT_FORWARD);
            }
        }
        for (int d = 0; d < ndefocus; d++) {
            cudaMemcpyAsync(e, psi, plane * sizeof(float2), cudaMemcpyDeviceToDevice, sm);
            FFT(e, CUFFT_INVERSE);
            k_plain_mul<<<G, TB, 0, sm>>>(e, ctx->fresnel.as<float2>() + (size_t)d * plane, plane);
            FFT(e, CUFFT_FORWARD);
            k_plain_accum<<<G, TB, 0, sm>>>(e, plane, c == 0, c == nconfig - 1 && nconfig > 1,
                                           (float)nconfig,
                                           d_images + ((size_t)a * ndefocus + d) * plane);
        }
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(sm) != cudaSuccess)
            status = fail(ctx, MSK_ECUDA, "per-orientation form: CUDA error");
    }
    fft.destroy(plan);
    if (status) return status;
    if (ndefocus > 0 && !img_dev)
        MSK_CUDA(ctx, cudaMemcpyAsync(images, d_images, img_bytes, cudaMemcpyDeviceToHost, sm));
    MSK_CUDA(ctx, cudaStreamSynchronize(sm));
    return MSK_OK;
}
