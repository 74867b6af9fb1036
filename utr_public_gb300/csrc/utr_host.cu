// utr_host.cu -- the UTR reconstruction (include/msk_utr.h): host geometry,
// the gridding kernel, the pointwise Fourier-space kernels and the schedule
// of passes.
//
// Data layout in HBM for one call (nimg images of ny x nx, a volume of
// nz x ny x nx):
//   images   float   [nimg][ny][nx]     (the caller's, or a staged copy)
//   k2       complex [nimg][ny][nx]     centred image spectra
//   acc      UtrAcc  [nz][ny][nx]       gridding sums (re, im, weight, -), 16 B
//   vol      complex [nz][ny][nx]       the spectrum, then its inverse in place
//   out      float   [nz][ny][nx]       the caller's, or a staged copy
// The gridding sums are float, as the reference accumulates them, with one
// 16-byte vector atomic per voxel update: the summation order (and so the last
// bits) follows the schedule, as in the reference's threaded loop over
// orientations.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "msk_ctx.h"
#include "msk_utr.h"
#include "utr_launch.cuh"

namespace msk {

const UtrOps *utr_ops_16();
const UtrOps *utr_ops_32();
const UtrOps *utr_ops_64();
const UtrOps *utr_ops_128();
const UtrOps *utr_ops_256();
const UtrOps *utr_ops_512();
const UtrOps *utr_ops_1024();
const UtrOps *utr_ops_2048();
const UtrOps *utr_ops_4096();

const UtrOps *utr_ops(int n)
{
    switch (n) {
    case 16: return utr_ops_16();
    case 32: return utr_ops_32();
    case 64: return utr_ops_64();
    case 128: return utr_ops_128();
    case 256: return utr_ops_256();
    case 512: return utr_ops_512();
    case 1024: return utr_ops_1024();
    case 2048: return utr_ops_2048();
    case 4096: return utr_ops_4096();
    default: return nullptr;
    }
}

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kScal = 10;  // per-image scalars of the gridding: sinY cosY sinZ cosZ, Fxc Fyc Fzc

// ------------------------------------------------------------------ kernels

struct UtrGridP {
    int nx, ny, nz, nimg;
    const float2 *k2;
    const float *tabs;  // [nimg][xxx2 | xsy | xcy (nx each) | yyy2 | ysz | ycz (ny each)]
    const float *scal;  // [nimg][kScal]
    float fxlo, fxst, fylo, fyst, fzlo, fzst;
    int rotshift, escc;
    UtrAcc *acc;
};

// CT_3Dgridding (UTR.h:199-307) of every pixel of every image: the pixel's
// frequency coordinates rotated back (about Y' then Z), on the Ewald sphere
// with the curvature correction, the enclosing voxel cell, and trilinear
// weights, all in float with the reference's operation order; each of the
// eight corners gets (weight * value, weight) by one vector atomic.
__global__ void __launch_bounds__(256) k_utr_grid(const UtrGridP p)
{
    const size_t npix = (size_t)p.nx * p.ny, total = npix * p.nimg;
    const size_t nxny = npix;
    const int tstride = 3 * p.nx + 3 * p.ny;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total;
         q += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / npix);
        const int r = (int)(q - (size_t)a * npix);
        const int j = r / p.nx, i = r - j * p.nx;
        const float *tb = p.tabs + (size_t)a * tstride;
        const float *sc = p.scal + (size_t)a * kScal;
        const float sinY = sc[0], cosY = sc[1], sinZ = sc[2], cosZ = sc[3];
        float zz = 0.0f;
        if (p.escc) zz = __fadd_rn(tb[i], tb[3 * p.nx + j]);
        const float xx = __fsub_rn(tb[2 * p.nx + i], __fmul_rn(zz, sinY));
        const float zzz = __fadd_rn(tb[p.nx + i], __fmul_rn(zz, cosY));
        float dz1 = __fdiv_rn(__fsub_rn(zzz, p.fzlo), p.fzst);
        const int nn = (int)floorf(dz1);
        if (nn < 0 || nn > p.nz - 2) continue;
        const float xxx = __fadd_rn(__fmul_rn(xx, cosZ), tb[3 * p.nx + p.ny + j]);
        float dx1 = __fdiv_rn(__fsub_rn(xxx, p.fxlo), p.fxst);
        const int ii = (int)floorf(dx1);
        if (ii < 0 || ii > p.nx - 2) continue;
        const float yyy = __fadd_rn(__fmul_rn(-xx, sinZ), tb[3 * p.nx + 2 * p.ny + j]);
        float dy1 = __fdiv_rn(__fsub_rn(yyy, p.fylo), p.fyst);
        const int jj = (int)floorf(dy1);
        if (jj < 0 || jj > p.ny - 2) continue;
        dx1 = __fsub_rn(dx1, (float)ii);
        dy1 = __fsub_rn(dy1, (float)jj);
        dz1 = __fsub_rn(dz1, (float)nn);
        const float dx[2] = {__fsub_rn(1.0f, dx1), dx1};
        const float dy[2] = {__fsub_rn(1.0f, dy1), dy1};
        const float dz[2] = {__fsub_rn(1.0f, dz1), dz1};
        float2 cd = p.k2[q];
        if (p.rotshift) {
            // exp(Fxc qx + Fyc qy + Fzc qz), the F purely imaginary
            const float ph = __fadd_rn(__fadd_rn(__fmul_rn(sc[5], xxx), __fmul_rn(sc[7], yyy)),
                                       __fmul_rn(sc[9], zzz));
            float s, c;
            sincosf(ph, &s, &c);
            cd = cmul_rn(cd, make_float2(c, s));
        }
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
            for (int zc = 0; zc < 2; zc++)
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const float w = __fmul_rn(__fmul_rn(dx[e], dy[b]), dz[zc]);
                    // a zero weight adds exact zeros: skip it (for a tilt about y
                    // alone the pixel rows fall on voxel rows, dy1 = 0)
                    if (w == 0.0f) continue;
                    UtrAcc *v = p.acc + (size_t)(nn + zc) * nxny + (size_t)(jj + b) * p.nx + (ii + e);
                    atomicAdd(reinterpret_cast<float4 *>(v),
                              make_float4(__fmul_rn(cd.x, w), __fmul_rn(cd.y, w), w, 0.0f));
                }
    }
}

// ------------------------------------------------------------------ input image plane
// UTR.cpp:920-950 for images with a Z'' rotation or a shift: the normalised
// image (input / f1 + f2, negatives to 0), its edge mean (NormAverEdge(5)),
// the shift by whole pixels, then the rotation back by -Z'' (XArray2DMove,
// XArray2DSpln::Rotate; XArrayLibrary is not part of the reference, so these
// are this library's definitions, those of MsctKirkland's image plane):
//   shift:  s(j, i) = v(j - dy, i - dx), the edge mean outside;
//   rotate: out(p) = s(c + R(-t)(p - c)), t = -Z'', Catmull-Rom bicubic on
//           (x, y) = (i, j), the edge mean outside, c the rotation centre.
struct UtrPlaneP {
    int nx, ny, nimg;
    float f1, f2;
    int use_f1, use_f2;
    double cx, cy;          // rotation centre in pixels
    const double *par;      // [nimg][4]: cos t, sin t, dx, dy
    const int *op;          // [nimg]: 0 none, 1 shift only, 2 rotate (and shift)
    const float *fill;      // [nimg] edge means
};

__device__ __forceinline__ float utr_norm(const UtrPlaneP &p, float v)
{
    if (p.use_f1) v = __fdiv_rn(v, p.f1);
    if (p.use_f2) v = __fadd_rn(v, p.f2);
    return v < 0.0f ? 0.0f : v;
}

// One CTA per image: the mean of the normalised pixels within 5 of an edge.
__global__ void __launch_bounds__(256) k_utr_edge_mean(const UtrPlaneP p, const float *__restrict__ img,
                                                       float *__restrict__ fill)
{
    const int a = blockIdx.x;
    if (!p.op[a]) return;
    const float *src = img + (size_t)a * p.nx * p.ny;
    double sum = 0.0;
    long long cnt = 0;
    for (int q = threadIdx.x; q < p.nx * p.ny; q += blockDim.x) {
        const int j = q / p.nx, i = q - j * p.nx;
        if (i < 5 || i >= p.nx - 5 || j < 5 || j >= p.ny - 5) {
            sum += utr_norm(p, src[q]);
            cnt++;
        }
    }
    __shared__ double s_sum[256];
    __shared__ long long s_cnt[256];
    s_sum[threadIdx.x] = sum;
    s_cnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s_sum[threadIdx.x] += s_sum[threadIdx.x + o];
            s_cnt[threadIdx.x] += s_cnt[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) fill[a] = s_cnt[0] ? (float)(s_sum[0] / (double)s_cnt[0]) : 0.0f;
}

__device__ __forceinline__ float cr_weight_f(float t, int k)
{
    // Catmull-Rom weights of the samples at -1, 0, 1, 2 for a fraction t
    const float t2 = t * t, t3 = t2 * t;
    switch (k) {
    case 0: return 0.5f * (-t3 + 2.0f * t2 - t);
    case 1: return 0.5f * (3.0f * t3 - 5.0f * t2 + 2.0f);
    case 2: return 0.5f * (-3.0f * t3 + 4.0f * t2 + t);
    default: return 0.5f * (t3 - t2);
    }
}

// Normalised images with their plane operations into `out` (every image).
__global__ void k_utr_img_plane(const UtrPlaneP p, const float *__restrict__ img,
                                float *__restrict__ out)
{
    const size_t plane = (size_t)p.nx * p.ny;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < plane * p.nimg;
         q += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / plane);
        const int r = (int)(q - (size_t)a * plane);
        const int j = r / p.nx, i = r - j * p.nx;
        const float *src = img + (size_t)a * plane;
        const int op = p.op[a];
        if (!op) {
            out[q] = utr_norm(p, src[r]);
            continue;
        }
        const double *pr = p.par + 4 * (size_t)a;
        const long dx = (long)pr[2], dy = (long)pr[3];
        const float f = p.fill[a];
        // the shifted image s at (yy, xx), the edge mean outside
        auto sval = [&](long yy, long xx) -> float {
            if (yy < 0 || yy >= p.ny || xx < 0 || xx >= p.nx) return f;
            const long sy = yy - dy, sx = xx - dx;
            if (sy < 0 || sy >= p.ny || sx < 0 || sx >= p.nx) return f;
            return utr_norm(p, src[(size_t)sy * p.nx + sx]);
        };
        if (op == 1) {
            out[q] = sval(j, i);
            continue;
        }
        const double c = pr[0], sn = pr[1];
        const double ddx = i - p.cx, ddy = j - p.cy;
        const double fx = p.cx + c * ddx + sn * ddy, fy = p.cy - sn * ddx + c * ddy;  // R(-t)
        const long x0 = (long)floor(fx), y0 = (long)floor(fy);
        const float tx = (float)(fx - x0), ty = (float)(fy - y0);
        float acc = 0.0f;
        for (int b = 0; b < 4; b++) {
            const float wy = cr_weight_f(ty, b);
            for (int e = 0; e < 4; e++) acc += cr_weight_f(tx, e) * wy * sval(y0 - 1 + b, x0 - 1 + e);
        }
        out[q] = acc;
    }
}

// gridding sums -> the caller's V3, Samp3 (msk_utr_grid)
__global__ void k_utr_acc_split(const UtrAcc *__restrict__ acc, size_t n, float2 *__restrict__ v3,
                                float *__restrict__ samp3)
{
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const UtrAcc a = acc[q];
        v3[q] = make_float2(a.re, a.im);
        samp3[q] = a.w;
    }
}

// the 3D corrections alone, in place (msk_utr_ctf_correction3d,
// msk_utr_inverse_mlaplacian3d)
__global__ void k_utr_point(const UtrFourier f, float2 *v3)
{
    const size_t n = (size_t)f.nx * f.ny * f.nz;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % f.nx);
        const size_t kj = q / f.nx;
        const int j = (int)(kj % f.ny), k = (int)(kj / f.ny);
        const UtrRow r = utr_row(f, k, j);
        v3[q] = utr_correct(f, r, i, v3[q]);
    }
}

// ------------------------------------------------------------------ host geometry

int ilog2i(int n)
{
    int b = 0;
    while ((1 << b) < n) b++;
    return b;
}

// The quantities UTR.cpp derives from its parameters (UTR.cpp:208-372, 388).
struct Geo {
    int nx, ny, nz;
    double xst, xlo, xhi, ylo, yhi, zlo, zhi;
    double fxst, fyst, fzst, fxlo, fylo, fzlo;
    long long ic, jc, kc;
    double ee, k2maxo, cs3, cs5, zout;
    bool rot_y_only, rot_z_only, rot_z2_only;
};

int depth_of(const msk_utr *p, double *zlo_out, double *zhi_out)
{
    if (!p || !(p->xst > 0.0) || p->nx < 1 || p->ny < 1) return MSK_EINVAL;
    double zlo = p->zlo, zhi = p->zhi;
    if (p->modality == 1 && zlo == 0.0 && zhi == 0.0) {  // the .xri default [xlo, xhi]
        zlo = -0.5 * p->xst * p->nx;
        zhi = zlo + p->xst * p->nx;
    }
    if (zlo > zhi) std::swap(zlo, zhi);
    const int nz = (int)((zhi - zlo) / p->xst + 0.5);
    if (nz <= 0) return MSK_EINVAL;
    if (zlo_out) *zlo_out = zlo;
    if (zhi_out) *zhi_out = zhi;
    return nz;
}

int make_geo(msk_context *ctx, const msk_utr *p, int nangles, const double *angles,
             const double *defocus, Geo &g, const double *zrot = nullptr)
{
    const int nz = depth_of(p, &g.zlo, &g.zhi);
    if (nz < 0) return fail(ctx, MSK_EINVAL, "bad UTR geometry (pixel size, sizes or z range)");
    g.nx = p->nx;
    g.ny = p->ny;
    g.nz = nz;
    g.xst = p->xst;
    g.xlo = -0.5 * p->xst * g.nx;
    g.xhi = g.xlo + p->xst * g.nx;
    g.ylo = -0.5 * p->xst * g.ny;
    g.yhi = g.ylo + p->xst * g.ny;
    g.fxst = 1.0 / (g.xhi - g.xlo);
    g.fyst = 1.0 / (g.yhi - g.ylo);
    g.fxlo = -g.fxst * (g.nx / 2);
    g.fylo = -g.fyst * (g.ny / 2);
    g.fzst = 1.0 / (g.zhi - g.zlo);
    g.fzlo = -g.fzst * (g.nz / 2);
    const double xc = (g.xhi + g.xlo) / 2.0 + p->dxc, yc = (g.yhi + g.ylo) / 2.0 + p->dyc,
                 zc = (g.zhi + g.zlo) / 2.0 + p->dzc;
    g.ic = (long long)(size_t)((xc - g.xlo) / p->xst + 0.5);
    g.jc = (long long)(size_t)((yc - g.ylo) / p->xst + 0.5);
    g.kc = (long long)(size_t)((zc - g.zlo) / p->xst + 0.5);
    if (p->modality == 0) {  // UTR.cpp:355-363
        const double hp = 6.62607004e-34, cc = 299792458, ee = 1.602176634e-19,
                     m0 = 9.1093837015e-31;
        const long double mc2 = m0 * cc * cc;
        const long double chl2 =
            (long double)(cc * cc * hp * hp) / (long double)(p->wl * p->wl * 1.e-20);
        const long double abra = sqrtl(mc2 * mc2 + chl2);
        g.ee = (double)((-mc2 + abra) / (long double)(ee));
    } else {
        g.ee = 0.001239841662513396 / p->wl;
    }
    g.k2maxo = pow(p->aobj * 0.001f / p->wl, 2.0);
    g.cs3 = p->cs3 * 1.e+7;
    g.cs5 = p->cs5 * 1.e+7;
    // UTR.cpp:211-238 (the flags are set from the second orientation on)
    g.rot_z_only = g.rot_y_only = g.rot_z2_only = true;
    double zav = defocus[0];
    for (int i = 1; i < nangles; i++) {
        if (angles[2 * i] != 0) g.rot_y_only = g.rot_z2_only = false;
        if (angles[2 * i + 1] != 0) g.rot_z_only = g.rot_z2_only = false;
        zav += defocus[i];
    }
    zav /= nangles;
    g.zout = zav - p->dzextra;
    if (zrot)  // UTR.cpp:221: a Z'' rotation (from the second orientation on)
        for (int i = 1; i < nangles; i++)
            if (zrot[i] != 0) g.rot_y_only = g.rot_z_only = false;
    return MSK_OK;
}

// Host tables of one 3D correction (uploaded with the call's other tables).
struct CorrTabs {
    std::vector<double> lx, cx, ilx;
    std::vector<float> cxf;
    std::vector<float2> ex, ey, ez;
};

// (cos, sin) of a double phase, rounded to float
float2 expi_d(double ph) { return make_float2((float)cos(ph), (float)sin(ph)); }

// CTFcorrection3D's constants (UTR.h:27-83); MSK_EINVAL where it throws.
// The phase of voxel (k, j, i) is fac2 (ksi_i + eta_j + zeta_k) - omega (+ the
// Cs terms of ksi^2): its exponential is a product of per-axis factors.
int ctf_setup(UtrFourier &f, int nx, int ny, int nz, double wl, double zlo, double zhi,
              double ylo, double yhi, double xlo, double xhi, double defocdist, double q2max,
              double cs3, double cs5, double sigma, double epsilon, int escc, CorrTabs &t)
{
    if ((nx & 1) || (ny & 1) || (nz & 1)) return MSK_EINVAL;
    const double xst = (xhi - xlo) / nx, yst = (yhi - ylo) / ny, zst = (zhi - zlo) / ny;
    const double srad = sqrt(0.25 / (xst * xst) + 0.25 / (yst * yst) + 0.25 / (zst * zst));
    if (srad * wl > 1.0) return MSK_EINVAL;
    const double dksi2 = 1.0 / ((xhi - xlo) * (xhi - xlo));
    f.deta2 = 1.0 / ((yhi - ylo) * (yhi - ylo));
    f.dzeta2 = 1.0 / ((zhi - zlo) * (zhi - zlo));
    const double fac2 = kPi * wl * defocdist;
    if (epsilon <= 0)
        epsilon = 0.1 * pow(fabs(fac2) * std::min(dksi2, std::min(f.deta2, f.dzeta2)), 2);
    f.eps = (float)epsilon;
    f.fac3 = kPi * pow(wl, 3) / 2.0 * cs3;
    f.fac5 = kPi * pow(wl, 5) / 3.0 * cs5;
    const double omega = atan(sigma);
    f.c35 = (cs3 != 0) || (cs5 != 0);
    f.aper = q2max > 0;
    f.q2max = q2max;
    f.q2maxf = (float)q2max;
    f.escc = escc;
    t.cx.resize(nx);
    t.cxf.resize(nx);
    t.ex.resize(nx);
    for (int i = 0; i < nx; i++) {
        const int i1 = i - nx / 2;
        t.cx[i] = dksi2 * i1 * i1;
        t.cxf[i] = (float)t.cx[i];
        t.ex[i] = expi_d(fac2 * t.cx[i]);
    }
    t.ey.resize(ny);
    for (int j = 0; j < ny; j++) {
        const int j1 = j - ny / 2;
        t.ey[j] = expi_d(fac2 * (f.deta2 * j1 * j1));
    }
    t.ez.resize(nz);
    for (int k = 0; k < nz; k++) {
        const int k1 = k - nz / 2;
        t.ez[k] = expi_d(fac2 * (f.dzeta2 * k1 * k1) - omega);
    }
    f.corr = 4;
    return MSK_OK;
}

// InverseMLaplacian3D's constants (UTR.h:141-163) into (x table, y, z, alpha, norm).
int invlap_setup(int nx, int ny, int nz, double zaper, double yaper, double xaper, double alpha,
                 std::vector<double> &lx, double &ly, double &lz)
{
    if (alpha <= 0 || xaper == 0 || yaper == 0 || zaper == 0) return MSK_EINVAL;
    if ((nx & 1) || (ny & 1) || (nz & 1)) return MSK_EINVAL;
    const double fact = 4.0 * kPi * kPi;
    const double dksi2 = fact / (xaper * xaper);
    ly = fact / (yaper * yaper);
    lz = fact / (zaper * zaper);
    lx.resize(nx);
    for (int i = 0; i < nx; i++) {
        const int i1 = i - nx / 2;
        lx[i] = dksi2 * i1 * i1;
    }
    return MSK_OK;
}

// Per-image coordinate tables and scalars of CT_3Dgridding (UTR.h:214-236;
// UTR.cpp:880-898 for the angles and the centre-of-rotation factors).
void grid_tables(const msk_utr *p, const Geo &g, int nangles, const double *angles,
                 std::vector<float> &tabs, std::vector<float> &scal)
{
    const int nx = g.nx, ny = g.ny;
    const size_t ts = 3 * (size_t)nx + 3 * (size_t)ny;
    tabs.resize(ts * nangles);
    scal.resize((size_t)kScal * nangles);
    const float fxlo = (float)g.fxlo, fxst = (float)g.fxst, fylo = (float)g.fylo,
                fyst = (float)g.fyst;
    const double wl2 = 0.5 * p->wl, pi180 = kPi / 180.0, tpi = 2.0 * kPi;
    for (int a = 0; a < nangles; a++) {
        const double angleZ = angles[2 * a] * pi180, angleY = angles[2 * a + 1] * pi180;
        const float sinY = (float)sin(angleY), cosY = (float)cos(angleY);
        const float sinZ = (float)sin(angleZ), cosZ = (float)cos(angleZ);
        float *tb = tabs.data() + ts * a;
        for (int i = 0; i < nx; i++) {
            const float fs = fxst * (float)i;
            const double x = (double)(fxlo + fs);
            tb[i] = (float)(-wl2 * x * x);
            tb[nx + i] = (float)(x * (double)sinY);
            tb[2 * nx + i] = (float)(x * (double)cosY);
        }
        for (int j = 0; j < ny; j++) {
            const float fs = fyst * (float)j;
            const double y = (double)(fylo + fs);
            tb[3 * nx + j] = (float)(-wl2 * y * y);
            tb[3 * nx + ny + j] = (float)(y * (double)sinZ);
            tb[3 * nx + 2 * ny + j] = (float)(y * (double)cosZ);
        }
        const double cy = cos(angleY), sy = sin(angleY), cz = cos(angleZ), sz = sin(angleZ);
        const float ax = (float)(tpi * (p->dxc * (1.0 - cy * cz) - p->dyc * sz + p->dzc * sy * cz));
        const float ay = (float)(tpi * (p->dxc * cy * sz + p->dyc * (1.0 - cz) - p->dzc * sy * sz));
        const float az = (float)(tpi * (-p->dxc * sy + p->dzc * (1.0 - cy)));
        float *sc = scal.data() + (size_t)kScal * a;
        sc[0] = sinY;
        sc[1] = cosY;
        sc[2] = sinZ;
        sc[3] = cosZ;
        // fcomplex(0, -1) * float(a) = (0 * a, -1 * a)
        sc[4] = 0.0f * ax;
        sc[5] = -1.0f * ax;
        sc[6] = 0.0f * ay;
        sc[7] = -1.0f * ay;
        sc[8] = 0.0f * az;
        sc[9] = -1.0f * az;
    }
}

bool sizes_ok(int n) { return utr_ops(n) != nullptr && size_ops(n) != nullptr; }

// 2D view of `units` blocks of `lines` rows x `width` complex64 for a UTR
// column pass over lines of length `lines` (box: its UtrColCfg tile).
int utr_column_map(msk_context *ctx, ColView *view, void *base, int lines, size_t width,
                   size_t units, bool final_pass = false)
{
    auto enc = tensor_map_encoder();
    if (!enc) return fail(ctx, MSK_ECUDA, "cuTensorMapEncodeTiled is not available");
    const UtrOps *op = utr_ops(lines);
    const cuuint64_t dims[2] = {(cuuint64_t)2 * width, (cuuint64_t)units * lines};
    const cuuint64_t strides[1] = {(cuuint64_t)width * 8};
    const cuuint32_t box[2] = {(cuuint32_t)(2 * (final_pass ? op->col_c_final : op->col_c)),
                               (cuuint32_t)op->col_box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&view->map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box,
                     estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return fail(ctx, MSK_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    view->v = 0;
    return MSK_OK;
}

// Device tables of one call, packed into ctx->utr_tab (256-byte aligned).
struct TabPack {
    std::vector<unsigned char> host;
    size_t put(const void *p, size_t bytes)
    {
        const size_t at = host.size();
        host.resize(at + ((bytes + 255) & ~(size_t)255));
        if (bytes) std::memcpy(host.data() + at, p, bytes);
        return at;
    }
    template <typename T> size_t put(const std::vector<T> &v) { return put(v.data(), v.size() * sizeof(T)); }
};

// The 3D-correction tables of `t` into the pack, pointers resolved against `base`.
struct CorrOffsets {
    size_t lx, cx, cxf, ilx, ex, ey, ez;
};
CorrOffsets put_corr(TabPack &pk, CorrTabs &t, int nx, int ny, int nz)
{
    if (t.lx.empty()) t.lx.assign(nx, 0.0);
    if (t.cx.empty()) t.cx.assign(nx, 0.0);
    if (t.cxf.empty()) t.cxf.assign(nx, 0.0f);
    if (t.ilx.empty()) t.ilx.assign(nx, 0.0);
    if (t.ex.empty()) t.ex.assign(nx, make_float2(1.0f, 0.0f));
    if (t.ey.empty()) t.ey.assign(ny, make_float2(1.0f, 0.0f));
    if (t.ez.empty()) t.ez.assign(nz, make_float2(1.0f, 0.0f));
    CorrOffsets o;
    o.lx = pk.put(t.lx);
    o.cx = pk.put(t.cx);
    o.cxf = pk.put(t.cxf);
    o.ilx = pk.put(t.ilx);
    o.ex = pk.put(t.ex);
    o.ey = pk.put(t.ey);
    o.ez = pk.put(t.ez);
    return o;
}
void bind_corr(UtrFourier &f, const unsigned char *base, const CorrOffsets &o)
{
    f.lx = reinterpret_cast<const double *>(base + o.lx);
    f.cx = reinterpret_cast<const double *>(base + o.cx);
    f.cxf = reinterpret_cast<const float *>(base + o.cxf);
    f.ilx = reinterpret_cast<const double *>(base + o.ilx);
    f.ex = reinterpret_cast<const float2 *>(base + o.ex);
    f.ey = reinterpret_cast<const float2 *>(base + o.ey);
    f.ez = reinterpret_cast<const float2 *>(base + o.ez);
}

// Uploads a pack into ctx->utr_tab; returns its device base (null on failure).
unsigned char *upload_pack(msk_context *ctx, const TabPack &pk, int *st)
{
    *st = MSK_OK;
    cudaError_t e = ctx->utr_tab.reserve(std::max<size_t>(pk.host.size(), 256));
    if (e != cudaSuccess) {
        *st = fail(ctx, e == cudaErrorMemoryAllocation ? MSK_ENOMEM : MSK_ECUDA, "table allocation failed");
        return nullptr;
    }
    e = cudaMemcpyAsync(ctx->utr_tab.p, pk.host.data(), pk.host.size(), cudaMemcpyHostToDevice,
                        ctx->stream);
    if (e != cudaSuccess) {
        *st = fail(ctx, MSK_ECUDA, std::string("table upload: ") + cudaGetErrorString(e));
        return nullptr;
    }
    count_copy(ctx, 0, (double)pk.host.size());
    return ctx->utr_tab.as<unsigned char>();
}

int upload(msk_context *ctx, void *dst, const void *src, size_t bytes)
{
    if (!bytes) return MSK_OK;
    MSK_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    count_copy(ctx, 0, (double)bytes);
    return MSK_OK;
}

int grid_blocks(size_t n)
{
    return (int)std::min<size_t>((n + 255) / 256, (size_t)152 * 16);
}

// Images (device) -> centred spectra in ctx->utr_k2 and the magnitude bound.
// Images (device) -> centred spectra in ctx->utr_k2.
// Images a0 .. a0 + nangles - 1 (img_d points at image a0) -> their spectra in
// ctx->utr_k2, which the caller has reserved for every image; err: the
// call's device error flag.
int spectra(msk_context *ctx, const msk_utr *p, int a0, int nangles, const float *img_d,
            const float2 *tw_x, const float2 *tw_y, int *err)
{
    const int nx = p->nx, ny = p->ny;
    const size_t plane = (size_t)nx * ny;
    float2 *k2 = ctx->utr_k2.as<float2>() + (size_t)a0 * plane;
    UtrImg ip{};
    ip.nx = nx;
    ip.ny = ny;
    ip.nrows = ny * nangles;
    ip.f1 = (float)p->f1;
    ip.f2 = (float)p->f2;
    ip.use_f1 = p->f1 != 1.0;
    ip.use_f2 = p->f2 != 0.0;
    ip.tw = tw_x;
    {
        Prof pr(ctx, kUtrImgRows, 12.0 * plane * nangles);
        utr_ops(nx)->img_rows(ip, img_d, k2, ctx->stream);
    }
    ColView view;
    int st = utr_column_map(ctx, &view, k2, ny, nx, (size_t)nangles);
    if (st) return st;
    UtrCol cp{};
    cp.width = nx;
    cp.tw = tw_y;
    cp.err = err;
    Prof pr(ctx, kUtrImgCols, 16.0 * plane * nangles);
    utr_ops(ny)->col_img(cp, view.map, view.map, nangles, ctx->stream);
    return MSK_OK;
}

int grid_launch(msk_context *ctx, const msk_utr *p, const Geo &g, int nangles, const float2 *k2,
                const float *tabs_d, const float *scal_d, UtrAcc *acc)
{
    UtrGridP gp{};
    gp.nx = g.nx;
    gp.ny = g.ny;
    gp.nz = g.nz;
    gp.nimg = nangles;
    gp.k2 = k2;
    gp.tabs = tabs_d;
    gp.scal = scal_d;
    gp.fxlo = (float)g.fxlo;
    gp.fxst = (float)g.fxst;
    gp.fylo = (float)g.fylo;
    gp.fyst = (float)g.fyst;
    gp.fzlo = (float)g.fzlo;
    gp.fzst = (float)g.fzst;
    gp.rotshift = p->dxc != 0 || p->dyc != 0 || p->dzc != 0;
    gp.escc = p->escc != 0;
    gp.acc = acc;
    const size_t n = (size_t)g.nx * g.ny * nangles;
    Prof pr(ctx, kUtrGrid, 8.0 * n);
    k_utr_grid<<<grid_blocks(n), 256, 0, ctx->stream>>>(gp);
    return MSK_OK;
}

int check_params(msk_context *ctx, const msk_utr *p, int nangles, const double *angles,
                 const double *defocus)
{
    if (!p || nangles < 1 || !angles || !defocus) return fail(ctx, MSK_EINVAL, "bad UTR arguments");
    if (p->modality != 0 && p->modality != 1) return fail(ctx, MSK_EINVAL, "modality must be 0 or 1");
    if (p->f1 == 0.0) return fail(ctx, MSK_EINVAL, "the first normalisation factor cannot be zero");
    if (!(p->wl > 0.0) || p->wl > 1.0) return fail(ctx, MSK_EINVAL, "wavelength out of range");
    if (p->aobj < 0 || p->aobj > 1000) return fail(ctx, MSK_EINVAL, "objective aperture out of range");
    if (p->nsr < 0) return fail(ctx, MSK_EINVAL, "noise-to-signal ratio must be non-negative");
    if (p->epsilon < 0) return fail(ctx, MSK_EINVAL, "regularisation must be non-negative");
    if (p->epsilon == 0 && p->asigma == 0)
        return fail(ctx, MSK_EINVAL, "with beta/delta = 0, epsilon must be positive");
    if (p->modality == 0 && p->asigma < 0) return fail(ctx, MSK_EINVAL, "beta/delta must be >= 0 (TEM)");
    if (p->modality == 1 && p->asigma >= 0) return fail(ctx, MSK_EINVAL, "beta/delta must be < 0 (X-ray)");
    if (p->ctf_mode == 1 || p->ctf_mode == 3)
        return fail(ctx, MSK_EUNSUPPORTED, "2D TIE-Hom / CTF phase retrieval is not provided");
    if (p->ctf_mode != 0 && p->ctf_mode != 2 && p->ctf_mode != 4)
        return fail(ctx, MSK_EINVAL, "unknown phase retrieval mode");
    if (p->asigma >= 0 && p->ctf_mode == 2)
        return fail(ctx, MSK_EINVAL, "beta/delta must be negative in TIE-Hom phase retrieval");
    if (nangles > (1 << 20)) return fail(ctx, MSK_EINVAL, "too many orientations");
    return MSK_OK;
}

}  // namespace
}  // namespace msk

using namespace msk;

extern "C" {

int msk_utr_depth(const msk_utr *p) { return depth_of(p, nullptr, nullptr); }

int msk_utr_reconstruct(msk_context *ctx, const msk_utr *p, int nangles, const double *angles,
                        const double *defocus, const float *images, float *volume)
{
    return msk_utr_reconstruct_planes(ctx, p, nangles, angles, defocus, nullptr, nullptr, images,
                                      volume);
}

int msk_utr_reconstruct_planes(msk_context *ctx, const msk_utr *p, int nangles,
                               const double *angles, const double *defocus, const double *zrot,
                               const double *shifts, const float *images, float *volume)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    int st = check_params(ctx, p, nangles, angles, defocus);
    if (st) return st;
    if (!images || !volume) return fail(ctx, MSK_EINVAL, "null image or volume pointer");
    Geo g{};
    st = make_geo(ctx, p, nangles, angles, defocus, g, zrot);
    if (st) return st;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (!sizes_ok(nx) || !sizes_ok(ny) || !sizes_ok(nz))
        return fail(ctx, MSK_EUNSUPPORTED, "nx, ny and the depth must be powers of two from 16 to 4096");
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));

    // Fourier-space stage constants (UTR.cpp:1052-1201)
    UtrFourier fr{};
    fr.nx = nx;
    fr.ny = ny;
    fr.nz = nz;
    fr.nsr = (float)(p->nsr * sqrt((double)nx * ny));
    fr.inv_nsr = fr.nsr != 0.0f ? (float)(1.0 / (p->nsr * sqrt((double)nx * ny))) : 0.0f;
    CorrTabs ct;
    // the x extent passed to InverseMLaplacian3D is xhi - ylo, as UTR.cpp:1186
    // and 1200 pass it (equal to xhi - xlo for the square images it reads)
    if (g.zout != 0) {
        if (p->ctf_mode == 2) {
            const double alpha = -4.0 * kPi * p->asigma / (g.zout * p->wl);
            const double norm = -alpha * sqrt(1.0 + p->asigma * p->asigma) / p->asigma;
            if (invlap_setup(nx, ny, nz, g.zhi - g.zlo, g.yhi - g.ylo, g.xhi - g.ylo, alpha, ct.lx,
                             fr.ly, fr.lz))
                return fail(ctx, MSK_EINVAL, "InverseMLaplacian3D: alpha <= 0 or a zero aperture");
            fr.corr = 2;
            fr.lalpha = alpha;
            fr.lnorm = norm;
        } else if (p->ctf_mode == 4) {
            if (ctf_setup(fr, nx, ny, nz, p->wl, g.zlo, g.zhi, g.ylo, g.yhi, g.xlo, g.xhi, g.zout,
                          g.k2maxo, g.cs3, g.cs5, p->asigma, p->epsilon, p->escc, ct))
                return fail(ctx, MSK_EINVAL, "CTFcorrection3D: evanescent waves present");
        }
    }
    if (p->inv_laplace && p->ctf_mode != 1 && p->ctf_mode != 2) {
        if (invlap_setup(nx, ny, nz, g.zhi - g.zlo, g.yhi - g.ylo, g.xhi - g.ylo, p->epsilon,
                         ct.ilx, fr.ily, fr.ilz))
            return fail(ctx, MSK_EINVAL, "inverse Laplacian filter: epsilon must be positive");
        fr.invlap = 1;
        fr.ilalpha = p->epsilon;
        fr.ilnorm = p->epsilon;
    }
    fr.nyq = 1;
    fr.modulate = 1;

    // output stage (UTR.cpp:1235-1278): the mask radius, exp(dtemp d^2) per
    // axis (1 for an axis the mask leaves out) and the output scale
    const bool use_y = !g.rot_y_only, use_z = !(g.rot_z_only || g.rot_z2_only);
    const long long nxd2 = nx / 2, nyd2 = ny / 2, nzd2 = nz / 2;
    const long long nxR2 = g.ic <= nxd2 ? g.ic * g.ic : (nx - g.ic) * (nx - g.ic);
    const long long nyR2 = g.jc <= nyd2 ? g.jc * g.jc : (ny - g.jc) * (ny - g.jc);
    const long long nzR2 = g.kc <= nzd2 ? g.kc * g.kc : (nz - g.kc) * (nz - g.kc);
    long long nR2;
    if (g.rot_y_only) nR2 = std::min(nxR2, nzR2);
    else if (g.rot_z_only || g.rot_z2_only) nR2 = std::min(nxR2, nyR2);
    else nR2 = std::min(std::min(nxR2, nyR2), nzR2);
    const double dtemp = 2.0 / (double)(g.kc * g.kc + g.jc * g.jc + g.ic * g.ic);
    std::vector<float> mx(nx), my(ny), mz(nz);
    for (int i = 0; i < nx; i++) mx[i] = (float)exp(dtemp * (double)((i - g.ic) * (i - g.ic)));
    for (int j = 0; j < ny; j++) my[j] = use_y ? (float)exp(dtemp * (double)((j - g.jc) * (j - g.jc))) : 1.0f;
    for (int k = 0; k < nz; k++) mz[k] = use_z ? (float)exp(dtemp * (double)((k - g.kc) * (k - g.kc))) : 1.0f;
    const double fnorm =
        p->modality == 0
            ? g.ee * p->wl / (2.0 * kPi * sqrt(1.0 + p->asigma * p->asigma) * g.xst)
            : p->asigma * p->wl / (4.0 * kPi * sqrt(1.0 + p->asigma * p->asigma) * g.xst);

    // tables
    std::vector<float> tabs, scal;
    grid_tables(p, g, nangles, angles, tabs, scal);
    std::vector<float2> twx, twy, twz;
    if (!twiddles(nx, twx) || !twiddles(ny, twy) || !twiddles(nz, twz))
        return fail(ctx, MSK_EUNSUPPORTED, "no FFT for this size");
    // input image planes (UTR.cpp:920-940): per image the operation, cos and
    // sin of t = -Z'', and the whole-pixel shift back
    std::vector<int> pop(nangles, 0);
    std::vector<double> ppar(4 * (size_t)nangles, 0.0);
    bool any_plane = false;
    for (int a = 0; a < nangles; a++) {
        const double z2 = zrot ? zrot[a] : 0.0;
        const double shx = shifts ? shifts[2 * a] : 0.0, shy = shifts ? shifts[2 * a + 1] : 0.0;
        if (z2 == 0.0 && shx == 0.0 && shy == 0.0) continue;
        const double t = -z2 * kPi / 180.0;
        pop[a] = z2 != 0.0 ? 2 : 1;
        ppar[4 * a] = cos(t);
        ppar[4 * a + 1] = sin(t);
        ppar[4 * a + 2] = floor(-shx / p->xst + 0.5);
        ppar[4 * a + 3] = floor(-shy / p->xst + 0.5);
        any_plane = true;
    }
    TabPack pk;
    const size_t o_pop = pk.put(pop), o_ppar = pk.put(ppar);
    std::vector<float> fill0(nangles, 0.0f);
    const size_t o_fill = pk.put(fill0);
    const size_t o_twx = pk.put(twx), o_twy = pk.put(twy), o_twz = pk.put(twz);
    const CorrOffsets oc = put_corr(pk, ct, nx, ny, nz);
    const size_t o_mx = pk.put(mx), o_my = pk.put(my), o_mz = pk.put(mz);
    const size_t o_tabs = pk.put(tabs), o_scal = pk.put(scal);
    unsigned char *tb = upload_pack(ctx, pk, &st);
    if (!tb) return st;
    const float2 *tw_x = reinterpret_cast<const float2 *>(tb + o_twx);
    const float2 *tw_y = reinterpret_cast<const float2 *>(tb + o_twy);
    const float2 *tw_z = reinterpret_cast<const float2 *>(tb + o_twz);
    bind_corr(fr, tb, oc);

    // images in, spectra, gridding
    const size_t plane = (size_t)nx * ny, nvox = plane * nz;
    Geom gflags{};  // the call's device error flag, cleared once
    if ((st = flags_reset(ctx, gflags))) return st;
    MSK_CUDA(ctx, ctx->utr_k2.reserve(sizeof(float2) * plane * nangles));
    MSK_CUDA(ctx, ctx->utr_acc.reserve(sizeof(UtrAcc) * nvox));
    UtrAcc *acc = ctx->utr_acc.as<UtrAcc>();
    MSK_CUDA(ctx, cudaMemsetAsync(acc, 0, sizeof(UtrAcc) * nvox, ctx->stream));
    const float *tabs_d = reinterpret_cast<const float *>(tb + o_tabs);
    const float *scal_d = reinterpret_cast<const float *>(tb + o_scal);
    const int tstride = 3 * nx + 3 * ny;
    const float *img_d = images;
    const bool img_host = !is_device_ptr(images);
    if (img_host) {
        MSK_CUDA(ctx, ctx->utr_img.reserve(sizeof(float) * plane * nangles));
        img_d = ctx->utr_img.as<float>();
    }
    if (img_host && !any_plane) {
        // host images in chunks on the copy-in stream: each chunk's spectra
        // and gridding run while the next chunk comes in
        const int nch = std::min(nangles, 8), per = (nangles + nch - 1) / nch;
        if (!ctx->stk_ev[0])
            for (cudaEvent_t &e : ctx->stk_ev)
                MSK_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        MSK_CUDA(ctx, cudaEventRecord(ctx->stk_ev[6], ctx->stream));
        MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->aux, ctx->stk_ev[6], 0));
        for (int a0 = 0, c = 0; a0 < nangles; a0 += per, c++) {
            const int na = std::min(per, nangles - a0);
            float *dst = ctx->utr_img.as<float>() + (size_t)a0 * plane;
            MSK_CUDA(ctx, cudaMemcpyAsync(dst, images + (size_t)a0 * plane,
                                          sizeof(float) * plane * na, cudaMemcpyHostToDevice,
                                          ctx->aux));
            count_copy(ctx, 0, (double)sizeof(float) * plane * na);
            cudaEvent_t ev = ctx->stk_ev[c & 1];
            MSK_CUDA(ctx, cudaEventRecord(ev, ctx->aux));
            MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev, 0));
            if ((st = spectra(ctx, p, a0, na, dst, tw_x, tw_y, gflags.err))) return st;
            if ((st = grid_launch(ctx, p, g, na, ctx->utr_k2.as<float2>() + (size_t)a0 * plane,
                                  tabs_d + (size_t)a0 * tstride, scal_d + (size_t)a0 * kScal,
                                  acc)))
                return st;
        }
    } else {
        if (img_host &&
            (st = upload(ctx, ctx->utr_img.p, images, sizeof(float) * plane * nangles)))
            return st;
        if (any_plane) {
            UtrPlaneP pp{};
            pp.nx = nx;
            pp.ny = ny;
            pp.nimg = nangles;
            pp.f1 = (float)p->f1;
            pp.f2 = (float)p->f2;
            pp.use_f1 = p->f1 != 1.0;
            pp.use_f2 = p->f2 != 0.0;
            pp.cx = (((g.xhi + g.xlo) / 2.0 + p->dxc) - g.xlo) / p->xst;
            pp.cy = (((g.yhi + g.ylo) / 2.0 + p->dyc) - g.ylo) / p->xst;
            pp.par = reinterpret_cast<const double *>(tb + o_ppar);
            pp.op = reinterpret_cast<const int *>(tb + o_pop);
            float *fill = reinterpret_cast<float *>(tb + o_fill);
            pp.fill = fill;
            MSK_CUDA(ctx, ctx->utr_stage.reserve(sizeof(float) * plane * nangles));
            float *staged = ctx->utr_stage.as<float>();
            {
                Prof pr(ctx, kUtrPoint, 8.0 * plane * nangles);
                k_utr_edge_mean<<<nangles, 256, 0, ctx->stream>>>(pp, img_d, fill);
                k_utr_img_plane<<<grid_blocks(plane * nangles), 256, 0, ctx->stream>>>(pp, img_d, staged);
            }
            msk_utr q = *p;  // the staged images are normalised
            q.f1 = 1.0;
            q.f2 = 0.0;
            if ((st = spectra(ctx, &q, 0, nangles, staged, tw_x, tw_y, gflags.err))) return st;
        } else if ((st = spectra(ctx, p, 0, nangles, img_d, tw_x, tw_y, gflags.err))) {
            return st;
        }
        if ((st = grid_launch(ctx, p, g, nangles, ctx->utr_k2.as<float2>(), tabs_d, scal_d, acc)))
            return st;
    }

    // Fourier-space processing and the inverse 3D transform
    MSK_CUDA(ctx, ctx->utr_vol.reserve(sizeof(float2) * nvox));
    float2 *vol = ctx->utr_vol.as<float2>();
    {
        Prof pr(ctx, kUtrFourier, 24.0 * nvox);
        utr_ops(nx)->fourier_rows(fr, tw_x, acc, vol, ny * nz, ctx->stream);
    }
    ColView vy, vz;
    if ((st = utr_column_map(ctx, &vy, vol, ny, nx, (size_t)nz))) return st;
    if ((st = utr_column_map(ctx, &vz, vol, nz, (size_t)nx * ny, 1, true))) return st;
    UtrCol cy{};
    cy.width = nx;
    cy.tw = tw_y;
    cy.err = gflags.err;
    {
        Prof pr(ctx, kUtrVolCols, 16.0 * nvox);
        utr_ops(ny)->col_vol(cy, vy.map, vy.map, nz, ctx->stream);
    }
    float *out_d = volume;
    const bool out_dev = is_device_ptr(volume);
    if (!out_dev) {
        MSK_CUDA(ctx, ctx->utr_out.reserve(sizeof(float) * nvox));
        out_d = ctx->utr_out.as<float>();
    }
    UtrCol cz{};
    cz.width = nx * ny;
    cz.tw = tw_z;
    cz.err = gflags.err;
    cz.out = out_d;
    cz.nx = nx;
    cz.ny = ny;
    cz.nxlog = ilog2i(nx);
    cz.inv_n = (float)(1.0 / ((double)nvox));
    cz.fnorm = (float)fnorm;
    cz.ic = g.ic;
    cz.jc = g.jc;
    cz.kc = g.kc;
    cz.nr2 = nR2;
    cz.use_y = use_y;
    cz.use_z = use_z;
    cz.ex = reinterpret_cast<const float *>(tb + o_mx);
    cz.ey = reinterpret_cast<const float *>(tb + o_my);
    cz.ez = reinterpret_cast<const float *>(tb + o_mz);
    // A host volume goes out in chunks of rows y: chunk c's z pass, then its
    // copy (nz rows of the chunk's ny/nch x nx floats, one 2D copy) on the
    // copy-out stream while the z pass of chunk c + 1 runs.
    const int nch = out_dev ? 1 : std::min(8, ny);
    const int cpc = utr_ops(nz)->col_c_final;                 // columns per block
    const int ncb = (int)((size_t)nx * (ny / nch) / cpc);     // blocks per chunk
    if (!out_dev && !ctx->stk_ev[0])
        for (cudaEvent_t &e : ctx->stk_ev)
            MSK_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!out_dev) {  // the copies start after the work already queued on the library's stream
        MSK_CUDA(ctx, cudaEventRecord(ctx->stk_ev[6], ctx->stream));
        MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->aux2, ctx->stk_ev[6], 0));
    }
    for (int c = 0; c < nch; c++) {
        cz.cb0 = c * ncb;
        cz.ncb = nch > 1 ? ncb : 0;
        {
            Prof pr(ctx, kUtrFinal, 12.0 * nvox / nch);
            utr_ops(nz)->col_final(cz, vz.map, 1, ctx->stream);
        }
        if (!out_dev) {
            const size_t y0 = (size_t)c * (ny / nch), pitch = sizeof(float) * plane;
            cudaEvent_t ev = ctx->stk_ev[c & 1];
            MSK_CUDA(ctx, cudaEventRecord(ev, ctx->stream));
            MSK_CUDA(ctx, cudaStreamWaitEvent(ctx->aux2, ev, 0));
            MSK_CUDA(ctx, cudaMemcpy2DAsync(volume + y0 * nx, pitch, out_d + y0 * nx, pitch,
                                            sizeof(float) * nx * (ny / nch), nz,
                                            cudaMemcpyDeviceToHost, ctx->aux2));
        }
    }
    MSK_CUDA(ctx, cudaGetLastError());
    if (!out_dev) {
        count_copy(ctx, 1, (double)sizeof(float) * nvox);
        MSK_CUDA(ctx, cudaStreamSynchronize(ctx->aux2));
    }
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    return flags_check(ctx);
}

int msk_utr_grid(msk_context *ctx, const msk_utr *p, int nangles, const double *angles,
                 const float *k2four, float *v3, float *samp3)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!p || nangles < 1 || !angles || !k2four || !v3 || !samp3)
        return fail(ctx, MSK_EINVAL, "bad UTR gridding arguments");
    std::vector<double> defocus(nangles, 0.0);
    Geo g{};
    int st = make_geo(ctx, p, nangles, angles, defocus.data(), g);
    if (st) return st;
    if (g.nx < 2 || g.ny < 2 || g.nz < 2) return fail(ctx, MSK_EINVAL, "volume too small");
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<float> tabs, scal;
    grid_tables(p, g, nangles, angles, tabs, scal);
    TabPack pk;
    const size_t o_tabs = pk.put(tabs), o_scal = pk.put(scal);
    unsigned char *tb = upload_pack(ctx, pk, &st);
    if (!tb) return st;
    const size_t plane = (size_t)g.nx * g.ny, nvox = plane * g.nz;
    const float2 *k2_d = reinterpret_cast<const float2 *>(k2four);
    if (!is_device_ptr(k2four)) {
        MSK_CUDA(ctx, ctx->utr_k2.reserve(sizeof(float2) * plane * nangles));
        if ((st = upload(ctx, ctx->utr_k2.p, k2four, sizeof(float2) * plane * nangles))) return st;
        k2_d = ctx->utr_k2.as<float2>();
    }
    MSK_CUDA(ctx, ctx->utr_acc.reserve(sizeof(UtrAcc) * nvox));
    UtrAcc *acc = ctx->utr_acc.as<UtrAcc>();
    MSK_CUDA(ctx, cudaMemsetAsync(acc, 0, sizeof(UtrAcc) * nvox, ctx->stream));
    if ((st = grid_launch(ctx, p, g, nangles, k2_d, reinterpret_cast<const float *>(tb + o_tabs),
                          reinterpret_cast<const float *>(tb + o_scal), acc)))
        return st;
    const bool vdev = is_device_ptr(v3), sdev = is_device_ptr(samp3);
    float2 *v_d = reinterpret_cast<float2 *>(v3);
    float *s_d = samp3;
    if (!vdev || !sdev) {
        MSK_CUDA(ctx, ctx->utr_vol.reserve(sizeof(float2) * nvox + sizeof(float) * nvox));
        if (!vdev) v_d = ctx->utr_vol.as<float2>();
        if (!sdev) s_d = reinterpret_cast<float *>(ctx->utr_vol.as<float2>() + nvox);
    }
    {
        Prof pr(ctx, kUtrPoint, 28.0 * nvox);
        k_utr_acc_split<<<grid_blocks(nvox), 256, 0, ctx->stream>>>(acc, nvox, v_d, s_d);
    }
    MSK_CUDA(ctx, cudaGetLastError());
    if (!vdev) {
        MSK_CUDA(ctx, cudaMemcpyAsync(v3, v_d, sizeof(float2) * nvox, cudaMemcpyDeviceToHost, ctx->stream));
        count_copy(ctx, 1, (double)sizeof(float2) * nvox);
    }
    if (!sdev) {
        MSK_CUDA(ctx, cudaMemcpyAsync(samp3, s_d, sizeof(float) * nvox, cudaMemcpyDeviceToHost, ctx->stream));
        count_copy(ctx, 1, (double)sizeof(float) * nvox);
    }
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    return MSK_OK;
}

}  // extern "C"

namespace {

// One pointwise pass over a caller's complex volume, staged through the
// context when it is in host memory.
int point_pass(msk_context *ctx, float *v3, size_t nvox, UtrFourier &f, CorrTabs &t)
{
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    TabPack pk;
    const CorrOffsets oc = put_corr(pk, t, f.nx, f.ny, f.nz);
    int st;
    unsigned char *tb = upload_pack(ctx, pk, &st);
    if (!tb) return st;
    bind_corr(f, tb, oc);
    float2 *v_d = reinterpret_cast<float2 *>(v3);
    const bool dev = is_device_ptr(v3);
    if (!dev) {
        MSK_CUDA(ctx, ctx->utr_vol.reserve(sizeof(float2) * nvox));
        v_d = ctx->utr_vol.as<float2>();
        if ((st = upload(ctx, v_d, v3, sizeof(float2) * nvox))) return st;
    }
    {
        Prof pr(ctx, kUtrPoint, 16.0 * nvox);
        k_utr_point<<<grid_blocks(nvox), 256, 0, ctx->stream>>>(f, v_d);
    }
    MSK_CUDA(ctx, cudaGetLastError());
    if (!dev) {
        MSK_CUDA(ctx, cudaMemcpyAsync(v3, v_d, sizeof(float2) * nvox, cudaMemcpyDeviceToHost, ctx->stream));
        count_copy(ctx, 1, (double)sizeof(float2) * nvox);
    }
    MSK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    return MSK_OK;
}

}  // namespace

extern "C" {

int msk_utr_ctf_correction3d(msk_context *ctx, float *v3, int nx, int ny, int nz, double wl,
                             double zlo, double zhi, double ylo, double yhi, double xlo,
                             double xhi, double defocdist, double q2max, double cs3, double cs5,
                             double sigma, double epsilon, int escc)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!v3 || nx < 2 || ny < 2 || nz < 2) return fail(ctx, MSK_EINVAL, "bad volume");
    UtrFourier f{};
    f.nx = nx;
    f.ny = ny;
    f.nz = nz;
    CorrTabs t;
    if (ctf_setup(f, nx, ny, nz, wl, zlo, zhi, ylo, yhi, xlo, xhi, defocdist, q2max, cs3, cs5,
                  sigma, epsilon, escc, t))
        return fail(ctx, MSK_EINVAL, "CTFcorrection3D: odd sizes or evanescent waves");
    return point_pass(ctx, v3, (size_t)nx * ny * nz, f, t);
}

int msk_utr_inverse_mlaplacian3d(msk_context *ctx, float *v3, int nx, int ny, int nz,
                                 double zaper, double yaper, double xaper, double alpha,
                                 double norm)
{
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    if (!v3 || nx < 2 || ny < 2 || nz < 2) return fail(ctx, MSK_EINVAL, "bad volume");
    UtrFourier f{};
    f.nx = nx;
    f.ny = ny;
    f.nz = nz;
    CorrTabs t;
    if (invlap_setup(nx, ny, nz, zaper, yaper, xaper, alpha, t.lx, f.ly, f.lz))
        return fail(ctx, MSK_EINVAL, "InverseMLaplacian3D: alpha <= 0, a zero aperture or odd sizes");
    f.corr = 2;
    f.lalpha = alpha;
    f.lnorm = norm;
    return point_pass(ctx, v3, (size_t)nx * ny * nz, f, t);
}

}  // extern "C"
