// utr_host.cu -- the UTR reconstruction (include/msk_utr.h): host geometry,
// the gridding kernel, the pointwise Fourier-space kernels and the schedule
// of passes.
//
// Data layout in HBM for one call (nimg images of ny x nx, a volume of
// nz x ny x nx):
//   images   float   [nimg][ny][nx]     (the caller's, or a staged copy)
//   k2       complex [nimg][ny][nx]     centred image spectra
//   acc      UtrAcc  [nz][ny][nx]       fixed-point gridding sums (32 B)
//   vol      complex [nz][ny][nx]       the spectrum, then its inverse in place
//   out      float   [nz][ny][nx]       the caller's, or a staged copy
// Gridding sums are int64 fixed point (atomic adds are exact and order-free,
// so the result does not depend on the schedule); the scale is a power of
// two chosen from the largest spectrum magnitude, with headroom for 16
// contributions per image and voxel.
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
    int rotshift, escc, hb;
    const unsigned *maxbits;
    UtrAcc *acc;
};

__device__ __forceinline__ void red_add(long long *p, long long v)
{
    atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}

// CT_3Dgridding (UTR.h:199-307) of every pixel of every image: the pixel's
// frequency coordinates rotated back (about Y' then Z), on the Ewald sphere
// with the curvature correction, the enclosing voxel cell, and trilinear
// weights, all in float with the reference's operation order; each of the
// eight corners gets weight * value and the weight, as fixed-point atomics.
__global__ void __launch_bounds__(256) k_utr_grid(const UtrGridP p)
{
    const size_t npix = (size_t)p.nx * p.ny, total = npix * p.nimg;
    const size_t nxny = npix;
    const float vs = utr_pow2f(utr_vexp(*p.maxbits, p.hb)), ws = utr_pow2f(61 - p.hb);
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
                    UtrAcc *v = p.acc + (size_t)(nn + zc) * nxny + (size_t)(jj + b) * p.nx + (ii + e);
                    red_add(&v->re, __float2ll_rn(__fmul_rn(__fmul_rn(cd.x, w), vs)));
                    red_add(&v->im, __float2ll_rn(__fmul_rn(__fmul_rn(cd.y, w), vs)));
                    red_add(&v->w, __float2ll_rn(__fmul_rn(w, ws)));
                }
    }
}

// max |re|, |im| of complex data (for spectra the caller supplies)
__global__ void k_utr_maxabs(const float2 *__restrict__ a, size_t n, unsigned *maxbits)
{
    float mx = 0.0f;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const float2 v = a[q];
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    const unsigned bits = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, bits);
}

// gridding sums -> float volumes (msk_utr_grid)
__global__ void k_utr_acc_float(const UtrAcc *__restrict__ acc, size_t n, const unsigned *maxbits,
                                int hb, float2 *__restrict__ v3, float *__restrict__ samp3)
{
    const float vinv = utr_pow2f(-utr_vexp(*maxbits, hb)), winv = utr_pow2f(-(61 - hb));
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const UtrAcc a = acc[q];
        v3[q] = make_float2(__fmul_rn(__ll2float_rn(a.re), vinv), __fmul_rn(__ll2float_rn(a.im), vinv));
        samp3[q] = __fmul_rn(__ll2float_rn(a.w), winv);
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
             const double *defocus, Geo &g)
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
    return MSK_OK;
}

// CTFcorrection3D's constants (UTR.h:27-83); MSK_EINVAL where it throws.
int ctf_setup(UtrFourier &f, int nx, int ny, int nz, double wl, double zlo, double zhi,
              double ylo, double yhi, double xlo, double xhi, double defocdist, double q2max,
              double cs3, double cs5, double sigma, double epsilon, int escc,
              std::vector<double> &cx, std::vector<double> &cfx)
{
    if ((nx & 1) || (ny & 1) || (nz & 1)) return MSK_EINVAL;
    const double xst = (xhi - xlo) / nx, yst = (yhi - ylo) / ny, zst = (zhi - zlo) / ny;
    const double srad = sqrt(0.25 / (xst * xst) + 0.25 / (yst * yst) + 0.25 / (zst * zst));
    if (srad * wl > 1.0) return MSK_EINVAL;
    const double dksi2 = 1.0 / ((xhi - xlo) * (xhi - xlo));
    f.deta2 = 1.0 / ((yhi - ylo) * (yhi - ylo));
    f.dzeta2 = 1.0 / ((zhi - zlo) * (zhi - zlo));
    f.fac2 = kPi * wl * defocdist;
    if (epsilon <= 0)
        epsilon = 0.1 * pow(fabs(f.fac2) * std::min(dksi2, std::min(f.deta2, f.dzeta2)), 2);
    f.eps = epsilon;
    f.fac3 = kPi * pow(wl, 3) / 2.0 * cs3;
    f.fac5 = kPi * pow(wl, 5) / 3.0 * cs5;
    f.omega = atan(sigma);
    f.c35 = (cs3 != 0) || (cs5 != 0);
    f.aper = q2max > 0;
    f.q2max = q2max;
    f.escc = escc;
    cx.resize(nx);
    cfx.resize(nx);
    for (int i = 0; i < nx; i++) {
        const int i1 = i - nx / 2;
        cx[i] = dksi2 * i1 * i1;
        cfx[i] = f.fac2 * cx[i];
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

int headroom_bits(int nangles) { return 5 + ilog2i(std::max(1, nangles)); }

bool sizes_ok(int n) { return utr_ops(n) != nullptr && size_ops(n) != nullptr; }

// Device scratch of one call: tables at fixed offsets in ctx->utr_tab.
struct TabLayout {
    size_t maxbits, tw_x, tw_y, tw_z, lx, cx, cfx, ilx, ex, ey, ez, tabs, scal, total;
};

TabLayout tab_layout(int nx, int ny, int nz, size_t ntabs, size_t nscal, size_t ntw = 0)
{
    TabLayout o{};
    size_t at = 0;
    auto put = [&](size_t bytes) {
        const size_t here = at;
        at += (bytes + 255) & ~(size_t)255;
        return here;
    };
    o.maxbits = put(256);
    o.tw_x = put(sizeof(float2) * std::max<size_t>(ntw, 2 * (size_t)nx));
    o.tw_y = put(sizeof(float2) * std::max<size_t>(ntw, 2 * (size_t)ny));
    o.tw_z = put(sizeof(float2) * std::max<size_t>(ntw, 2 * (size_t)nz));
    o.lx = put(sizeof(double) * nx);
    o.cx = put(sizeof(double) * nx);
    o.cfx = put(sizeof(double) * nx);
    o.ilx = put(sizeof(double) * nx);
    o.ex = put(sizeof(double) * nx);
    o.ey = put(sizeof(double) * ny);
    o.ez = put(sizeof(double) * nz);
    o.tabs = put(sizeof(float) * ntabs);
    o.scal = put(sizeof(float) * nscal);
    o.total = at;
    return o;
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
int spectra(msk_context *ctx, const msk_utr *p, int nangles, const float *img_d,
            const float2 *tw_x, const float2 *tw_y, unsigned *maxbits)
{
    const int nx = p->nx, ny = p->ny;
    const size_t plane = (size_t)nx * ny;
    MSK_CUDA(ctx, ctx->utr_k2.reserve(sizeof(float2) * plane * nangles));
    float2 *k2 = ctx->utr_k2.as<float2>();
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
    int st = column_map(ctx, &view, k2, ny, nx, (size_t)nangles, size_ops(ny), 0);
    if (st) return st;
    Geom gdummy{};
    st = flags_reset(ctx, gdummy);
    if (st) return st;
    UtrCol cp{};
    cp.width = nx;
    cp.tw = tw_y;
    cp.err = gdummy.err;
    cp.maxbits = maxbits;
    Prof pr(ctx, kUtrImgCols, 16.0 * plane * nangles);
    utr_ops(ny)->col_img(cp, view.map, view.map, nangles, ctx->stream);
    return MSK_OK;
}

int grid_launch(msk_context *ctx, const msk_utr *p, const Geo &g, int nangles, const float2 *k2,
                const float *tabs_d, const float *scal_d, const unsigned *maxbits, UtrAcc *acc)
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
    gp.hb = headroom_bits(nangles);
    gp.maxbits = maxbits;
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
    if (!ctx) return MSK_EINVAL;
    ctx->err.clear();
    int st = check_params(ctx, p, nangles, angles, defocus);
    if (st) return st;
    if (!images || !volume) return fail(ctx, MSK_EINVAL, "null image or volume pointer");
    Geo g{};
    st = make_geo(ctx, p, nangles, angles, defocus, g);
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
    fr.hb = headroom_bits(nangles);
    fr.nsr = p->nsr * sqrt((double)nx * ny);
    std::vector<double> cx, cfx, lx, ilx(nx, 0.0);
    if (g.zout != 0) {
        if (p->ctf_mode == 2) {
            const double alpha = -4.0 * kPi * p->asigma / (g.zout * p->wl);
            const double norm = -alpha * sqrt(1.0 + p->asigma * p->asigma) / p->asigma;
            if (invlap_setup(nx, ny, nz, g.zhi - g.zlo, g.yhi - g.ylo, g.xhi - g.ylo, alpha, lx,
                             fr.ly, fr.lz))
                return fail(ctx, MSK_EINVAL, "InverseMLaplacian3D: alpha <= 0 or a zero aperture");
            fr.corr = 2;
            fr.lalpha = alpha;
            fr.lnorm = norm;
        } else if (p->ctf_mode == 4) {
            if (ctf_setup(fr, nx, ny, nz, p->wl, g.zlo, g.zhi, g.ylo, g.yhi, g.xlo, g.xhi, g.zout,
                          g.k2maxo, g.cs3, g.cs5, p->asigma, p->epsilon, p->escc, cx, cfx))
                return fail(ctx, MSK_EINVAL, "CTFcorrection3D: evanescent waves present");
        }
    }
    if (p->inv_laplace && p->ctf_mode != 1 && p->ctf_mode != 2) {
        if (invlap_setup(nx, ny, nz, g.zhi - g.zlo, g.yhi - g.ylo, g.xhi - g.ylo, p->epsilon, ilx,
                         fr.ily, fr.ilz))
            return fail(ctx, MSK_EINVAL, "inverse Laplacian filter: epsilon must be positive");
        fr.invlap = 1;
        fr.ilalpha = p->epsilon;
        fr.ilnorm = p->epsilon;
    }
    fr.nyq = 1;
    fr.modulate = 1;
    if (lx.empty()) lx.assign(nx, 0.0);
    if (cx.empty()) {
        cx.assign(nx, 0.0);
        cfx.assign(nx, 0.0);
    }

    // output stage (UTR.cpp:1235-1278)
    const long long nxd2 = nx / 2, nyd2 = ny / 2, nzd2 = nz / 2;
    const long long nxR2 = g.ic <= nxd2 ? g.ic * g.ic : (nx - g.ic) * (nx - g.ic);
    const long long nyR2 = g.jc <= nyd2 ? g.jc * g.jc : (ny - g.jc) * (ny - g.jc);
    const long long nzR2 = g.kc <= nzd2 ? g.kc * g.kc : (nz - g.kc) * (nz - g.kc);
    long long nR2;
    if (g.rot_y_only) nR2 = std::min(nxR2, nzR2);
    else if (g.rot_z_only || g.rot_z2_only) nR2 = std::min(nxR2, nyR2);
    else nR2 = std::min(std::min(nxR2, nyR2), nzR2);
    const double dtemp = 2.0 / (double)(g.kc * g.kc + g.jc * g.jc + g.ic * g.ic);
    std::vector<double> ex(nx), ey(ny), ez(nz);
    for (int i = 0; i < nx; i++) ex[i] = exp(dtemp * (double)((i - g.ic) * (i - g.ic)));
    for (int j = 0; j < ny; j++) ey[j] = exp(dtemp * (double)((j - g.jc) * (j - g.jc)));
    for (int k = 0; k < nz; k++) ez[k] = exp(dtemp * (double)((k - g.kc) * (k - g.kc)));
    const double fnorm =
        p->modality == 0
            ? g.ee * p->wl / (2.0 * kPi * sqrt(1.0 + p->asigma * p->asigma) * g.xst)
            : p->asigma * p->wl / (4.0 * kPi * sqrt(1.0 + p->asigma * p->asigma) * g.xst);

    std::vector<float> tabs, scal;
    grid_tables(p, g, nangles, angles, tabs, scal);
    std::vector<float2> twx, twy, twz;
    if (!twiddles(nx, twx) || !twiddles(ny, twy) || !twiddles(nz, twz))
        return fail(ctx, MSK_EUNSUPPORTED, "no FFT for this size");

    const TabLayout o = tab_layout(nx, ny, nz, tabs.size(), scal.size(),
                                   std::max(twx.size(), std::max(twy.size(), twz.size())));
    MSK_CUDA(ctx, ctx->utr_tab.reserve(o.total));
    unsigned char *tb = ctx->utr_tab.as<unsigned char>();
    MSK_CUDA(ctx, cudaMemsetAsync(tb + o.maxbits, 0, 256, ctx->stream));
    if ((st = upload(ctx, tb + o.tw_x, twx.data(), twx.size() * sizeof(float2))) ||
        (st = upload(ctx, tb + o.tw_y, twy.data(), twy.size() * sizeof(float2))) ||
        (st = upload(ctx, tb + o.tw_z, twz.data(), twz.size() * sizeof(float2))) ||
        (st = upload(ctx, tb + o.lx, lx.data(), nx * sizeof(double))) ||
        (st = upload(ctx, tb + o.cx, cx.data(), nx * sizeof(double))) ||
        (st = upload(ctx, tb + o.cfx, cfx.data(), nx * sizeof(double))) ||
        (st = upload(ctx, tb + o.ilx, ilx.data(), nx * sizeof(double))) ||
        (st = upload(ctx, tb + o.ex, ex.data(), nx * sizeof(double))) ||
        (st = upload(ctx, tb + o.ey, ey.data(), ny * sizeof(double))) ||
        (st = upload(ctx, tb + o.ez, ez.data(), nz * sizeof(double))) ||
        (st = upload(ctx, tb + o.tabs, tabs.data(), tabs.size() * sizeof(float))) ||
        (st = upload(ctx, tb + o.scal, scal.data(), scal.size() * sizeof(float))))
        return st;
    unsigned *maxbits = reinterpret_cast<unsigned *>(tb + o.maxbits);
    const float2 *tw_x = reinterpret_cast<const float2 *>(tb + o.tw_x);
    const float2 *tw_y = reinterpret_cast<const float2 *>(tb + o.tw_y);
    const float2 *tw_z = reinterpret_cast<const float2 *>(tb + o.tw_z);
    fr.maxbits = maxbits;
    fr.lx = reinterpret_cast<const double *>(tb + o.lx);
    fr.cx = reinterpret_cast<const double *>(tb + o.cx);
    fr.cfx = reinterpret_cast<const double *>(tb + o.cfx);
    fr.ilx = reinterpret_cast<const double *>(tb + o.ilx);

    // images in, spectra, gridding
    const size_t plane = (size_t)nx * ny, nvox = plane * nz;
    const float *img_d = images;
    if (!is_device_ptr(images)) {
        MSK_CUDA(ctx, ctx->utr_img.reserve(sizeof(float) * plane * nangles));
        if ((st = upload(ctx, ctx->utr_img.p, images, sizeof(float) * plane * nangles))) return st;
        img_d = ctx->utr_img.as<float>();
    }
    if ((st = spectra(ctx, p, nangles, img_d, tw_x, tw_y, maxbits))) return st;
    MSK_CUDA(ctx, ctx->utr_acc.reserve(sizeof(UtrAcc) * nvox));
    UtrAcc *acc = ctx->utr_acc.as<UtrAcc>();
    MSK_CUDA(ctx, cudaMemsetAsync(acc, 0, sizeof(UtrAcc) * nvox, ctx->stream));
    if ((st = grid_launch(ctx, p, g, nangles, ctx->utr_k2.as<float2>(),
                          reinterpret_cast<const float *>(tb + o.tabs),
                          reinterpret_cast<const float *>(tb + o.scal), maxbits, acc)))
        return st;

    // Fourier-space processing and the inverse 3D transform
    MSK_CUDA(ctx, ctx->utr_vol.reserve(sizeof(float2) * nvox));
    float2 *vol = ctx->utr_vol.as<float2>();
    {
        Prof pr(ctx, kUtrFourier, 40.0 * nvox);
        utr_ops(nx)->fourier_rows(fr, tw_x, acc, vol, ny * nz, ctx->stream);
    }
    Geom gdummy{};
    if ((st = flags_reset(ctx, gdummy))) return st;
    ColView vy, vz;
    if ((st = column_map(ctx, &vy, vol, ny, nx, (size_t)nz, size_ops(ny), 0))) return st;
    if ((st = column_map(ctx, &vz, vol, nz, nx * ny, 1, size_ops(nz), 0))) return st;
    UtrCol cy{};
    cy.width = nx;
    cy.tw = tw_y;
    cy.err = gdummy.err;
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
    cz.err = gdummy.err;
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
    cz.use_y = !g.rot_y_only;
    cz.use_z = !(g.rot_z_only || g.rot_z2_only);
    cz.ex = reinterpret_cast<const double *>(tb + o.ex);
    cz.ey = reinterpret_cast<const double *>(tb + o.ey);
    cz.ez = reinterpret_cast<const double *>(tb + o.ez);
    {
        Prof pr(ctx, kUtrFinal, 12.0 * nvox);
        utr_ops(nz)->col_final(cz, vz.map, 1, ctx->stream);
    }
    MSK_CUDA(ctx, cudaGetLastError());
    if (!out_dev) {
        MSK_CUDA(ctx, cudaMemcpyAsync(volume, out_d, sizeof(float) * nvox, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        count_copy(ctx, 1, (double)sizeof(float) * nvox);
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
    const TabLayout o = tab_layout(2, 2, 2, tabs.size(), scal.size());
    MSK_CUDA(ctx, ctx->utr_tab.reserve(o.total));
    unsigned char *tb = ctx->utr_tab.as<unsigned char>();
    MSK_CUDA(ctx, cudaMemsetAsync(tb + o.maxbits, 0, 256, ctx->stream));
    if ((st = upload(ctx, tb + o.tabs, tabs.data(), tabs.size() * sizeof(float))) ||
        (st = upload(ctx, tb + o.scal, scal.data(), scal.size() * sizeof(float))))
        return st;
    unsigned *maxbits = reinterpret_cast<unsigned *>(tb + o.maxbits);
    const size_t plane = (size_t)g.nx * g.ny, nvox = plane * g.nz;
    const float2 *k2_d = reinterpret_cast<const float2 *>(k2four);
    if (!is_device_ptr(k2four)) {
        MSK_CUDA(ctx, ctx->utr_k2.reserve(sizeof(float2) * plane * nangles));
        if ((st = upload(ctx, ctx->utr_k2.p, k2four, sizeof(float2) * plane * nangles))) return st;
        k2_d = ctx->utr_k2.as<float2>();
    }
    k_utr_maxabs<<<grid_blocks(plane * nangles), 256, 0, ctx->stream>>>(k2_d, plane * nangles, maxbits);
    MSK_CUDA(ctx, ctx->utr_acc.reserve(sizeof(UtrAcc) * nvox));
    UtrAcc *acc = ctx->utr_acc.as<UtrAcc>();
    MSK_CUDA(ctx, cudaMemsetAsync(acc, 0, sizeof(UtrAcc) * nvox, ctx->stream));
    if ((st = grid_launch(ctx, p, g, nangles, k2_d, reinterpret_cast<const float *>(tb + o.tabs),
                          reinterpret_cast<const float *>(tb + o.scal), maxbits, acc)))
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
        Prof pr(ctx, kUtrPoint, 44.0 * nvox);
        k_utr_acc_float<<<grid_blocks(nvox), 256, 0, ctx->stream>>>(acc, nvox, maxbits,
                                                                     headroom_bits(nangles), v_d, s_d);
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
int point_pass(msk_context *ctx, float *v3, size_t nvox, UtrFourier &f,
               const std::vector<double> &tab_a, const std::vector<double> &tab_b)
{
    MSK_CUDA(ctx, cudaSetDevice(ctx->device));
    const TabLayout o = tab_layout(f.nx, 2, 2, 0, 0);
    MSK_CUDA(ctx, ctx->utr_tab.reserve(o.total));
    unsigned char *tb = ctx->utr_tab.as<unsigned char>();
    int st;
    if ((st = upload(ctx, tb + o.lx, tab_a.data(), f.nx * sizeof(double))) ||
        (st = upload(ctx, tb + o.cfx, tab_b.data(), f.nx * sizeof(double))))
        return st;
    f.lx = f.cx = f.ilx = reinterpret_cast<const double *>(tb + o.lx);
    f.cfx = reinterpret_cast<const double *>(tb + o.cfx);
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
    std::vector<double> cx, cfx;
    if (ctf_setup(f, nx, ny, nz, wl, zlo, zhi, ylo, yhi, xlo, xhi, defocdist, q2max, cs3, cs5,
                  sigma, epsilon, escc, cx, cfx))
        return fail(ctx, MSK_EINVAL, "CTFcorrection3D: odd sizes or evanescent waves");
    return point_pass(ctx, v3, (size_t)nx * ny * nz, f, cx, cfx);
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
    std::vector<double> lx;
    if (invlap_setup(nx, ny, nz, zaper, yaper, xaper, alpha, lx, f.ly, f.lz))
        return fail(ctx, MSK_EINVAL, "InverseMLaplacian3D: alpha <= 0, a zero aperture or odd sizes");
    f.corr = 2;
    f.lalpha = alpha;
    f.lnorm = norm;
    return point_pass(ctx, v3, (size_t)nx * ny * nz, f, lx, lx);
}

}  // extern "C"
