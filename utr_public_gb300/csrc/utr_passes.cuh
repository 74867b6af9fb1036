// utr_passes.cuh -- line passes of the UTR reconstruction (UTR.exe,
// MultisliceCppTest/PhaseRetrieval/UTR.cpp and UTR.h) for one line length N.
//
// Centred transforms without data movement: for even n, the centred DFT
// (UTR.cpp's Shuffle, FFT, Shuffle) of x is (-1)^k DFT((-1)^i x)[k] when
// n/2 is even (every size here, n >= 16), so each pass multiplies by the
// sign of its own index instead of shifting quadrants.
//
// Image spectra (UTR.cpp:989-996):  k_utr_img_rows (normalise, threshold,
//   log, (-1)^(x+y), FFT along x, FFTW's forward sign) then k_utr_col<N,
//   kUtrColImg> (FFT along y, (-1)^(kx+ky)).
// Volume inverse (UTR.cpp:1200-1272): k_utr_fourier_rows (gridding sums ->
//   sampling normalisation, SNR filter, 3D correction, (-1)^(i+j+k), inverse
//   FFT along x), k_utr_col<N, kUtrColVol> (along y, in place), k_utr_col<N,
//   kUtrColFinal> (along z, then (-1)^(x+y+z), the real part / (nx ny nz), the
//   reconstruction-sphere mask, the cupping compensation and the output scale,
//   stored as float).
#pragma once

#include <cuda_runtime.h>

#include "fft_line.cuh"
#include "msk_passes.cuh"
#include "tma.cuh"

namespace msk {

// One voxel of the gridding sums (float, as the reference accumulates them):
// real part, imaginary part, weight -- one 16-byte vector atomic per update.
struct __align__(16) UtrAcc {
    float re, im, w, pad;
};

// Per-voxel Fourier-space processing of UTR.cpp:1052-1217 and UTR.h:15-175.
struct UtrFourier {
    int nx, ny, nz;
    float nsr;                // dInputNSR * sqrt(nx * ny); 0: plain normalisation
    float inv_nsr;            // 1 / nsr
    int corr;                 // 0 none, 2 TIE-Hom (inverse Laplacian), 4 CTF
    // InverseMLaplacian3D of the 3D TIE-Hom step: den = lx[i] + (j1 j1 ly + (k1 k1 lz + alpha))
    const double *lx;         // [nx] (dksi2 * i1) * i1
    double ly, lz, lalpha, lnorm;
    // CTFcorrection3D: the phase dtemp = fac2 ksi^2 - omega (+ the Cs terms) of
    // voxel (k, j, i) is a sum of per-axis parts; exp(i dtemp) = ex[i] ey[j]
    // ez[k] from tables made in double (ez holds -omega).  cx: [nx] (dksi2 *
    // i1) * i1 for the aperture test and the Cs terms.
    const float2 *ex, *ey, *ez;
    const double *cx;
    const float *cxf;  // cx in float
    double fac3, fac5, deta2, dzeta2, q2max;
    float eps, q2maxf;
    int aper, c35, escc;
    // the optional inverse Laplacian filter (parameter 22), as lx/ly/lz
    int invlap;
    const double *ilx;
    double ily, ilz, ilalpha, ilnorm;
    int nyq;       // apply the Hermitian step's factor on the x-Nyquist plane
    int modulate;  // multiply by (-1)^(i+j+k) for the centred inverse
};

__device__ __forceinline__ float2 cmul_rn(float2 a, float2 b)
{
    return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                       __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

// Double helpers without contraction (the reference's expressions round
// after every operation).
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

// sin and cos of a double phase: reduced modulo 2 pi in double (two-part
// 2 pi), then evaluated in float.
__device__ __forceinline__ void sincos_reduced(double ph, float *s, float *c)
{
    const double n = rint(ph * 0.15915494309189535);
    double r = fma(-n, 6.283185307179586, ph);
    r = fma(-n, 2.4492935982947064e-16, r);
    sincosf((float)r, s, c);
}

// Row constants of the 3D corrections for row (k, j).
struct UtrRow {
    double eta2;            // CTF: the (j, k) part of ksi^2
    float eta2f;
    float2 e;               // CTF: ey[j] ez[k]
    double lden, ilden;     // inverse Laplacians: the (j, k) part of the denominator
};

__device__ __forceinline__ UtrRow utr_row(const UtrFourier &f, int k, int j)
{
    UtrRow r{};
    const int k1 = k - f.nz / 2, j1 = j - f.ny / 2;
    if (f.corr == 4) {  // (the FP64 pipe is narrow: only what the mode uses)
        const double zeta2 = dmul(dmul(f.dzeta2, (double)k1), (double)k1);
        const double eta2 = dmul(dmul(f.deta2, (double)j1), (double)j1);
        r.eta2 = dadd(eta2, zeta2);
        r.eta2f = (float)r.eta2;
        r.e = cmul_rn(__ldg(&f.ey[j]), __ldg(&f.ez[k]));
    }
    if (f.corr == 2)
        r.lden = dadd(dmul((double)(j1 * j1), f.ly), dadd(dmul((double)(k1 * k1), f.lz), f.lalpha));
    if (f.invlap)
        r.ilden = dadd(dmul((double)(j1 * j1), f.ily), dadd(dmul((double)(k1 * k1), f.ilz), f.ilalpha));
    return r;
}

// The 3D corrections of one voxel (UTR.cpp:1177-1201).
__device__ __forceinline__ float2 utr_correct(const UtrFourier &f, const UtrRow &r, int i, float2 v)
{
    if (f.corr == 4) {
        bool in = true;
        double ksi2 = 0.0;
        if (f.c35) ksi2 = dadd(__ldg(&f.cx[i]), r.eta2);
        if (f.aper) {
            // ksi^2 < q2max in double (UTR.h:106); decided in float away from
            // the boundary
            const float kf = __fadd_rn(__ldg(&f.cxf[i]), r.eta2f), qf = f.q2maxf;
            if (fabsf(kf - qf) > 1e-5f * qf) {
                in = kf < qf;
            } else {
                if (!f.c35) ksi2 = dadd(__ldg(&f.cx[i]), r.eta2);
                in = ksi2 < f.q2max;
            }
        }
        if (in) {
            float2 e = cmul_rn(__ldg(&f.ex[i]), r.e);  // (cos, sin) of the phase
            if (f.c35) {
                float s, c;
                const double k4 = dmul(ksi2, ksi2);
                sincos_reduced(dadd(dmul(dmul(f.fac3, ksi2), ksi2), dmul(f.fac5, dmul(k4, ksi2))),
                               &s, &c);
                e = cmul_rn(e, make_float2(c, s));
            }
            const float sinreg = __fdividef(e.y, fmaf(e.y, e.y, f.eps));
            float cosreg = 0.0f;
            if (f.escc) cosreg = __fdividef(e.x, fmaf(e.x, e.x, f.eps));
            v = cmul_rn(v, make_float2(sinreg, -cosreg));
        }
    } else if (f.corr == 2) {
        const double den = dadd(__ldg(&f.lx[i]), r.lden);
        const float sc = __fdividef((float)f.lnorm, (float)den);
        v = make_float2(__fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
    }
    if (f.invlap) {
        const double den = dadd(__ldg(&f.ilx[i]), r.ilden);
        const float sc = __fdividef((float)f.ilnorm, (float)den);
        v = make_float2(__fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
    }
    return v;
}

// Sampling normalisation and the SNR filter of UTR.cpp:1052-1093 (float,
// as the reference): x = the summed weight.
__device__ __forceinline__ float2 utr_filter(const UtrFourier &f, float2 v, float x)
{
    if (x == 0.0f) return make_float2(0.0f, 0.0f);
    float s = __frcp_rn(x);  // 1/x, correctly rounded as the reference's division
    if (f.nsr != 0.0f) {
        // y = |v| / (nsr sqrt(x)), the SNR of the coefficient
        const float y = sqrtf(fmaf(v.x, v.x, v.y * v.y)) * rsqrtf(x) * f.inv_nsr;
        const float a = atanf(__fmul_rn(100.0f, __fsub_rn(y, 1.41421354f)));
        s = __fmul_rn(s, fmaf(a, 0.318309873f, 0.5f));  // 0.5 + atan / pi
    }
    return make_float2(__fmul_rn(v.x, s), __fmul_rn(v.y, s));
}

// The Hermitian step of UTR.cpp:1203-1217 before the complex-to-real inverse
// transform.  Off the x-Nyquist plane it changes nothing the real part of a
// complex inverse transform sees.  On that plane (centred index i = 0) it
// runs in place in the reference's (k, j) order: of a pair p, q = -p the
// earlier a becomes (a + conj b)/2, then the later b becomes (b + conj a')/2
// = 3b/4 + conj(a)/4, which for the real part of the transform equals
// scaling a by 3/4 and b by 5/4; a self-paired point keeps its real part,
// all that part of the transform reads of it.
__device__ __forceinline__ float utr_nyquist_factor(int k, int j, int ny, int nz)
{
    const int ka = k == 0 ? 0 : nz - k, ja = j == 0 ? 0 : ny - j;
    if (ka == k && ja == j) return 1.0f;
    return (k < ka || (k == ka && j < ja)) ? 0.75f : 1.25f;
}

// ---------------------------------------------------------------- image rows
// images [nimg][ny][nx] float -> k2 [nimg][ny][nx] complex: per row y of
// image a, v = input / f1 + f2, v < 0 -> 0, Log0, (-1)^(x+y), FFT along x
// with FFTW's forward sign (UTR.cpp:940-950, 989-996).
struct UtrImg {
    int nx, ny, nrows;  // rows = nimg * ny
    float f1, f2;
    int use_f1, use_f2;
    const float2 *tw;
};

template <int NX>
__global__ void __launch_bounds__(RowCfg<NX>::L * FftPlan<NX>::T)
k_utr_img_rows(const UtrImg p, const float *__restrict__ img, float2 *__restrict__ k2)
{
    using P = FftPlan<NX>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NX>::L;
    constexpr bool BLK = RowCfg<NX>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int row = blockIdx.x * L + l;
    const bool ok = row < p.nrows;
    const int y = (ok ? row : 0) % p.ny;
    const float *src = img + (size_t)(ok ? row : 0) * NX;
    float2 w[E];
#pragma unroll
    for (int m = 0; m < E; m++) {
        const int x = t + m * T;
        float v = src[x];
        if (p.use_f1) v = __fdiv_rn(v, p.f1);
        if (p.use_f2) v = __fadd_rn(v, p.f2);
        v = v > 0.0f ? logf(v) : 0.0f;
        w[m] = make_float2(((x + y) & 1) ? -v : v, 0.0f);
    }
    fft_line<NX, true, 1, BLK>(w, s_lines + l * P::PADN, 0, t, p.tw);
    if (ok) {
        float2 *dst = k2 + (size_t)row * NX;
#pragma unroll
        for (int m = 0; m < E; m++) dst[t + m * T] = w[m];
    }
}

// ---------------------------------------------------------------- Fourier rows
// Row (k, j) of the volume: the gridding sums -> the processed spectrum ->
// inverse FFT along x (FFTW's backward sign) into vol.
template <int NX>
__global__ void __launch_bounds__(RowCfg<NX>::L * FftPlan<NX>::T, RowCfg<NX>::MB)
k_utr_fourier_rows(const UtrFourier f, const float2 *__restrict__ tw, const UtrAcc *__restrict__ acc,
                   float2 *__restrict__ vol)
{
    using P = FftPlan<NX>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NX>::L;
    constexpr bool BLK = RowCfg<NX>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nrows = f.ny * f.nz;
    const int row = blockIdx.x * L + l;
    const bool ok = row < nrows;
    const int rr = ok ? row : 0;
    const int k = rr / f.ny, j = rr % f.ny;
    const UtrRow r = utr_row(f, k, j);
    const UtrAcc *src = acc + (size_t)rr * NX;
    float2 *line = s_lines + l * P::PADN;
    // per-voxel work in a rolled loop (one copy of the code: the unrolled form
    // overflowed the instruction cache), staged in the line's shared buffer;
    // the sums are loaded three iterations ahead (four 16-byte loads in flight
    // a thread: one alone left the pass waiting on HBM latency)
    UtrAcc a1 = src[t], a2 = src[t + T], a3 = src[t + 2 * T];
#pragma unroll 1
    for (int m = 0; m < E; m++) {
        const int i = t + m * T;
        const UtrAcc a = a1;
        a1 = a2;
        a2 = a3;
        if (m + 3 < E) a3 = src[i + 3 * T];
        float2 v = utr_filter(f, make_float2(a.re, a.im), a.w);
        v = utr_correct(f, r, i, v);
        if (f.nyq && i == 0) {
            const float q = utr_nyquist_factor(k, j, f.ny, f.nz);
            v = make_float2(v.x * q, v.y * q);
        }
        if (f.modulate && ((i + j + k) & 1)) v = make_float2(-v.x, -v.y);
        line[i] = v;
    }
    group_sync<BLK>();
    float2 w[E];
#pragma unroll
    for (int m = 0; m < E; m++) w[m] = line[t + m * T];
    fft_line<NX, false, 1, BLK>(w, line, 0, t, tw);
    if (ok) {
        float2 *dst = vol + (size_t)rr * NX;
#pragma unroll
        for (int m = 0; m < E; m++) dst[t + m * T] = w[m];
    }
}

// ---------------------------------------------------------------- column passes
enum { kUtrColImg = 0, kUtrColVol = 1, kUtrColFinal = 2 };

// Column tiles of the UTR passes: C lines of N points with 256 threads
// (capped at 16 lines), so that every row of a tile is C * 8 >= 32 bytes;
// WIDE (the final z pass, whose line points lie nx * ny * 8 bytes apart):
// 512 threads, twice the lines, 128-byte tile rows at 1024 points.
template <int N, bool WIDE = false> struct UtrColCfg {
    static constexpr int T = FftPlan<N>::T;
    static constexpr int TH = WIDE ? 512 : 256;
    static constexpr int C = (TH / T) < 2 ? 2 : ((TH / T) > 16 ? 16 : TH / T);
    static constexpr int NT = C * T;
    static constexpr int BR = N < 256 ? N : 256;  // rows per TMA box
    static constexpr int NBOX = N / BR;
    static constexpr uint32_t TILE_BYTES = (uint32_t)N * C * 8;
    static constexpr size_t SMEM = (size_t)C * FftPlan<N>::PADN * 8 + 16;
};

struct UtrCol {
    int width;  // complex columns of the 2D view
    int cb0, ncb;  // column blocks cb0 .. cb0 + ncb - 1 of each unit (ncb 0: all)
    const float2 *tw;
    int *err;
    // kUtrColFinal: the volume [nz][ny][nx] (width = nx * ny, lines = nz)
    float *out;
    int nx, ny, nxlog;
    float inv_n, fnorm;
    long long ic, jc, kc, nr2;
    int use_y, use_z;
    const float *ex, *ey, *ez;  // exp(dtemp * d^2) per axis (1 for an axis left out)
};

template <int N, int MODE>
__global__ void __launch_bounds__(UtrColCfg<N, MODE == kUtrColFinal>::NT)
k_utr_col(const UtrCol p, const __grid_constant__ CUtensorMap in_map,
          const __grid_constant__ CUtensorMap out_map)
{
    using P = FftPlan<N>;
    using CC = UtrColCfg<N, MODE == kUtrColFinal>;
    constexpr int T = P::T, E = P::E, C = CC::C;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *buf = reinterpret_cast<float2 *>(smem);
    uint64_t *bar = reinterpret_cast<uint64_t *>(buf + P::PADN * C);
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const int bpu = p.ncb > 0 ? p.ncb : p.width / C;
    const int u = blockIdx.x / bpu, cb = blockIdx.x % bpu + p.cb0;
    const int col = cb * C + c;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, CC::TILE_BYTES);
#pragma unroll
        for (int jb = 0; jb < CC::NBOX; jb++)
            tma_load_2d(buf + jb * CC::BR * C, &in_map, 2 * cb * C, u * N + jb * CC::BR, bar);
    }
    if (!cta_wait(bar, 0, p.err)) {
        cta_drain(bar, 0);
        return;
    }
    float2 v[E];
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = buf[(t + m * T) * C + c];
    fft_line<N, MODE == kUtrColImg, C, true>(v, buf, c, t, p.tw);
    if constexpr (MODE == kUtrColFinal) {
        const int x = col & (p.nx - 1), y = col >> p.nxlog;
        const long long dx = x - p.ic, dy = y - p.jc;
        const float fxy = __fmul_rn(__ldg(&p.ex[x]), __ldg(&p.ey[y]));
#pragma unroll
        for (int m = 0; m < E; m++) {
            const int z = t + m * T;
            const long long dz = z - p.kc;
            const long long kk2 = p.use_z ? dz * dz : 0;
            const long long jj2 = p.use_y ? dy * dy + kk2 : kk2;
            const long long ii2 = dx * dx + jj2;
            float r = __fmul_rn(((x + y + z) & 1) ? -v[m].x : v[m].x, p.inv_n);
            if (ii2 > p.nr2) {
                r = 0.0f;
            } else {
                r = __fmul_rn(__fmul_rn(r, __fmul_rn(fxy, __ldg(&p.ez[z]))), p.fnorm);
            }
            p.out[((size_t)z * p.ny * p.nx) + col] = r;
        }
        return;
    } else {
        if constexpr (MODE == kUtrColImg) {
#pragma unroll
            for (int m = 0; m < E; m++)
                if ((col + t + m * T) & 1) v[m] = make_float2(-v[m].x, -v[m].y);
        }
        __syncthreads();  // every thread is done with the exchange layout
#pragma unroll
        for (int m = 0; m < E; m++) buf[(t + m * T) * C + c] = v[m];
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
#pragma unroll
            for (int jb = 0; jb < CC::NBOX; jb++)
                tma_store_2d(&out_map, 2 * cb * C, u * N + jb * CC::BR, buf + jb * CC::BR * C);
            bulk_commit();
            bulk_wait_read();
        }
    }
}

}  // namespace msk
