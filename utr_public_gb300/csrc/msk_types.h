// msk_types.h -- host/device descriptors shared by the launchers and kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace msk {

// Everything a pass needs to know about one grid (one plan).  Passed to the
// kernels by value.  Float members hold exactly the float values the
// reference computes (TemsimLibrary/autoslic.cpp:326-414, 929-941), so that
// band-limit and aperture decisions are bit-identical with it.
struct Geom {
    int nx, ny;
    float k2max;        // (2/3 * min(nx/2ax, ny/2by))^2, float
    float inv_n;        // 1/(nx*ny)
    float sigma_f;      // sigma(keV)/1000, rad/(V*Angstrom)
    float scalex_f;     // ax/nx as float (pixel pitch used by the splat)
    float scaley_f;
    float rminsq;       // (rmin)^2, rmin = 1/4 sqrt((dx^2+dy^2)/2)
    int idx, idy;       // splat window half widths int(n*3/a)+1
    const float *kx2;   // [nx] kx^2 (freqn, float)
    const float *ky2;   // [ny]
    const float2 *propx;  // [nx] (cos t, -sin t) / nx, t = pi dz (kx^2 lambda - kx 2 tan(tilt_x))
    const float2 *propy;  // [ny]
    const int2 *kband;    // [ny] (A, B): kx2[ix] + ky2[iy] < k2max  <=>  ix <= A or ix >= B
    // Columns iy with ky2[iy] >= k2max are zeroed whole by the band limit and
    // by the propagator: in band <=> iy <= band_p or iy >= band_q.  Column
    // passes in band mode run only the column blocks [0, cb_lo) and
    // [cb_hi0, ny/C) (C columns per block); cb_n blocks per unit; one set per
    // column-pass variant (tile width and FFT plan).
    int band_p, band_q;
    int cb_lo[4], cb_hi0[4], cb_n[4];
    // Row segments [0, seg_e1) and [seg_s2, ny) with even bounds that cover
    // the in-band columns: what a band-mode row pass loads and stores.
    int seg_e1, seg_s2;
    const float2 *zeros;  // >= 4096 zero complex values: the source of zero fills
    const float2 *tw_row;  // twiddles for line length ny
    const float2 *tw_col;  // twiddles for line length nx
    const float2 *tw_row16;  // the same for the 16-points-a-thread plan (null above 2048)
    const float2 *tw_col16;
    const float *knots;    // [100] spline knots in r^2
    const float4 *coef;    // [nz][100] spline {y, b, c, d} per compact atomic number
    int *err;              // device error flags (kErrWaitTimeout ...), 0 when all is well
};

// Atoms of one (unit, slice) for the splat: x and y relative to the pixel
// that contains them, computed on the host in double.
//   geom = {fx = x - ixo*scalex, fy = y - iyo*scaley, occ, bits(meta)}
//   meta = ixo | iyo << 13 | zidx << 26
struct SplatAtom {
    float fx, fy, occ;
    uint32_t meta;
};
static_assert(sizeof(SplatAtom) == 16, "SplatAtom layout");

constexpr int kMetaBits = 13;
constexpr uint32_t kMetaMask = (1u << kMetaBits) - 1u;
constexpr int kMaxZidx = 64;

// Free-space step to one detector plane (this library's FresnelA definition):
// chi = a1 k^2 + a3 k^4 + a5 k^6 + a2c (kx^2 - ky^2) + a2s 2 kx ky,
// multiplier exp(-i chi) where k^2 < k2maxo (k2maxo == 0: everywhere).
// k_fresnel_table evaluates it once per plane in double into `table`
// ([nx][ny] complex64, times a scale); the column pass then reads the table.
struct Fresnel {
    double a1, a3, a5, a2c, a2s;
    float k2maxo;
    const float *kx;  // [nx]
    const float *ky;  // [ny]
    const float2 *table;
    // Debye-Waller column pass (kColDW): -B/4 per (unit, slice) at
    // dw[u * dw_stride] (the caller offsets dw to the slice)
    const float *dw;
    int dw_stride;
};

}  // namespace msk
