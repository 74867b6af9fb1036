// msk_passes.cuh -- the fused row and column passes of the batched multislice.
//
// HBM layout: every wave / transmission buffer is complex64 [unit][ix][iy],
// iy contiguous (the reference's cfpix layout, data[iy + ix*ny]).  A "row"
// is one ix (ny contiguous points), a "column" one iy (nx points, stride ny).
//
// State kept between passes (S = the row transform along iy, unnormalised,
// kernel exp(+2 pi i ..); iS its inverse, unnormalised, kernel exp(-..);
// F, iF the same along ix; iS(S(f)) = ny f):
//   psi buffer:  W = S(psi)          (between slices; psi = iS(W)/ny)
//   t buffer:    A = S(t)            (after P1)
//                B = S(t_bl)         (after P2, t_bl the band-limited t)
// One slice (TemsimLibrary/autoslic.cpp:756-830, trlayer 917-1013):
//   P1 k_row_splat     potential v by splat, t = exp(i sigma v), A = S(t)
//   P2 k_col_pass<0>   B = iF(M F(A))/nx        (M: 2/3 band limit)
//   P3 k_row_transmit  W = S(iS(W) * iS(B))/ny^2          (wave *= trans)
//   P4 k_col_pass<1>   W = iF(P F(W))/nx        (P: propagator + aperture)
// With unnormalised transforms these scalings are exactly the reference's
// fft / ifft-with-1/(nx*ny) pairs.  An empty slice is P4 alone: the
// wave's row iFFT and FFT around a missing transmit cancel.
//
// Scattered form (the potential-stack path and its adjoint): the buffers hold
// phi = psi - 1 and tau = t - 1 instead of psi and t.  The band limit, the
// propagator and the free-space multiplier are 1 at k = 0, so they map 1 to 1
// and act on phi and tau alone; the transmit becomes phi' = phi + (tau +
// phi tau) and I = |1 + phi|^2.  Same FP32 arithmetic, but every rounding
// scales with |phi| (the scattered part) instead of with the unit plane
// wave, which leaves ~10x less error in I -- the figure the image residuals
// I - T of the adjoint's loss, a few 1e-4 of I, depend on.
#pragma once

#include <cuda_runtime.h>

#include "fft_line.cuh"
#include "msk_types.h"
#include "sincos_poly.cuh"
#include "tma.cuh"

namespace msk {

// a mod n in [0, n) for a power-of-two n (every grid size here is one)
__device__ __forceinline__ int pmod(int a, int n) { return a & (n - 1); }

// Column iy lies outside the band: the band limit and the propagator zero it
// whole, so a row pass whose output only feeds them may store zeros there.
__device__ __forceinline__ bool out_of_band(const Geom &g, int iy)
{
    return iy > g.band_p && iy < g.band_q;
}

// True when no thread of the line group holds a non-zero `nz`: a warp vote
// for lines of <= 32 threads (several lines a warp below 32: the group
// transforms share warp barriers), a CTA vote for larger lines (their
// transforms use CTA barriers).  Uniform over everything a line FFT syncs.
template <bool BLK>
__device__ __forceinline__ bool group_none(bool nz)
{
    if constexpr (BLK) return !__syncthreads_or(nz);
    else return !__any_sync(0xffffffffu, nz);
}

// Store `rows` dense rows of length NY from shared memory as their in-band
// segments [0, seg_e1) and [seg_s2, NY); the (at most two) out-of-band
// elements inside the segments are zeroed first.  Called by every thread;
// ends with the stores committed and shared memory read.
template <int NY>
__device__ __forceinline__ void store_band_rows(const Geom &g, float2 *rows_smem, int rows,
                                                float2 *dst)
{
    const int e1 = g.seg_e1, s2 = g.seg_s2;
    __syncthreads();  // every element written before the fix-up
    if (threadIdx.x < 2 * rows) {
        const int r = threadIdx.x >> 1;
        const int iy = (threadIdx.x & 1) ? s2 : e1 - 1;
        if (iy >= 0 && iy < NY && out_of_band(g, iy)) rows_smem[r * NY + iy] = make_float2(0.0f, 0.0f);
    }
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int r = 0; r < rows; r++) {
            bulk_store(dst + (size_t)r * NY, rows_smem + r * NY, (uint32_t)e1 * 8u);
            if (s2 < NY)
                bulk_store(dst + (size_t)r * NY + s2, rows_smem + r * NY + s2, (uint32_t)(NY - s2) * 8u);
        }
        bulk_commit();
        bulk_wait_read();
    }
}

// exp(i*ph) by the polynomial form of sincos_poly.cuh (the library's sincosf
// beyond its range), kept out of line: 32 inlined bodies per thread would
// overflow the instruction cache of the splat
static __device__ __noinline__ float2 expi(float ph)
{
    if (fabsf(ph) <= kExpiMax) return expi_poly(ph);
    float s, c;
    sincosf(ph, &s, &c);
    return make_float2(c, s);
}

// exp(i*ph) - 1 = (-2 sin^2(ph/2), 2 sin(ph/2) cos(ph/2)): both parts with a
// relative error of a few ulp of their own size (no cancellation against 1)
static __device__ __noinline__ float2 expm1i(float ph)
{
    float s, c;
    if (fabsf(0.5f * ph) <= kExpiMax) {
        const float2 e = expi_poly(0.5f * ph);
        c = e.x;
        s = e.y;
    } else {
        sincosf(0.5f * ph, &s, &c);
    }
    return make_float2(-2.0f * s * s, 2.0f * s * c);
}

// phi' = phi + tau (1 + phi) of the scattered form, on a = n phi, b = n tau
// (row transforms of W-states), inv_n = 1/n: returns n phi'.  Rounding 1 + phi
// costs eps |tau| in the product, as small as the other roundings.
__device__ __forceinline__ float2 scat_transmit(float2 a, float2 b, float inv_n)
{
    const float2 bc = cmul(b, make_float2(fmaf(a.x, inv_n, 1.0f), a.y * inv_n));
    return make_float2(a.x + bc.x, a.y + bc.y);
}

// conj(1 + x) g on c = n g, x = n x', inv_n = 1/n: returns n conj(1 + x') g
__device__ __forceinline__ float2 scat_conj_mul(float2 c, float2 x, float inv_n)
{
    return cmul_conj(c, make_float2(fmaf(x.x, inv_n, 1.0f), x.y * inv_n));
}

// |1 + phi|^2 - 1 = phi_r (2 + phi_r) + phi_i^2, without forming 1 + phi
__device__ __forceinline__ float scat_dI(float2 phi)
{
    return fmaf(phi.x, phi.x + 2.0f, phi.y * phi.y);
}

// Rows (lines of length NY) per CTA for the row passes.
template <int NY> struct RowCfg {
    static constexpr int T = FftPlan<NY>::T;
    static constexpr int L = (256 / T) > 0 ? 256 / T : 1;   // P1 and the row utilities
    static constexpr int LT = (128 / T) > 0 ? 128 / T : 1;  // P3 (two tiles in flight)
    static constexpr bool BLK = T > 32;
    // resident CTAs per SM the latency-bound utilities are compiled for
    // (80 registers a thread at 256 threads); fewer where that would spill
    static constexpr int MB = NY <= 1024 ? 3 : 2;
};
// The transmit's schedules, chosen per row length at run time by timing them
// (the row tuner of the host code): the FFT plan EV and the CTA width W.
//   variant 0: EV = 0 (32 points a thread), CTAs of 64 threads (rows of up to
//              32 threads: two or more rows a CTA, so a CTA barrier waits for
//              fewer warps; the registers of six CTAs per SM)
//   variant 1: EV = 0, CTAs of 128 threads (three per SM)
//   variant 2: (64 to 2048 points) EV = 16 (16 points a thread), CTAs of 128
//              threads, four per SM at 128 registers; a 2048-point row is one
//              CTA of 128 threads instead of a 64-thread row that spills
// Shared memory (two rows of complex64 per row in flight) holds every variant
// to ~12-16 resident warps per SM at 1024 points.
constexpr int kRowVariants = 3;
__host__ __device__ constexpr bool row_plan16_ok(int n) { return n >= 64 && n <= 2048; }
template <int NY, int EV = 0, int W = 128> struct TrCfg {
    using P = FftPlan<NY, EV>;
    static constexpr int T = P::T;
    static constexpr int LT = (W / T) > 0 ? W / T : 1;  // rows per CTA
    static constexpr bool BLK = T > 32;
    static constexpr int MB = EV ? 4 : 3 * (128 / (LT * T) > 0 ? 128 / (LT * T) : 1);
};
// Columns per CTA for the column passes, and the TMA boxes of a column tile.
// Per line length up to four variants, chosen per pass at run time by timing
// them (the column tuner of the host code): the FFT plan EV (0: 32 points a
// thread, 16: 16 points a thread), and the tile width V = 0 (the width that
// gives a 128-thread CTA, clamped to 2..16) or V = 1 (half of it, or twice
// where half would be < 2).
template <int NX, int V = 0, int EV = 0> struct ColCfg {
    static constexpr int T = FftPlan<NX, EV>::T;
    static constexpr int C0 = (128 / T) < 2 ? 2 : ((128 / T) > 16 ? 16 : 128 / T);
    static constexpr int C = V == 0 ? C0 : (C0 / 2 >= 2 ? C0 / 2 : 2 * C0);
    static constexpr int NT = C * T;
    static constexpr int BR = NX < 256 ? NX : 256;  // rows per box (TMA boxes are <= 256)
    static constexpr int NBOX = NX / BR;
    static constexpr uint32_t TILE_BYTES = (uint32_t)NX * C * 8;
};
// Column-pass variant index: tile width + 2 x plan (16 points a thread).
constexpr int kColVariants = 4;
__host__ __device__ constexpr bool col_plan16_ok(int n) { return n >= 64 && n <= 2048; }

// One thread arms the CTA's barrier; everyone waits for the phase with a
// bound.  On a timeout the flag is raised and every thread returns false.
__device__ __forceinline__ bool cta_wait(uint64_t *bar, uint32_t parity, int *err)
{
    const bool ok = mbar_wait(bar, parity);
    const bool all = __syncthreads_and(ok) != 0;
    if (!all && threadIdx.x == 0) atomicOr(err, kErrWaitTimeout);
    return all;
}

// After a timeout: wait (bounded) for the copy to land so the CTA does not
// exit under an in-flight write to its shared memory.
__device__ __forceinline__ void cta_drain(uint64_t *bar, uint32_t parity)
{
    if (threadIdx.x == 0) (void)mbar_wait(bar, parity);
    __syncthreads();
}

// Resident CTAs per SM the column pass is compiled for (its register budget):
// with 32 points a thread the propagator pass fits 128 registers, the
// band-limit and free-space passes need ~168 to stay free of spills at 1024
// points.
// With 16 points a thread, five 128-thread CTAs (102 registers).
template <int NX, int MODE, int V, int EV = 0> struct ColMinBlocks {
    static constexpr int per = (EV ? 640 : (MODE == 1 ? 512 : 384)) / ColCfg<NX, V, EV>::NT;
    static constexpr int value = per > 0 ? per : 1;
};

constexpr int kKnots = 100;
// The knot piece of the grid tables (and its shared-memory copy): the 100
// knots of r^2 (float), padding to 128 words, then the interval table of
// spline_vz -- one byte per bucket of r^2, a bucket being 1/16 of an octave
// (the float's exponent and top four mantissa bits), from 2^-20 to 2^5: the
// knots are 13% apart, so a bucket holds at most one of them.
constexpr int kKnotBucketShift = 23 - 4;
constexpr int kKnotBucketBase = (127 - 20) << 4;  // the bucket of 2^-20
constexpr int kKnotBuckets = 25 << 4;
constexpr int kKnotWords = 128 + kKnotBuckets / 4;

// Spline of the projected potential vs r^2 (TemsimLibrary/slicelib.cpp:2402-2425,
// 2812-2875), evaluated in float.  The interval is the one seval's bisection
// finds (knot[i] <= r^2 < knot[i+1], clamped to [0, 98]): the bucket of r^2
// gives the last knot at or below the bucket's start, and one compare with
// the next knot settles it.  `knots` is the knot piece (kKnotWords words).
__device__ __forceinline__ float spline_vz(const float *knots, const float4 *coef, float rsq)
{
    const unsigned char *bucket = reinterpret_cast<const unsigned char *>(knots + 128);
    const int b = min(max((int)(__float_as_uint(rsq) >> kKnotBucketShift) - kKnotBucketBase, 0),
                      kKnotBuckets - 1);
    int i = bucket[b];
    const float k0 = knots[i], k1 = knots[i + 1];
    const bool up = rsq >= k1 && i < kKnots - 2;
    i += up ? 1 : 0;
    const float4 c = __ldg(&coef[i]);
    const float z = rsq - (up ? k1 : k0);
    return c.x + (c.y + (c.z + c.w * z) * z) * z;
}

// ---------------------------------------------------------------- P1
// One CTA = L rows of one unit.  Every thread adds the potential of each atom
// of the (unit, slice) whose window touches its row to the pixels it owns
// (iy = t mod T of its row) -- a gather with a fixed pixel owner, so the sum
// order per pixel is the atom order and the result is deterministic, with no
// atomics (autoslic.cpp:950-984 is a racy scatter in the reference).  Then
// t = exp(i sigma v) and the row FFT.
//   Lines of <= 32 threads (NY <= 1024): every warp owns RW = 32/T whole rows
//   and works alone -- it scans the slice's atom list 32 at a time, a ballot
//   picks the atoms whose window touches its rows, each is broadcast by
//   shuffles -- and stores its own rows, so no row waits for another.
//   Longer lines (a row spans several warps): the atoms touching the CTA's
//   rows are staged into shared memory in slice order (ordered block
//   compaction) and every row's threads loop over them.
// MODE kSplatTrans: A = S(exp(i sigma v)), in-band row segments to tbuf
//      kSplatPot:   v itself (float) to vout + u * vstride
//      kSplatSpec:  S(v) (v as a complex field), whole rows to tbuf (the
//                   Debye-Waller branch filters it before the phase)
enum { kSplatTrans = 0, kSplatPot = 1, kSplatSpec = 2 };

// Per-row shared-memory stride of the splat (float2 units): the padded line,
// rounded to an even count so every row starts 16-byte aligned (bulk copies).
template <int NY> struct SplatCfg {
    static constexpr int SROW = (FftPlan<NY>::PADN + 1) & ~1;
};

// The potential of atom `sa` at this thread's pixels of row ix.
__device__ __forceinline__ void splat_atom(const Geom &g, const SplatAtom &sa, int ix, int t,
                                           int T, int NY, int W, float *vacc, const float *s_knots)
{
    const int nx = g.nx;
    const int ixo = (int)(sa.meta & kMetaMask);
    const int iyo = (int)((sa.meta >> kMetaBits) & kMetaMask);
    const float4 *coef = g.coef + (sa.meta >> (2 * kMetaBits)) * kKnots;
    const int ws = ixo - g.idx;
    for (int ixp = ws + pmod(ix - ws, nx); ixp < ws + W; ixp += nx) {
        const float dx = sa.fx - (float)(ixp - ixo) * g.scalex_f;
        const float dx2 = dx * dx;
        const int ys = iyo - g.idy;
        for (int iyp = ys + pmod(t - ys, T); iyp <= iyo + g.idy; iyp += T) {
            const float dy = sa.fy - (float)(iyp - iyo) * g.scaley_f;
            float rsq = dx2 + dy * dy;
            if (rsq <= 9.0f) {
                rsq = fmaxf(rsq, g.rminsq);
                vacc[pmod(iyp, NY)] += sa.occ * spline_vz(s_knots, coef, rsq);
            }
        }
    }
}

// The atoms [a0, a1) of a (unit, slice) whose window touches this warp's RW
// rows (from wx0), added to the pixels of the row each thread owns (lines of
// <= 32 threads): the list is scanned 32 atoms at a time, a ballot picks the
// atoms that touch the warp's rows, each is broadcast by shuffles; per pixel
// the sums keep the atom order.  vacc = this thread's row (float), zeroed.
template <int NY, int EV = 0>
__device__ __forceinline__ void splat_scan_warp(const Geom &g, const SplatAtom *__restrict__ atoms,
                                                int a0, int a1, int wx0, int RW, int ix,
                                                bool row_ok, int t, float *vacc,
                                                const float *s_knots)
{
    constexpr int T = FftPlan<NY, EV>::T;
    const int nx = g.nx, lane = threadIdx.x & 31;
    const int W = 2 * g.idx + 1;
    for (int base = a0; base < a1; base += 32) {
        const int a = base + lane;
        bool hit = false;
        SplatAtom at = {};
        if (a < a1) {
            at = atoms[a];
            const int ixo = (int)(at.meta & kMetaMask);
            const int rel = pmod(ixo - g.idx - wx0, nx);
            hit = (W >= nx) || (rel < RW) || (rel + W > nx);
        }
        unsigned bal = __ballot_sync(0xffffffffu, hit);
        while (bal) {  // in atom order: the per-pixel sums keep the slice order
            const int k = __ffs(bal) - 1;
            bal &= bal - 1;
            SplatAtom sa;
            sa.fx = __shfl_sync(0xffffffffu, at.fx, k);
            sa.fy = __shfl_sync(0xffffffffu, at.fy, k);
            sa.occ = __shfl_sync(0xffffffffu, at.occ, k);
            sa.meta = __shfl_sync(0xffffffffu, at.meta, k);
            if (row_ok) splat_atom(g, sa, ix, t, T, NY, W, vacc, s_knots);
        }
    }
    __syncwarp();
}

// A = S(exp(i sigma v)) of this thread's row from its potential vacc (float;
// the row's shared region, which the transform then uses as its exchange
// buffer): exp(i 0) = 1 exactly where the potential is 0, and rows without
// atoms take S(1) = NY at iy = 0 directly (what the transform of ones gives).
template <int NY, int SYNC, int EV = 0>
__device__ __forceinline__ void trans_row(const Geom &g, int t, const float *vacc, float2 *xbuf,
                                          float2 (&v)[FftPlan<NY, EV>::E])
{
    constexpr int T = FftPlan<NY, EV>::T, E = FftPlan<NY, EV>::E;
    bool nz = false;
#pragma unroll
    for (int m = 0; m < E; m++) {
        const float ph = vacc[t + m * T] * g.sigma_f;
        v[m] = make_float2(1.0f, 0.0f);
        nz |= ph != 0.0f;
        if (__any_sync(0xffffffffu, ph != 0.0f)) v[m] = expi(ph);
    }
    if (group_none<SYNC == 1>(nz)) {
#pragma unroll
        for (int m = 0; m < E; m++) v[m] = make_float2(m == 0 && t == 0 ? (float)NY : 0.0f, 0.0f);
    } else {
        fft_line<NY, false, 1, SYNC, EV>(v, xbuf, 0, t, EV ? g.tw_row16 : g.tw_row);
    }
}

// This warp's `rows` dense rows (row r at rows_smem + r * stride, 16-byte
// aligned) as their in-band segments [0, seg_e1) and [seg_s2, NY), the (at
// most two) out-of-band elements inside the segments zeroed first; lane 0
// issues the bulk copies and waits until they have read shared memory.
template <int NY>
__device__ __forceinline__ void warp_store_band_rows(const Geom &g, float2 *rows_smem, int stride,
                                                     int rows, float2 *dst)
{
    const int e1 = g.seg_e1, s2 = g.seg_s2, lane = threadIdx.x & 31;
    __syncwarp();  // every element written before the fix-up
    for (int q = lane; q < 2 * rows; q += 32) {
        const int r = q >> 1;
        const int iy = (q & 1) ? s2 : e1 - 1;
        if (iy >= 0 && iy < NY && out_of_band(g, iy)) rows_smem[r * stride + iy] = make_float2(0.0f, 0.0f);
    }
    fence_proxy_async();
    __syncwarp();
    if (lane == 0 && rows > 0) {
        for (int r = 0; r < rows; r++) {
            bulk_store(dst + (size_t)r * NY, rows_smem + r * stride, (uint32_t)e1 * 8u);
            if (s2 < NY)
                bulk_store(dst + (size_t)r * NY + s2, rows_smem + r * stride + s2, (uint32_t)(NY - s2) * 8u);
        }
        bulk_commit();
        bulk_wait_read();
    }
    __syncwarp();
}

// The same for whole rows.
template <int NY>
__device__ __forceinline__ void warp_store_rows(float2 *rows_smem, int stride, int rows, float2 *dst)
{
    fence_proxy_async();
    __syncwarp();
    if ((threadIdx.x & 31) == 0 && rows > 0) {
        for (int r = 0; r < rows; r++)
            bulk_store(dst + (size_t)r * NY, rows_smem + r * stride, (uint32_t)NY * 8u);
        bulk_commit();
        bulk_wait_read();
    }
    __syncwarp();
}

template <int NY, int MODE>
__global__ void __launch_bounds__(RowCfg<NY>::L * FftPlan<NY>::T)
k_row_splat(const Geom g, const int *__restrict__ units, int slice, int nsl1,
            const int *__restrict__ slice_off, const SplatAtom *__restrict__ atoms,
            float2 *__restrict__ tbuf, float *__restrict__ vout, size_t vstride)
{
    using P = FftPlan<NY>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NY>::L, NT = L * T, NW = (NT + 31) / 32;
    constexpr int SROW = SplatCfg<NY>::SROW;
    constexpr bool BLK = RowCfg<NY>::BLK;
    constexpr int RW = BLK ? 1 : 32 / T;  // rows per warp (lines of <= 32 threads)
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    SplatAtom *s_atoms = reinterpret_cast<SplatAtom *>(s_lines + L * SROW);
    float *s_knots = reinterpret_cast<float *>(s_atoms + NT);
    int *s_cnt = reinterpret_cast<int *>(s_knots + kKnotWords);

    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int u = units[blockIdx.x / bpu];
    const int ix0 = (blockIdx.x % bpu) * L;
    const int ix = ix0 + l;
    const bool row_ok = ix < nx;
    const int lane = tid & 31, warp = tid >> 5;

    for (int i = tid; i < kKnotWords; i += NT) s_knots[i] = g.knots[i];
    float *vacc = reinterpret_cast<float *>(s_lines + l * SROW);
#pragma unroll
    for (int m = 0; m < E; m++) vacc[t + m * T] = 0.0f;
    __syncthreads();

    const int a0 = slice_off[u * nsl1 + slice], a1 = slice_off[u * nsl1 + slice + 1];
    const int W = 2 * g.idx + 1;
    if constexpr (!BLK) {
        splat_scan_warp<NY>(g, atoms, a0, a1, ix0 + warp * RW, RW, ix, row_ok, t, vacc, s_knots);
    } else {
        for (int base = a0; base < a1; base += NT) {
            const int a = base + tid;
            bool hit = false;
            SplatAtom at;
            if (a < a1) {
                at = atoms[a];
                const int ixo = (int)(at.meta & kMetaMask);
                const int rel = pmod(ixo - g.idx - ix0, nx);
                hit = (W >= nx) || (rel < L) || (rel + W > nx);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) s_cnt[warp] = __popc(bal);
            __syncthreads();
            if (warp == 0) {
                int c = lane < NW ? s_cnt[lane] : 0;
                int incl = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                if (lane < NW) s_cnt[lane] = incl - c;
                if (lane == 31) s_cnt[NW] = incl;
            }
            __syncthreads();
            if (hit) s_atoms[s_cnt[warp] + __popc(bal & ((1u << lane) - 1u))] = at;
            const int nsel = s_cnt[NW];
            __syncthreads();
            if (row_ok)
                for (int k = 0; k < nsel; k++) splat_atom(g, s_atoms[k], ix, t, T, NY, W, vacc, s_knots);
            __syncthreads();
        }
    }
    // rows of this warp (lines <= 32 threads) or of the CTA that exist
    const int wrow0 = BLK ? 0 : warp * RW;
    const int wrows = BLK ? min(L, nx - ix0) : min(RW, nx - ix0 - wrow0);
    if constexpr (MODE == kSplatPot) {
        // the projected potential itself: vout -> slice `slice` of unit 0
        if (row_ok) {
            float *dst = vout + (size_t)u * vstride + (size_t)ix * NY;
#pragma unroll
            for (int m = 0; m < E; m++) dst[t + m * T] = vacc[t + m * T];
        }
    } else if constexpr (MODE == kSplatSpec) {
        float2 v[E];
        bool nz = false;
#pragma unroll
        for (int m = 0; m < E; m++) {
            v[m] = make_float2(vacc[t + m * T], 0.0f);
            nz |= v[m].x != 0.0f;
        }
        if (!group_none<BLK>(nz))  // S(0) = 0: rows without atoms skip the transform
            fft_line<NY, false, 1, BLK>(v, s_lines + l * SROW, 0, t, g.tw_row);
        if constexpr (BLK) {
            __syncthreads();
#pragma unroll
            for (int m = 0; m < E; m++) s_lines[l * NY + t + m * T] = v[m];
            fence_proxy_async();
            __syncthreads();
            if (tid == 0) {
                bulk_store(tbuf + ((size_t)u * nx + ix0) * NY, s_lines, (uint32_t)wrows * NY * 8u);
                bulk_commit();
                bulk_wait_read();
            }
        } else {
            __syncwarp();  // the row's reads of its region are done
#pragma unroll
            for (int m = 0; m < E; m++) s_lines[l * SROW + t + m * T] = v[m];
            warp_store_rows<NY>(s_lines + wrow0 * SROW, SROW, wrows,
                                tbuf + ((size_t)u * nx + ix0 + wrow0) * NY);
        }
    } else {
        float2 v[E];
        trans_row<NY, BLK ? 1 : 0>(g, t, vacc, s_lines + l * SROW, v);
        // dense rows into shared memory, then their in-band segments to the
        // buffer (its out-of-band columns hold zeros: the band limit zeroes them)
        if constexpr (BLK) {
            __syncthreads();
#pragma unroll
            for (int m = 0; m < E; m++) s_lines[l * NY + t + m * T] = v[m];
            store_band_rows<NY>(g, s_lines, wrows, tbuf + ((size_t)u * nx + ix0) * NY);
        } else {
            __syncwarp();  // the row's reads of its region are done
#pragma unroll
            for (int m = 0; m < E; m++) s_lines[l * SROW + t + m * T] = v[m];
            warp_store_band_rows<NY>(g, s_lines + wrow0 * SROW, SROW, wrows,
                                     tbuf + ((size_t)u * nx + ix0 + wrow0) * NY);
        }
    }
}

// ---------------------------------------------------------------- P2 / P4 / free space
// Column FFT, pointwise multiplier times fscale, column inverse FFT.  One
// CTA = C adjacent columns of one unit; C columns interleave in shared
// memory so each half-warp moves whole 32-byte sectors.
//   MODE 0: 2/3 band limit of the transmission function
//           (autoslic.cpp:999-1009)
//   MODE 1: Fresnel propagator p_y then p_x with the 2/3 aperture
//           (slicelib.cpp:811-849)
//   MODE 2: free-space step exp(-i chi) with the objective aperture
//   MODE 3: Debye-Waller damping (float)exp(-B k^2/4) of a potential's
//           spectrum (autoslic.cpp:1098-1106), -B/4 per unit in fr.dw
enum { kColMask = 0, kColProp = 1, kColFresnel = 2, kColDW = 3 };

template <int NX, int MODE, int V, int EV = 0>
__global__ void __launch_bounds__(ColCfg<NX, V, EV>::NT, ColMinBlocks<NX, MODE, V, EV>::value)
k_col_pass(const Geom g, const __grid_constant__ CUtensorMap in_map,
           const __grid_constant__ CUtensorMap out_map, const int *__restrict__ units,
           const Fresnel fr, float fscale, int band)
{
    using P = FftPlan<NX, EV>;
    using CC = ColCfg<NX, V, EV>;
    constexpr int VI = V + 2 * (EV ? 1 : 0);  // the variant's index in Geom::cb_*
    const float2 *tw = EV ? g.tw_col16 : g.tw_col;
    constexpr int T = P::T, E = P::E, C = CC::C;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *buf = reinterpret_cast<float2 *>(smem);                       // PADN*C
    uint64_t *bar = reinterpret_cast<uint64_t *>(buf + P::PADN * C);

    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const int ny = g.ny;
    // band mode: only the column blocks that hold in-band columns (the others
    // are zero on input and output)
    const int bpu = band ? g.cb_n[VI] : ny / C;
    const int u = units ? units[blockIdx.x / bpu] : (int)(blockIdx.x / bpu);
    int cb = blockIdx.x % bpu;
    if (band && cb >= g.cb_lo[VI]) cb = g.cb_hi0[VI] + (cb - g.cb_lo[VI]);
    const int iy = cb * C + c;
    // tile = rows u*NX .. u*NX+NX-1, float columns 2*cb*C .. 2*cb*C+2C-1
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, CC::TILE_BYTES);
#pragma unroll
        for (int j = 0; j < CC::NBOX; j++)
            tma_load_2d(buf + j * CC::BR * C, &in_map, 2 * cb * C, u * NX + j * CC::BR, bar);
    }
    if (!cta_wait(bar, 0, g.err)) {
        cta_drain(bar, 0);
        return;
    }
    float2 v[E];
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = buf[(t + m * T) * C + c];
    fft_line<NX, false, C, true, EV>(v, buf, c, t, tw);

    if constexpr (MODE == kColMask) {
        // the band limit ky2 + kx2 < k2max keeps ix <= A or ix >= B (host-exact)
        const int2 ab = __ldg(&g.kband[iy]);
#pragma unroll
        for (int m = 0; m < E; m++) {
            const int ix = t + m * T;
            v[m] = (ix <= ab.x || ix >= ab.y) ? cscale(v[m], fscale) : make_float2(0.0f, 0.0f);
        }
    } else if constexpr (MODE == kColProp) {
        // kx2 < k2max and kx2 + ky2 < k2max: the same index set as the band
        // limit; propx carries the 1/nx of the transforms (fscale is 1)
        const int2 ab = __ldg(&g.kband[iy]);
        const float2 py = __ldg(&g.propy[iy]);
#pragma unroll
        for (int m = 0; m < E; m++) {
            const int ix = t + m * T;
            v[m] = (ix <= ab.x || ix >= ab.y) ? cmul(cmul(v[m], py), __ldg(&g.propx[ix]))
                                              : make_float2(0.0f, 0.0f);
        }
    } else if constexpr (MODE == kColDW) {
        const float mb4 = __ldg(&fr.dw[(size_t)u * fr.dw_stride]);
        const float ky2 = __ldg(&g.ky2[iy]);
#pragma unroll
        for (int m = 0; m < E; m++) {
            const float k2 = __fadd_rn(ky2, __ldg(&g.kx2[t + m * T]));
            v[m] = cscale(v[m], expf(mb4 * k2) * fscale);
        }
    } else {
        const float2 *tab = fr.table + iy;
#pragma unroll
        for (int m = 0; m < E; m++) v[m] = cmul(v[m], __ldg(&tab[(size_t)(t + m * T) * ny]));
    }
    fft_line<NX, true, C, true, EV>(v, buf, c, t, tw);
    __syncthreads();  // every thread is done with the exchange layout
#pragma unroll
    for (int m = 0; m < E; m++) buf[(t + m * T) * C + c] = v[m];
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int j = 0; j < CC::NBOX; j++)
            tma_store_2d(&out_map, 2 * cb * C, u * NX + j * CC::BR, buf + j * CC::BR * C);
        bulk_commit();
        bulk_wait_read();
    }
}

// ---------------------------------------------------------------- P3
// W' = S(iS(W) * iS(B)) * out_scale (out_scale = 1/ny^2): wave *= trans
// (cfpix.cpp:349-372) between the transmission's and the wave's row
// transforms.  `out` may be `psi` (in place).  SCAT: the scattered form,
// W = S(phi), B = S(tau_bl), out = S(phi + tau + phi tau) * out_scale * ny.
// EV, W: the line FFT plan and the CTA width (TrCfg).
template <int NY, bool SCAT = false, int EV = 0, int W = 128>
__global__ void __launch_bounds__(TrCfg<NY, EV, W>::LT * TrCfg<NY, EV, W>::T, TrCfg<NY, EV, W>::MB)
k_row_transmit(const Geom g, const int *__restrict__ units, const float2 *__restrict__ tbuf,
               const float2 *psi, float2 *out, float out_scale, int band)
{
    using P = FftPlan<NY, EV>;
    constexpr int T = P::T, E = P::E, L = TrCfg<NY, EV, W>::LT;
    constexpr bool BLK = TrCfg<NY, EV, W>::BLK;
    const float2 *tw = EV ? g.tw_row16 : g.tw_row;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *bufB = reinterpret_cast<float2 *>(smem);   // transmission rows, then t_bl
    float2 *bufW = bufB + L * P::PADN;                  // wave rows
    uint64_t *bar = reinterpret_cast<uint64_t *>(bufW + L * P::PADN);

    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int u = units ? units[blockIdx.x / bpu] : (int)(blockIdx.x / bpu);
    const int ix0 = (blockIdx.x % bpu) * L;
    const int rows = min(L, nx - ix0);
    const uint32_t bytes = (uint32_t)rows * NY * 8u;
    const size_t off = ((size_t)u * nx + ix0) * NY;
    // band: only the row segments [0, e1) and [s2, NY) move (even bounds, so
    // every copy is 16-byte aligned); the rest is zero in B and W
    const int e1 = band ? g.seg_e1 : NY, s2 = band ? g.seg_s2 : NY;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        if (band) {  // segments from the buffers, the middle from the zero source
            mbar_arrive_expect_tx(bar, 2u * bytes);
            for (int r = 0; r < rows; r++) {
                const size_t ro = off + (size_t)r * NY;
                bulk_load(bufB + r * NY, tbuf + ro, (uint32_t)e1 * 8u, bar);
                bulk_load(bufW + r * NY, psi + ro, (uint32_t)e1 * 8u, bar);
                if (s2 > e1) {
                    bulk_load(bufB + r * NY + e1, g.zeros, (uint32_t)(s2 - e1) * 8u, bar);
                    bulk_load(bufW + r * NY + e1, g.zeros, (uint32_t)(s2 - e1) * 8u, bar);
                }
                if (s2 < NY) {
                    bulk_load(bufB + r * NY + s2, tbuf + ro + s2, (uint32_t)(NY - s2) * 8u, bar);
                    bulk_load(bufW + r * NY + s2, psi + ro + s2, (uint32_t)(NY - s2) * 8u, bar);
                }
            }
        } else {
            mbar_arrive_expect_tx(bar, 2u * bytes);
            bulk_load(bufB, tbuf + off, bytes, bar);
            bulk_load(bufW, psi + off, bytes, bar);
        }
    }
    if (!cta_wait(bar, 0, g.err)) {
        cta_drain(bar, 0);
        return;
    }
    float2 v[E];
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = bufB[l * NY + t + m * T];
    __syncthreads();  // dense rows read before any line's exchange overwrites them
    fft_line<NY, true, 1, BLK, EV>(v, bufB + l * P::PADN, 0, t, tw);
    __syncthreads();
#pragma unroll
    for (int m = 0; m < E; m++) bufB[l * NY + t + m * T] = v[m];  // t_bl, own elements only
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = bufW[l * NY + t + m * T];
    __syncthreads();
    fft_line<NY, true, 1, BLK, EV>(v, bufW + l * P::PADN, 0, t, tw);
#pragma unroll
    for (int m = 0; m < E; m++)
        v[m] = SCAT ? scat_transmit(v[m], bufB[l * NY + t + m * T], 1.0f / (float)NY)
                    : cmul(v[m], bufB[l * NY + t + m * T]);
    fft_line<NY, false, 1, BLK, EV>(v, bufW + l * P::PADN, 0, t, tw);
    __syncthreads();
    if (out_scale == 1.0f) {  // the scale already carried by B (no multiply)
#pragma unroll
        for (int m = 0; m < E; m++) bufW[l * NY + t + m * T] = v[m];
    } else {
#pragma unroll
        for (int m = 0; m < E; m++) bufW[l * NY + t + m * T] = cscale(v[m], out_scale);
    }
    if (band) {  // in-band segments only: `out` holds zeros out of band, the
                 // propagator that follows zeroes those columns
        store_band_rows<NY>(g, bufW, rows, out + off);
        return;
    }
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
        bulk_store(out + off, bufW, bytes);
        bulk_commit();
        bulk_wait_read();
    }
}

// ---------------------------------------------------------------- row utilities
// MODE 0: W0 = S(wave0) * scale (start state from an incident wave; wave0
//         shared by all units, units[i] selects the destination)
// MODE 1: psi = iS(W) * scale, scale = 1/ny (exit wave)
enum { kRowInit = 0, kRowExit = 1 };

template <int NY, int MODE>
__global__ void __launch_bounds__(RowCfg<NY>::L * FftPlan<NY>::T)
k_row_simple(const Geom g, const int *__restrict__ units, const float2 *__restrict__ in,
             float2 *__restrict__ out, float scale)
{
    using P = FftPlan<NY>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NY>::L;
    constexpr bool BLK = RowCfg<NY>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int ui = blockIdx.x / bpu;
    const int u = units ? units[ui] : ui;
    const int ix = (blockIdx.x % bpu) * L + l;
    const bool row_ok = ix < nx;
    const size_t row = (size_t)(row_ok ? ix : 0) * NY;
    const float2 *src = (MODE == kRowInit) ? in + row : in + (size_t)u * nx * NY + row;
    float2 v[E];
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = src[t + m * T];
    fft_line<NY, MODE == kRowExit, 1, BLK>(v, s_lines + l * P::PADN, 0, t, g.tw_row);
    if (row_ok) {
        float2 *dst = out + (size_t)u * nx * NY + row;
#pragma unroll
        for (int m = 0; m < E; m++) dst[t + m * T] = cscale(v[m], scale);
    }
}

// Detector intensity, averaged over thermal configurations
// (autosliccmd.cpp:1205-1224: I = |psi|^2, summed in configuration order,
// divided by the configuration count after the last one).
//   img_units[img_off[i] .. img_off[i+1]) : units (configurations, in order)
//                                           whose free-space waves make image i
//   img_dst[i]: destination image index; img_flags[i]: 1 = add onto the
//   partial sum already stored, 2 = divide by nconf after adding.
// SCAT: the waves are the scattered parts phi of psi = 1 + phi.
template <int NY, bool SCAT = false>
__global__ void __launch_bounds__(RowCfg<NY>::L * FftPlan<NY>::T)
k_row_intensity(const Geom g, const int *__restrict__ img_off, const int *__restrict__ img_units,
                const int *__restrict__ img_dst, const int *__restrict__ img_flags,
                const float2 *__restrict__ ebuf, float *__restrict__ images, float nconf)
{
    using P = FftPlan<NY>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NY>::L;
    constexpr bool BLK = RowCfg<NY>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int img = blockIdx.x / bpu;
    const int ix = (blockIdx.x % bpu) * L + l;
    const bool row_ok = ix < nx;
    const size_t row = (size_t)(row_ok ? ix : 0) * NY;
    float acc[E];
    const int flags = img_flags[img];
    float *dst = images + (size_t)img_dst[img] * nx * NY + row;
#pragma unroll
    for (int m = 0; m < E; m++) acc[m] = (flags & 1) && row_ok ? dst[t + m * T] : 0.0f;
    for (int k = img_off[img]; k < img_off[img + 1]; k++) {
        const float2 *src = ebuf + (size_t)img_units[k] * nx * NY + row;
        float2 v[E];
#pragma unroll
        for (int m = 0; m < E; m++) v[m] = src[t + m * T];
        fft_line<NY, true, 1, BLK>(v, s_lines + l * P::PADN, 0, t, g.tw_row);
#pragma unroll
        for (int m = 0; m < E; m++)
            acc[m] += SCAT ? 1.0f + scat_dI(v[m]) : v[m].x * v[m].x + v[m].y * v[m].y;
    }
    if (row_ok) {
#pragma unroll
        for (int m = 0; m < E; m++) dst[t + m * T] = (flags & 2) ? __fdiv_rn(acc[m], nconf) : acc[m];
    }
}

// ---------------------------------------------------------------- potential stacks
// Rows of a per-slice potential stack v[u][k][ix][iy] (float, V*Angstrom):
// A = S(exp(i sigma v) - 1), the scattered part tau of the transmission
// before its band limit.  `v` points at slice k of unit 0; units are
// `ustride` floats apart.
template <int NY>
__global__ void __launch_bounds__(RowCfg<NY>::L * FftPlan<NY>::T, RowCfg<NY>::MB)
k_row_expv(const Geom g, const float *__restrict__ v, size_t ustride, float2 *__restrict__ out)
{
    using P = FftPlan<NY>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NY>::L;
    constexpr bool BLK = RowCfg<NY>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int u = blockIdx.x / bpu;
    const int ix = (blockIdx.x % bpu) * L + l;
    const float *src = v + (size_t)u * ustride + (size_t)(ix < nx ? ix : 0) * NY;
    float2 w[E];
    bool nz = false;
    // every load in flight before the first vote on a value (a vote per load
    // would send them out one memory latency apart); the potentials wait in
    // the real parts
#pragma unroll
    for (int m = 0; m < E; m++) w[m].x = src[t + m * T];
#pragma unroll
    for (int m = 0; m < E; m++) {
        const float ph = w[m].x * g.sigma_f;
        w[m] = make_float2(0.0f, 0.0f);
        nz |= ph != 0.0f;
        if (__any_sync(0xffffffffu, ph != 0.0f)) w[m] = expm1i(ph);
    }
    if (!group_none<BLK>(nz))  // S(0) = 0: empty rows skip the transform
        fft_line<NY, false, 1, BLK>(w, s_lines + l * P::PADN, 0, t, g.tw_row);
    if (ix < nx) {  // out-of-band columns as zeros: the band limit zeroes them
        float2 *dst = out + ((size_t)u * nx + ix) * NY;
#pragma unroll
        for (int m = 0; m < E; m++)
            dst[t + m * T] = out_of_band(g, t + m * T) ? make_float2(0.0f, 0.0f) : w[m];
    }
}

// Debye-Waller branch, last step (autoslic.cpp:1107-1118): from C = the
// damped spectrum after the column pass (iF(D F(S v))/nx), the damped
// potential v' = Re(iS(C))/ny, t = exp(i sigma v'), A = S(t) stored as the
// in-band row segments of `out` (as the splat stores them).
template <int NY>
__global__ void __launch_bounds__(RowCfg<NY>::L * FftPlan<NY>::T)
k_row_dwexp(const Geom g, const int *__restrict__ units, const float2 *__restrict__ spec,
            float2 *__restrict__ out)
{
    using P = FftPlan<NY>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NY>::L;
    constexpr bool BLK = RowCfg<NY>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int u = units[blockIdx.x / bpu];
    const int ix0 = (blockIdx.x % bpu) * L;
    const int ix = ix0 + l;
    const bool row_ok = ix < nx;
    const float2 *src = spec + ((size_t)u * nx + (row_ok ? ix : 0)) * NY;
    float2 w[E];
#pragma unroll
    for (int m = 0; m < E; m++) w[m] = src[t + m * T];
    fft_line<NY, true, 1, BLK>(w, s_lines + l * P::PADN, 0, t, g.tw_row);
    const float sc = g.sigma_f / (float)NY;
#pragma unroll
    for (int m = 0; m < E; m++) {
        const float ph = w[m].x * sc;
        w[m] = make_float2(1.0f, 0.0f);
        if (__any_sync(0xffffffffu, ph != 0.0f)) w[m] = expi(ph);
    }
    fft_line<NY, false, 1, BLK>(w, s_lines + l * P::PADN, 0, t, g.tw_row);
    __syncthreads();
#pragma unroll
    for (int m = 0; m < E; m++) s_lines[l * NY + t + m * T] = w[m];
    store_band_rows<NY>(g, s_lines, min(L, nx - ix0), out + ((size_t)u * nx + ix0) * NY);
}

// Adjoint of transmit, scattered form.  In W-states (W(f) = S(f)): from
// Gu = W(g_u), B = W(tau_k), Wp = W(phi_{k-1}):  Gu <- W(conj(1 + tau) g_u)
// (dL/dconj psi_{k-1}) and B <- W(conj(1 + phi_{k-1}) g_u) (dL/dconj t_k),
// both in place.  Its five row transforms run as one forward transform in a
// loop that is not unrolled (the three inverse ones as conj(S(conj x))): one
// copy of the transform's code instead of five, which ncu showed stalling on
// instruction fetch (15.2 -> 14.3 ms of the C5 call).
template <int NY>
__global__ void __launch_bounds__(RowCfg<NY>::LT * FftPlan<NY>::T)
k_row_adj_transmit(const Geom g, float2 *Gu, float2 *B, const float2 *__restrict__ Wp)
{
    using P = FftPlan<NY>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NY>::LT;
    constexpr bool BLK = RowCfg<NY>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    float2 *s_stash = s_lines + L * P::PADN;
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int u = blockIdx.x / bpu;
    const int ix = (blockIdx.x % bpu) * L + l;
    const bool row_ok = ix < nx;
    const size_t off = ((size_t)u * nx + (row_ok ? ix : 0)) * NY;
    const float sc = 1.0f / (float)NY, inv_n = 1.0f / (float)NY;
    float2 *buf = s_lines + l * P::PADN;
    float2 *stash = s_stash + l * NY;
    float2 a[E];
#pragma unroll 1
    for (int ph = 0; ph < 5; ph++) {
        if (ph == 0 || ph == 1 || ph == 3) {
            const float2 *src = ph == 0 ? Gu : (ph == 1 ? B : Wp);
#pragma unroll
            for (int m = 0; m < E; m++) {
                const float2 x = src[off + t + m * T];
                a[m] = make_float2(x.x, -x.y);
            }
        }
        fft_line<NY, false, 1, BLK>(a, buf, 0, t, g.tw_row);
        if (ph == 0) {
#pragma unroll
            for (int m = 0; m < E; m++) stash[t + m * T] = make_float2(a[m].x, -a[m].y);
        } else if (ph == 1 || ph == 3) {
#pragma unroll
            for (int m = 0; m < E; m++)
                a[m] = scat_conj_mul(stash[t + m * T], make_float2(a[m].x, -a[m].y), inv_n);
        } else if (row_ok) {
            float2 *dst = ph == 2 ? Gu : B;
#pragma unroll
            for (int m = 0; m < E; m++) dst[off + t + m * T] = cscale(a[m], sc);
        }
    }
}

// dL/dv_k = 2 sigma Im(g_e conj(e_k)), e_k = exp(i sigma v_k), from
// Ge = W(g_e).  `v` and `grad` point at slice k of unit 0, units `ustride`
// floats apart.
template <int NY>
__global__ void __launch_bounds__(RowCfg<NY>::L * FftPlan<NY>::T, RowCfg<NY>::MB)
k_row_grad(const Geom g, const float2 *__restrict__ Ge, const float *__restrict__ v,
           size_t ustride, float *__restrict__ grad)
{
    using P = FftPlan<NY>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NY>::L;
    constexpr bool BLK = RowCfg<NY>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int u = blockIdx.x / bpu;
    const int ix = (blockIdx.x % bpu) * L + l;
    const bool row_ok = ix < nx;
    const size_t row = (size_t)(row_ok ? ix : 0) * NY;
    float2 a[E];
#pragma unroll
    for (int m = 0; m < E; m++) a[m] = Ge[(size_t)u * nx * NY + row + t + m * T];
    fft_line<NY, true, 1, BLK>(a, s_lines + l * P::PADN, 0, t, g.tw_row);
    const float c = 2.0f * g.sigma_f / (float)NY;
    const float *vr = v + (size_t)u * ustride + row;
    float *gr = grad + (size_t)u * ustride + row;
    // the potentials in groups of G loads in flight before their votes (the
    // transformed row holds the registers a whole line would need)
    constexpr int G = E < 8 ? E : 8;
#pragma unroll
    for (int m0 = 0; m0 < E; m0 += G) {
        float vv[G];
#pragma unroll
        for (int j = 0; j < G; j++) vv[j] = vr[t + (m0 + j) * T];
#pragma unroll
        for (int j = 0; j < G; j++) {
            const int m = m0 + j;
            const float ph = vv[j] * g.sigma_f;
            float2 e = make_float2(1.0f, 0.0f);
            if (__any_sync(0xffffffffu, ph != 0.0f)) e = expi(ph);
            if (row_ok) gr[t + m * T] = c * (a[m].y * e.x - a[m].x * e.y);
        }
    }
}

// Image residual of the loss L = sum (|psi|^2 - T)^2, scattered form: from E
// with phi = iS(E) (the free-space column pass output, psi = 1 + phi),
// r = I - T = (1 - T) + (|1 + phi|^2 - 1), G = S(2 r psi) = W(dL/dconj psi);
// per-CTA partial sums of r^2 go to partial[block].
// G may be Ein: every CTA reads its rows before it writes them.
template <int NY>
__global__ void __launch_bounds__(RowCfg<NY>::L * FftPlan<NY>::T)
k_row_imgrad(const Geom g, const float2 *Ein, const float *__restrict__ target, size_t tstride,
             float2 *G, double *__restrict__ partial)
{
    using P = FftPlan<NY>;
    constexpr int T = P::T, E = P::E, L = RowCfg<NY>::L, NT = L * T;
    constexpr bool BLK = RowCfg<NY>::BLK;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *s_lines = reinterpret_cast<float2 *>(smem);
    double *s_red = reinterpret_cast<double *>(s_lines + L * P::PADN);
    const int tid = threadIdx.x, l = tid / T, t = tid % T;
    const int nx = g.nx;
    const int bpu = (nx + L - 1) / L;
    const int u = blockIdx.x / bpu;
    const int ix = (blockIdx.x % bpu) * L + l;
    const bool row_ok = ix < nx;
    const size_t row = (size_t)(row_ok ? ix : 0) * NY;
    float2 a[E];
#pragma unroll
    for (int m = 0; m < E; m++) a[m] = Ein[(size_t)u * nx * NY + row + t + m * T];
    fft_line<NY, true, 1, BLK>(a, s_lines + l * P::PADN, 0, t, g.tw_row);  // phi
    const float *tr = target + (size_t)u * tstride + row;
    double acc = 0.0;
#pragma unroll
    for (int m = 0; m < E; m++) {
        const float r = row_ok ? (1.0f - tr[t + m * T]) + scat_dI(a[m]) : 0.0f;
        acc += (double)r * (double)r;
        a[m] = make_float2(2.0f * r * (1.0f + a[m].x), 2.0f * r * a[m].y);
    }
    fft_line<NY, false, 1, BLK>(a, s_lines + l * P::PADN, 0, t, g.tw_row);
    if (row_ok) {
#pragma unroll
        for (int m = 0; m < E; m++) G[(size_t)u * nx * NY + row + t + m * T] = a[m];
    }
    // fixed-order block reduction: deterministic loss
    __syncthreads();
    s_red[tid] = acc;
    __syncthreads();
    for (int w = NT / 2; w > 0; w >>= 1) {
        if (tid < w) s_red[tid] += s_red[tid + w];
        __syncthreads();
    }
    if (tid == 0) partial[blockIdx.x] = s_red[0];
}

// The free-space multiplier of one detector plane, in double, reduced modulo
// 2 pi before the single-precision sine and cosine: table[ix*ny + iy] =
// scale * exp(-i chi(kx, ky)) inside the aperture, 0 outside.
__global__ void k_fresnel_table(const Geom g, const Fresnel fr, float scale, float2 *table);
__global__ void k_plane_init(float2 *psi, const int *__restrict__ units, int nunits, int nx, int ny);

}  // namespace msk
