// msk_small.cuh -- the whole slice loop of a small grid in one launch: one
// thread-block cluster per unit (orientation x configuration).
//
// For N x N grids with N <= 256 a unit's buffers (the wave W = S(psi) and two
// transmission buffers, 0.5 MB each at 256^2) stay in L2, and a slice-step is
// too small to fill the GPU from one launch per pass: the multi-launch loop
// spends most of its time in launch latency.  Here a cluster of Q = N/16 CTAs
// owns one unit; CTA r owns rows [16r, 16r+16) and columns [16r, 16r+16).  Each
// slice is two phases separated by cluster barriers (release / acquire at
// cluster scope, so every CTA's global writes of one phase are visible to the
// others in the next):
//
//   row phase k:    half 0  transmit of slice k on the CTA's rows
//                           W = S(iS(W) iS(B_k))                 (P3)
//                   half 1  splat of slice k+1 on the same rows
//                           A_{k+1} = S(exp(i sigma v))          (P1)
//   column phase k: half 0  propagator of slice k on the CTA's columns
//                           W = iF(P F(W))/nx                    (P4)
//                   half 1  band limit of slice k+1
//                           B_{k+1} = iF(M F(A_{k+1}))/(nx ny^2) (P2)
//
// (slices without atoms skip P1-P3).  The two CTA halves run different passes
// at once, each with its own named barrier for its column transforms; the
// transmissions of consecutive slices with atoms alternate between the two
// buffers.  Every row and column is computed with the same line transforms,
// multipliers and atom order as the multi-launch passes (k_row_splat,
// k_col_pass, k_row_transmit), whole rows and columns instead of the in-band
// segments.  Loads of data another CTA wrote go through L2 (ld.global.cg).
//
// The line transforms use the 16-points-a-thread plan (FftPlan<N, 16>: twice
// the threads per line of the multi-launch passes, half the registers and the
// serial chain per thread), so a CTA of 2 x 16 lines has 512 threads at 256^2;
// the results equal the multi-launch loop's to FP32 rounding (the same
// potentials, multipliers and atom order; another radix split of the FFT).
// The grid is `units x Q` CTAs in clusters of Q (Q = 16 for 256^2 needs the
// non-portable cluster size); no CTA leaves the slice loop early, so every one
// arrives at every cluster barrier.
#pragma once

#include "msk_passes.cuh"

namespace msk {

template <int N>
struct SmallCfg {
    static constexpr int EV = 16;  // the plan's elements per thread
    using P = FftPlan<N, EV>;
    static constexpr int T = P::T, E = P::E;
    static constexpr int LPC = 16;        // rows (and columns) one CTA owns
    static constexpr int Q = N / LPC;     // CTAs per cluster: one unit
    static constexpr int HALF = LPC * T;  // threads of one half
    static constexpr int NT = 2 * HALF;
    static constexpr int RW = 32 / T;     // rows per warp in the row phase
    static constexpr int PADN = P::PADN;
    static constexpr int SROW = (P::PADN + 1) & ~1;
    // shared memory in float2 units.  Row phase: half 0 a transform buffer and
    // a stash of iS(B) per row; half 1 the splat row (potential, then the
    // transform's exchange).  Column phase: one tile of LPC interleaved columns
    // per half.
    static constexpr int ROW0 = LPC * (PADN + N);
    static constexpr int ROW1 = LPC * SROW;
    static constexpr int COL = LPC * PADN;
    static constexpr int F2 = (ROW0 + ROW1) > 2 * COL ? (ROW0 + ROW1) : 2 * COL;
    static constexpr size_t SMEM = (size_t)F2 * 8 + kKnotWords * 4;
    static_assert(N >= 64 && N <= 256, "small-grid sizes");
    static_assert(T <= 32 && 32 % T == 0, "a warp holds whole lines");
    static_assert(HALF % 32 == 0, "halves of whole warps");
};

__device__ __forceinline__ unsigned cluster_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Every thread of the cluster: this CTA's earlier writes (global and shared)
// visible to every CTA of the cluster after it.
__device__ __forceinline__ void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int N>
__global__ void __launch_bounds__(SmallCfg<N>::NT, 1)
k_small_slices(const Geom g, int nslices, int nsl1, const int *__restrict__ slice_off,
               const SplatAtom *__restrict__ atoms, float2 *W, float2 *Tb0, float2 *Tb1)
{
    using C = SmallCfg<N>;
    constexpr int T = C::T, E = C::E, LPC = C::LPC, HALF = C::HALF, EV = C::EV;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *sm = reinterpret_cast<float2 *>(smem);
    float *s_knots = reinterpret_cast<float *>(sm + C::F2);

    const int rank = (int)cluster_rank();
    const int u = blockIdx.x / C::Q;
    const int half = threadIdx.x / HALF, ht = threadIdx.x % HALF;
    const size_t plane = (size_t)N * N;
    float2 *Wu = W + (size_t)u * plane;
    float2 *Tu[2] = {Tb0 + (size_t)u * plane, Tb1 + (size_t)u * plane};
    const int *so = slice_off + (size_t)u * nsl1;
    for (int i = threadIdx.x; i < kKnotWords; i += C::NT) s_knots[i] = g.knots[i];
    __syncthreads();

    // row phase: line l of the CTA's rows, thread t of the line
    const int rl = ht / T, rt = ht % T, row = rank * LPC + rl;
    // column phase: column c of the CTA's columns, thread t of the line
    const int cc = ht % LPC, ct = ht / LPC, col = rank * LPC + cc;
    const float mask_scale = (1.0f / ((float)N * (float)N)) / (float)N;

    // slice k's transmission lives in buffer tb[k] = (slices with atoms before k) & 1
    int tb_next = 0;  // buffer of slice k+1, updated as the loop advances
    int tb_cur = 0;
    for (int k = -1; k < nslices; k++) {
        const bool has_k = k >= 0 && so[k + 1] > so[k];
        const bool has_n = k + 1 < nslices && so[k + 2] > so[k + 1];
        if (k >= 0) {
            tb_cur = tb_next;
            tb_next = has_k ? (tb_cur ^ 1) : tb_cur;
        }
        // ---- row phase
        if (half == 0) {
            if (has_k) {  // W = S(iS(W) iS(B_k)) on this row
                float2 *xb = sm + rl * (C::PADN + N), *stash = xb + C::PADN;
                const float2 *brow = Tu[tb_cur] + (size_t)row * N;
                float2 *wrow = Wu + (size_t)row * N;
                float2 v[E];
#pragma unroll
                for (int m = 0; m < E; m++) v[m] = __ldcg(&brow[rt + m * T]);
                fft_line<N, true, 1, 0, EV>(v, xb, 0, rt, g.tw_row16);
#pragma unroll
                for (int m = 0; m < E; m++) stash[rt + m * T] = v[m];
#pragma unroll
                for (int m = 0; m < E; m++) v[m] = __ldcg(&wrow[rt + m * T]);
                fft_line<N, true, 1, 0, EV>(v, xb, 0, rt, g.tw_row16);
#pragma unroll
                for (int m = 0; m < E; m++) v[m] = cmul(v[m], stash[rt + m * T]);
                fft_line<N, false, 1, 0, EV>(v, xb, 0, rt, g.tw_row16);
#pragma unroll
                for (int m = 0; m < E; m++) wrow[rt + m * T] = v[m];
            }
        } else if (has_n) {  // A_{k+1} = S(exp(i sigma v)) on this row
            float2 *xb = sm + C::ROW0 + rl * C::SROW;
            float *vacc = reinterpret_cast<float *>(xb);
#pragma unroll
            for (int m = 0; m < E; m++) vacc[rt + m * T] = 0.0f;
            __syncwarp();
            const int wx0 = rank * LPC + ((ht >> 5) * C::RW);  // this warp's first row
            splat_scan_warp<N, EV>(g, atoms, so[k + 1], so[k + 2], wx0, C::RW, row, true, rt,
                                   vacc, s_knots);
            float2 v[E];
            trans_row<N, 0, EV>(g, rt, vacc, xb, v);
            float2 *arow = Tu[tb_next] + (size_t)row * N;
#pragma unroll
            for (int m = 0; m < E; m++)
                arow[rt + m * T] = out_of_band(g, rt + m * T) ? make_float2(0.0f, 0.0f) : v[m];
        }
        cluster_sync();
        // ---- column phase (whole columns of the unit's grid)
        if (half == 0) {
            if (k >= 0) {  // W = iF(P F(W))/nx: propagator p_y then p_x, 2/3 aperture
                float2 *buf = sm;
                float2 v[E];
#pragma unroll
                for (int m = 0; m < E; m++) v[m] = __ldcg(&Wu[(size_t)(ct + m * T) * N + col]);
                fft_line<N, false, LPC, 2, EV>(v, buf, cc, ct, g.tw_col16);
                const int2 ab = __ldg(&g.kband[col]);
                const float2 py = __ldg(&g.propy[col]);
#pragma unroll
                for (int m = 0; m < E; m++) {
                    const int ix = ct + m * T;
                    v[m] = (ix <= ab.x || ix >= ab.y) ? cmul(cmul(v[m], py), __ldg(&g.propx[ix]))
                                                      : make_float2(0.0f, 0.0f);
                }
                fft_line<N, true, LPC, 2, EV>(v, buf, cc, ct, g.tw_col16);
#pragma unroll
                for (int m = 0; m < E; m++) Wu[(size_t)(ct + m * T) * N + col] = v[m];
            }
        } else if (has_n) {  // B_{k+1} = iF(M F(A_{k+1})) / (nx ny^2)
            float2 *buf = sm + C::COL;
            float2 *tu = Tu[tb_next];
            float2 v[E];
#pragma unroll
            for (int m = 0; m < E; m++) v[m] = __ldcg(&tu[(size_t)(ct + m * T) * N + col]);
            fft_line<N, false, LPC, 2, EV>(v, buf, cc, ct, g.tw_col16);
            const int2 ab = __ldg(&g.kband[col]);
#pragma unroll
            for (int m = 0; m < E; m++) {
                const int ix = ct + m * T;
                v[m] = (ix <= ab.x || ix >= ab.y) ? cscale(v[m], mask_scale) : make_float2(0.0f, 0.0f);
            }
            fft_line<N, true, LPC, 2, EV>(v, buf, cc, ct, g.tw_col16);
#pragma unroll
            for (int m = 0; m < E; m++) tu[(size_t)(ct + m * T) * N + col] = v[m];
        }
        cluster_sync();
    }
}

}  // namespace msk
