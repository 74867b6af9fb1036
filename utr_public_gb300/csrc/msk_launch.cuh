// msk_launch.cuh -- host launchers for the passes of one line length N.
// Each msk_size_<N>.cu instantiates SizeOps for its N; the dispatcher picks
// row passes by ny and column passes by nx.
#pragma once

#include <mutex>

#include "msk_passes.cuh"
#include "msk_small.cuh"
#include "msk_types.h"

namespace msk {

// A column pass's view of a wave buffer: the TMA map (its box as wide as the
// pass's column tile) and the tile variant it was encoded for.
struct ColView {
    CUtensorMap map;
    int v;
};

struct SizeOps {
    int n;
    int col_c[kColVariants], col_box_rows;  // column tile widths per variant, TMA box height
    int col_nv;                             // variants with kernels (2, or 4 with the 16-point plan)
    int row_nv;                             // transmit schedules with kernels (2, or 3: TrCfg)
    void (*splat)(const Geom &, const int *units, int nunits, int slice, int nsl1,
                  const int *slice_off, const SplatAtom *atoms, float2 *tbuf, cudaStream_t);
    // the same splat writing the projected potential of the slice (float) to
    // vout + u * vstride instead of its transmission
    void (*splat_potential)(const Geom &, const int *units, int nunits, int slice, int nsl1,
                            const int *slice_off, const SplatAtom *atoms, float *vout,
                            size_t vstride, cudaStream_t);
    // Debye-Waller branch: S(v) to `spec`, the damping column pass on it
    // (in place), then A = S(exp(i sigma v')) into `tbuf`
    void (*splat_spec)(const Geom &, const int *units, int nunits, int slice, int nsl1,
                       const int *slice_off, const SplatAtom *atoms, float2 *spec, cudaStream_t);
    void (*col_dw)(const Geom &, const ColView &spec, const int *units, int nunits,
                   const float *dw, int dw_stride, cudaStream_t);
    void (*row_dwexp)(const Geom &, const int *units, int nunits, const float2 *spec,
                      float2 *tbuf, cudaStream_t);
    // band != 0: only the in-band column blocks (Geom::cb_*); the others must
    // be zero in the input and stay zero in the output buffer.  col_mask scales
    // its output by post / nx (post: a power of two the next pass would apply)
    void (*col_mask)(const Geom &, const ColView &in, const ColView &out,
                     const int *units, int nunits, int band, float post, cudaStream_t);
    void (*col_prop)(const Geom &, const ColView &in, const ColView &out,
                     const int *units, int nunits, int band, cudaStream_t);
    void (*col_fresnel)(const Geom &, const ColView &in, const ColView &out,
                        const int *units, int nunits, const Fresnel &, float scale, cudaStream_t);
    // band != 0: only the in-band row segments are loaded and stored (B and
    // W must be zero out of band, and `out` too; a propagator pass follows).
    // rv: the schedule (0 .. row_nv-1, as TrCfg numbers them)
    void (*row_transmit)(const Geom &, const int *units, int nunits, const float2 *tbuf,
                         const float2 *psi, float2 *out, float out_scale, int band, int rv,
                         cudaStream_t);
    // the same in the scattered form (phi, tau; the potential-stack path)
    void (*row_transmit_scat)(const Geom &, const int *units, int nunits, const float2 *tbuf,
                              const float2 *psi, float2 *out, float out_scale, int band, int rv,
                              cudaStream_t);
    void (*row_init)(const Geom &, const int *units, int nunits, const float2 *wave0,
                     float2 *psi, float scale, cudaStream_t);
    void (*row_exit)(const Geom &, const int *units, int nunits, const float2 *psi,
                     float2 *out, cudaStream_t);
    // out = iS(in) * scale (the real-space wave of a W-state, unnormalised)
    void (*row_inverse)(const Geom &, const int *units, int nunits, const float2 *in,
                        float2 *out, float scale, cudaStream_t);
    void (*row_intensity)(const Geom &, int nimg, const int *img_off, const int *img_units,
                          const int *img_dst, const int *img_flags, const float2 *ebuf,
                          float *images, float nconf, cudaStream_t);
    // potential stacks and the adjoint (row length n), all in the scattered form
    void (*row_intensity_scat)(const Geom &, int nimg, const int *img_off, const int *img_units,
                               const int *img_dst, const int *img_flags, const float2 *ebuf,
                               float *images, float nconf, cudaStream_t);
    void (*row_expv)(const Geom &, int nunits, const float *v, size_t ustride, float2 *out,
                     cudaStream_t);
    void (*row_adj_transmit)(const Geom &, int nunits, float2 *Gu, float2 *B, const float2 *Wp,
                             cudaStream_t);
    void (*row_grad)(const Geom &, int nunits, const float2 *Ge, const float *v, size_t ustride,
                     float *grad, cudaStream_t);
    // returns the number of loss partials written
    int (*row_imgrad)(const Geom &, int nunits, const float2 *E, const float *target,
                      size_t tstride, float2 *G, double *partial, cudaStream_t);
    // square grids of N <= 256: every slice of every unit in one cluster launch
    // (msk_small.cuh); W holds S(psi) on entry and exit, T0 / T1 scratch of the
    // same size.  small_ok: how many of its clusters the device runs at once
    // (0: none fit).  Both null for other sizes.
    cudaError_t (*small_slices)(const Geom &, int nunits, int nslices, int nsl1,
                                const int *slice_off, const SplatAtom *atoms, float2 *W,
                                float2 *T0, float2 *T1, cudaStream_t);
    int (*small_ok)(int device);  // clusters of this size active at once (0: none fit)
};

// Line lengths with kernels: 16 .. 4096, powers of two.
const SizeOps *size_ops(int n);

template <int N> struct Smem {
    using P = FftPlan<N>;
    static constexpr int NTS = RowCfg<N>::L * P::T;
    static constexpr size_t splat = (size_t)RowCfg<N>::L * SplatCfg<N>::SROW * 8 + NTS * 16 +
                                    kKnotWords * 4 + ((NTS + 31) / 32 + 1) * 4;
    template <int V, int EV = 0>
    static constexpr size_t col() { return (size_t)ColCfg<N, V, EV>::C * FftPlan<N, EV>::PADN * 8 + 16; }
    template <int EV = 0, int W = 128>
    static constexpr size_t transmit()
    {
        return (size_t)2 * TrCfg<N, EV, W>::LT * FftPlan<N, EV>::PADN * 8 + 16;
    }
    static constexpr size_t row = (size_t)RowCfg<N>::L * P::PADN * 8;
    static constexpr size_t adj = (size_t)RowCfg<N>::LT * (P::PADN + N) * 8;
    static constexpr size_t imgrad = row + (size_t)RowCfg<N>::L * P::T * 8;
};

template <typename K>
inline void set_smem(K kernel, size_t bytes, std::once_flag &flag)
{
    std::call_once(flag, [&] {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        // the default carve-out leaves ~100 KB of shared memory per SM, one
        // CTA of the larger passes; ask for the whole 228 KB
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    });
}

template <int N>
struct Launch {
    using P = FftPlan<N>;
    static int row_blocks(const Geom &g, int L) { return (g.nx + L - 1) / L; }

    static void splat(const Geom &g, const int *units, int nunits, int slice, int nsl1,
                      const int *slice_off, const SplatAtom *atoms, float2 *tbuf, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_splat<N, kSplatTrans>, Smem<N>::splat, f);
        const int L = RowCfg<N>::L;
        k_row_splat<N, kSplatTrans><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::splat, s>>>(
            g, units, slice, nsl1, slice_off, atoms, tbuf, nullptr, 0);
    }
    static void splat_potential(const Geom &g, const int *units, int nunits, int slice, int nsl1,
                                const int *slice_off, const SplatAtom *atoms, float *vout,
                                size_t vstride, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_splat<N, kSplatPot>, Smem<N>::splat, f);
        const int L = RowCfg<N>::L;
        k_row_splat<N, kSplatPot><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::splat, s>>>(
            g, units, slice, nsl1, slice_off, atoms, nullptr, vout, vstride);
    }
    static void splat_spec(const Geom &g, const int *units, int nunits, int slice, int nsl1,
                           const int *slice_off, const SplatAtom *atoms, float2 *spec,
                           cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_splat<N, kSplatSpec>, Smem<N>::splat, f);
        const int L = RowCfg<N>::L;
        k_row_splat<N, kSplatSpec><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::splat, s>>>(
            g, units, slice, nsl1, slice_off, atoms, spec, nullptr, 0);
    }
    static void row_dwexp(const Geom &g, const int *units, int nunits, const float2 *spec,
                          float2 *tbuf, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_dwexp<N>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_row_dwexp<N><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::row, s>>>(g, units, spec,
                                                                                tbuf);
    }
    template <int MODE, int V, int EV>
    static void colv(const Geom &g, const CUtensorMap &in, const CUtensorMap &out,
                     const int *units, int nunits, const Fresnel &fr, float scale, int band,
                     cudaStream_t s)
    {
        if (EV && !g.tw_col16) return;  // no table for the plan: nothing may run
        static std::once_flag f;
        constexpr size_t sm = Smem<N>::template col<V, EV>();
        set_smem(k_col_pass<N, MODE, V, EV>, sm, f);
        using CC = ColCfg<N, V, EV>;
        const int vi = V + (EV ? 2 : 0);
        const int bpu = band ? g.cb_n[vi] : g.ny / CC::C;
        k_col_pass<N, MODE, V, EV><<<nunits * bpu, CC::NT, sm, s>>>(g, in, out, units, fr, scale,
                                                                     band);
    }
    // in and out must be views of the same variant (the kernel's box)
    template <int MODE>
    static void col(const Geom &g, const ColView &in, const ColView &out, const int *units,
                    int nunits, const Fresnel &fr, float scale, int band, cudaStream_t s)
    {
        if (in.v != out.v) return;
        switch (in.v) {
        case 1: colv<MODE, 1, 0>(g, in.map, out.map, units, nunits, fr, scale, band, s); return;
        case 2:
        case 3:
            if constexpr (col_plan16_ok(N)) {
                if (in.v == 2) colv<MODE, 0, 16>(g, in.map, out.map, units, nunits, fr, scale, band, s);
                else colv<MODE, 1, 16>(g, in.map, out.map, units, nunits, fr, scale, band, s);
            }
            return;
        default: colv<MODE, 0, 0>(g, in.map, out.map, units, nunits, fr, scale, band, s); return;
        }
    }
    static void col_mask(const Geom &g, const ColView &in, const ColView &out,
                         const int *units, int nunits, int band, float post, cudaStream_t s)
    {
        col<kColMask>(g, in, out, units, nunits, Fresnel{}, post / (float)g.nx, band, s);
    }
    static void col_prop(const Geom &g, const ColView &in, const ColView &out,
                         const int *units, int nunits, int band, cudaStream_t s)
    {
        // the 1/nx of the column transforms is in the propx table
        col<kColProp>(g, in, out, units, nunits, Fresnel{}, 1.0f, band, s);
    }
    static void col_dw(const Geom &g, const ColView &spec, const int *units, int nunits,
                       const float *dw, int dw_stride, cudaStream_t s)
    {
        Fresnel fr{};
        fr.dw = dw;
        fr.dw_stride = dw_stride;
        col<kColDW>(g, spec, spec, units, nunits, fr, 1.0f / (float)g.nx, 0, s);
    }
    static void col_fresnel(const Geom &g, const ColView &in, const ColView &out,
                            const int *units, int nunits, const Fresnel &fr, float scale,
                            cudaStream_t s)
    {
        if (!fr.table) return;  // the pass multiplies by fr.table; nothing to run without it
        col<kColFresnel>(g, in, out, units, nunits, fr, scale, 0, s);
    }
    template <bool SCAT, int EV, int W>
    static void row_transmit_v(const Geom &g, const int *units, int nunits, const float2 *tbuf,
                               const float2 *psi, float2 *out, float out_scale, int band,
                               cudaStream_t s)
    {
        if (EV && !g.tw_row16) return;  // no 16-point twiddles bound: nothing to run
        static std::once_flag f;
        constexpr size_t sm = Smem<N>::template transmit<EV, W>();
        set_smem(k_row_transmit<N, SCAT, EV, W>, sm, f);
        constexpr int L = TrCfg<N, EV, W>::LT;
        k_row_transmit<N, SCAT, EV, W><<<nunits * row_blocks(g, L), L * TrCfg<N, EV, W>::T, sm, s>>>(
            g, units, tbuf, psi, out, out_scale, band);
    }
    template <bool SCAT>
    static void row_transmit_t(const Geom &g, const int *units, int nunits, const float2 *tbuf,
                               const float2 *psi, float2 *out, float out_scale, int band, int rv,
                               cudaStream_t s)
    {
        if constexpr (row_plan16_ok(N)) {
            if (rv == 2) {
                row_transmit_v<SCAT, 16, 128>(g, units, nunits, tbuf, psi, out, out_scale, band, s);
                return;
            }
        }
        if (rv == 1)
            row_transmit_v<SCAT, 0, 128>(g, units, nunits, tbuf, psi, out, out_scale, band, s);
        else
            row_transmit_v<SCAT, 0, 64>(g, units, nunits, tbuf, psi, out, out_scale, band, s);
    }
    static void row_init(const Geom &g, const int *units, int nunits, const float2 *wave0,
                         float2 *psi, float scale, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_simple<N, kRowInit>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_row_simple<N, kRowInit><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::row, s>>>(
            g, units, wave0, psi, scale);
    }
    static void row_inverse(const Geom &g, const int *units, int nunits, const float2 *in,
                            float2 *out, float scale, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_simple<N, kRowExit>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_row_simple<N, kRowExit><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::row, s>>>(
            g, units, in, out, scale);
    }
    static void row_exit(const Geom &g, const int *units, int nunits, const float2 *psi,
                         float2 *out, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_simple<N, kRowExit>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_row_simple<N, kRowExit><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::row, s>>>(
            g, units, psi, out, 1.0f / (float)g.ny);
    }
    template <bool SCAT>
    static void row_intensity_t(const Geom &g, int nimg, const int *img_off,
                                const int *img_units, const int *img_dst, const int *img_flags,
                                const float2 *ebuf, float *images, float nconf, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_intensity<N, SCAT>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_row_intensity<N, SCAT><<<nimg * row_blocks(g, L), L * P::T, Smem<N>::row, s>>>(
            g, img_off, img_units, img_dst, img_flags, ebuf, images, nconf);
    }

    static void row_expv(const Geom &g, int nunits, const float *v, size_t ustride, float2 *out,
                         cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_expv<N>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_row_expv<N><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::row, s>>>(g, v, ustride, out);
    }
    static void row_adj_transmit(const Geom &g, int nunits, float2 *Gu, float2 *B,
                                 const float2 *Wp, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_adj_transmit<N>, Smem<N>::adj, f);
        const int L = RowCfg<N>::LT;
        k_row_adj_transmit<N><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::adj, s>>>(g, Gu, B, Wp);
    }
    static void row_grad(const Geom &g, int nunits, const float2 *Ge, const float *v,
                         size_t ustride, float *grad, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_grad<N>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_row_grad<N><<<nunits * row_blocks(g, L), L * P::T, Smem<N>::row, s>>>(g, Ge, v, ustride,
                                                                               grad);
    }
    static int row_imgrad(const Geom &g, int nunits, const float2 *E, const float *target,
                          size_t tstride, float2 *G, double *partial, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_row_imgrad<N>, Smem<N>::imgrad, f);
        const int L = RowCfg<N>::L;
        const int nb = nunits * row_blocks(g, L);
        k_row_imgrad<N><<<nb, L * P::T, Smem<N>::imgrad, s>>>(g, E, target, tstride, G, partial);
        return nb;
    }

    static cudaLaunchConfig_t small_cfg(int nunits, cudaStream_t s, cudaLaunchAttribute *at)
    {
        using C = SmallCfg<N>;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(nunits * C::Q));
        cfg.blockDim = dim3(C::NT);
        cfg.dynamicSmemBytes = C::SMEM;
        cfg.stream = s;
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = C::Q;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cfg;
    }
    static void small_attrs()
    {
        static std::once_flag f;
        std::call_once(f, [] {
            using C = SmallCfg<N>;
            cudaFuncSetAttribute(k_small_slices<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)C::SMEM);
            if (C::Q > 8)
                cudaFuncSetAttribute(k_small_slices<N>,
                                     cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        });
    }
    static cudaError_t small_slices(const Geom &g, int nunits, int nslices, int nsl1,
                                    const int *slice_off, const SplatAtom *atoms, float2 *W,
                                    float2 *T0, float2 *T1, cudaStream_t s)
    {
        if constexpr (N >= 64 && N <= 256) {
            small_attrs();
            cudaLaunchAttribute at[1];
            cudaLaunchConfig_t cfg = small_cfg(nunits, s, at);
            return cudaLaunchKernelEx(&cfg, k_small_slices<N>, g, nslices, nsl1, slice_off, atoms,
                                      W, T0, T1);
        } else {
            return cudaErrorNotSupported;
        }
    }
    // clusters the device runs at once (cluster size and shared memory), 0 if none fit
    static int small_ok(int device)
    {
        if constexpr (N >= 64 && N <= 256) {
            static std::mutex m;
            static int known[64];  // -1 unknown
            static bool init = false;
            if (device < 0 || device >= 64) return 0;
            std::lock_guard<std::mutex> lk(m);
            if (!init) {
                for (int &k : known) k = -1;
                init = true;
            }
            if (known[device] < 0) {
                small_attrs();
                cudaLaunchAttribute at[1];
                cudaLaunchConfig_t cfg = small_cfg(1, nullptr, at);
                int n = 0;
                const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, k_small_slices<N>, &cfg);
                if (e != cudaSuccess) cudaGetLastError();
                known[device] = e == cudaSuccess ? n : 0;
            }
            return known[device];
        } else {
            (void)device;
            return 0;
        }
    }

    static const SizeOps *ops()
    {
        static const SizeOps o = {N,
                                  {ColCfg<N, 0>::C, ColCfg<N, 1>::C,
                                   col_plan16_ok(N) ? ColCfg<N, 0, col_plan16_ok(N) ? 16 : 0>::C : ColCfg<N, 0>::C,
                                   col_plan16_ok(N) ? ColCfg<N, 1, col_plan16_ok(N) ? 16 : 0>::C : ColCfg<N, 1>::C},
                                  ColCfg<N>::BR, col_plan16_ok(N) ? kColVariants : 2,
                                  row_plan16_ok(N) ? kRowVariants : 2, splat,
                                  splat_potential, splat_spec, col_dw, row_dwexp,
                                  col_mask, col_prop,     col_fresnel,      row_transmit_t<false>,
                                  row_transmit_t<true>,   row_init, row_exit, row_inverse,
                                  row_intensity_t<false>, row_intensity_t<true>, row_expv,
                                  row_adj_transmit,       row_grad,         row_imgrad,
                                  (N >= 64 && N <= 256) ? small_slices : nullptr,
                                  (N >= 64 && N <= 256) ? small_ok : nullptr};
        return &o;
    }
};

}  // namespace msk

#define MSK_INSTANTIATE_SIZE(N) \
    namespace msk { const SizeOps *size_ops_##N() { return Launch<N>::ops(); } }
