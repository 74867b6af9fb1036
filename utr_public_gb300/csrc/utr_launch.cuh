// utr_launch.cuh -- host launchers of the UTR line passes for one line
// length N (instantiated with the multislice passes in msk_size_<N>.cu).
#pragma once

#include <mutex>

#include "msk_launch.cuh"
#include "utr_passes.cuh"

namespace msk {

struct UtrOps {
    int n;
    int col_c, col_box_rows;  // column tile width and TMA box height (UtrColCfg)
    int col_c_final;          // the final z pass's tile width (UtrColCfg<n, true>)
    // rows of images (x lines of length n)
    void (*img_rows)(const UtrImg &, const float *img, float2 *k2, cudaStream_t);
    // rows of the volume (x lines of length n): gridding sums -> inverse FFT
    void (*fourier_rows)(const UtrFourier &, const float2 *tw, const UtrAcc *acc, float2 *vol,
                         int nrows, cudaStream_t);
    // column passes over lines of length n (units x width columns of a 2D view)
    void (*col_img)(const UtrCol &, const CUtensorMap &in, const CUtensorMap &out, int units,
                    cudaStream_t);
    void (*col_vol)(const UtrCol &, const CUtensorMap &in, const CUtensorMap &out, int units,
                    cudaStream_t);
    void (*col_final)(const UtrCol &, const CUtensorMap &in, int units, cudaStream_t);
};

const UtrOps *utr_ops(int n);

template <int N> struct UtrLaunch {
    using P = FftPlan<N>;
    static void img_rows(const UtrImg &p, const float *img, float2 *k2, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_utr_img_rows<N>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_utr_img_rows<N><<<(p.nrows + L - 1) / L, L * P::T, Smem<N>::row, s>>>(p, img, k2);
    }
    static void fourier_rows(const UtrFourier &fr, const float2 *tw, const UtrAcc *acc,
                             float2 *vol, int nrows, cudaStream_t s)
    {
        static std::once_flag f;
        set_smem(k_utr_fourier_rows<N>, Smem<N>::row, f);
        const int L = RowCfg<N>::L;
        k_utr_fourier_rows<N><<<(nrows + L - 1) / L, L * P::T, Smem<N>::row, s>>>(fr, tw, acc, vol);
    }
    template <int MODE>
    static void col(const UtrCol &p, const CUtensorMap &in, const CUtensorMap &out, int units,
                    cudaStream_t s)
    {
        static std::once_flag f;
        using CC = UtrColCfg<N, MODE == kUtrColFinal>;
        set_smem(k_utr_col<N, MODE>, CC::SMEM, f);
        const int bpu = p.ncb > 0 ? p.ncb : p.width / CC::C;
        k_utr_col<N, MODE><<<units * bpu, CC::NT, CC::SMEM, s>>>(p, in, out);
    }
    static void col_img(const UtrCol &p, const CUtensorMap &in, const CUtensorMap &out, int units,
                        cudaStream_t s)
    {
        col<kUtrColImg>(p, in, out, units, s);
    }
    static void col_vol(const UtrCol &p, const CUtensorMap &in, const CUtensorMap &out, int units,
                        cudaStream_t s)
    {
        col<kUtrColVol>(p, in, out, units, s);
    }
    static void col_final(const UtrCol &p, const CUtensorMap &in, int units, cudaStream_t s)
    {
        col<kUtrColFinal>(p, in, in, units, s);
    }
    static const UtrOps *ops()
    {
        static const UtrOps o = {N,       UtrColCfg<N>::C, UtrColCfg<N>::BR, UtrColCfg<N, true>::C,
                                 img_rows,
                                 fourier_rows, col_img, col_vol, col_final};
        return &o;
    }
};

}  // namespace msk

#define UTR_INSTANTIATE_SIZE(N) \
    namespace msk { const UtrOps *utr_ops_##N() { return UtrLaunch<N>::ops(); } }
