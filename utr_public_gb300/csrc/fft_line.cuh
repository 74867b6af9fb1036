// fft_line.cuh -- shared-memory staged complex FFT of one line held across a
// group of threads (the building block of every row and column pass).
//
// Convention (the reference's cfpix, TemsimLibrary/cfpix.cpp:137-193):
//   forward  X[k] = sum_j x[j] exp(+2 pi i jk/N)     (cfpix::fft, FFTW_BACKWARD)
//   inverse  x[j] = sum_k X[k] exp(-2 pi i jk/N)     (cfpix::ifft before its 1/N)
// Both are unnormalised; callers fold 1/N into their pointwise multipliers.
//
// Work distribution: a line of N points is owned by T = N/E threads, E = 32
// (E = N below 32).  Thread t holds elements t + m*T, m = 0..E-1, in registers
// ("strided order") both before and after a transform, so a row pass loads and
// stores fully coalesced and a forward transform, a pointwise multiply and an
// inverse transform chain without any extra exchange.
//
// Algorithm: Stockham autosort.  Stage 1 is a radix-32 DFT in registers; the
// remaining stages (radix 2..32) read the line from shared memory, apply
// twiddles from a precomputed per-stage table and write back (or, for the
// last stage, keep the result in registers).  1024 = 32*32 needs a single
// shared-memory round trip per transform.
//
// Shared-memory layout of a line group: element idx of column c (of C lines
// interleaved column-fastest) lives at (idx + idx/32)*C + c.  The one-in-32
// padding makes the radix-32 scatter of stage 1 bank-conflict free; with C
// columns innermost, a half-warp of a column pass touches 128 contiguous bytes.
#pragma once

#include <cuda_runtime.h>

namespace msk {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmul_conj(float2 a, float2 b)  // a * conj(b)
{
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

__host__ __device__ constexpr int ilog2(int n)
{
    int b = 0;
    while ((1 << b) < n) b++;
    return b;
}
__host__ __device__ __forceinline__ constexpr int brev(int x, int bits)
{
    int r = 0;
    for (int i = 0; i < bits; i++) r |= ((x >> i) & 1) << (bits - 1 - i);
    return r;
}

// cos(pi k/16), k = 0..16, to 20 significant digits (exact mathematical values:
// cos(pi/16), cos(pi/8) = sqrt(2 + sqrt 2)/2, cos(3 pi/16), sqrt(1/2), ...).
__host__ __device__ constexpr double cos16(int k)
{
    constexpr double c[9] = {1.0,
                             0.98078528040323044913,
                             0.92387953251128675613,
                             0.83146961230254523708,
                             0.70710678118654752440,
                             0.55557023301960222474,
                             0.38268343236508977173,
                             0.19509032201612826785,
                             0.0};
    return k <= 8 ? c[k] : -c[16 - k];
}
__host__ __device__ constexpr double sin16(int k) { return k <= 8 ? cos16(8 - k) : cos16(k - 8); }
__host__ __device__ constexpr double dabs(double x) { return x < 0 ? -x : x; }

// The radix-2 butterfly (a, b) -> (a + w b, a - w b) with the twiddle
// w = exp(+-2 pi i K/32) = c + i s (K < 16 known at compile time) folded into
// fused multiply-adds (the tangent form of the FMA-optimised FFT, Linzer and
// Feig 1993 / Goedecker 1997): with |c| >= |s|, w b = c (b + i (s/c) b); else
// w b = s ((c/s) b + i b).  Two FMAs form the bracket and four apply the common
// factor with the sums: 6 operations against the 8 of a complex multiply
// followed by two complex additions.  K = 0 and K = 8 (w = +-i) take 4 adds.
template <int K, bool INV>
__host__ __device__ __forceinline__ void bfly(float2 &a, float2 &b)
{
    const float2 u = a;
    if constexpr (K == 0) {
        a = make_float2(u.x + b.x, u.y + b.y);
        b = make_float2(u.x - b.x, u.y - b.y);
    } else if constexpr (K == 8) {
        // w b = (-b.y, b.x) forward, (b.y, -b.x) inverse
        const float2 wb = INV ? make_float2(b.y, -b.x) : make_float2(-b.y, b.x);
        a = make_float2(u.x + wb.x, u.y + wb.y);
        b = make_float2(u.x - wb.x, u.y - wb.y);
    } else {
        constexpr double c = cos16(K), s = INV ? -sin16(K) : sin16(K);
        constexpr bool TAN = dabs(c) >= dabs(s);
        constexpr float r = (float)(TAN ? s / c : c / s);  // tan or cot of the angle
        constexpr float m = (float)(TAN ? c : s);
        float2 t;
        if constexpr (TAN) t = make_float2(fmaf(-r, b.y, b.x), fmaf(r, b.x, b.y));
        else t = make_float2(fmaf(r, b.x, -b.y), fmaf(r, b.y, b.x));
        a = make_float2(fmaf(m, t.x, u.x), fmaf(m, t.y, u.y));
        b = make_float2(fmaf(-m, t.x, u.x), fmaf(-m, t.y, u.y));
    }
}

// In-register DFT of R points v[0], v[S], ..., v[(R-1)*S], natural order in
// and out.  Radix-2 decimation in time, all indices compile-time.
template <int R, bool INV, int S, int LEN = 2>
__host__ __device__ __forceinline__ void dft_levels(float2 *a)
{
    if constexpr (LEN <= R) {
#pragma unroll
        for (int i = 0; i < R; i += LEN) {
#pragma unroll
            for (int j = 0; j < LEN / 2; j++) {
                // twiddle exp(+-2 pi i j/LEN) = exp(+-2 pi i K/32), K = j * 32/LEN
                float2 &x = a[i + j], &y = a[i + j + LEN / 2];
                switch (j * (32 / LEN)) {
#define MSK_BFCASE(K) case K: bfly<K, INV>(x, y); break;
                    MSK_BFCASE(0) MSK_BFCASE(1) MSK_BFCASE(2) MSK_BFCASE(3)
                    MSK_BFCASE(4) MSK_BFCASE(5) MSK_BFCASE(6) MSK_BFCASE(7)
                    MSK_BFCASE(8) MSK_BFCASE(9) MSK_BFCASE(10) MSK_BFCASE(11)
                    MSK_BFCASE(12) MSK_BFCASE(13) MSK_BFCASE(14) MSK_BFCASE(15)
#undef MSK_BFCASE
                    default: break;
                }
            }
        }
        dft_levels<R, INV, S, LEN * 2>(a);
    }
}

template <int R, bool INV, int S>
__host__ __device__ __forceinline__ void dft(float2 *v)
{
    static_assert(R >= 1 && R <= 32 && (R & (R - 1)) == 0, "radix");
    if constexpr (R == 1) return;
    float2 a[R];
    constexpr int B = ilog2(R);
#pragma unroll
    for (int i = 0; i < R; i++) a[brev(i, B)] = v[i * S];
    dft_levels<R, INV, S>(a);
#pragma unroll
    for (int i = 0; i < R; i++) v[i * S] = a[i];
}

// Radix plan per line length.  EV = 0: E = 32 elements per thread (the
// default plan of every pass: 1024 = 32 x 32, 2048 = 32 x 8 x 8, ...); EV = 16:
// 16 elements per thread and twice the threads per line (lines up to 2048
// points: 256 = 16 x 16, 1024 = 16 x 8 x 8, 2048 = 16 x 16 x 8), for passes
// that need more threads per line and fewer registers per thread.
template <int N, int EV = 0>
struct FftPlan {
    static_assert(N >= 16 && N <= 4096 && (N & (N - 1)) == 0, "line length");
    static_assert(EV == 0 || (EV == 16 && N >= 16 && N <= 2048), "plan variant");
    static constexpr int E = EV ? (N >= EV ? EV : N) : (N >= 32 ? 32 : N);  // elements per thread
    static constexpr int T = N / E;              // threads per line
    static constexpr int REST = N / E;
    // stages after the first: REST <= E -> one stage of radix REST; else two,
    // the last of radix 8
    static constexpr int S = (REST == 1) ? 1 : (REST <= E ? 2 : 3);
    static constexpr int R2 = (S >= 2) ? (REST <= E ? REST : REST / 8) : 1;
    static constexpr int R3 = (S == 3) ? REST / R2 : 1;
    static_assert(R2 <= E && R3 <= E, "stage radix within a thread's elements");
    static constexpr int NS2 = E;          // sub-transform size entering stage 2
    static constexpr int NS3 = E * R2;     // entering stage 3
    // per-stage twiddle tables tw[r*Ns + j], r < R, j < Ns
    static constexpr int TW2 = (S >= 2) ? NS2 * R2 : 0;
    static constexpr int TW3 = (S == 3) ? NS3 * R3 : 0;
    static constexpr int TWN = TW2 + TW3;
    // shared memory: one padding element every PER (conflict-free exchanges;
    // 32 for the default plan, E for the others)
    static constexpr int PER = EV ? E : 32;
    static constexpr int PADN = N + N / PER;
};

// Padded shared-memory index of line element idx.
template <int N, int EV = 0>
__device__ __forceinline__ int pidx(int idx)
{
    constexpr int PER = FftPlan<N, EV>::PER;
    return idx + idx / PER;
}

// Barrier among the threads that share a line group: SYNC 0 the warp (lines of
// <= 32 threads), 1 the CTA, 2 the half of the CTA the thread is in (named
// barriers 1 and 2, for CTAs whose halves run different passes).
template <int SYNC>
__device__ __forceinline__ void group_sync()
{
    if constexpr (SYNC == 1) {
        __syncthreads();
    } else if constexpr (SYNC == 2) {
        const unsigned h = blockDim.x >> 1;
        asm volatile("bar.sync %0, %1;" ::"r"(1u + (threadIdx.x >= h ? 1u : 0u)), "r"(h) : "memory");
    } else {
        __syncwarp();
    }
}

// Stage twiddles are fetched in groups of kTwG 16-byte loads (two twiddles
// each), one group ahead of the multiplies that use it: the first group of
// stage 2 is requested before stage 1's register DFT, and every later group
// while the previous one is being applied, so the L1 latency of a load hides
// behind arithmetic instead of stalling the warp.
constexpr int kTwG = 4;

template <int N, int R, int NS, int EV = 0>
struct StageTw {
    static constexpr int E = FftPlan<N, EV>::E, T = FftPlan<N, EV>::T, KB = E / R;
    static constexpr int NP = R / 2;                    // twiddle pairs per sub-transform
    static constexpr int GPK = (NP + kTwG - 1) / kTwG;  // load groups per sub-transform
    static constexpr int NG = KB * GPK;                 // load groups in the stage
};

// Group gi (compile-time once unrolled) of a stage's twiddles into w.
template <int N, int R, int NS, int EV = 0>
__device__ __forceinline__ void tw_fetch(float4 (&w)[kTwG], const float2 *tw, int t, int gi)
{
    using S = StageTw<N, R, NS, EV>;
    const int k = gi / S::GPK, p0 = (gi % S::GPK) * kTwG;
    const int j = (t + k * S::T) % NS;
    const float4 *tw4 = reinterpret_cast<const float4 *>(tw);
#pragma unroll
    for (int q = 0; q < kTwG; q++)
        if (p0 + q < S::NP) w[q] = __ldg(&tw4[(p0 + q) * NS + j]);
}

// One middle/last Stockham stage.  Reads the line from shared memory into
// registers (all reads before any write), twiddles, radix-R DFT; a middle
// stage writes back, the last stage leaves the result in strided order.
// `pre` holds the stage's first twiddle group, fetched by the caller.
template <int N, int R, int NS, bool LAST, bool INV, int C, int BLOCK, int EV = 0>
__device__ __forceinline__ void fft_stage(float2 (&v)[FftPlan<N, EV>::E], float2 *buf, int c,
                                          int t, const float2 *tw, const float4 (&pre)[kTwG])
{
    using S = StageTw<N, R, NS, EV>;
    constexpr int E = FftPlan<N, EV>::E, T = FftPlan<N, EV>::T, KB = E / R;
#pragma unroll
    for (int k = 0; k < KB; k++) {
        const int b = t + k * T;
#pragma unroll
        for (int r = 0; r < R; r++) v[k + r * KB] = buf[pidx<N, EV>(b + r * (N / R)) * C + c];
    }
    if constexpr (!LAST) group_sync<BLOCK>();
    float4 cur[kTwG], nxt[kTwG];
#pragma unroll
    for (int q = 0; q < kTwG; q++) cur[q] = pre[q];
#pragma unroll
    for (int gi = 0; gi < S::NG; gi++) {
        if (gi + 1 < S::NG) tw_fetch<N, R, NS, EV>(nxt, tw, t, gi + 1);
        const int k = gi / S::GPK, p0 = (gi % S::GPK) * kTwG;
#pragma unroll
        for (int q = 0; q < kTwG; q++) {
            const int p = p0 + q;
            if (p < S::NP) {
                const int r1 = 2 * p + 1, r2 = 2 * p + 2;
                const float2 w = make_float2(cur[q].x, cur[q].y), w_ = make_float2(cur[q].z, cur[q].w);
                v[k + r1 * KB] = INV ? cmul_conj(v[k + r1 * KB], w) : cmul(v[k + r1 * KB], w);
                if (r2 < R)
                    v[k + r2 * KB] = INV ? cmul_conj(v[k + r2 * KB], w_) : cmul(v[k + r2 * KB], w_);
            }
        }
        if (gi % S::GPK == S::GPK - 1) dft<R, INV, KB>(&v[k]);
        // keeps the compiler from hoisting later groups' loads (4 registers each)
        asm volatile("" ::: "memory");
#pragma unroll
        for (int q = 0; q < kTwG; q++) cur[q] = nxt[q];
    }
    if constexpr (!LAST) {
#pragma unroll
        for (int k = 0; k < KB; k++) {
            const int b = t + k * T;
            const int j = b % NS;
            const int o = (b / NS) * NS * R + j;
#pragma unroll
            for (int r = 0; r < R; r++) buf[pidx<N, EV>(o + r * NS) * C + c] = v[k + r * KB];
        }
        group_sync<BLOCK>();
    }
}

// Full transform of one line: strided order in, strided order out.
//   buf: the line group's shared buffer (C interleaved lines, padded)
//   c:   this thread's line within the group; t: index within the line
//   tw:  FftPlan<N>::TWN twiddles in global memory (stage 2 table, then
//        stage 3 table; each in pairs, see the host's twiddle tables), read
//        through the L1 cache; 16-byte aligned
//   BLOCK: the group barrier (group_sync's SYNC)
// Every thread of the group must call it (it contains group barriers).
template <int N, bool INV, int C, int BLOCK, int EV = 0>
__device__ __forceinline__ void fft_line(float2 (&v)[FftPlan<N, EV>::E], float2 *buf, int c, int t,
                                         const float2 *tw)
{
    using P = FftPlan<N, EV>;
    constexpr int E = P::E;
    float4 pre2[kTwG];
    if constexpr (P::S >= 2) tw_fetch<N, P::R2, P::NS2, EV>(pre2, tw, t, 0);
    dft<E, INV, 1>(v);
    if constexpr (P::S >= 2) {
        group_sync<BLOCK>();  // earlier readers of buf are done
#pragma unroll
        for (int r = 0; r < E; r++) buf[pidx<N, EV>(t * E + r) * C + c] = v[r];
        group_sync<BLOCK>();
        if constexpr (P::S == 2) {
            fft_stage<N, P::R2, P::NS2, true, INV, C, BLOCK, EV>(v, buf, c, t, tw, pre2);
        } else {
            float4 pre3[kTwG];
            tw_fetch<N, P::R3, P::NS3, EV>(pre3, tw + P::TW2, t, 0);
            fft_stage<N, P::R2, P::NS2, false, INV, C, BLOCK, EV>(v, buf, c, t, tw, pre2);
            fft_stage<N, P::R3, P::NS3, true, INV, C, BLOCK, EV>(v, buf, c, t, tw + P::TW2, pre3);
        }
    }
}

}  // namespace msk
