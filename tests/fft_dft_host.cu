// fft_dft_host.cu -- runs the line FFT's in-register DFT (dft<R, INV, 1> of
// utr_public_gb300/csrc/fft_line.cuh, compiled for the host) on the inputs in
// argv[1] and writes the results to argv[2].  TEST ONLY: lets the CPU tests
// check the butterfly arithmetic against numpy without a GPU.
//
// Input: float32 (re, im) pairs, 62 blocks: for R = 2, 4, 8, 16, 32 and
// INV = 0, 1 in that order, one block of R points each ... repeated
// `reps` times (argv[3]).  Output: the same layout, transformed.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fft_line.cuh"

template <int R, bool INV>
static void run(float2 *v)
{
    msk::dft<R, INV, 1>(v);
}

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    const int reps = atoi(argv[3]);
    const size_t per = 2 * (2 + 4 + 8 + 16 + 32);
    std::vector<float2> buf(per * reps);
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(buf.data(), sizeof(float2), buf.size(), f) != buf.size()) return 3;
    fclose(f);
    float2 *p = buf.data();
    for (int k = 0; k < reps; k++) {
        run<2, false>(p); p += 2;   run<2, true>(p); p += 2;
        run<4, false>(p); p += 4;   run<4, true>(p); p += 4;
        run<8, false>(p); p += 8;   run<8, true>(p); p += 8;
        run<16, false>(p); p += 16; run<16, true>(p); p += 16;
        run<32, false>(p); p += 32; run<32, true>(p); p += 32;
    }
    f = fopen(argv[2], "wb");
    if (!f || fwrite(buf.data(), sizeof(float2), buf.size(), f) != buf.size()) return 4;
    fclose(f);
    return 0;
}
