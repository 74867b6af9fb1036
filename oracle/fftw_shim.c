/*
 * fftw_shim.c -- the few FFTW 3 single-precision entry points that the
 * reference's cfpix class calls (TemsimLibrary/cfpix.cpp:110,140,157,172,
 * 225-236,252,259,448,451), implemented on the oracle's own CPU FFT.
 *
 * TEST INFRASTRUCTURE ONLY: it exists so that the reference's autoslic.cpp,
 * slicelib.cpp and cfpix.cpp can be compiled unmodified into oracle/_ref.
 * FFTW itself is not installed; its semantics are taken from its public
 * interface: fftwf_plan_dft_2d(n0, n1, in, out, sign, flags) is a row-major
 * n0 x n1 unnormalised transform with kernel exp(sign*2*pi*i*...), and
 * fftwf_execute_dft may be given new arrays of the planned size.
 * Compiled against the reference's own fftw3.h header (-I in place).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"
#include "fft_cpu.h"

struct fftwf_plan_s {
    int n0, n1, sign, c2r;
    fftwf_complex *in, *out;
};

fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out,
                             int sign, unsigned flags)
{
    (void)flags;
    fftwf_plan p = (fftwf_plan)calloc(1, sizeof(*p));
    p->n0 = n0;
    p->n1 = n1;
    p->sign = sign;
    p->in = in;
    p->out = out;
    return p;
}

fftwf_plan fftwf_plan_dft_c2r_2d(int n0, int n1, fftwf_complex *in, float *out, unsigned flags)
{
    (void)flags;
    (void)out;
    fftwf_plan p = (fftwf_plan)calloc(1, sizeof(*p));
    p->n0 = n0;
    p->n1 = n1;
    p->c2r = 1;
    p->in = in;
    return p;
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out)
{
    if (p->c2r) {
        fprintf(stderr, "fftw_shim: complex-to-real transforms are not provided\n");
        abort();
    }
    if (in != out) memcpy(out, in, sizeof(fftwf_complex) * (size_t)p->n0 * (size_t)p->n1);
    ocfft2d_f((float *)out, p->n0, p->n1, p->sign);
}

void fftwf_execute(const fftwf_plan p) { fftwf_execute_dft(p, p->in, p->out); }

void fftwf_destroy_plan(fftwf_plan p) { free(p); }

void *fftwf_malloc(size_t n)
{
    void *ptr = NULL;
    if (posix_memalign(&ptr, 64, n ? n : 64) != 0) return NULL;
    return ptr;
}

void fftwf_free(void *p) { free(p); }
