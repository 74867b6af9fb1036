/*
 * fft_cpu.h -- CPU complex FFTs used only by the test oracle.
 *
 * TEST INFRASTRUCTURE ONLY: nothing in the shipped library links this file.
 *
 * Definition (the one FFTW documents for fftw_plan_dft_2d): for a row-major
 * n0 x n1 array a[i0*n1 + i1],
 *     A[k0,k1] = sum_{i0,i1} a[i0,i1] * exp(sign * 2*pi*i*(i0*k0/n0 + i1*k1/n1))
 * unnormalised, sign = -1 or +1.  Power-of-two lengths use an iterative
 * radix-2 Cooley-Tukey transform with twiddles computed in double precision;
 * any other length falls back to a direct O(n^2) sum accumulated in double.
 */
#ifndef ORACLE_FFT_CPU_H
#define ORACLE_FFT_CPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* In-place 2D transform of interleaved complex data (re,im pairs). */
void ocfft2d_f(float *data, int n0, int n1, int sign);
void ocfft2d_d(double *data, int n0, int n1, int sign);

/* In-place 1D transform of `howmany` lines; element j of line l is at
 * data[2*(l*dist + j*stride)]. */
void ocfft1d_many_f(float *data, int n, int howmany, int stride, int dist, int sign);
void ocfft1d_many_d(double *data, int n, int howmany, int stride, int dist, int sign);

#ifdef __cplusplus
}
#endif

#endif
