/*
 * utr_oracle.h -- CPU restatement of UTR.exe's reconstruction core
 * (MultisliceCppTest/PhaseRetrieval/UTR.cpp, UTR.h).
 *
 * TEST INFRASTRUCTURE ONLY: what the GPU reconstruction in libmsk.so is
 * compared with; nothing in the shipped library links this file.
 *
 * Layouts as in msk_utr.h: images [ny][nx], volumes [nz][ny][nx] (x
 * fastest), complex data interleaved, Fourier volumes centred.
 */
#ifndef UTR_ORACLE_H
#define UTR_ORACLE_H

#include "msk_utr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Quantities UTR.cpp derives from its parameters (UTR.cpp:208-372, 388). */
typedef struct {
    int nx, ny, nz;
    double xst, xlo, xhi, ylo, yhi, zlo, zhi;
    double fxst, fyst, fzst, fxlo, fylo, fzlo;
    double xc, yc, zc;
    long ic, jc, kc;
    double wl, ee, k2maxo, cs3, cs5;  /* cs in length units */
    double zout_aver;
    int rot_y_only, rot_z_only, rot_z2_only;
} mo_utr_geom;

int mo_utr_geom_make(const msk_utr *p, int nangles, const double *angles, const double *defocus,
                     mo_utr_geom *g);

/* Input normalisation, threshold, log and centred forward 2D FFT of one
 * image (UTR.cpp:940-996): k2 complex [ny][nx].  _f32 mirrors the float
 * steps up to the log (the FFT in double, then rounded to float); _f64 is
 * double throughout. */
void mo_utr_k2four_f32(const float *img, int nx, int ny, double f1, double f2, float *k2);
void mo_utr_k2four_f64(const float *img, int nx, int ny, double f1, double f2, double *k2);

/* CT_3Dgridding (UTR.h:199-307) of one image: float coordinates, weights
 * and products exactly as the reference; _f32 accumulates in float in the
 * reference's pixel order (bit for bit the reference template), _acc64 adds
 * the same float products into double sums, _f64 takes a double spectrum
 * and a double phase factor.  fc = {Fxc, Fyc, Fzc} (re, im pairs). */
void mo_utr_grid_f32(const float *k2four, int nx, int ny, int nz, double angleY, double angleZ,
                     float fxlo, float fxst, float fylo, float fyst, float fzlo, float fzst,
                     const float *fc, double wl, int rotshift, int escc, float *v3, float *samp3);
void mo_utr_grid_acc64(const float *k2four, int nx, int ny, int nz, double angleY,
                       double angleZ, float fxlo, float fxst, float fylo, float fyst, float fzlo,
                       float fzst, const float *fc, double wl, int rotshift, int escc,
                       double *v3, double *samp3);
void mo_utr_grid_f64(const double *k2four, int nx, int ny, int nz, double angleY,
                     double angleZ, float fxlo, float fxst, float fylo, float fyst, float fzlo,
                     float fzst, const double *fcd, double wl, int rotshift, int escc,
                     double *v3, double *samp3);

/* CTFcorrection3D (UTR.h:15-123) and InverseMLaplacian3D (UTR.h:126-175)
 * on a float volume (bit for bit the reference templates) and on a double
 * one.  Return 0, or -1 where the reference throws. */
int mo_utr_ctf3d_f32(float *v3, int nx, int ny, int nz, double wl, double zlo, double zhi,
                     double ylo, double yhi, double xlo, double xhi, double defocdist,
                     double q2max, double cs3, double cs5, double sigma, double epsilon,
                     int escc);
int mo_utr_ctf3d_f64(double *v3, int nx, int ny, int nz, double wl, double zlo, double zhi,
                     double ylo, double yhi, double xlo, double xhi, double defocdist,
                     double q2max, double cs3, double cs5, double sigma, double epsilon,
                     int escc);
int mo_utr_invlap3d_f32(float *v3, int nx, int ny, int nz, double zaper, double yaper,
                        double xaper, double alpha, double norm);
int mo_utr_invlap3d_f64(double *v3, int nx, int ny, int nz, double zaper, double yaper,
                        double xaper, double alpha, double norm);

/* The whole reconstruction in double (UTR.cpp:862-1282): the spectra, the
 * gridding with double sums, the sampling normalisation and SNR filter, the
 * 3D correction, the Hermitian symmetrisation in the reference's loop order,
 * an FFTW-style complex-to-real inverse 3D FFT of the half spectrum, the
 * sphere mask and the output scale.  volume: double [nz][ny][nx].
 * nthreads: host threads for the gridding (its sums are per-thread partial
 * volumes added in thread order, so the result does not depend on timing).
 * zrot, shifts (may be NULL): the Z'' rotation (degrees) and the x, y shift
 * of each image, undone before its spectrum (UTR.cpp:920-940). */
int mo_utr_reconstruct_f64(const msk_utr *p, int nangles, const double *angles,
                           const double *defocus, const double *zrot, const double *shifts,
                           const float *images, double *volume, int nthreads);

/* UTR.cpp:920-940 on a normalised image [ny][nx] (definitions in the
 * utr_oracle.c header): zrot (degrees, may be NULL) and shifts ([n][2] x, y,
 * may be NULL) in mo_utr_reconstruct_f64 select it per image. */
void mo_utr_image_plane_f64(double *img, int nx, int ny, double cx, double cy, double t,
                            long dx, long dy);

/* Only the Fourier-space and output stages of mo_utr_reconstruct_f64, from
 * gridded sums: v3 complex, samp3 [nz][ny][nx] (v3 is overwritten). */
int mo_utr_finish_f64(const msk_utr *p, int nangles, const double *angles,
                      const double *defocus, double *v3, const double *samp3, double *volume);

#ifdef __cplusplus
}
#endif

#endif
