/*
 * msk_utr.h -- C ABI of the GB300 UTR reconstruction in libmsk.so.
 *
 * Drop-in for the numerical core of timg021/UTR_public's UTR.exe
 * (MultisliceCppTest/PhaseRetrieval/UTR.cpp, UTR.h): the unified tomographic
 * reconstruction of a 3D potential from one defocused image per orientation
 * -- log of the flat-field corrected image, its centred 2D FFT, trilinear
 * gridding of every image onto its (Ewald) plane in 3D Fourier space, the
 * sampling normalisation with the SNR filter, the 3D TIE-Hom or CTF
 * correction, an inverse 3D FFT, the reconstruction-sphere mask and the
 * output scaling.  Parameter files, image files, symmetry averaging, volume
 * rotation, peak search and 16-bit output stay with the caller.
 *
 * Conventions:
 *   - images are float [nangles][ny][nx], x fastest (the layout UTR.exe reads
 *     from its GRD / TIFF files, UTR.cpp:915-917);
 *   - volumes are [nz][ny][nx], x fastest (XArray3D, UTR.cpp:864-867),
 *     complex ones interleaved (re, im), Fourier-space ones centred ("non
 *     wrapped": index i is frequency (i - nx/2) / (nx * xst));
 *   - every pointer may be host or device memory;
 *   - nx, ny and the volume depth nz: powers of two from 16 to 4096;
 *   - status codes and the context are those of msk.h.
 * zlo = zhi = 0 with modality 1 selects the ".xri" default z range [xlo, xhi].
 */
#ifndef MSK_UTR_H
#define MSK_UTR_H

#include "msk.h"

#ifdef __cplusplus
extern "C" {
#endif

/* UTR.exe's input parameters the reconstruction reads (ReadmeUTR.txt; the
 * ".txt" parameter file, UTR.cpp:240-530), in the file's units.  Numbers in
 * brackets are the parameter lines. */
typedef struct {
    int modality;          /* [1] 0: TEM, lengths in Angstrom; 1: X-ray CT, microns */
    double f1, f2;         /* [7] input normalisation: input / f1 + f2 */
    int nx, ny;            /* [8] image width and height = volume x, y extents */
    double xst;            /* [9] pixel size = voxel edge */
    double zlo, zhi;       /* [10] output defocus range (the volume's z extent) */
    double dzextra;        /* [10] defocus offset */
    double dxc, dyc, dzc;  /* [11] centre-of-rotation shifts */
    double wl;             /* [12] wavelength */
    double aobj;           /* [13] objective aperture, mrad (0: none) */
    double cs3, cs5;       /* [14] spherical aberrations, mm */
    int ctf_mode;          /* [15] 0 none, 2 TIE-Hom-3D, 4 CTF-3D (1, 3: MSK_EUNSUPPORTED) */
    int escc;              /* [16] Ewald sphere curvature correction */
    double asigma;         /* [17] beta / delta */
    double nsr;            /* [18] noise-to-signal ratio of the input images */
    double epsilon;        /* [19] Tikhonov regularisation */
    int inv_laplace;       /* [22] inverse 3D Laplacian filter */
} msk_utr;

/* Volume depth nz = int((zhi - zlo) / xst + 0.5) (UTR.cpp:321), or a
 * negative status for bad parameters. */
int msk_utr_depth(const msk_utr *p);

/* The reconstruction of UTR.cpp:862-1282 for one defocus plane per
 * orientation and no Z'' rotation or image shift:
 *   angles: [nangles][2] rotations about Z and Y' (degrees), as in the
 *           orientation file
 *   defocus: [nangles] defocus distances
 *   images: float [nangles][ny][nx], flat-field corrected
 *   volume out: float [nz][ny][nx], the potential (TEM) or beta (X-ray) */
int msk_utr_reconstruct(msk_context *ctx, const msk_utr *p, int nangles, const double *angles,
                        const double *defocus, const float *images, float *volume);

/* msk_utr_reconstruct with each image's Z'' rotation and shift undone first
 * (UTR.cpp:920-940, the orientation file's Z'' angle and the .relionnew
 * shifts): the normalised image is shifted back by whole pixels, then
 * rotated by -Z'' about the rotation centre (Catmull-Rom bicubic), the mean
 * of its pixels within 5 of an edge filling in (XArray2DMove, XArray2DSpln:
 * XArrayLibrary is not part of the reference; this library's definitions).
 *   zrot: [nangles] Z'' angles (degrees), may be NULL
 *   shifts: [nangles][2] x, y shifts, may be NULL */
int msk_utr_reconstruct_planes(msk_context *ctx, const msk_utr *p, int nangles,
                               const double *angles, const double *defocus, const double *zrot,
                               const double *shifts, const float *images, float *volume);

/* CT_3Dgridding (UTR.h:199-307) of nangles centred image spectra into a
 * zeroed volume: v3 = sum of weight * K2four, samp3 = sum of weights,
 * accumulated in float as the reference does (by atomics: the order of the
 * sums, and so their last bits, follow the schedule, as in the reference's
 * threaded loop over orientations).
 *   k2four: complex [nangles][ny][nx]; v3 out: complex [nz][ny][nx];
 *   samp3 out: float [nz][ny][nx] */
int msk_utr_grid(msk_context *ctx, const msk_utr *p, int nangles, const double *angles,
                 const float *k2four, float *v3, float *samp3);

/* CTFcorrection3D (UTR.h:15-123) on a centred complex volume, in place;
 * cs3, cs5 in the units of the other lengths (UTR.cpp applies the mm
 * conversion before the call). */
int msk_utr_ctf_correction3d(msk_context *ctx, float *v3, int nx, int ny, int nz, double wl,
                             double zlo, double zhi, double ylo, double yhi, double xlo,
                             double xhi, double defocdist, double q2max, double cs3, double cs5,
                             double sigma, double epsilon, int escc);

/* InverseMLaplacian3D (UTR.h:126-175) on a centred complex volume, in place. */
int msk_utr_inverse_mlaplacian3d(msk_context *ctx, float *v3, int nx, int ny, int nz,
                                 double zaper, double yaper, double xaper, double alpha,
                                 double norm);

#ifdef __cplusplus
}
#endif

#endif /* MSK_UTR_H */
