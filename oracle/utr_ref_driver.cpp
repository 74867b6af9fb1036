/*
 * utr_ref_driver.cpp -- C-linkage entry points into the reference's own
 * PhaseRetrieval/UTR.h templates (CT_3Dgridding, CTFcorrection3D,
 * InverseMLaplacian3D), compiled unmodified from the reference tree against
 * the XArray stand-ins in oracle/utr_include into oracle/_ref/libutr_ref.so.
 *
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement and to make
 * golden fixtures; never linked into the shipped library.
 *
 * Arrays are dense, slowest index first, complex as interleaved float pairs:
 * k2four [ny][nx], v3 [nz][ny][nx] complex, samp3 [nz][ny][nx].
 */
#include <cstring>

#include "UTR.h"

extern "C" {

/* CT_3Dgridding<float> (UTR.h:199-307) of one image into v3 / samp3, which
 * hold the sums so far (in and out).  fc = {Fxc, Fyc, Fzc} as re, im pairs. */
void ref_utr_grid_f(const float *k2four, int nx, int ny, int nz, double angleY, double angleZ,
                    float fxlo, float fxst, float fylo, float fyst, float fzlo, float fzst,
                    const float *fc, double wl, int rotshift, int escc, float *v3, float *samp3)
{
    xar::XArray2D<xar::fcomplex> K2(ny, nx);
    std::memcpy(K2.data(), k2four, sizeof(float) * 2 * (size_t)nx * ny);
    const size_t nv = (size_t)nx * ny * nz;
    xar::XArray3D<std::complex<float>> V3(nz, ny, nx);
    xar::XArray3D<float> S3(nz, ny, nx);
    std::memcpy(V3.data(), v3, sizeof(float) * 2 * nv);
    std::memcpy(S3.data(), samp3, sizeof(float) * nv);
    CT_3Dgridding<float>(K2, V3, S3, angleY, angleZ, fxlo, fxst, fylo, fyst, fzlo, fzst,
                         std::complex<float>(fc[0], fc[1]), std::complex<float>(fc[2], fc[3]),
                         std::complex<float>(fc[4], fc[5]), wl, rotshift != 0, escc != 0);
    std::memcpy(v3, V3.data(), sizeof(float) * 2 * nv);
    std::memcpy(samp3, S3.data(), sizeof(float) * nv);
}

/* CTFcorrection3D<float> (UTR.h:15-123), in place. */
void ref_utr_ctf3d_f(float *v3, int nx, int ny, int nz, double wl, double zlo, double zhi,
                     double ylo, double yhi, double xlo, double xhi, double defocdist,
                     double q2max, double cs3, double cs5, double sigma, double epsilon, int escc)
{
    const size_t nv = (size_t)nx * ny * nz;
    xar::XArray3D<std::complex<float>> V3(nz, ny, nx);
    std::memcpy(V3.data(), v3, sizeof(float) * 2 * nv);
    CTFcorrection3D<float>(V3, xar::Wavehead3D(wl, zlo, zhi, ylo, yhi, xlo, xhi), defocdist, q2max,
                           cs3, cs5, sigma, epsilon, escc != 0);
    std::memcpy(v3, V3.data(), sizeof(float) * 2 * nv);
}

/* InverseMLaplacian3D<float> (UTR.h:126-175), in place. */
void ref_utr_invlap3d_f(float *v3, int nx, int ny, int nz, double zaper, double yaper,
                        double xaper, double alpha, double norm)
{
    const size_t nv = (size_t)nx * ny * nz;
    xar::XArray3D<std::complex<float>> V3(nz, ny, nx);
    std::memcpy(V3.data(), v3, sizeof(float) * 2 * nv);
    InverseMLaplacian3D<float>(V3, zaper, yaper, xaper, alpha, norm);
    std::memcpy(v3, V3.data(), sizeof(float) * 2 * nv);
}

}  // extern "C"
