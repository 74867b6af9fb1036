/*
 * ref_driver.cpp -- C-linkage entry points into the reference's own
 * TemsimLibrary code (autoslic.cpp, slicelib.cpp, cfpix.cpp compiled
 * unmodified from the reference tree into oracle/_ref/libautoslic_ref.so).
 *
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement and to make
 * golden fixtures; never linked into the shipped library.
 *
 * The reference's calculate() calls exit(0) on bad input
 * (TemsimLibrary/autoslic.cpp:258-262,288-299,734-739); callers of this
 * driver must only pass specimens that lie inside the box.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "autoslic.hpp"
#include "slicelib.hpp"
#include "XA_nrrand.h"

/* Gaussian deviate for the reference's wobble branch (autoslic.cpp:701-713),
 * which the parity cases never enable.  Box-Muller on a 64-bit LCG. */
double gasdev(long *idum)
{
    uint64_t s = (uint64_t)(*idum) * 6364136223846793005ULL + 1442695040888963407ULL;
    uint64_t s2 = s * 6364136223846793005ULL + 1442695040888963407ULL;
    *idum = (long)s2;
    double u1 = ((s >> 11) + 1.0) / 9007199254740993.0;
    double u2 = (s2 >> 11) / 9007199254740992.0;
    return sqrt(-2.0 * log(u1)) * cos(8.0 * atan(1.0) * u2);
}

extern "C" {

/* autoslic::calculate coherent branch (autoslic.hpp:166-169).
 * pix_out, wave0_in: nx*ny interleaved complex64, x-major (data[iy + ix*ny]).
 * The atom arrays are read only (calculate copies them, autoslic.cpp:689-720). */
void ref_calculate(float *pix_out, const float *wave0_in, float *param, int natom,
                   int *Znum, float *x, float *y, float *z, float *occ, float *wobble,
                   float ctblength, float ctblengthz, int nmode, int lwobble,
                   long *iseed, int nfftwinit)
{
    const int nx = ToInt(param[pNX]), ny = ToInt(param[pNY]);
    cfpix pix, wave0, depthpix, beams;
    wave0.resize(nx, ny);
    std::memcpy(&wave0.re(0, 0), wave0_in, sizeof(float) * 2 * (size_t)nx * ny);
    autoslic aslice;
    aslice.lwobble = lwobble;
    long seed_local = -1;
    aslice.calculate(pix, wave0, depthpix, param, 0, natom, iseed ? iseed : &seed_local,
                     Znum, x, y, z, occ, wobble, beams, nullptr, nullptr, 0, 0.0f, 0.0f,
                     ctblength, ctblengthz, nfftwinit, nmode);
    std::memcpy(pix_out, &pix.re(0, 0), sizeof(float) * 2 * (size_t)nx * ny);
}

/* Many independent orientations at once, one host thread per orientation as
 * MsctKirkland drives them (MultisliceT.cpp:403-448).  Atom arrays are
 * [n][natom[i]] packed at offsets off[i]; outputs pix_out[n][nx*ny*2].
 * Call ref_calculate once first (nfftwinit=1) so that the shared static
 * plans and spline tables are built before threads start. */
void ref_calculate_many(int n, int nthreads, float *pix_out, const float *wave0_in,
                        const float *param_in, const int *natom, const long *off,
                        int *Znum, float *x, float *y, float *z, float *occ, float *wobble,
                        float ctblength, float ctblengthz, int nmode)
{
    const int nx = ToInt(param_in[pNX]), ny = ToInt(param_in[pNY]);
    const size_t npix2 = (size_t)2 * nx * ny;
    int next = 0;
    auto work = [&](int) {
        std::vector<float> param(param_in, param_in + 200);
        for (;;) {
            int i = __atomic_fetch_add(&next, 1, __ATOMIC_RELAXED);
            if (i >= n) break;
            ref_calculate(pix_out + npix2 * i, wave0_in, param.data(), natom[i], Znum + off[i],
                          x + off[i], y + off[i], z + off[i], occ + off[i], wobble + off[i],
                          ctblength, ctblengthz, nmode, 0, nullptr, 0);
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back(work, t);
    for (auto &t : th) t.join();
}

void ref_sortByZ(float *x, float *y, float *z, float *occ, int *Znum, int natom)
{
    sortByZ(x, y, z, occ, Znum, natom);
}

double ref_vzatomLUT(int Z, double rsq) { return vzatomLUT(Z, rsq); }
double ref_vzatom(int Z, double r) { return vzatom(Z, r); }
double ref_wavelength(double kev) { return wavelength(kev); }
double ref_sigma(double kev) { return sigma(kev); }
double ref_bessk0(double x) { return bessk0(x); }
double ref_bessi0(double x) { return bessi0(x); }
void ref_freqn(float *k, float *k2, float *xpos, int n, double a) { freqn(k, k2, xpos, n, a); }
void ref_splinh(double *x, double *y, double *b, double *c, double *d, int n)
{
    splinh(x, y, b, c, d, n);
}
double ref_seval(double *x, double *y, double *b, double *c, double *d, int n, double x0)
{
    return seval(x, y, b, c, d, n, x0);
}

}  // extern "C"
