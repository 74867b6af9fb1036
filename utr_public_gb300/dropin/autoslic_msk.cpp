// autoslic_msk.cpp -- drop-in definition of the reference's `autoslic` class
// (TemsimLibrary/autoslic.hpp) whose calculate() runs on the GPU through
// libmsk's C ABI (include/msk.h).
//
// Build it in place of TemsimLibrary/autoslic.cpp, against the reference's own
// autoslic.hpp / cfpix.hpp / slicelib.hpp, and link libmsk.so:
//
//   g++ -std=gnu++17 -I<TemsimLibrary> -I<fftwlib> -I<this repo>/include \
//       -c autoslic_msk.cpp && link with libmsk.so
//
// The class layout comes from the reference's header, so autosliccmd.cpp
// (autosliccmd.cpp:936-937) calls it unchanged.  Only the coherent branch is
// provided (lpartl = lbeams = lcross = 0), with its thermal branches (lwobble,
// iseed and wobble are forwarded to msk_calculate); the partial-coherence,
// beam and cross-section branches, and every error the reference answers with
// exit(0), become an exception.
#include <cstring>
#include <stdexcept>
#include <string>

#include "autoslic.hpp"
#include "msk.h"

namespace {

// One libmsk context per host thread: MsctKirkland runs one worker thread per
// orientation (MultisliceT.cpp:431), and a context is single-threaded.
msk_context *thread_context()
{
    static thread_local struct Holder {
        msk_context *ctx = nullptr;
        ~Holder() { msk_destroy(ctx); }
    } h;
    if (!h.ctx) {
        const int st = msk_create(0, &h.ctx);
        if (st != MSK_OK) throw std::runtime_error(std::string("msk_create: ") + msk_status_string(st));
    }
    return h.ctx;
}

}  // namespace

autoslic::autoslic()
{
    BW = (2.0F / 3.0F);
    ABERR = 1.0e-4;
    NSMAX = 1000;
    NCMAX = 256;
    NZMAX = 103;
    twopi = 2.0 * (4.0 * atan(1.0));
    lcross = lpartl = lstart = lwobble = lbeams = 0;
    nillum = 0;
}

autoslic::~autoslic() {}

void autoslic::calculate(cfpix &pix, cfpix &wave0, cfpix &depthpix, float param[], int multiMode,
                         int natom, long *iseed, int Znum[], float x[], float y[], float z[],
                         float occ[], float wobble[], cfpix &beams, int hb[], int kb[], int nbeams,
                         float ycross, float dfdelt, float ctblength, float ctblengthz,
                         int nfftwinit, int nmode)
{
    (void)depthpix; (void)multiMode; (void)beams; (void)hb; (void)kb;
    (void)nbeams; (void)ycross; (void)dfdelt; (void)nfftwinit;
    if (lpartl || lbeams || lcross)
        throw std::runtime_error("autoslic (GPU): only the coherent branch is provided");
    const int nx = ToInt(param[pNX]), ny = ToInt(param[pNY]);
    if (wave0.nx() != nx || wave0.ny() != ny)
        throw std::runtime_error("autoslic (GPU): wave0 must be nx x ny");
    pix.resize(nx, ny);
    // cfpix keeps interleaved complex floats, x-major: &re(0,0) is its data
    const int st = msk_calculate(thread_context(), &pix.re(0, 0), &wave0.re(0, 0), param, natom,
                                 Znum, x, y, z, occ, wobble, ctblength, ctblengthz, nmode,
                                 lwobble, iseed);
    if (st != MSK_OK)
        throw std::runtime_error(std::string("autoslic (GPU): ") + msk_last_error(thread_context()));
}
