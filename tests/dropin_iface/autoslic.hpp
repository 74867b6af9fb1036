// autoslic.hpp -- stand-in for the reference's autoslic class declaration
// (TemsimLibrary/autoslic.hpp:140-183), for building the drop-in where the
// reference tree is absent.  TEST ONLY.
//
// The public surface is the reference's: the control flags, nillum and the
// calculate() signature (autoslic.hpp:152-169).  The private members are the
// ones the drop-in's constructor sets.
#ifndef MSK_TEST_AUTOSLIC_HPP
#define MSK_TEST_AUTOSLIC_HPP

#include <cmath>
#include <string>

#include "cfpix.hpp"
#include "slicelib.hpp"

class autoslic {
public:
    autoslic();
    ~autoslic();

    int lbeams, lcross, lpartl, lstart, lwobble;
    int nillum;

    void calculate(cfpix &pix, cfpix &wave0, cfpix &depthpix, float param[], int multiMode,
                   int natom, long *iseed1, int Znum[], float x[], float y[], float z[],
                   float occ[], float wobble[], cfpix &beams, int hb[], int kb[], int nbeams,
                   float ycross, float dfdelt, float ctblength, float ctblengthz, int nfftwinit,
                   int nmode);

private:
    int NZMAX, NSMAX, NCMAX;
    float BW;
    double twopi, ABERR;
    std::string sbuffer;
};

#endif
