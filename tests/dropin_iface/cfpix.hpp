// cfpix.hpp -- stand-in for the reference's complex image class, for building
// the autoslic drop-in where the reference tree is absent.  TEST ONLY.
//
// Written from the interface the drop-in relies on (TemsimLibrary/cfpix.hpp:
// constructor / destructor 97-99, nx() / ny() 101-102, re() / im() 105-134,
// resize() 152): a complex image of nx x ny single-precision pixels kept as
// interleaved (re, im) float pairs, x-major -- pixel (ix, iy) at
// data[iy + ix*ny] -- so &re(0, 0) is the start of the whole image.  No FFT
// plans: the drop-in never transforms on the host.
#ifndef MSK_TEST_CFPIX_HPP
#define MSK_TEST_CFPIX_HPP

class cfpix {
public:
    cfpix(int nx = 0, int ny = 0);
    ~cfpix();
    cfpix(const cfpix &) = delete;
    cfpix &operator=(const cfpix &) = delete;

    inline int nx() const { return nxl; }
    inline int ny() const { return nyl; }
    inline float &re(const int ix, const int iy) { return data[iy + ix * nyl][0]; }
    inline float &im(const int ix, const int iy) { return data[iy + ix * nyl][1]; }

    int resize(const int nx, const int ny);

private:
    int nxl = 0, nyl = 0;
    float (*data)[2] = nullptr;
};

#endif
