/*
 * XA_ini.h (shim) -- the few XArrayLibrary declarations that the reference's
 * PhaseRetrieval/UTR.h templates use, so that those templates compile
 * unmodified into the test-only reference build (oracle/_ref/libutr_ref.so).
 *
 * TEST INFRASTRUCTURE ONLY.  XArrayLibrary itself is not part of the
 * reference tree; these are interface stand-ins written from how UTR.h and
 * UTR.cpp call them (array indexing [k][j][i] with i fastest, GetDim1/2/3 =
 * slowest..fastest extent, Wavehead3D(wl, zlo, zhi, ylo, yhi, xlo, xhi) with
 * step = extent / points, as UTR.cpp:299-330 sets xhi = xlo + xst * nx).
 * UTR.h calls abs() on doubles (UTR.h:55-59, 81); in UTR.cpp the XArray
 * headers included before it make the floating-point overloads visible, as
 * MSVC's headers do, so this stand-in does too (with only <complex.h> in
 * scope, g++ would pick the C library's int abs()).
 */
#pragma once
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdlib>
#include <vector>

using std::abs;

namespace xar {
typedef std::size_t index_t;
constexpr double PI = 3.14159265358979323846;
typedef std::complex<float> fcomplex;
}  // namespace xar
using xar::index_t;
