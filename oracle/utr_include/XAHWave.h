/* XAHWave.h (shim) -- the 3D header object UTR.h reads.  See XA_ini.h.
 * TEST INFRASTRUCTURE ONLY. */
#pragma once
#include "XA_ini.h"

namespace xar {
class Wavehead3D {
public:
    Wavehead3D(double wl, double zlo, double zhi, double ylo, double yhi, double xlo, double xhi)
        : wl_(wl), zlo_(zlo), zhi_(zhi), ylo_(ylo), yhi_(yhi), xlo_(xlo), xhi_(xhi) {}
    double GetWl() const { return wl_; }
    double GetXlo() const { return xlo_; }
    double GetXhi() const { return xhi_; }
    double GetYlo() const { return ylo_; }
    double GetYhi() const { return yhi_; }
    double GetZlo() const { return zlo_; }
    double GetZhi() const { return zhi_; }
    double GetXStep(index_t n) const { return (xhi_ - xlo_) / double(n); }
    double GetYStep(index_t n) const { return (yhi_ - ylo_) / double(n); }
    double GetZStep(index_t n) const { return (zhi_ - zlo_) / double(n); }

private:
    double wl_, zlo_, zhi_, ylo_, yhi_, xlo_, xhi_;
};
}  // namespace xar
