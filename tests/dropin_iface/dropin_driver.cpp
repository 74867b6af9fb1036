// dropin_driver.cpp -- drives the autoslic drop-in the way MsctKirkland does:
// one autoslic object per worker thread, each calling calculate() on its own
// cfpix images (MultisliceT.cpp:403-448, autosliccmd.cpp:642-649, 936-937).
// TEST ONLY: built with the stand-in headers of this folder, the drop-in
// (utr_public_gb300/dropin/autoslic_msk.cpp) and libmsk.so.
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "autoslic.hpp"

cfpix::cfpix(int nx, int ny) { resize(nx, ny); }
cfpix::~cfpix() { delete[] data; }

int cfpix::resize(const int nx, const int ny)
{
    if (nx == nxl && ny == nyl && data) return 1;
    delete[] data;
    data = nullptr;
    nxl = nx;
    nyl = ny;
    if (nx > 0 && ny > 0) data = new float[(size_t)nx * ny][2]();
    return 1;
}

namespace {

// One worker: a plane incident wave of amplitude 1 (autosliccmd.cpp:642-649),
// calculate(), the exit wave copied out as interleaved x-major floats.
void worker(const float *param_in, int natom, const int *Znum, const float *x, const float *y,
            const float *z, const float *occ, float ctblength, float ctblengthz, float *out,
            std::string *err)
{
    try {
        std::vector<float> param(param_in, param_in + 200);
        const int nx = ToInt(param[pNX]), ny = ToInt(param[pNY]);
        cfpix pix, depth, beams, wave0(nx, ny);
        for (int ix = 0; ix < nx; ix++)
            for (int iy = 0; iy < ny; iy++) {
                wave0.re(ix, iy) = 1.0F;
                wave0.im(ix, iy) = 0.0F;
            }
        // calculate() takes non-const arrays (the reference reads them only)
        std::vector<int> Z(Znum, Znum + natom);
        std::vector<float> xs(x, x + natom), ys(y, y + natom), zs(z, z + natom),
            os(occ, occ + natom), wob(natom, 0.0F);
        long iseed = 0;
        autoslic aslic;
        aslic.lbeams = aslic.lcross = aslic.lpartl = aslic.lwobble = 0;
        aslic.lstart = 0;
        aslic.calculate(pix, wave0, depth, param.data(), 0, natom, &iseed, Z.data(), xs.data(),
                        ys.data(), zs.data(), os.data(), wob.data(), beams, nullptr, nullptr, 0,
                        0.0F, 0.0F, ctblength, ctblengthz, 0, 0);
        std::memcpy(out, &pix.re(0, 0), sizeof(float) * 2 * (size_t)nx * ny);
    } catch (const std::exception &e) {
        *err = e.what();
    }
}

}  // namespace

// Runs `nthreads` workers at once on the same inputs; out holds nthreads exit
// waves.  Returns 0, or 1 with the first worker's error in errbuf.
extern "C" int dropin_threads(int nthreads, const float *param, int natom, const int *Znum,
                              const float *x, const float *y, const float *z, const float *occ,
                              float ctblength, float ctblengthz, float *out, char *errbuf,
                              int errlen)
{
    const int nx = ToInt(param[pNX]), ny = ToInt(param[pNY]);
    std::vector<std::string> errs(nthreads);
    std::vector<std::thread> th;
    for (int i = 0; i < nthreads; i++)
        th.emplace_back(worker, param, natom, Znum, x, y, z, occ, ctblength, ctblengthz,
                        out + (size_t)i * 2 * nx * ny, &errs[i]);
    for (auto &t : th) t.join();
    for (auto &e : errs)
        if (!e.empty()) {
            std::strncpy(errbuf, e.c_str(), errlen - 1);
            errbuf[errlen - 1] = 0;
            return 1;
        }
    return 0;
}
