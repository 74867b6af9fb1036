// msk_io.cpp -- MsctKirkland's file formats: image writers (GRD, GRC, 32-bit
// float TIFF) and the orientation files (.txt, .relionnew).
//
// The reference reads and writes them through its XArrayLibrary, which is not
// part of it; the formats follow ReadmeMsctKirkland.txt (GRD/GRC layouts,
// orientation columns) and the TIFF 6.0 baseline.  Images are the library's
// [nx][ny] arrays (iy fastest); a file's rows run along y and its fastest index
// along x, as the reference transposes its cfpix data into [iy][ix] arrays
// before writing (autosliccmd.cpp:1053-1055).  Little-endian byte order.
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "msk.h"

namespace {

template <typename T> void put(std::vector<unsigned char> &b, T v)
{
    unsigned char raw[sizeof(T)];
    std::memcpy(raw, &v, sizeof(T));
    b.insert(b.end(), raw, raw + sizeof(T));
}

int write_all(const char *path, const std::vector<unsigned char> &b)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) return MSK_EINVAL;
    const size_t n = std::fwrite(b.data(), 1, b.size(), f);
    const int rc = std::fclose(f);
    return (n == b.size() && rc == 0) ? MSK_OK : MSK_EINVAL;
}

bool little_endian()
{
    const uint16_t one = 1;
    unsigned char c;
    std::memcpy(&c, &one, 1);
    return c == 1;
}

// the image transposed to rows along y: out[iy][ix]
void rows_y(const float *img, int nx, int ny, int comps, std::vector<float> &out)
{
    out.resize((size_t)nx * ny * comps);
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++)
            for (int c = 0; c < comps; c++)
                out[((size_t)iy * nx + ix) * comps + c] = img[((size_t)ix * ny + iy) * comps + c];
}

}  // namespace

extern "C" {

int msk_write_grd(const char *path, const float *img, int nx, int ny, double xlo, double xhi,
                  double ylo, double yhi)
{
    if (!path || !img || nx < 1 || ny < 1 || nx > 32767 || ny > 32767 || !little_endian())
        return MSK_EINVAL;
    std::vector<float> t;
    rows_y(img, nx, ny, 1, t);
    double zlo = t[0], zhi = t[0];
    for (float v : t) {
        zlo = std::fmin(zlo, (double)v);
        zhi = std::fmax(zhi, (double)v);
    }
    std::vector<unsigned char> b;
    b.insert(b.end(), {'D', 'S', 'B', 'B'});
    put<int16_t>(b, (int16_t)nx);
    put<int16_t>(b, (int16_t)ny);
    put(b, xlo);
    put(b, xhi);
    put(b, ylo);
    put(b, yhi);
    put(b, zlo);
    put(b, zhi);
    for (float v : t) put(b, v);
    return write_all(path, b);
}

int msk_write_grc(const char *path, const float *amp, int nx, int ny, double wavelength,
                  double xlo, double xhi, double ylo, double yhi)
{
    if (!path || !amp || nx < 1 || ny < 1 || nx > 32767 || ny > 32767 || !little_endian())
        return MSK_EINVAL;
    std::vector<float> t;
    rows_y(amp, nx, ny, 2, t);
    std::vector<unsigned char> b;
    put<int16_t>(b, -5);
    put(b, wavelength);
    put<int16_t>(b, (int16_t)nx);
    put<int16_t>(b, (int16_t)ny);
    put(b, xlo);
    put(b, xhi);
    put(b, ylo);
    put(b, yhi);
    for (float v : t) put(b, v);
    return write_all(path, b);
}

int msk_write_tiff32(const char *path, const float *img, int nx, int ny)
{
    if (!path || !img || nx < 1 || ny < 1 || !little_endian()) return MSK_EINVAL;
    std::vector<float> t;
    rows_y(img, nx, ny, 1, t);
    // header, the pixel strip, then one image file directory
    const uint32_t data_off = 8, data_bytes = (uint32_t)(t.size() * 4);
    const uint32_t ifd_off = data_off + data_bytes;  // a multiple of 4: word aligned
    std::vector<unsigned char> b;
    b.insert(b.end(), {'I', 'I'});
    put<uint16_t>(b, 42);
    put<uint32_t>(b, ifd_off);
    for (float v : t) put(b, v);
    struct Tag {
        uint16_t tag, type;
        uint32_t value;
    };
    const Tag tags[] = {
        {256, 4, (uint32_t)nx},   // ImageWidth (LONG)
        {257, 4, (uint32_t)ny},   // ImageLength
        {258, 3, 32},             // BitsPerSample (SHORT)
        {259, 3, 1},              // Compression: none
        {262, 3, 1},              // PhotometricInterpretation: black is zero
        {273, 4, data_off},       // StripOffsets
        {277, 3, 1},              // SamplesPerPixel
        {278, 4, (uint32_t)ny},   // RowsPerStrip: one strip
        {279, 4, data_bytes},     // StripByteCounts
        {284, 3, 1},              // PlanarConfiguration: chunky
        {339, 3, 3},              // SampleFormat: IEEE floating point
    };
    put<uint16_t>(b, (uint16_t)(sizeof(tags) / sizeof(tags[0])));
    for (const Tag &g : tags) {
        put(b, g.tag);
        put(b, g.type);
        put<uint32_t>(b, 1);  // count
        if (g.type == 3) {    // a SHORT sits in the first two bytes of the value field
            put<uint16_t>(b, (uint16_t)g.value);
            put<uint16_t>(b, 0);
        } else {
            put(b, g.value);
        }
    }
    put<uint32_t>(b, 0);  // no further directory
    return write_all(path, b);
}

int msk_read_orientations(const char *path, int *nangles, int *nplanes, double *angles,
                          int *plane_off, double *planes, double *shifts)
{
    if (!path || !nangles || !nplanes) return MSK_EINVAL;
    std::ifstream in(path);
    if (!in) return MSK_EINVAL;
    const std::string p(path);
    std::string ext;
    const size_t dot = p.rfind('.');
    if (dot != std::string::npos)
        for (size_t i = dot; i < p.size(); i++) ext += (char)std::tolower((unsigned char)p[i]);
    const bool relion = ext == ".relionnew";
    if (!relion && ext != ".txt") return MSK_EINVAL;
    const bool fill = angles && plane_off && planes && shifts;
    const int cap_a = fill ? *nangles : 0, cap_p = fill ? *nplanes : 0;
    int na = 0, np = 0;
    std::string line;
    while (std::getline(in, line)) {
        const size_t s0 = line.find_first_not_of(" \t\r");
        if (s0 == std::string::npos || line.compare(s0, 2, "//") == 0) continue;
        std::istringstream ls(line);
        int kplanes;
        double a[2], sh[2] = {0.0, 0.0};
        std::vector<double> pl;  // 5 per plane
        if (relion) {
            std::string idx, name;
            double v[8];
            if (!(ls >> idx >> name)) return MSK_EINVAL;
            for (double &x : v)
                if (!(ls >> x)) return MSK_EINVAL;
            // every number but the astigmatism angle changes sign (the readme's rule)
            a[0] = -v[5];
            a[1] = -v[6];
            sh[0] = -v[0];
            sh[1] = -v[1];
            const double U = -v[2], V = -v[3];
            pl = {-v[7], 0.5 * (U + V), 0.5 * (U - V), v[4], 0.0};
            kplanes = 1;
        } else {
            std::vector<double> v;
            double x;
            while (ls >> x) v.push_back(x);
            if (v.size() < 2 || (v.size() % 2) != 0) return MSK_EINVAL;
            a[0] = v[0];
            a[1] = v[1];
            kplanes = (int)(v.size() - 2) / 2;
            for (int k = 0; k < kplanes; k++) pl.insert(pl.end(), {v[2 + 2 * k], v[3 + 2 * k], 0.0, 0.0, 0.0});
        }
        if (fill) {
            if (na >= cap_a || np + kplanes > cap_p) return MSK_EINVAL;  // the file changed
            angles[2 * na] = a[0];
            angles[2 * na + 1] = a[1];
            shifts[2 * na] = sh[0];
            shifts[2 * na + 1] = sh[1];
            plane_off[na] = np;
            std::memcpy(planes + 5 * (size_t)np, pl.data(), pl.size() * sizeof(double));
        }
        np += kplanes;
        na++;
    }
    if (fill) plane_off[na] = np;
    *nangles = na;
    *nplanes = np;
    return MSK_OK;
}

}  // extern "C"
