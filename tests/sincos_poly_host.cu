// sincos_poly_host.cu -- evaluates msk::expi_poly (sincos_poly.cuh, compiled
// for the host) on the float32 arguments in argv[1], writing (cos, sin) pairs
// to argv[2].  TEST ONLY.
#include <cstdio>
#include <vector>

#include "sincos_poly.cuh"

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 3;
    std::vector<float> x;
    float v;
    while (fread(&v, 4, 1, f) == 1) x.push_back(v);
    fclose(f);
    std::vector<float2> y(x.size());
    for (size_t i = 0; i < x.size(); i++) y[i] = msk::expi_poly(x[i]);
    f = fopen(argv[2], "wb");
    if (!f || fwrite(y.data(), sizeof(float2), y.size(), f) != y.size()) return 4;
    fclose(f);
    return 0;
}
