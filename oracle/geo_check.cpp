// Byte-identity check of sph_write_geo against the reference's own writer.
// Linked with the reference's test/src/main.cpp compiled with main renamed
// (oracle/ref_fluidtest.sh), so dumpToGeo here is the reference's code.
// Writes the same synthetic frame through both and compares the files.
// Test infrastructure only.  Exit status 0 = identical.
#include <cstdio>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>
#include <sys/types.h>
#include <vector_types.h>

#include "sph_c.h"

void dumpToGeo(const std::string& filebase, const std::vector<float3>& points, const std::vector<float3>& colour,
               const std::vector<float3>& velocity, const float& pscale, const uint cnt);

static std::string slurp(const std::string& p) {
    std::ifstream f(p, std::ios::binary);
    return std::string(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

int main(int argc, char** argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    const unsigned n = 1537;
    std::vector<float3> p(n), c(n), v(n);
    unsigned s = 12345;
    auto rnd = [&]() { s = s * 1664525u + 1013904223u; return (float)(s >> 8) / 16777216.0f; };
    for (unsigned i = 0; i < n; ++i) {
        p[i] = float3{rnd(), rnd() * 0.9f, 1e-3f * rnd()};
        c[i] = float3{0.0f, rnd(), 1.0f - rnd()};
        v[i] = float3{rnd() - 0.5f, -12.345678f * rnd(), 1e-7f * (rnd() - 0.5f)};
    }
    const float pscale = 0.0123456789f;
    dumpToGeo(dir + "/ref", p, c, v, pscale, 7);
    char path[4096];
    sph_geo_path(path, sizeof(path), (dir + "/ours").c_str(), 7);
    if (sph_write_geo(path, &p[0].x, &c[0].x, &v[0].x, n, pscale) != SPH_OK) return 2;
    const std::string a = slurp(dir + "/ref.0007.geo"), b = slurp(path);
    if (a.empty() || a != b) {
        std::printf("geo files differ (%zu vs %zu bytes)\n", a.size(), b.size());
        return 1;
    }
    std::printf("geo identical (%zu bytes)\n", a.size());
    return 0;
}
