// Houdini PGEOMETRY V5 ASCII export of a particle frame: the file format
// fluidtest writes (test/src/main.cpp:10-74) — one point per particle with
// position, diffuse colour Cd, velocity v and pscale, and one particle
// primitive listing every point.  Output is byte-identical to the
// reference's for the same data (tested against its own writer).
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/sph_c.h"

extern "C" int sph_geo_path(char* out, uint64_t cap, const char* filebase, uint32_t frame) {
    if (!out || !filebase) return SPH_EINVAL;
    const int k = std::snprintf(out, (size_t)cap, "%s.%04d.geo", filebase, (int)frame);
    return (k < 0 || (uint64_t)k >= cap) ? SPH_EINVAL : SPH_OK;
}

extern "C" int sph_write_geo(const char* path, const float* pos, const float* colour, const float* vel, uint32_t n,
                             float pscale) {
    if (!path || (n && (!pos || !colour || !vel))) return SPH_EINVAL;
    std::ofstream file(path);
    if (!file.is_open()) return SPH_EINVAL;
    std::stringstream ss;
    ss << "PGEOMETRY V5\n";
    ss << "NPoints " << (size_t)n << " NPrims 1\n";
    ss << "NPointGroups 0 NPrimGroups 1\n";
    ss << "NPointAttrib 3  NVertexAttrib 0 NPrimAttrib 2 NAttrib 0\n";
    ss << "PointAttrib \n";
    ss << "Cd 3 float 1 1 1\n";
    ss << "v 3 float 0 0 0\n";
    ss << "pscale 1 float 1\n";
    for (uint32_t i = 0; i < n; ++i) {
        const float* p = pos + 3 * (size_t)i;
        const float* c = colour + 3 * (size_t)i;
        const float* v = vel + 3 * (size_t)i;
        ss << p[0] << " " << p[1] << " " << p[2] << " 1 ";
        ss << "(" << c[0] << " " << c[1] << " " << c[2] << " " << v[0] << " " << v[1] << " " << v[2] << " "
           << pscale << ")\n";
    }
    ss << "PrimitiveAttrib\n";
    ss << "generator 1 index 1 location1\n";
    ss << "dopobject 1 index 1 /obj/AutoDopNetwork:1\n";
    ss << "Part " << (size_t)n << " ";
    for (size_t i = 0; i < n; ++i) ss << i << " ";
    ss << " [0\t0]\n";
    ss << "box_object1 unordered\n";
    ss << "1 1\n";
    ss << "beginExtra\n";
    ss << "endExtra\n";
    file << ss.rdbuf();
    return file.good() ? SPH_OK : SPH_EINVAL;
}
