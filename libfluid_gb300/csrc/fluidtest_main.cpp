// fluidtest: the reference's demo driver (test/src/main.cpp:76-158) on the
// GB300 step.  Builds the double dam break of test/src/myfluidsystem.cpp:6-30
// through the FluidSystem drop-in, advances it frame by frame, times each
// advance() and writes one Houdini .geo file per frame.
//
//   fluidtest -f <filebase> [-n particles=10000] [-g res=16] [-a adhesion=0.1]
//             [-v viscosity=0.2] [-s tension=1.0] [-d damp=0.5] [-t dt=0.002]
//             [-p substeps=1] [-q steps=500] [--no-geo]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "fluidsystem.h"
#include "sph_c.h"

namespace {

class DamBreak : public FluidSystem {
public:
    // test/src/myfluidsystem.cpp:6-30
    void setupDoubleDamBreak(uint n, uint res, float adhesion, float viscosity, float tension, float vdamp) {
        init(n, res);
        setAdhesion(adhesion);
        setViscosity(viscosity);
        setSurfaceTension(tension);
        setVDamp(vdamp);
        createFluidBlock(0, n / 2, 0.0f, 0.0f, 0.0f, 0.33f, 0.9f, 0.33f);
        createFluidBlock(n / 2, n - n / 2, 0.66f, 0.0f, 0.66f, 1.0f, 0.9f, 1.0f);
    }
};

void usage() {
    std::cerr << "usage: fluidtest -f <filebase> [-n 10000] [-g 16] [-a 0.1] [-v 0.2] [-s 1.0] [-d 0.5]"
                 " [-t 0.002] [-p 1] [-q 500] [--no-geo]\n";
}

}  // namespace

int main(int argc, char** argv) {
    uint n = 10000, res = 16, substeps = 1, steps = 500;
    float adhesion = 0.1f, viscosity = 0.2f, tension = 1.0f, damp = 0.5f, dt = 0.002f;
    std::string filebase;
    bool geo = true;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() -> const char* {
            if (i + 1 >= argc) { usage(); std::exit(EXIT_FAILURE); }
            return argv[++i];
        };
        if (a == "-n" || a == "--num") n = (uint)std::strtoul(next(), nullptr, 10);
        else if (a == "-g" || a == "--grid") res = (uint)std::strtoul(next(), nullptr, 10);
        else if (a == "-a" || a == "--adhesion") adhesion = std::strtof(next(), nullptr);
        else if (a == "-v" || a == "--viscosity") viscosity = std::strtof(next(), nullptr);
        else if (a == "-s" || a == "--tension") tension = std::strtof(next(), nullptr);
        else if (a == "-d" || a == "--damp") damp = std::strtof(next(), nullptr);
        else if (a == "-t" || a == "--timestep") dt = std::strtof(next(), nullptr);
        else if (a == "-p" || a == "--substeps") substeps = (uint)std::strtoul(next(), nullptr, 10);
        else if (a == "-q" || a == "--numsteps") steps = (uint)std::strtoul(next(), nullptr, 10);
        else if (a == "-f" || a == "--filebase") filebase = next();
        else if (a == "--no-geo") geo = false;
        else { usage(); return EXIT_FAILURE; }
    }
    if (filebase.empty() && geo) { usage(); return EXIT_FAILURE; }

    DamBreak splash;
    splash.setupDoubleDamBreak(n, res, adhesion, viscosity, tension, damp);
    std::vector<float3> points(n), colour(n), velocity(n);
    const float pscale = splash.getPscale();
    double t_tot = 0.0;
    std::vector<char> path(filebase.size() + 32);
    for (uint i = 1; i <= steps; ++i) {
        std::cout << "---Step " << i << ", Timestep " << dt * float(i) << ", Substeps " << substeps << " pscale "
                  << pscale << " ";
        const auto t1 = std::chrono::high_resolution_clock::now();
        splash.advance(dt, substeps);
        const auto t2 = std::chrono::high_resolution_clock::now();
        const std::chrono::duration<double, std::milli> ms = t2 - t1;
        std::cout << " step time " << ms.count() << "ms----\n";
        t_tot += ms.count();
        splash.exportToData(points, colour, velocity);
        if (geo) {
            sph_geo_path(path.data(), path.size(), filebase.c_str(), i);
            if (sph_write_geo(path.data(), &points[0].x, &colour[0].x, &velocity[0].x, n, pscale) != SPH_OK) {
                std::cout << "Failed to open file " << path.data() << '\n';
                return EXIT_FAILURE;
            }
        }
    }
    std::cout << "TOTAL TIME " << t_tot << "\n";
    return EXIT_SUCCESS;
}
