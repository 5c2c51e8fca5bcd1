/*
 * fluidsystem.h - C++ drop-in for NCCA/libfluid's FluidSystem
 * (libfluid/include/fluidsystem.h:16-126) over the C ABI in sph_c.h.
 *
 * Same class name, public and protected members, signatures and default
 * arguments, so code written against the reference (its test/src/main.cpp and
 * test/src/myfluidsystem.*) compiles unchanged.  The reference's
 * thrust::device_vector members are not part of the interface any caller
 * uses; the device state lives behind an opaque sph_system handle.
 * Link with -lfluid -lsph_gb300.  Needs the CUDA include path for float3.
 */
#ifndef FLUIDSYSTEM_H
#define FLUIDSYSTEM_H

#include <sys/types.h>
#include <vector>
#include <vector_types.h>

#include "fluiddefines.h"

struct sph_system;

class FluidSystem
{
public:
    typedef enum
    {
        STATIC = 1,
        DYNAMIC = 2
    } ParticleState;

    /// Construct an empty fluid system (fluidsystem.cu:18-22)
    FluidSystem();

    /// Destroy it (fluidsystem.cu:27-31)
    virtual ~FluidSystem();

    /// Dam-break set-up: init + one block [0.1,0.9]^3 (fluidsystem.cu:132-147)
    virtual void setup(const uint &_numPoints, const uint &_res);

    /// Initialise from external data (fluidsystem.cu:179-189)
    void setupFromData(const std::vector<float3> & /*points*/,
                       const std::vector<float3> & /*velocity*/,
                       const uint &_res = 32);

    /// Copy positions, density colours and velocities out (fluidsystem.cu:154-173).
    /// Vectors smaller than the particle count are resized.
    void exportToData(std::vector<float3> & /*points*/,
                      std::vector<float3> & /*colour*/,
                      std::vector<float3> & /*velocity*/);

    /// Particle radius (fluidsystem.cu:406-409)
    float getPscale() const;

    /// Advance by dt in `substeps` substeps (fluidsystem.cu:273-399)
    void advance(const float & /*dt*/ = DEFAULT_TIMESTEP, const uint & /*substeps*/ = 10);

    void setRestDensity(const float &_restDensity);
    void setParticleSize(const float &_particleSize);
    void setGasConstant(const float &_gasConstant);
    void setLimits(const float &_velLimit, const float &_accLimit);
    void setXSPHScale(const float &_xsphScale);
    void setSurfaceTension(const float &_surfaceTension);
    void setViscosity(const float &_viscosity);
    void setAdhesion(const float &_adhesion);
    void setVDamp(const float &_vdamp);
    void setGamma(const float &_gamma);
    void setMass(const float &_mass);

    /// The C ABI handle, for calls beyond the reference interface
    /// (gravity, box domain, debug taps; see sph_c.h).
    sph_system *handle() const { return m_sys; }

protected:
    /// Whether advance() does anything (fluidsystem.h:84)
    bool m_isInit;

    /// Allocate for _numPoints particles on a res^3 grid and reset the
    /// parameters (fluidsystem.cu:196-265)
    void init(const uint &_numPoints, const uint &_res);

    /// Drop all particle data (fluidsystem.cu:36-52)
    void clear();

    /// Place a lattice block of particles and set mass and particle size
    /// from it (fluidsystem.cu:66-127)
    void createFluidBlock(const uint & /*firstPtIdx*/,
                          const uint & /*numPoints*/,
                          const float &min_x, const float &min_y, const float &min_z,
                          const float &max_x, const float &max_y, const float &max_z);

private:
    sph_system *m_sys;
    FluidSystem(const FluidSystem &);
    FluidSystem &operator=(const FluidSystem &);
};

#endif // FLUIDSYSTEM_H
