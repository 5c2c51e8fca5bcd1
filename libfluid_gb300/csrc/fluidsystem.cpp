// C++ FluidSystem drop-in (include/fluidsystem.h) over the C ABI.
// Errors are reported on stderr; nothing here exits the process (the
// reference calls exit(0) on CUDA errors, fluidsystem.cu:253-258).
#include "fluidsystem.h"

#include <iostream>

#include "sph_c.h"

namespace {
void report(const sph_system* s, int rc, const char* what) {
    if (rc != SPH_OK)
        std::cerr << "FluidSystem::" << what << " failed (" << rc << "): " << sph_last_error(s) << "\n";
}
}  // namespace

FluidSystem::FluidSystem() : m_isInit(false), m_sys(nullptr) {
    const int rc = sph_create(&m_sys, -1);
    if (rc != SPH_OK) std::cerr << "FluidSystem: no CUDA device available (" << rc << ")\n";
}

FluidSystem::~FluidSystem() {
    clear();
    if (m_sys) sph_destroy(m_sys);
}

void FluidSystem::clear() {
    if (m_sys) report(m_sys, sph_clear(m_sys), "clear");
}

void FluidSystem::init(const uint& _numPoints, const uint& _res) {
    if (!m_sys) return;
    const int rc = sph_init(m_sys, _numPoints, _res);
    report(m_sys, rc, "init");
    if (rc == SPH_OK) m_isInit = true;
}

void FluidSystem::createFluidBlock(const uint& firstPtIdx, const uint& numPoints, const float& min_x,
                                   const float& min_y, const float& min_z, const float& max_x, const float& max_y,
                                   const float& max_z) {
    if (!m_sys) return;
    report(m_sys, sph_create_block(m_sys, firstPtIdx, numPoints, min_x, min_y, min_z, max_x, max_y, max_z),
           "createFluidBlock");
}

void FluidSystem::setup(const uint& _numPoints, const uint& _res) {
    // fluidsystem.cu:132-147
    init(_numPoints, _res);
    setAdhesion(0.0f);
    setViscosity(0.0f);
    setSurfaceTension(0.0f);
    setVDamp(0.5f);
    createFluidBlock(0, _numPoints, 0.1f, 0.1f, 0.1f, 0.9f, 0.9f, 0.9f);
}

void FluidSystem::setupFromData(const std::vector<float3>& points, const std::vector<float3>& velocity,
                                const uint& _res) {
    init((uint)points.size(), _res);
    if (!m_sys || points.empty()) return;
    // velocities beyond the given ones stay zero, as after init
    const float3 zero = {0.f, 0.f, 0.f};
    std::vector<float3> vel(points.size(), zero);
    for (size_t i = 0; i < vel.size() && i < velocity.size(); ++i) vel[i] = velocity[i];
    report(m_sys, sph_set_state(m_sys, &points[0].x, &vel[0].x, (uint32_t)points.size()), "setupFromData");
}

void FluidSystem::exportToData(std::vector<float3>& points, std::vector<float3>& colour,
                               std::vector<float3>& velocity) {
    if (!m_sys) return;
    const uint32_t n = sph_num_particles(m_sys);
    if (points.size() < n) points.resize(n);
    if (colour.size() < n) colour.resize(n);
    if (velocity.size() < n) velocity.resize(n);
    if (n == 0) return;
    report(m_sys, sph_export(m_sys, &points[0].x, &colour[0].x, &velocity[0].x, n), "exportToData");
}

float FluidSystem::getPscale() const {
    float v = 0.f;
    if (m_sys) sph_get_pscale(m_sys, &v);
    return v;
}

void FluidSystem::advance(const float& dt, const uint& substeps) {
    if (!m_isInit || !m_sys) return;   // fluidsystem.cu:276-277
    report(m_sys, sph_advance(m_sys, dt, substeps, nullptr), "advance");
}

#define FS_SETTER(method, cfn)                                  \
    void FluidSystem::method(const float& v) {                  \
        if (m_sys) report(m_sys, cfn(m_sys, v), #method);       \
    }
FS_SETTER(setRestDensity, sph_set_rest_density)
FS_SETTER(setParticleSize, sph_set_particle_size)
FS_SETTER(setGasConstant, sph_set_gas_constant)
FS_SETTER(setXSPHScale, sph_set_xsph_scale)
FS_SETTER(setSurfaceTension, sph_set_surface_tension)
FS_SETTER(setViscosity, sph_set_viscosity)
FS_SETTER(setAdhesion, sph_set_adhesion)
FS_SETTER(setVDamp, sph_set_vdamp)
FS_SETTER(setGamma, sph_set_gamma)
FS_SETTER(setMass, sph_set_mass)

void FluidSystem::setLimits(const float& velLimit, const float& accLimit) {
    if (m_sys) report(m_sys, sph_set_limits(m_sys, velLimit, accLimit), "setLimits");
}
