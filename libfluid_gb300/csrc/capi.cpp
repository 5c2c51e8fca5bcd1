// C ABI of the plain WCSPH step (include/sph_c.h): a FluidSystem
// (libfluid/cudasrc/fluidsystem.cu) over an Engine with one scene.
#include "../../include/sph_c.h"

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"
#include "snapshot_fmt.h"

using sph::Engine;
using sph::SceneConfig;

struct sph_system {
    std::unique_ptr<Engine> eng;
    SceneConfig cfg;        // the FluidParams host copy (fluidparams.cuh:140)
    bool is_init = false;   // FluidSystem::m_isInit
    int scene = -1;
    uint32_t n = 0;
    std::string err;
};

namespace {

int set_err(sph_system* s, int code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}
int eng_err(sph_system* s, int code) {
    if (code && s && s->eng) s->err = s->eng->last_error();
    return code;
}

// FluidParams constructor defaults (fluidparams.cuh:81-97, fluidparams.cu:11-49).
void ctor_defaults(SceneConfig& c) {
    c = SceneConfig();
    c.box_mode = 0;
    c.res = 1;
    c.rest_density = 1.0f;     // DEFAULT_REST_DENSITY
    c.gas_constant = 1.0f;     // DEFAULT_GAS_CONSTANT
    c.gamma = 1.0f;
    c.mass = 1.0f;
    c.xsph = 0.5f;
    c.surface_tension = 1.0f;  // DEFAULT_SURFACE_TENSION_FORCE
    c.viscosity = 0.1f;        // DEFAULT_VISCOSITY_FORCE
    c.adhesion = 1.0f;         // DEFAULT_ADHESION_FORCE
    c.vel_limit = 5.0f;
    c.acc_limit = 150.0f;
    c.vdamp = 1.0f;
    c.particle_size = 1.0f;
    c.dt = 0.01f;              // DEFAULT_TIMESTEP
    c.gravity[0] = 0.0f; c.gravity[1] = -9.8f; c.gravity[2] = 0.0f;
}

// Push the host parameter copy to the scene (the FluidParams dirty flag;
// the device copy is refreshed before the next substep).
int push_cfg(sph_system* s) {
    if (!s->is_init || s->scene < 0) return SPH_OK;
    return eng_err(s, s->eng->set_config(s->scene, s->cfg));
}

// createFluidBlock placement and parameter side effects (fluidsystem.cu:66-127).
void block_points(const SceneConfig& cfg, uint32_t n, float mnx, float mny, float mnz, float mxx, float mxy,
                  float mxz, std::vector<float>& pts, float* mass, float* psize) {
    const float dx = mxx - mnx, dy = mxy - mny, dz = mxz - mnz;
    const float volume = dx * dy * dz;
    const float part_volume = volume / float(n);
    const float approx = std::cbrt(part_volume);
    const float rx = dx / approx + 0.5f, ry = dy / approx + 0.5f, rz = dz / approx + 0.5f;
    const float diam = std::fmin(std::fmin(dx / rx, dy / ry), dz / rz);
    *mass = part_volume * cfg.rest_density;
    *psize = diam * 0.5f;
    pts.clear();
    uint32_t cnt = 0;
    float px, py, pz;
    for (px = mnx + 0.5f * diam; px <= mxx; px += diam)
        for (py = mny + 0.5f * diam; py <= mxy; py += diam)
            for (pz = mnz + 0.5f * diam; pz <= mxz; pz += diam)
                if (cnt < n) {
                    pts.push_back(px); pts.push_back(py); pts.push_back(pz);
                    cnt++;
                }
}

}  // namespace

extern "C" {

int64_t sph_substep_count(float full_dt, uint32_t substeps) {
    // fluidsystem.cu:294-301: for (dt = part_dt; dt <= full_dt; dt += part_dt)
    volatile float part = full_dt / float(substeps);
    volatile float dt = part;
    int64_t cnt = 0;
    while (dt <= full_dt) {
        cnt++;
        volatile float nx = dt + part;
        if (nx == dt) return -1;   // the reference loop would never end
        dt = nx;
        if (cnt > ((int64_t)1 << 40)) return -1;
    }
    return cnt;
}

int sph_create(sph_system** out, int device) {
    if (!out) return SPH_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SPH_ECUDA;
    if (device >= ndev) return SPH_EINVAL;
    sph_system* s = new sph_system();
    s->eng.reset(new Engine(device));
    ctor_defaults(s->cfg);
    *out = s;
    return SPH_OK;
}

int sph_destroy(sph_system* s) {
    delete s;
    return SPH_OK;
}

int sph_clear(sph_system* s) {
    if (!s) return SPH_EINVAL;
    if (s->scene >= 0) s->eng->remove_scene(s->scene);
    s->scene = -1;
    s->n = 0;
    return SPH_OK;
}

int sph_init(sph_system* s, uint32_t num_points, uint32_t res) {
    if (!s) return SPH_EINVAL;
    sph_clear(s);
    // fluidparams.cu:53-54: res == 0 keeps the current grid
    if (res != 0) { s->cfg.box_mode = 0; s->cfg.res = res; }
    // fluidsystem.cu:210-235
    s->cfg.gas_constant = 100.0f;
    s->cfg.vdamp = 0.0f;
    s->cfg.gamma = 7.0f;
    s->cfg.vel_limit = 5.0f;
    s->cfg.acc_limit = 150.0f;
    s->cfg.dt = 1.0f;
    s->cfg.xsph = 0.5f;
    s->cfg.particle_size = 1.0f;
    s->cfg.rest_density = 1000.0f;
    s->cfg.mass = 1.0f;
    s->n = num_points;
    if (num_points) {
        int rc = s->eng->add_scene(s->cfg, num_points, &s->scene);
        if (rc) { s->scene = -1; s->n = 0; return eng_err(s, rc); }
        std::vector<float> zero((size_t)num_points * 3, 0.0f);
        rc = s->eng->set_state(s->scene, zero.data(), zero.data(), num_points);
        if (rc) return eng_err(s, rc);
    }
    s->is_init = true;
    return SPH_OK;
}

int sph_create_block(sph_system* s, uint32_t first, uint32_t n, float min_x, float min_y, float min_z, float max_x,
                     float max_y, float max_z) {
    if (!s) return SPH_EINVAL;
    if ((uint64_t)first + n > s->n)
        return set_err(s, SPH_EINVAL, "createFluidBlock: not enough space for the requested points");
    if (n == 0) return SPH_OK;
    std::vector<float> pts;
    float mass = 0.f, psize = 0.f;
    block_points(s->cfg, n, min_x, min_y, min_z, max_x, max_y, max_z, pts, &mass, &psize);
    s->cfg.mass = mass;
    s->cfg.particle_size = psize;
    int rc = push_cfg(s);
    if (rc) return rc;
    if (s->scene >= 0 && !pts.empty())
        return eng_err(s, s->eng->set_positions(s->scene, first, pts.data(), (uint32_t)(pts.size() / 3)));
    return SPH_OK;
}

int sph_setup(sph_system* s, uint32_t num_points, uint32_t res) {
    int rc = sph_init(s, num_points, res);
    if (rc) return rc;
    // fluidsystem.cu:137-146
    s->cfg.adhesion = 0.0f;
    s->cfg.viscosity = 0.0f;
    s->cfg.surface_tension = 0.0f;
    s->cfg.vdamp = 0.5f;
    rc = push_cfg(s);
    if (rc) return rc;
    return sph_create_block(s, 0, num_points, 0.1f, 0.1f, 0.1f, 0.9f, 0.9f, 0.9f);
}

int sph_set_state(sph_system* s, const float* pos, const float* vel, uint32_t n) {
    if (!s || !pos) return SPH_EINVAL;
    if (!s->is_init) return set_err(s, SPH_ENOTINIT, "system is not initialised");
    if (n != s->n) return set_err(s, SPH_EINVAL, "particle count mismatch");
    if (n == 0) return SPH_OK;
    return eng_err(s, s->eng->set_state(s->scene, pos, vel, n));
}

int sph_setup_from_data(sph_system* s, const float* pos, const float* vel, uint32_t n, uint32_t res) {
    int rc = sph_init(s, n, res);
    if (rc) return rc;
    if (n == 0) return SPH_OK;
    return sph_set_state(s, pos, vel, n);
}

static int advance_impl(sph_system* s, float full_dt, uint32_t substeps, uint32_t* executed, bool sync) {
    if (executed) *executed = 0;
    if (!s) return SPH_EINVAL;
    if (!s->is_init) return set_err(s, SPH_ENOTINIT, "advance before init");
    const int64_t cnt = sph_substep_count(full_dt, substeps);
    if (cnt < 0) return set_err(s, SPH_EINVAL, "the substep loop of advance() would not terminate for these arguments");
    if (cnt > 0xFFFFFFFFll) return set_err(s, SPH_EINVAL, "too many substeps");
    // fluidsystem.cu:295-299
    s->cfg.dt = full_dt / float(substeps);
    int rc = push_cfg(s);
    if (rc) return rc;
    if (s->scene < 0 || cnt == 0) return SPH_OK;
    rc = s->eng->step((uint32_t)cnt, sync);
    if (executed) *executed = (uint32_t)cnt;
    return eng_err(s, rc);
}

int sph_advance(sph_system* s, float full_dt, uint32_t substeps, uint32_t* executed) {
    return advance_impl(s, full_dt, substeps, executed, true);
}
int sph_advance_async(sph_system* s, float full_dt, uint32_t substeps, uint32_t* executed) {
    return advance_impl(s, full_dt, substeps, executed, false);
}
int sph_sync(sph_system* s) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->sync());
}

int sph_export(sph_system* s, float* pos, float* colour, float* vel, uint32_t n) {
    if (!s) return SPH_EINVAL;
    if (!s->is_init) return set_err(s, SPH_ENOTINIT, "export before init");
    if (n < s->n) return set_err(s, SPH_EINVAL, "export buffers hold fewer than num_particles entries");
    if (s->n == 0) return SPH_OK;
    return eng_err(s, s->eng->get_state(s->scene, pos, colour, vel, s->n));
}

int sph_get_pscale(const sph_system* s, float* out) {
    if (!s || !out) return SPH_EINVAL;
    *out = s->cfg.particle_size;
    return SPH_OK;
}
uint32_t sph_num_particles(const sph_system* s) { return s ? s->n : 0; }
int sph_is_init(const sph_system* s) { return (s && s->is_init) ? 1 : 0; }

uint64_t sph_snapshot_bytes(uint32_t n) { return sph::snapshot_total_bytes(n); }

int sph_snapshot(sph_system* s, void* buf, uint64_t cap, uint64_t* written) {
    if (!s || !buf) return SPH_EINVAL;
    if (!s->is_init) return set_err(s, SPH_ENOTINIT, "snapshot before init");
    const uint64_t need = sph::snapshot_total_bytes(s->n);
    if (cap < need) return set_err(s, SPH_EINVAL, "snapshot buffer smaller than sph_snapshot_bytes(n)");
    sph_params p;
    sph_get_params(s, &p);
    sph_snapshot_header h;
    sph::snapshot_make_header(h, s->n, p);
    h.reserved[0] = (uint32_t)s->cfg.boundary;
    std::memcpy(buf, &h, sizeof(h));
    float4* body = reinterpret_cast<float4*>(static_cast<char*>(buf) + sizeof(h));
    int rc = eng_err(s, s->eng->save_state(s->scene, body, s->n));
    if (rc == SPH_OK && written) *written = need;
    return rc;
}

int sph_restore(sph_system* s, const void* buf, uint64_t bytes) {
    if (!s || !buf) return SPH_EINVAL;
    if (!s->is_init) return set_err(s, SPH_ENOTINIT, "restore before init");
    sph_snapshot_header h;
    std::string why;
    if (!sph::snapshot_parse(buf, bytes, &h, &why)) return set_err(s, SPH_EINVAL, why);
    if (h.n != s->n) return set_err(s, SPH_EINVAL, "snapshot particle count differs from the system's");
    s->cfg.boundary = (int)h.reserved[0];
    int rc = sph_set_params(s, &h.params);
    if (rc) return rc;
    const float4* body = reinterpret_cast<const float4*>(static_cast<const char*>(buf) + sizeof(h));
    return eng_err(s, s->eng->load_state(s->scene, body, s->n));
}

#define SPH_SETTER(name, field)                     \
    int name(sph_system* s, float v) {              \
        if (!s) return SPH_EINVAL;                  \
        s->cfg.field = v;                           \
        return push_cfg(s);                         \
    }
SPH_SETTER(sph_set_rest_density, rest_density)
SPH_SETTER(sph_set_particle_size, particle_size)
SPH_SETTER(sph_set_gas_constant, gas_constant)
SPH_SETTER(sph_set_xsph_scale, xsph)
SPH_SETTER(sph_set_surface_tension, surface_tension)
SPH_SETTER(sph_set_viscosity, viscosity)
SPH_SETTER(sph_set_adhesion, adhesion)
SPH_SETTER(sph_set_vdamp, vdamp)
SPH_SETTER(sph_set_gamma, gamma)
SPH_SETTER(sph_set_mass, mass)

int sph_set_limits(sph_system* s, float vel_limit, float acc_limit) {
    if (!s) return SPH_EINVAL;
    s->cfg.vel_limit = vel_limit;
    s->cfg.acc_limit = acc_limit;
    return push_cfg(s);
}
int sph_set_gravity(sph_system* s, float gx, float gy, float gz) {
    if (!s) return SPH_EINVAL;
    s->cfg.gravity[0] = gx; s->cfg.gravity[1] = gy; s->cfg.gravity[2] = gz;
    return push_cfg(s);
}
int sph_set_domain(sph_system* s, float lx, float ly, float lz, float h) {
    if (!s) return SPH_EINVAL;
    SceneConfig c = s->cfg;
    c.box_mode = 1;
    c.lx = lx; c.ly = ly; c.lz = lz; c.h = h;
    DevParams dp;
    std::string e;
    if (!sph::derive_params(c, dp, &e)) return set_err(s, SPH_EINVAL, e);
    s->cfg = c;
    return push_cfg(s);
}

int sph_get_params(const sph_system* s, sph_params* o) {
    if (!s || !o) return SPH_EINVAL;
    const SceneConfig& c = s->cfg;
    o->box_mode = (uint32_t)c.box_mode;
    o->res = c.res;
    o->lx = c.lx; o->ly = c.ly; o->lz = c.lz; o->h = c.h;
    o->rest_density = c.rest_density; o->gas_constant = c.gas_constant; o->gamma = c.gamma;
    o->mass = c.mass; o->particle_size = c.particle_size;
    o->xsph = c.xsph; o->surface_tension = c.surface_tension; o->viscosity = c.viscosity;
    o->adhesion = c.adhesion; o->vdamp = c.vdamp;
    o->vel_limit = c.vel_limit; o->acc_limit = c.acc_limit; o->dt = c.dt;
    o->gravity[0] = c.gravity[0]; o->gravity[1] = c.gravity[1]; o->gravity[2] = c.gravity[2];
    return SPH_OK;
}

int sph_set_params(sph_system* s, const sph_params* o) {
    if (!s || !o) return SPH_EINVAL;
    SceneConfig c;
    c.box_mode = (int)o->box_mode;
    c.res = o->res;
    c.lx = o->lx; c.ly = o->ly; c.lz = o->lz; c.h = o->h;
    c.rest_density = o->rest_density; c.gas_constant = o->gas_constant; c.gamma = o->gamma;
    c.mass = o->mass; c.particle_size = o->particle_size;
    c.xsph = o->xsph; c.surface_tension = o->surface_tension; c.viscosity = o->viscosity;
    c.adhesion = o->adhesion; c.vdamp = o->vdamp;
    c.vel_limit = o->vel_limit; c.acc_limit = o->acc_limit; c.dt = o->dt;
    c.gravity[0] = o->gravity[0]; c.gravity[1] = o->gravity[1]; c.gravity[2] = o->gravity[2];
    c.boundary = s->cfg.boundary;   // not part of sph_params: sph_set_boundary
    DevParams dp;
    std::string e;
    if (!sph::derive_params(c, dp, &e)) return set_err(s, SPH_EINVAL, e);
    s->cfg = c;
    return push_cfg(s);
}

int sph_set_boundary(sph_system* s, int shape) {
    if (!s) return SPH_EINVAL;
    if (shape != SPH_BOUNDARY_BOX && shape != SPH_BOUNDARY_SPHERE)
        return set_err(s, SPH_EINVAL, "boundary must be SPH_BOUNDARY_BOX or SPH_BOUNDARY_SPHERE");
    s->cfg.boundary = shape;
    return push_cfg(s);
}
int sph_get_boundary(const sph_system* s, int* shape) {
    if (!s || !shape) return SPH_EINVAL;
    *shape = s->cfg.boundary;
    return SPH_OK;
}

static int derived_values(const SceneConfig& cfg, double* out, int cap);

int sph_get_derived(const sph_system* s, double* out, int cap) {
    if (!s || !out) return 0;
    return derived_values(s->cfg, out, cap);
}

int sph_derive_params(const sph_params* o, double* out, int cap) {
    if (!o || !out) return 0;
    SceneConfig c;
    c.box_mode = (int)o->box_mode;
    c.res = o->res;
    c.lx = o->lx; c.ly = o->ly; c.lz = o->lz; c.h = o->h;
    c.rest_density = o->rest_density; c.gas_constant = o->gas_constant; c.gamma = o->gamma;
    c.mass = o->mass; c.particle_size = o->particle_size;
    c.xsph = o->xsph; c.surface_tension = o->surface_tension; c.viscosity = o->viscosity;
    c.adhesion = o->adhesion; c.vdamp = o->vdamp;
    c.vel_limit = o->vel_limit; c.acc_limit = o->acc_limit; c.dt = o->dt;
    c.gravity[0] = o->gravity[0]; c.gravity[1] = o->gravity[1]; c.gravity[2] = o->gravity[2];
    return derived_values(c, out, cap);
}

static int derived_values(const SceneConfig& cfg, double* out, int cap) {
    DevParams p;
    if (!sph::derive_params(cfg, p, nullptr)) return 0;
    const double v[] = {double(p.gx), double(p.gy), double(p.gz), double(p.inv_cell), double(p.h), double(p.h2),
                        double(p.poly6), double(p.grad_poly6), double(p.grad_spiky), double(p.cohesion),
                        double(p.invh9), double(p.rest_density), double(p.gas_constant), double(p.gamma),
                        double(p.mass), double(p.particle_size), double(p.dt), double(p.xsph),
                        double(p.surface_tension), double(p.viscosity), double(p.adhesion), double(p.vdamp),
                        double(p.vel_limit), double(p.acc_limit), double(p.grav_x), double(p.grav_y),
                        double(p.grav_z), double(p.eps)};
    int k = 0;
    for (; k < cap && k < (int)(sizeof(v) / sizeof(v[0])); ++k) out[k] = v[k];
    return k;
}

int sph_debug_enable(sph_system* s, int on) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->debug_enable(on != 0));
}
int sph_debug_get(sph_system* s, int field, void* buf, uint64_t count) {
    if (!s || !buf) return SPH_EINVAL;
    if (!s->is_init || s->scene < 0) return set_err(s, SPH_ENOTINIT, "no particles");
    return eng_err(s, s->eng->debug_get(s->scene, field, buf, count));
}
int sph_debug_scan_fault(sph_system* s, uint32_t spin_limit, int withhold_first_tile) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->set_scan_fault(spin_limit, withhold_first_tile != 0));
}
int sph_set_use_graph(sph_system* s, int on) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->set_use_graph(on != 0));
}
int sph_set_export_ahead(sph_system* s, int on) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->set_export_ahead(on != 0));
}
int sph_export_ahead_stats(const sph_system* s, uint64_t* out) {
    if (!s || !out || !s->eng) return SPH_EINVAL;
    s->eng->export_ahead_stats(out);
    return SPH_OK;
}
int sph_set_deferred_xsph(sph_system* s, int on) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->set_deferred_xsph(on != 0));
}
int sph_set_exec(sph_system* s, const sph_exec_config* e) {
    if (!s || !e) return SPH_EINVAL;
    sph::ExecConfig x;
    x.tile = e->tile;
    x.persistent = e->persistent;
    x.skin = e->skin;
    x.variant = e->variant;
    return eng_err(s, s->eng->set_exec(x));
}
int sph_get_exec(const sph_system* s, sph_exec_config* e) {
    if (!s || !e) return SPH_EINVAL;
    const sph::ExecConfig& x = s->eng->exec();
    e->tile = x.tile;
    e->persistent = x.persistent;
    e->skin = x.skin;
    e->variant = x.variant;
    return SPH_OK;
}
int sph_set_profiling(sph_system* s, int on) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->set_profiling(on != 0));
}
int sph_get_pass_times(sph_system* s, double* ms, int cap, uint64_t* substeps) {
    if (!s || !ms) return SPH_EINVAL;
    return eng_err(s, s->eng->get_pass_times(ms, cap, substeps));
}
const char* sph_pass_name(int i) { return Engine::pass_name(i); }
int sph_host_register(void* ptr, uint64_t bytes) {
    if (!ptr || bytes == 0) return SPH_EINVAL;
    return cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault) == cudaSuccess ? SPH_OK : SPH_ECUDA;
}
int sph_host_unregister(void* ptr) {
    if (!ptr) return SPH_EINVAL;
    return cudaHostUnregister(ptr) == cudaSuccess ? SPH_OK : SPH_ECUDA;
}
int sph_timer_mark(sph_system* s, int slot) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->timer_mark(slot));
}
int sph_timer_elapsed(sph_system* s, int a, int b, float* ms) {
    if (!s) return SPH_EINVAL;
    return eng_err(s, s->eng->timer_elapsed(a, b, ms));
}
const char* sph_last_error(const sph_system* s) { return s ? s->err.c_str() : "null handle"; }
const char* sph_version(void) { return "libsph_gb300 1.0 (sm_103a)"; }

}  // extern "C"
