// C ABI of the batched step (include/sph_c.h, sph_batch_*): many independent
// scenes in one Engine, every pass one launch over all of them.
#include <cstring>
#include <memory>
#include <string>

#include "../../include/sph_c.h"
#include "engine.h"
#include "snapshot_fmt.h"

using sph::Engine;
using sph::SceneConfig;

struct sph_batch {
    std::unique_ptr<Engine> eng;
    std::string err;
};

namespace {

int berr(sph_batch* b, int code) {
    if (code && b && b->eng) b->err = b->eng->last_error();
    return code;
}

bool to_config(const sph_params* p, SceneConfig& c, std::string* err) {
    c = SceneConfig();
    c.box_mode = (int)p->box_mode;
    c.res = p->res;
    c.lx = p->lx; c.ly = p->ly; c.lz = p->lz; c.h = p->h;
    c.rest_density = p->rest_density; c.gas_constant = p->gas_constant; c.gamma = p->gamma;
    c.mass = p->mass; c.particle_size = p->particle_size;
    c.xsph = p->xsph; c.surface_tension = p->surface_tension; c.viscosity = p->viscosity;
    c.adhesion = p->adhesion; c.vdamp = p->vdamp;
    c.vel_limit = p->vel_limit; c.acc_limit = p->acc_limit; c.dt = p->dt;
    c.gravity[0] = p->gravity[0]; c.gravity[1] = p->gravity[1]; c.gravity[2] = p->gravity[2];
    DevParams dp;
    return sph::derive_params(c, dp, err);
}

void from_config(const SceneConfig& c, sph_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->box_mode = (uint32_t)c.box_mode;
    p->res = c.res;
    p->lx = c.lx; p->ly = c.ly; p->lz = c.lz; p->h = c.h;
    p->rest_density = c.rest_density; p->gas_constant = c.gas_constant; p->gamma = c.gamma;
    p->mass = c.mass; p->particle_size = c.particle_size;
    p->xsph = c.xsph; p->surface_tension = c.surface_tension; p->viscosity = c.viscosity;
    p->adhesion = c.adhesion; p->vdamp = c.vdamp;
    p->vel_limit = c.vel_limit; p->acc_limit = c.acc_limit; p->dt = c.dt;
    p->gravity[0] = c.gravity[0]; p->gravity[1] = c.gravity[1]; p->gravity[2] = c.gravity[2];
}

}  // namespace

extern "C" {

int sph_batch_create(sph_batch** out, int device) {
    if (!out) return SPH_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SPH_ECUDA;
    if (device >= ndev) return SPH_EINVAL;
    sph_batch* b = new sph_batch();
    b->eng.reset(new Engine(device));
    *out = b;
    return SPH_OK;
}

int sph_batch_destroy(sph_batch* b) {
    delete b;
    return SPH_OK;
}

int sph_batch_add_scene(sph_batch* b, const sph_params* p, uint32_t n, int* scene_id) {
    if (!b || !p || !scene_id) return SPH_EINVAL;
    SceneConfig c;
    if (!to_config(p, c, &b->err)) return SPH_EINVAL;
    int rc = b->eng->add_scene(c, n, scene_id);
    if (rc) return berr(b, rc);
    return SPH_OK;
}

int sph_batch_remove_scene(sph_batch* b, int scene_id) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->remove_scene(scene_id));
}

int sph_batch_set_params(sph_batch* b, int scene_id, const sph_params* p) {
    if (!b || !p) return SPH_EINVAL;
    SceneConfig c;
    if (!to_config(p, c, &b->err)) return SPH_EINVAL;
    if (const sph::Scene* sc = b->eng->scene(scene_id)) c.boundary = sc->cfg.boundary;
    return berr(b, b->eng->set_config(scene_id, c));
}

int sph_batch_set_boundary(sph_batch* b, int scene_id, int shape) {
    if (!b) return SPH_EINVAL;
    const sph::Scene* sc = b->eng->scene(scene_id);
    if (!sc) { b->err = "unknown scene id"; return SPH_EINVAL; }
    if (shape != SPH_BOUNDARY_BOX && shape != SPH_BOUNDARY_SPHERE) {
        b->err = "boundary must be SPH_BOUNDARY_BOX or SPH_BOUNDARY_SPHERE";
        return SPH_EINVAL;
    }
    SceneConfig c = sc->cfg;
    c.boundary = shape;
    return berr(b, b->eng->set_config(scene_id, c));
}

int sph_batch_set_state(sph_batch* b, int scene_id, const float* pos, const float* vel, uint32_t n) {
    if (!b || !pos) return SPH_EINVAL;
    return berr(b, b->eng->set_state(scene_id, pos, vel, n));
}

int sph_batch_generate_lattice(sph_batch* b, int scene_id, const sph_lattice* spec, uint32_t first) {
    if (!b || !spec) return SPH_EINVAL;
    static_assert(sizeof(sph_lattice) == sizeof(LatticeSpec), "lattice layout");
    LatticeSpec s;
    std::memcpy(&s, spec, sizeof(s));
    return berr(b, b->eng->generate_lattice(scene_id, s, first));
}

int sph_batch_step(sph_batch* b, uint32_t substeps) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->step(substeps, true));
}
int sph_batch_step_async(sph_batch* b, uint32_t substeps) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->step(substeps, false));
}
int sph_batch_sync(sph_batch* b) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->sync());
}

int sph_batch_get_state(sph_batch* b, int scene_id, float* pos, float* colour, float* vel, uint32_t n) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->get_state(scene_id, pos, colour, vel, n));
}

int sph_batch_snapshot(sph_batch* b, int scene_id, void* buf, uint64_t cap, uint64_t* written) {
    if (!b || !buf) return SPH_EINVAL;
    const sph::Scene* sc = b->eng->scene(scene_id);
    if (!sc) { b->err = "unknown scene id"; return SPH_EINVAL; }
    const uint64_t need = sph::snapshot_total_bytes(sc->n);
    if (cap < need) { b->err = "snapshot buffer smaller than sph_snapshot_bytes(n)"; return SPH_EINVAL; }
    sph_params p;
    from_config(sc->cfg, &p);
    sph_snapshot_header h;
    sph::snapshot_make_header(h, sc->n, p);
    h.reserved[0] = (uint32_t)sc->cfg.boundary;
    std::memcpy(buf, &h, sizeof(h));
    float4* body = reinterpret_cast<float4*>(static_cast<char*>(buf) + sizeof(h));
    int rc = berr(b, b->eng->save_state(scene_id, body, sc->n));
    if (rc == SPH_OK && written) *written = need;
    return rc;
}

int sph_batch_restore(sph_batch* b, int scene_id, const void* buf, uint64_t bytes) {
    if (!b || !buf) return SPH_EINVAL;
    const sph::Scene* sc = b->eng->scene(scene_id);
    if (!sc) { b->err = "unknown scene id"; return SPH_EINVAL; }
    sph_snapshot_header h;
    if (!sph::snapshot_parse(buf, bytes, &h, &b->err)) return SPH_EINVAL;
    if (h.n != sc->n) { b->err = "snapshot particle count differs from the scene's"; return SPH_EINVAL; }
    int rc = sph_batch_set_boundary(b, scene_id, (int)h.reserved[0]);
    if (rc) return rc;
    rc = sph_batch_set_params(b, scene_id, &h.params);
    if (rc) return rc;
    const float4* body = reinterpret_cast<const float4*>(static_cast<const char*>(buf) + sizeof(h));
    return berr(b, b->eng->load_state(scene_id, body, h.n));
}

uint32_t sph_batch_num_scenes(const sph_batch* b) { return b ? (uint32_t)b->eng->num_scenes() : 0; }
uint64_t sph_batch_num_particles(const sph_batch* b) { return b ? b->eng->total_particles() : 0; }

int sph_batch_debug_enable(sph_batch* b, int on) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->debug_enable(on != 0));
}
int sph_batch_debug_get(sph_batch* b, int scene_id, int field, void* buf, uint64_t count) {
    if (!b || !buf) return SPH_EINVAL;
    return berr(b, b->eng->debug_get(scene_id, field, buf, count));
}
int sph_batch_set_use_graph(sph_batch* b, int on) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->set_use_graph(on != 0));
}
int sph_batch_set_deferred_xsph(sph_batch* b, int on) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->set_deferred_xsph(on != 0));
}
int sph_batch_set_exec(sph_batch* b, const sph_exec_config* e) {
    if (!b || !e) return SPH_EINVAL;
    sph::ExecConfig x;
    x.tile = e->tile;
    x.persistent = e->persistent;
    x.skin = e->skin;
    x.variant = e->variant;
    return berr(b, b->eng->set_exec(x));
}
int sph_batch_set_profiling(sph_batch* b, int on) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->set_profiling(on != 0));
}
int sph_batch_get_pass_times(sph_batch* b, double* ms, int cap, uint64_t* substeps) {
    if (!b || !ms) return SPH_EINVAL;
    return berr(b, b->eng->get_pass_times(ms, cap, substeps));
}
int sph_batch_timer_mark(sph_batch* b, int slot) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->timer_mark(slot));
}
int sph_batch_timer_elapsed(sph_batch* b, int a, int b2, float* ms) {
    if (!b) return SPH_EINVAL;
    return berr(b, b->eng->timer_elapsed(a, b2, ms));
}
const char* sph_batch_last_error(const sph_batch* b) { return b ? b->err.c_str() : "null handle"; }

}  // extern "C"
