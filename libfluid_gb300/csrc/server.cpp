// Served WCSPH step: a continuous-batching request loop (include/sph_c.h,
// sph_server_*).
//
// One host thread owns an Engine.  Each iteration it (1) admits queued
// requests in arrival order while the device-memory budget and the
// live-scene limit allow, creating their scenes on the GPU; (2) advances
// every live scene by one substep with one batched launch per pass; (3)
// copies finished scenes to the host and removes them, which frees arena
// slots for the queue.  Requests arriving meanwhile join at the next
// iteration, so their work overlaps on the device with the scenes already
// running.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/sph_c.h"
#include "engine.h"

using sph::Engine;
using sph::SceneConfig;

namespace {

struct Request {
    uint64_t id = 0;
    SceneConfig cfg;
    uint32_t n = 0, steps = 0, remaining = 0;
    std::vector<float> pos, vel;
    std::vector<LatticeSpec> blocks;
    int state = SPH_REQ_QUEUED;
    int scene = -1;
    uint64_t bytes = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    std::vector<float> out_pos, out_vel;
    std::string err;
};

bool to_config(const sph_params* p, SceneConfig& c, DevParams& dp, std::string* err) {
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
    return sph::derive_params(c, dp, err);
}

}  // namespace

struct sph_server {
    sph_server_config cfg{};
    std::unique_ptr<Engine> eng;
    std::thread th;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<Request*> live;
    uint64_t next_id = 1;
    bool stop = false;
    uint64_t used_bytes = 0;
    sph_server_stats st{};
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    std::string err;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    void loop();
    void fail_request(Request* r, const std::string& why) {
        r->state = SPH_REQ_FAILED;
        r->err = why;
        r->t_done = now();
        st.failed++;
    }
};

void sph_server::loop() {
    if (cfg.device >= 0) cudaSetDevice(cfg.device);
    const uint32_t per_iter = std::max<uint32_t>(1u, cfg.substeps_per_iteration);
    for (;;) {
        std::vector<Request*> admit;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stop || !queue.empty() || !live.empty(); });
            if (stop) return;
            while (!queue.empty()) {
                Request* r = queue.front();
                if (cfg.max_live_scenes && live.size() + admit.size() >= cfg.max_live_scenes) break;
                if (used_bytes + r->bytes > cfg.memory_budget) break;
                queue.pop_front();
                used_bytes += r->bytes;
                admit.push_back(r);
            }
        }
        // create admitted scenes (engine calls only on this thread)
        const double ta0 = now();
        for (size_t ai = 0; ai < admit.size(); ++ai) {
            Request* r = admit[ai];
            int rc = eng->add_scene(r->cfg, r->n, &r->scene);
            if (rc == sph::ENG_ENOMEM && !live.empty()) {
                // the arena is fragmented or full: wait for running scenes to leave
                std::lock_guard<std::mutex> lk(mu);
                st.admit_retries += admit.size() - ai;
                for (size_t b = admit.size(); b-- > ai;) {
                    used_bytes -= admit[b]->bytes;
                    queue.push_front(admit[b]);
                }
                break;
            }
            if (rc == sph::ENG_OK) {
                if (!r->pos.empty()) {
                    rc = eng->set_state(r->scene, r->pos.data(), r->vel.empty() ? nullptr : r->vel.data(), r->n);
                } else {
                    uint32_t first = 0;
                    for (const LatticeSpec& b : r->blocks) {
                        if (rc) break;
                        rc = eng->generate_lattice(r->scene, b, first);
                        first += b.nx * b.ny * b.nz;
                    }
                }
            }
            std::lock_guard<std::mutex> lk(mu);
            if (rc != sph::ENG_OK) {
                if (r->scene >= 0) eng->remove_scene(r->scene);
                used_bytes -= r->bytes;
                fail_request(r, eng->last_error());
                cv_done.notify_all();
                continue;
            }
            r->state = SPH_REQ_RUNNING;
            r->t_admit = now();
            st.admitted++;
            live.push_back(r);
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            st.admit_seconds += now() - ta0;
        }
        if (live.empty()) continue;
        uint32_t k = per_iter;
        for (Request* r : live) k = std::min(k, r->remaining);
        const double t1 = now();
        const int rc = eng->step(k, true);
        const double t2 = now();
        std::vector<Request*> finished;
        {
            std::lock_guard<std::mutex> lk(mu);
            st.busy_seconds += t2 - t1;
            st.iterations++;
            if (rc != sph::ENG_OK) {
                // a failed step leaves every live scene undefined
                for (Request* r : live) {
                    eng->remove_scene(r->scene);
                    used_bytes -= r->bytes;
                    fail_request(r, eng->last_error());
                }
                live.clear();
                cv_done.notify_all();
                continue;
            }
            uint64_t lp = 0;
            for (Request* r : live) {
                r->remaining -= k;
                st.particle_steps += (uint64_t)r->n * k;
                lp += r->n;
                if (r->remaining == 0) finished.push_back(r);
            }
            st.peak_live_particles = std::max(st.peak_live_particles, lp);
        }
        // Read every finished scene before removing any: the first read runs
        // the next substep's prefix (deferred XSPH) and the others reuse it.
        const double tr0 = now();
        std::vector<int> got(finished.size());
        for (size_t fi = 0; fi < finished.size(); ++fi) {
            Request* r = finished[fi];
            r->out_pos.resize((size_t)r->n * 3);
            r->out_vel.resize((size_t)r->n * 3);
            got[fi] = eng->get_state(r->scene, r->out_pos.data(), nullptr, r->out_vel.data(), r->n);
        }
        for (size_t fi = 0; fi < finished.size(); ++fi) {
            Request* r = finished[fi];
            const int g = got[fi];
            eng->remove_scene(r->scene);
            std::lock_guard<std::mutex> lk(mu);
            used_bytes -= r->bytes;
            if (g != sph::ENG_OK) {
                fail_request(r, eng->last_error());
            } else {
                r->state = SPH_REQ_DONE;
                r->t_done = now();
                st.completed++;
            }
            live.erase(std::find(live.begin(), live.end(), r));
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            st.read_seconds += now() - tr0;
            st.layout_seconds = eng->prep_seconds();
        }
        if (!finished.empty()) cv_done.notify_all();
    }
}

extern "C" {

int sph_server_create(sph_server** out, const sph_server_config* cfg) {
    if (!out || !cfg || cfg->memory_budget == 0) return SPH_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SPH_ECUDA;
    if (cfg->device >= ndev) return SPH_EINVAL;
    sph_server* s = new sph_server();
    s->cfg = *cfg;
    s->eng.reset(new Engine(cfg->device));
    if (s->cfg.device < 0) s->cfg.device = s->eng->device();
    // membership changes nearly every iteration: launch eagerly
    s->eng->set_use_graph(false);
    s->eng->set_byte_limit(cfg->memory_budget);
    // Cells for 1/16 of the budget up front: the cell count follows the live
    // scenes up and down, and regrowing the cell arrays near the budget
    // would reallocate them again and again (best effort: growth on demand
    // remains).
    s->eng->reserve(0, cfg->memory_budget / 16 / Engine::bytes_per_cell());
    s->th = std::thread([s] { s->loop(); });
    *out = s;
    return SPH_OK;
}

int sph_server_destroy(sph_server* s) {
    if (!s) return SPH_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->th.joinable()) s->th.join();
    delete s;
    return SPH_OK;
}

int sph_server_submit(sph_server* s, const sph_request* req, uint64_t* request_id) {
    if (!s || !req || req->n == 0) return SPH_EINVAL;
    std::unique_ptr<Request> r(new Request());
    DevParams dp;
    if (!to_config(&req->params, r->cfg, dp, &s->err)) return SPH_EINVAL;
    r->n = req->n;
    r->steps = r->remaining = req->steps;
    if (req->pos) {
        r->pos.assign(req->pos, req->pos + (size_t)req->n * 3);
        if (req->vel) r->vel.assign(req->vel, req->vel + (size_t)req->n * 3);
    } else {
        if (!req->blocks || req->num_blocks == 0) { s->err = "request has neither positions nor blocks"; return SPH_EINVAL; }
        uint64_t tot = 0;
        for (uint32_t b = 0; b < req->num_blocks; ++b) {
            LatticeSpec l;
            std::memcpy(&l, &req->blocks[b], sizeof(l));
            tot += (uint64_t)l.nx * l.ny * l.nz;
            r->blocks.push_back(l);
        }
        if (tot > req->n) { s->err = "lattice blocks exceed the particle count"; return SPH_EINVAL; }
    }
    r->bytes = (uint64_t)req->n * Engine::bytes_per_particle() + ((uint64_t)dp.ncells + 1) * 8ull +
               ((uint64_t)req->n / 64 + 1) * 16ull;
    std::lock_guard<std::mutex> lk(s->mu);
    s->st.submitted++;
    if (r->bytes > s->cfg.memory_budget) {
        s->st.rejected++;
        s->err = "request exceeds the memory budget";
        return SPH_EBUSY;
    }
    r->id = s->next_id++;
    r->t_submit = s->now();
    if (r->steps == 0) {
        r->state = SPH_REQ_DONE;
        r->t_admit = r->t_done = r->t_submit;
        r->out_pos = r->pos;
        r->out_vel = r->vel;
    } else {
        s->queue.push_back(r.get());
    }
    if (request_id) *request_id = r->id;
    s->reqs.emplace(r->id, std::move(r));
    s->cv_work.notify_all();
    return SPH_OK;
}

int sph_server_state(sph_server* s, uint64_t id) {
    if (!s) return SPH_REQ_UNKNOWN;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    return it == s->reqs.end() ? SPH_REQ_UNKNOWN : it->second->state;
}

int sph_server_wait(sph_server* s, uint64_t id, int64_t timeout_ms) {
    if (!s) return SPH_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return SPH_EINVAL;
    Request* r = it->second.get();
    auto ready = [&] { return r->state == SPH_REQ_DONE || r->state == SPH_REQ_FAILED; };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return SPH_ETIMEOUT;
    if (r->state == SPH_REQ_FAILED) { s->err = r->err; return SPH_ECUDA; }
    return SPH_OK;
}

int sph_server_fetch(sph_server* s, uint64_t id, float* pos, float* vel, uint32_t n) {
    if (!s) return SPH_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return SPH_EINVAL;
    Request* r = it->second.get();
    if (r->state != SPH_REQ_DONE) { s->err = "request not finished"; return SPH_EINVAL; }
    if (n < r->n) { s->err = "buffers too small"; return SPH_EINVAL; }
    if (pos && !r->out_pos.empty()) std::memcpy(pos, r->out_pos.data(), r->out_pos.size() * sizeof(float));
    if (vel && !r->out_vel.empty()) std::memcpy(vel, r->out_vel.data(), r->out_vel.size() * sizeof(float));
    s->reqs.erase(it);
    return SPH_OK;
}

int sph_server_times(sph_server* s, uint64_t id, double* t_submit, double* t_admit, double* t_done) {
    if (!s) return SPH_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return SPH_EINVAL;
    if (t_submit) *t_submit = it->second->t_submit;
    if (t_admit) *t_admit = it->second->t_admit;
    if (t_done) *t_done = it->second->t_done;
    return SPH_OK;
}

int sph_server_get_stats(sph_server* s, sph_server_stats* out) {
    if (!s || !out) return SPH_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->live_scenes = (uint32_t)s->live.size();
    out->queued = (uint32_t)s->queue.size();
    uint64_t lp = 0;
    for (const Request* r : s->live) lp += r->n;
    out->live_particles = lp;
    out->device_bytes = s->eng->device_bytes();
    return SPH_OK;
}

int sph_server_drain(sph_server* s, int64_t timeout_ms) {
    if (!s) return SPH_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto idle = [&] { return s->queue.empty() && s->live.empty(); };
    if (timeout_ms < 0) s->cv_done.wait(lk, idle);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle)) return SPH_ETIMEOUT;
    return SPH_OK;
}

const char* sph_server_last_error(sph_server* s) { return s ? s->err.c_str() : "null handle"; }

}  // extern "C"
